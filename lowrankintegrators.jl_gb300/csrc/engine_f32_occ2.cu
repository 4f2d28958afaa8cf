// engine_f32_occ2.cu - float instance engine sized for 2 CTAs per SM (up to
// 128 registers per thread), the autotuner's alternative to the default 3
// (own translation unit so it compiles in parallel with the others).
#include "engine_impl.cuh"

namespace lri {
template cudaError_t launch_step_occ<float, 2>(const StepArgs<float>&, int, cudaStream_t);
}  // namespace lri
