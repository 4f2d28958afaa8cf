// engine_f32.cu - float instantiation of the instance engine (one translation
// unit per precision so the two compile in parallel).
#include "engine_impl.cuh"

namespace lri {
template cudaError_t launch_step_occ<float, 3>(const StepArgs<float>&, int, cudaStream_t);
template size_t step_smem_bytes<float>();
}  // namespace lri
