// engine_f64.cu - double instantiation of the instance engine (one translation
// unit per precision so the two compile in parallel).
#include "engine_impl.cuh"

namespace lri {
template cudaError_t launch_step_occ<double, 3>(const StepArgs<double>&, int, cudaStream_t);
template size_t step_smem_bytes<double>();
}  // namespace lri
