// engine_df.cu - double-float instantiation of the instance engine and the
// double <-> double-float conversion kernels used at the ABI boundary.
#include "engine_impl.cuh"

namespace lri {

template cudaError_t launch_step_occ<dfloat, 3>(const StepArgs<dfloat>&, int, cudaStream_t);
template size_t step_smem_bytes<dfloat>();

__global__ void f64_to_df_kernel(const double* __restrict__ in, dfloat* __restrict__ out, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = dfloat(in[i]);
}

__global__ void df_to_f64_kernel(const dfloat* __restrict__ in, double* __restrict__ out, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = (double)in[i];
}

static int conv_grid(int64_t n) {
  int64_t g = (n + 255) / 256;
  if (g > 152 * 16) g = 152 * 16;
  return g < 1 ? 1 : (int)g;
}

cudaError_t convert_f64_to_df(const double* in, void* out, int64_t n, cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  f64_to_df_kernel<<<conv_grid(n), 256, 0, stream>>>(in, static_cast<dfloat*>(out), n);
  return cudaGetLastError();
}

cudaError_t convert_df_to_f64(const void* in, double* out, int64_t n, cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  df_to_f64_kernel<<<conv_grid(n), 256, 0, stream>>>(static_cast<const dfloat*>(in), out, n);
  return cudaGetLastError();
}

int local_flow_count() { return kLocalFlowCount; }

const char* local_flow_name(int id) {
  switch (id) {
#define LRI_FLOW_NAME(ID, TYPE, NAME) \
  case ID:                            \
    return NAME;
    LRI_LOCAL_FLOWS(LRI_FLOW_NAME)
#undef LRI_FLOW_NAME
    default:
      return nullptr;
  }
}

}  // namespace lri
