// noalloc.cu - lri_bug_step_noalloc: one BUG-integrated instance advanced
// without any device allocation.
//
// Some callers cannot call cudaMalloc: a host application whose device
// memory is owned by another allocator (a framework's caching pool that has
// reserved the whole device), or a time-stepping loop that must not trigger
// the implicit device-wide synchronisation cudaMalloc/cudaFree perform.  For
// them this entry point runs the same step kernel as lri_batch_step, with its
// workspace carved out of the file-scope array below instead of memory from
// lri_batch_create.
#include <cuda_runtime.h>

#include <atomic>
#include <cmath>
#include <cstdint>

#include "../../include/lri.h"
#include "engine_api.h"

namespace {

// Scratch of every call: 4 MiB, 256-byte aligned.  Every GPU that loads the
// library keeps this array until the process exits.
constexpr size_t kScratchBytes = size_t(4) << 20;
__device__ __align__(256) unsigned char lri_noalloc_scratch[kScratchBytes];

// Header at the start of the scratch: instance descriptor and bookkeeping
// words, written by noalloc_init_kernel on every call.
struct NoallocHeader {
  lri::InstDesc inst;
  int32_t order;
  int32_t rank;
  int32_t proj_valid;
  uint32_t status;
};
constexpr size_t kHeaderBytes = 256;
static_assert(sizeof(NoallocHeader) <= kHeaderBytes, "header must fit its slot");

// Device address of the scratch array, per device ordinal.  Host threads may
// look it up concurrently; they all store the same address.
constexpr int kMaxDevices = 64;
std::atomic<void*> g_scratch_addr[kMaxDevices];

__global__ void noalloc_init_kernel(NoallocHeader* h, lri::InstDesc d, int32_t r) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    h->inst = d;
    h->order = 0;
    h->rank = r;
    h->proj_valid = 0;  // the cached projections are recomputed by the first step
    h->status = 0u;
  }
}

lri::Scheme to_scheme(const lri_scheme& s) {
  lri::Scheme o{};
  o.nstages = s.nstages;
  o.nsub = s.nsub;
  for (int i = 0; i < 4; ++i) {
    o.a[i] = s.a[i];
    o.b[i] = s.b[i];
    o.c[i] = s.c[i];
  }
  return o;
}

template <typename T>
cudaError_t run_steps(unsigned char* base, const lri::InstDesc& d, void* U, void* S, void* V, const void* A,
                      const void* B, double dt, int nsteps, const lri::Scheme& sc, cudaStream_t st) {
  NoallocHeader* h = reinterpret_cast<NoallocHeader*>(base);
  lri::StepArgs<T> g{};
  g.inst = &h->inst;
  g.order = &h->order;
  g.rank = &h->rank;
  g.proj_valid = &h->proj_valid;
  g.status = &h->status;
  g.U = static_cast<T*>(U);
  g.S = static_cast<T*>(S);
  g.V = static_cast<T*>(V);
  g.opA = static_cast<const T*>(A);
  g.opB = static_cast<const T*>(B);
  g.work = reinterpret_cast<T*>(base + kHeaderBytes);
  g.small = g.work;  // offSmall is relative to the same base
  g.Yprev = nullptr;
  g.Ynext = nullptr;
  g.dt = dt;
  g.alg = lri::ALG_BUG;
  g.op = lri::OP_SYLVESTER;
  g.r_min = 1;
  g.sK = sc;
  g.sL = sc;
  g.sS = sc;
  for (int k = 0; k < nsteps; ++k) {
    g.t = k * dt;
    cudaError_t e = lri::launch_step<T>(g, 1, st);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

}  // namespace

extern "C" lri_status lri_bug_step_noalloc(int32_t dtype, int64_t n, int64_t m, int64_t r, void* U, void* S,
                                           void* V, const void* A, const void* B, double dt, int32_t nsteps,
                                           const lri_scheme* scheme, void* stream, int32_t* status_out) {
  if (!U || !S || !V || !A || !B || !scheme) return LRI_ERR_ARG;
  if (dtype != LRI_F32 && dtype != LRI_F64) return LRI_ERR_UNSUPPORTED;
  if (n < 1 || m < 1 || r < 1 || r > 64 || r > n || r > m || n >= (1 << 30) || m >= (1 << 30)) return LRI_ERR_ARG;
  if (nsteps < 0 || !std::isfinite(dt)) return LRI_ERR_ARG;
  if (scheme->nstages < 1 || scheme->nstages > 4 || scheme->nsub < 1) return LRI_ERR_ARG;
  const size_t es = dtype == LRI_F32 ? 4 : 8;
  auto al = [](int64_t x) { return (x + 3) & ~int64_t(3); };
  // same per-instance workspace layout as lri_batch_create (w = r for BUG)
  lri::InstDesc d{};
  d.n = (int32_t)n;
  d.m = (int32_t)m;
  d.rcap = (int32_t)r;
  d.wcap = (int32_t)r;
  d.offU = d.offS = d.offV = 0;
  d.offA = d.offB = 0;
  d.offWK = 0;
  d.offWL = al(n * (5 * r));
  d.offSmall = d.offWL + al(m * (5 * r));
  d.offY = 0;
  const int64_t elems = d.offSmall + lri::kSmallBlocks * al(r * r);
  if (kHeaderBytes + es * (size_t)elems > kScratchBytes) return LRI_ERR_ARG;  // beyond the fixed scratch
  if (nsteps == 0) {
    if (status_out) *status_out = LRI_OK;
    return LRI_OK;
  }

  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return LRI_ERR_CUDA;
  void* addr = g_scratch_addr[dev].load(std::memory_order_acquire);
  if (!addr) {
    // once per device, with that device current: the host-side symbol is a
    // stand-in, the kernels need the device address
    if (cudaGetSymbolAddress(&addr, lri_noalloc_scratch) != cudaSuccess || !addr) return LRI_ERR_CUDA;
    g_scratch_addr[dev].store(addr, std::memory_order_release);
  }
  unsigned char* base = static_cast<unsigned char*>(addr);
  cudaStream_t st = (cudaStream_t)stream;
  noalloc_init_kernel<<<1, 32, 0, st>>>(reinterpret_cast<NoallocHeader*>(base), d, (int32_t)r);
  if (cudaGetLastError() != cudaSuccess) return LRI_ERR_CUDA;
  const lri::Scheme sc = to_scheme(*scheme);
  cudaError_t e = (dtype == LRI_F32) ? run_steps<float>(base, d, U, S, V, A, B, dt, nsteps, sc, st)
                                     : run_steps<double>(base, d, U, S, V, A, B, dt, nsteps, sc, st);
  if (e != cudaSuccess) return LRI_ERR_CUDA;
  if (status_out) {
    // synchronous status report: wait for this call's steps, read the word
    uint32_t word = 0;
    const NoallocHeader* h = reinterpret_cast<const NoallocHeader*>(base);
    if (cudaMemcpyAsync(&word, &h->status, sizeof(word), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
      return LRI_ERR_CUDA;
    // same mapping as lri_batch_status
    *status_out = (word & lri::ST_BAD_SHAPE)      ? LRI_ERR_ARG
                  : (word & lri::ST_NONFINITE)    ? LRI_ERR_NONFINITE
                  : (word & lri::ST_SVD_NOCONV)   ? LRI_ERR_BREAKDOWN
                  : (word & lri::ST_RANK_OVERFLOW) ? LRI_ERR_RANK_OVERFLOW
                                                  : LRI_OK;
  }
  return LRI_OK;
}
