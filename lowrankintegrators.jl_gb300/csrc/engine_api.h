// engine_api.h - host/device shared definitions of the instance engine.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include <atomic>
#include <type_traits>

namespace lri_df {
struct dfloat;  // double-float value (dfloat.cuh); the host only passes pointers to it
}  // namespace lri_df

namespace lri {

using lri_df::dfloat;

// Blocks of W*W elements (each rounded up to 4 elements) in an instance's
// small scratch: projections, basis changes, core-step work matrices, and
// the double-float copies of M, N, P_U, P_V of the FP32 class.
constexpr int kSmallBlocks = 23;

enum AlgKind : int32_t { ALG_BUG = 0, ALG_RA_BUG = 1, ALG_KSL = 2, ALG_GREEDY = 3 };
enum KslOrder : int32_t { KSL_PRIMAL = 0, KSL_DUAL = 1, KSL_STRANG = 2 };
enum OpKind : int32_t { OP_ZERO = 0, OP_SYLVESTER = 1, OP_BURGERS = 2, OP_DATA = 3, OP_LOCAL = 4 };

// Device status bits (OR-ed into the batch status word).
enum StatusBits : uint32_t {
  ST_NONFINITE = 1u,
  ST_SVD_NOCONV = 2u,
  ST_RANK_OVERFLOW = 4u,
  ST_BAD_SHAPE = 8u,
  ST_TIMEOUT = 16u,  // a bounded device wait gave up
};

struct Scheme {
  int32_t nstages, nsub;
  double a[4], b[4], c[4];
};

// Per-instance descriptor (device resident).
struct InstDesc {
  int32_t n, m, rcap, wcap;  // wcap: widest panel (rcap, or 2*rcap for RA)
  int64_t offU, offS, offV;  // caller buffers
  int64_t offA, offB;        // operator coefficients
  int64_t offWK, offWL;      // K-side / L-side panel workspaces
  int64_t offSmall;          // small-matrix scratch
  int64_t offY;              // data snapshots (n x m)
};

template <typename T>
struct StepArgs {
  const InstDesc* inst;
  const int32_t* order;
  int32_t* rank;
  int32_t* proj_valid;
  uint32_t* status;
  T* U;
  T* S;
  T* V;
  const T* opA;
  const T* opB;
  T* work;
  T* small;
  T* Yprev;
  const T* Ynext;
  double t, dt;
  int32_t alg, ksl_order, op, r_min;
  int32_t two_factor;  // greedy: factors U Z^T (Z in V) instead of U S V^T
  int32_t flow;        // OP_LOCAL: registered flow id (flows.cuh)
  double tol;
  Scheme sK, sL, sS;
  double bh, balpha, bbeta;  // local flows: h, p0, p1 (Burgers: h, alpha, beta)
  int32_t split;             // set by the launcher: one 2-CTA cluster per instance (FP64 BUG, Sylvester)
};

// Registered local flow maps (flows.cuh): count and names.
int local_flow_count();
const char* local_flow_name(int id);

// Raises a kernel's dynamic shared-memory limit on the current device.  The
// attribute is per device, so `done` keeps one bit per device ordinal (< 64;
// higher ordinals set it on every call); several host threads may race to
// set the same bit, which is harmless.  cudaFuncSetAttribute is not a stream
// operation, so this is also safe while a stream is being captured.
template <typename F>
inline cudaError_t set_smem_limit(F* func, int bytes, std::atomic<uint64_t>& done) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const uint64_t bit = (dev >= 0 && dev < 64) ? (uint64_t(1) << dev) : 0;
  if (bit && (done.load(std::memory_order_acquire) & bit)) return cudaSuccess;
  e = cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e == cudaSuccess && bit) done.fetch_or(bit, std::memory_order_acq_rel);
  return e;
}

template <typename T, int MINB>
cudaError_t launch_step_occ(const StepArgs<T>& g, int count, cudaStream_t stream);

// One launch of the step kernel for `count` instances.  ctas_per_sm selects
// the register budget: 3 CTAs per SM (at most 80 registers per thread, the
// default) or 2 (at most 128); FP64 batches have the default only.
template <typename T>
inline cudaError_t launch_step(const StepArgs<T>& g, int count, cudaStream_t stream, int ctas_per_sm = 3) {
  if constexpr (std::is_same<T, double>::value) {
    return launch_step_occ<T, 3>(g, count, stream);
  } else {
    return ctas_per_sm == 2 ? launch_step_occ<T, 2>(g, count, stream) : launch_step_occ<T, 3>(g, count, stream);
  }
}

// double <-> double-float conversions of n elements (dfloat storage is a
// pair of floats, 8 bytes per element)
cudaError_t convert_f64_to_df(const double* in, void* out, int64_t n, cudaStream_t stream);
cudaError_t convert_df_to_f64(const void* in, double* out, int64_t n, cudaStream_t stream);
template <typename T>
size_t step_smem_bytes();

// Discrete adjoint of the FP64 BUG step (adjoint.cu): workspace elements per
// instance, the largest nstages * nsub it supports, and the launch.
size_t adjoint_work_elems(int64_t n, int64_t m, int64_t r, int ns_k, int ns_l);
int adjoint_max_stages();
cudaError_t launch_adjoint_step(const InstDesc* inst, const int64_t* adj_off, const int64_t* th_off, int count,
                                const double* U0, const double* S0, const double* V0, double* Ub, double* Sb,
                                double* Vb, double* thb, const double* opA, const double* opB, double* work,
                                const Scheme& sK, const Scheme& sL, const Scheme& sS, double dt, cudaStream_t st);

}  // namespace lri
