// core_svd.cu - SVD and truncation of the 2r x 2r core of the large engines'
// rank-adaptive step (src/integrators/rank_adaptive_unconventional.jl:
// 217-226: S~ = P Sigma Q^T, r1 from the truncation tolerance, U1 = Uhat P1,
// V1 = Vhat Q1) for FP32 panels, on one cluster of CS_C thread blocks.
//
// The one-sided Jacobi SVD (Hestenes) rotates pairs of columns of the core
// until all pairs are orthogonal.  A sweep over the 2r columns is 2r - 1
// rounds of disjoint pairs, each bound by the latency of a dot product, its
// reduction and the rotation; on one CTA (rank 64) that was 0.4 ms per FP32
// sweep and 1.5 ms per double-float sweep.  Here the columns (with their
// right vectors) are split into 2 CS_C blocks over the cluster: in each round
// of a sweep a CTA rotates the pairs across its two blocks (wb sub-rounds of
// wb disjoint pairs; the pairs inside a block in the sweep's first round),
// then every block moves to the CTA that holds it in the next round, through
// distributed shared memory.  The rounds place the blocks by the circle
// method, so every two blocks meet once per sweep.  Products of the whole
// matrices (Newton-Schulz, the basis changes) are split by output columns
// over the cluster and go through L2.
//
// Stages (as in the one-CTA form for FP32 panels): FP32 sweeps as a
// preconditioner give V32; X = V32 orthonormalised by two Newton-Schulz
// steps in double-float; AS = F X; double-float sweeps on AS (rotations V_p)
// until the rotations are below 1e-4, with the truncation-level skip rule;
// sigma_j = |AS_j|, left vectors AS_j / sigma_j, V = X V_p.  Every loop is
// bounded (sweep limits); the cluster barriers are reached the same number
// of times by every CTA (the convergence decisions are made from the same
// reduced values everywhere).
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstdint>

#include "core_svd.h"
#include "engine.cuh"
#include "engine_api.h"

namespace cg = cooperative_groups;

namespace lri {
namespace {

constexpr int CS_C = 8;                      // CTAs per cluster
constexpr int CS_NT = 256;                   // threads per CTA
constexpr int CS_NBLK = 2 * CS_C;            // column blocks
constexpr int CS_WBMAX = (CORE_SVD_MAX_WA + CS_NBLK - 1) / CS_NBLK;
// four blocks (two slots, two buffers) of wb columns and wb right vectors,
// double-float; the product stage reuses the area
constexpr int CS_SMEM = 4 * 2 * CS_WBMAX * CORE_SVD_MAX_WA * 8;

struct ClusterState {
  double fro[CS_C];          // partial ||A||_F^2 of every CTA
  unsigned flag[2][CS_C];    // per sweep parity: a CTA rotated
  unsigned dmax[2][CS_C];    // per sweep parity: its largest rotation measure (float bits)
  unsigned lflag, ldmax;     // this CTA, current sweep
};

// In round t (0 <= t < 2C - 1) CTA k holds blocks blk_first(k, t) (slot 0)
// and blk_second(k, t) (slot 1): block 2C - 1 stays, the others turn.
__device__ __forceinline__ int blk_first(int k, int t) {
  return (k == 0) ? t % (CS_NBLK - 1) : (t + k) % (CS_NBLK - 1);
}
__device__ __forceinline__ int blk_second(int k, int t) {
  return (k == 0) ? CS_NBLK - 1 : (t - k + CS_NBLK - 1) % (CS_NBLK - 1);
}
// the CTA and slot holding block b in round t
__device__ __forceinline__ void blk_home(int b, int t, int& k, int& slot) {
  if (b == CS_NBLK - 1) {
    k = 0;
    slot = 1;
    return;
  }
  const int d = (b - t + CS_NBLK - 1) % (CS_NBLK - 1);
  if (d == 0) {
    k = 0;
    slot = 0;
  } else if (d < CS_C) {
    k = d;
    slot = 0;
  } else {
    k = CS_NBLK - 1 - d;
    slot = 1;
  }
}

__device__ __forceinline__ double as_double(float x) { return (double)x; }
__device__ __forceinline__ double as_double(dfloat x) { return (double)x; }

__device__ __forceinline__ dfloat ld_cg(const dfloat* p) {
  const float2 v = __ldcg(reinterpret_cast<const float2*>(p));
  return dfloat(v.x, v.y);
}

// Rotation parameters of a pair with al = |x|^2, be = |y|^2, ga = x.y: the
// measure dl = |ga| / sqrt(al be), and, when dl > eps, tan = t of the
// rotation angle (zeta = (be - al) / 2 ga, t = sign(zeta) / (|zeta| +
// sqrt(1 + zeta^2))) with cs = (1 + t^2)^(-1/2), sn = cs t.  The angle needs
// FP32 accuracy only (an angle off by a relative delta leaves delta of the
// pair's product, far below the next sweep's quadratic residual); cs and sn
// are orthonormal to the working precision, so the right vectors stay
// orthogonal.  FP32 approximate intrinsics (MUFU) keep the rotation's
// dependency chain short.
// t = sign(d) 2ga / (|d| + sqrt(d^2 + 4ga^2)) (d = be - al; the same as
// sign(zeta) / (|zeta| + sqrt(1 + zeta^2)) with zeta = d / 2ga), after
// scaling d and 2ga by the larger of the two (no overflow; the root's
// argument lies in [1, 2])
__device__ __forceinline__ float rot_tan(float d, float ga) {
  const float g2 = 2.0f * ga;
  const float sc = __frcp_rn(fmaxf(fabsf(d), fabsf(g2)));
  const float dn = d * sc, gn = g2 * sc;
  const float h = fmaf(dn, dn, gn * gn);
  const float t = __fdividef(gn, fabsf(dn) + h * rsqrtf(h));
  return (d < 0.0f) ? -t : t;
}

__device__ __forceinline__ bool rot_params(float al, float be, float ga, float eps, float& cs, float& sn, float& dl) {
  dl = fabsf(ga) * rsqrtf(al) * rsqrtf(be);
  if (!(dl > eps) || ga == 0.0f) return false;
  const float t = rot_tan(be - al, ga);
  cs = rsqrtf(fmaf(t, t, 1.0f));
  sn = cs * t;
  return true;
}

// (1 + t^2)^(-1/2) in double-float: the FP32 estimate and one Newton step
// y (1 + e / 2), e = 1 - q y^2 (relative error about 1e-13)
__device__ __forceinline__ dfloat rsqrt_1pt2(float t) {
  const dfloat q = fma(dfloat(t), dfloat(t), dfloat(1.0f));
  const float y = rsqrtf(q.hi);
  const dfloat e = dfloat(1.0f) - q * (dfloat(y) * dfloat(y));
  return lri_df::fast_two_sum(y, 0.5f * y * e.hi);
}

__device__ __forceinline__ bool rot_params(dfloat al, dfloat be, dfloat ga, dfloat eps, dfloat& cs, dfloat& sn,
                                           float& dl) {
  dl = fabsf(ga.hi) * rsqrtf(al.hi) * rsqrtf(be.hi);
  if (!(dl > eps.hi) || ga.hi == 0.0f) return false;
  const float t = rot_tan((be - al).hi, ga.hi);  // be - al in double-float: no cancellation
  cs = rsqrt_1pt2(t);
  sn = cs * dfloat(t);
  return true;
}

// One Jacobi rotation of columns (ap, aq) with right vectors (vp, vq) by a
// group of G lanes (gl = lane in the group; the group's rows i = gl + k G of
// the columns and of the right vectors are loaded at once and stay in
// registers until the rotation); every lane of the
// warp takes part in the reductions.  Same test and rotation as the one-CTA
// sweeps, with the parameters above.  A rotation sets fl and raises dm (the
// rotation measure) in the lane's registers; the sweep reduces them once at
// its end.
template <typename T, int G>
__device__ __forceinline__ void rotate_pair(T* ap, T* aq, T* vp, T* vq, bool valid, int wa, int gl, T eps, T tiny,
                                            T reach, bool skip_noise, unsigned& fl, float& dm) {
  constexpr int KR = (CORE_SVD_MAX_WA + G - 1) / G;
  T x[KR], y[KR], u[KR], w[KR];  // the group's rows of the columns and of the right vectors
  T al = T(0), be = T(0), ga = T(0);
#pragma unroll
  for (int k = 0; k < KR; ++k) {
    const int i = gl + k * G;
    if (valid && i < wa) {
      x[k] = ap[i];
      y[k] = aq[i];
      u[k] = vp[i];
      w[k] = vq[i];
    } else {
      x[k] = T(0);
      y[k] = T(0);
      u[k] = T(0);
      w[k] = T(0);
    }
    al = fma_acc(x[k], x[k], al);
    be = fma_acc(y[k], y[k], be);
    ga = fma_acc(x[k], y[k], ga);
  }
  al = renorm(al);
  be = renorm(be);
  ga = renorm(ga);
#pragma unroll
  for (int o = G >> 1; o > 0; o >>= 1) {
    al += shfl_xor(al, o);
    be += shfl_xor(be, o);
    ga += shfl_xor(ga, o);
  }
  const bool live =
      valid && (skip_noise ? (al > tiny && be > tiny && (al > reach || be > reach)) : (al > tiny || be > tiny));
  T cs_, sn;
  float dl;
  if (live && rot_params(al, be, ga, eps, cs_, sn, dl)) {
#pragma unroll
    for (int k = 0; k < KR; ++k) {
      const int i = gl + k * G;
      if (i < wa) {
        ap[i] = cs_ * x[k] - sn * y[k];
        aq[i] = sn * x[k] + cs_ * y[k];
      }
    }
#pragma unroll
    for (int k = 0; k < KR; ++k) {
      const int i = gl + k * G;
      if (i < wa) {
        vp[i] = cs_ * u[k] - sn * w[k];
        vq[i] = sn * u[k] + cs_ * w[k];
      }
    }
    fl = 1u;
    dm = fmaxf(dm, dl);
  }
}

// Jacobi sweeps over the cluster.  On entry and on return the blocks sit in
// buffer `cur` in their round-0 places.  Returns whether the sweeps
// converged (no rotation, or the largest rotation measure of a sweep at most
// conv_delta; sqrt(eps) when negative).  The same on every CTA.
template <typename T>
__device__ bool cluster_jacobi(cg::cluster_group& cl, ClusterState& cs, T* base, int& cur, int wa, int wb,
                               int max_sweeps, bool skip_noise, double conv_delta, double tiny_abs) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int cr = (int)cl.block_rank();
  const size_t bstride = (size_t)2 * wb * wa;
  auto block = [&](int buf, int slot) { return base + (size_t)(buf * 2 + slot) * bstride; };

  // ||A||_F^2: every CTA adds the same partials in the same order
  __shared__ double red[CS_NT / 32];
  {
    double s = 0.0;
    for (int slot = 0; slot < 2; ++slot) {
      const int b = slot ? blk_second(cr, 0) : blk_first(cr, 0);
      const T* A = block(cur, slot);
      for (int e = tid; e < wb * wa; e += CS_NT)
        if (b * wb + e / wa < wa) {
          const double x = as_double(A[e]);
          s += x * x;
        }
    }
    s = warp_sum(s);
    if (lane == 0) red[warp] = s;
    __syncthreads();
    if (tid < CS_C) {
      double p = 0.0;
      for (int k = 0; k < CS_NT / 32; ++k) p += red[k];
      double* dst = cl.map_shared_rank(&cs.fro[cr], tid);
      *dst = p;
    }
    cl.sync();
  }
  double fro2 = 0.0;
  for (int k = 0; k < CS_C; ++k) fro2 += cs.fro[k];

  const T eps = T(Prec<T>::eps * wa);
  const T tiny = T(Prec<T>::eps * Prec<T>::eps * fro2);
  const T reach = T(tiny_abs);
  const float delta_stop = (float)((conv_delta >= 0.0) ? conv_delta : sqrt(Prec<T>::eps));
  const int wbe = wb + (wb & 1);  // even number of players inside a block
  const int G = (wbe <= CS_NT / 32) ? 32 : 16;
  const int gid = tid / G, gl = tid % G;
  auto rotate = [&](T* ap, T* aq, T* vp, T* vq, bool valid, unsigned& fl, float& dm) {
    if (G == 32)
      rotate_pair<T, 32>(ap, aq, vp, vq, valid, wa, gl, eps, tiny, reach, skip_noise, fl, dm);
    else
      rotate_pair<T, 16>(ap, aq, vp, vq, valid, wa, gl, eps, tiny, reach, skip_noise, fl, dm);
  };
  const size_t bsz16 = bstride * sizeof(T) / 16;
  bool converged = false;
  for (int sweep = 0; sweep < max_sweeps && !converged; ++sweep) {
    if (tid == 0) {
      cs.lflag = 0u;
      cs.ldmax = 0u;
    }
    unsigned fl = 0u;  // this lane's group rotated in this sweep
    float dm = 0.0f;   // and its largest rotation measure
    __syncthreads();
    for (int t = 0; t < CS_NBLK - 1; ++t) {
      const int b0 = blk_first(cr, t), b1 = blk_second(cr, t);
      T* B0 = block(cur, 0);
      T* B1 = block(cur, 1);
      if (t == 0) {
        // pairs inside each block (circle method over wbe players)
        const int half = wbe / 2;
        for (int u = 0; u < wbe - 1; ++u) {
          const int slot = gid / max(half, 1), k = gid % max(half, 1);
          int x, y;
          if (k == 0) {
            x = u % (wbe - 1);
            y = wbe - 1;
          } else {
            x = (u + k) % (wbe - 1);
            y = (u - k + wbe - 1) % (wbe - 1);
          }
          if (x > y) {
            const int tmp = x;
            x = y;
            y = tmp;
          }
          const int b = slot ? b1 : b0;
          const bool valid = gid < wbe && y < wb && b * wb + y < wa;
          T* Bk = slot ? B1 : B0;
          const int xs = valid ? x : 0, ys = valid ? y : 0;
          rotate(Bk + (size_t)xs * wa, Bk + (size_t)ys * wa, Bk + (size_t)(wb + xs) * wa, Bk + (size_t)(wb + ys) * wa,
                 valid, fl, dm);
          __syncthreads();
        }
      }
      // pairs across the two blocks: column x of slot 0 with (x + s) mod wb of slot 1
      for (int s = 0; s < wb; ++s) {
        const int x = gid, y = (gid + s) % wb;
        const bool valid = gid < wb && b0 * wb + x < wa && b1 * wb + y < wa;
        const int xs = valid ? x : 0, ys = valid ? y : 0;
        T* ap = B0 + (size_t)xs * wa;
        T* vp = B0 + (size_t)(wb + xs) * wa;
        T* aq = B1 + (size_t)ys * wa;
        T* vq = B1 + (size_t)(wb + ys) * wa;
        if (b0 * wb + x > b1 * wb + y) {  // the lower column index first
          T* t1 = ap;
          ap = aq;
          aq = t1;
          t1 = vp;
          vp = vq;
          vq = t1;
        }
        rotate(ap, aq, vp, vq, valid, fl, dm);
        __syncthreads();
      }
      // every block to its place in the next round (buffer cur ^ 1)
      const int tn = (t + 1) % (CS_NBLK - 1);
      for (int slot = 0; slot < 2; ++slot) {
        int dk, ds;
        blk_home(slot ? b1 : b0, tn, dk, ds);
        const float4* src = reinterpret_cast<const float4*>(block(cur, slot));
        float4* dst = cl.map_shared_rank(reinterpret_cast<float4*>(block(cur ^ 1, ds)), dk);
        for (size_t e = tid; e < bsz16; e += CS_NT) dst[e] = src[e];
      }
      if (t == CS_NBLK - 2) {
        // the sweep's flag and largest measure: lanes, warps, then every CTA
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          fl |= __shfl_xor_sync(0xffffffffu, fl, o);
          dm = fmaxf(dm, __shfl_xor_sync(0xffffffffu, dm, o));
        }
        if (lane == 0) {
          atomicOr(&cs.lflag, fl);
          atomicMax(&cs.ldmax, __float_as_uint(dm));  // non-negative: the bits order as the values
        }
        __syncthreads();
        if (tid < CS_C) {
          *cl.map_shared_rank(&cs.flag[sweep & 1][cr], tid) = cs.lflag;
          *cl.map_shared_rank(&cs.dmax[sweep & 1][cr], tid) = cs.ldmax;
        }
      }
      cl.sync();
      cur ^= 1;
    }
    unsigned any = 0u, dmc = 0u;
    for (int k = 0; k < CS_C; ++k) {
      any |= cs.flag[sweep & 1][k];
      dmc = max(dmc, cs.dmax[sweep & 1][k]);
    }
    converged = (any == 0u) || (__uint_as_float(dmc) <= delta_stop);
  }
  return converged;
}

// out[:, j] (j0 <= j < j1) = op(A) B[:, j] for wa x wa double-float matrices
// (ld wa) in global memory; A from AD (double-float) or A64 (FP64).
// ns: out = 1.5 [i == j] - 0.5 (A^T B) (a Newton-Schulz factor).  Tiles of
// 32 rows of op(A) and the CTA's columns of B in shared memory; reads of
// matrices other CTAs wrote bypass L1.
__device__ void prod_cols(int wa, const dfloat* AD, const double* A64, bool transA, const dfloat* B, int j0, int j1,
                          dfloat* out, bool ns, unsigned char* smem) {
  const int tid = threadIdx.x;
  const int nJ = j1 - j0;
  if (nJ <= 0) return;
  dfloat* Bs = reinterpret_cast<dfloat*>(smem);  // nJ x wa
  dfloat* As = Bs + (size_t)nJ * wa;             // [k][33]: rows i0..i0+31 of op(A)
  __syncthreads();
  for (int e = tid; e < nJ * wa; e += CS_NT) Bs[e] = ld_cg(B + (size_t)(j0 + e / wa) * wa + e % wa);
  auto A_at = [&](int i, int k) {  // A[i, k]
    return AD ? ld_cg(AD + i + (size_t)k * wa) : dfloat(A64[i + (size_t)k * wa]);
  };
  for (int i0 = 0; i0 < wa; i0 += 32) {
    __syncthreads();
    for (int e = tid; e < 32 * wa; e += CS_NT) {
      int ii, k;
      if (!transA) {
        ii = e & 31;
        k = e >> 5;
      } else {
        k = e % wa;
        ii = e / wa;
      }
      const int i = i0 + ii;
      As[k * 33 + ii] = (i < wa) ? (transA ? A_at(k, i) : A_at(i, k)) : dfloat(0.0f, 0.0f);
    }
    __syncthreads();
    for (int o = tid; o < 32 * nJ; o += CS_NT) {
      const int ii = o & 31, jj = o >> 5, i = i0 + ii;
      dfloat acc(0.0f, 0.0f);
      const dfloat* bj = Bs + (size_t)jj * wa;
      for (int k = 0; k < wa; ++k) acc = fma_acc(As[k * 33 + ii], bj[k], acc);
      acc = renorm(acc);
      if (i < wa) {
        const int j = j0 + jj;
        if (ns) acc = ((i == j) ? dfloat(1.5f, 0.0f) : dfloat(0.0f, 0.0f)) - dfloat(0.5f, 0.0f) * acc;
        out[i + (size_t)j * wa] = acc;
      }
    }
  }
  __syncthreads();
}

// singular values: the norms of the CTA's active columns to every CTA's sig[]
__device__ void broadcast_sigma(cg::cluster_group& cl, const dfloat* base, int cur, int wa, int wb, dfloat* sig) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int cr = (int)cl.block_rank();
  const size_t bstride = (size_t)2 * wb * wa;
  for (int c = warp; c < 2 * wb; c += CS_NT / 32) {
    const int slot = c / wb, q = c % wb;
    const int col = (slot ? blk_second(cr, 0) : blk_first(cr, 0)) * wb + q;
    if (col >= wa) continue;  // warp-uniform
    const dfloat* A = base + (size_t)(cur * 2 + slot) * bstride + (size_t)q * wa;
    dfloat s(0.0f, 0.0f);
    for (int i = lane; i < wa; i += 32) s = fma(A[i], A[i], s);
    s = warp_sum(s);
    const dfloat sv = sqrt(s);
    if (lane < CS_C) *cl.map_shared_rank(&sig[col], lane) = sv;
  }
  cl.sync();
}

// perm: column indices by descending sigma (ties by index), in parallel
__device__ void sort_sigma(int wa, const dfloat* sig, int* perm) {
  for (int j = threadIdx.x; j < wa; j += CS_NT) {
    const dfloat sj = sig[j];
    int rk = 0;
    for (int k = 0; k < wa; ++k) {
      const dfloat sk = sig[k];
      rk += (sk > sj || (sk == sj && k < j)) ? 1 : 0;
    }
    perm[rk] = j;
  }
  __syncthreads();
}

// smallest r1 with sum_{j > r1} sigma_j^2 < tol^2, clamped to [rmin, R] and wa
__device__ int decide_rank(int wa, int R, int rmin, double tol, const dfloat* sig, const int* perm) {
  const double tol2 = tol * tol;
  double acc = 0.0;
  int rr = wa;
  while (acc < tol2 && rr > 0) {
    const double sv = (double)sig[perm[rr - 1]];
    acc += sv * sv;
    --rr;
  }
  int r1 = rr + 1;
  if (r1 > R) r1 = R;
  if (r1 < rmin) r1 = rmin;
  if (r1 > wa) r1 = wa;
  return r1;
}

__global__ void __cluster_dims__(CS_C, 1, 1) __launch_bounds__(CS_NT, 1) core_svd_kernel(const CoreSvdArgs a) {
  cg::cluster_group cl = cg::this_cluster();
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ ClusterState cs;
  __shared__ dfloat sig[CORE_SVD_MAX_WA];
  __shared__ int perm[CORE_SVD_MAX_WA];
  __shared__ int r_new, redo;
  const int tid = threadIdx.x;
  const int cr = (int)cl.block_rank();
  const int R = a.R, w = 2 * R;
  const int r = min(R, (int)*a.rank), wa = 2 * r;
  const int wb = max(1, (wa + CS_NBLK - 1) / CS_NBLK);
  const size_t bstride = (size_t)2 * wb * wa;
  dfloat* X = reinterpret_cast<dfloat*>(a.scr[0]);
  dfloat* Xn = reinterpret_cast<dfloat*>(a.scr[1]);
  dfloat* T2 = reinterpret_cast<dfloat*>(a.scr[2]);
  dfloat* AF = reinterpret_cast<dfloat*>(a.scr[3]);
  dfloat* VF = reinterpret_cast<dfloat*>(a.scr[4]);
  // pairs whose columns both hold at most tol^2 / (4 wa) are left alone (the
  // kept singular directions are then those of the exact SVD)
  const double tiny_abs = a.tol * a.tol / (4.0 * max(wa, 1));
  cl.sync();  // every CTA of the cluster runs before any distributed access

  // ---- FP32 sweeps: V32 ----
  int cur = 0;
  {
    float* base = reinterpret_cast<float*>(smem);
    for (int slot = 0; slot < 2; ++slot) {
      const int b = slot ? blk_second(cr, 0) : blk_first(cr, 0);
      float* B = base + (size_t)slot * bstride;
      for (int e = tid; e < wb * wa; e += CS_NT) {
        const int q = e / wa, i = e % wa, col = b * wb + q;
        B[e] = (col < wa) ? __double2float_rn(a.F[i + (size_t)col * wa]) : 0.0f;
        B[(size_t)wb * wa + e] = (col < wa && i == col) ? 1.0f : 0.0f;
      }
    }
    __syncthreads();
    // a preconditioner: near FP32's resolution limit the sweeps need not
    // converge, so at most 12
    cluster_jacobi<float>(cl, cs, base, cur, wa, wb, 12, false, -1.0, 0.0);
    for (int slot = 0; slot < 2; ++slot) {
      const int b = slot ? blk_second(cr, 0) : blk_first(cr, 0);
      const float* V = base + (size_t)(cur * 2 + slot) * bstride + (size_t)wb * wa;
      for (int e = tid; e < wb * wa; e += CS_NT) {
        const int col = b * wb + e / wa;
        if (col < wa) X[(size_t)col * wa + e % wa] = dfloat(V[e], 0.0f);
      }
    }
    __threadfence();
    cl.sync();
  }

  // ---- X = Newton-Schulz(V32), two steps: X (3 I - X^T X) / 2; AS = F X ----
  const int jc = (wa + CS_C - 1) / CS_C;
  const int j0 = min(wa, cr * jc), j1 = min(wa, j0 + jc);
  for (int it = 0; it < 2; ++it) {
    prod_cols(wa, X, nullptr, true, X, j0, j1, T2, true, smem);  // own columns of (3 I - X^T X) / 2
    prod_cols(wa, X, nullptr, false, T2, j0, j1, Xn, false, smem);
    __threadfence();
    cl.sync();
    dfloat* tmp = X;
    X = Xn;
    Xn = tmp;
  }
  dfloat* AS = T2;
  prod_cols(wa, nullptr, a.F, false, X, j0, j1, AS, false, smem);
  __threadfence();
  cl.sync();

  // ---- double-float sweeps on AS: rotations V_p ----
  dfloat* base = reinterpret_cast<dfloat*>(smem);
  cur = 0;
  for (int slot = 0; slot < 2; ++slot) {
    const int b = slot ? blk_second(cr, 0) : blk_first(cr, 0);
    dfloat* B = base + (size_t)slot * bstride;
    for (int e = tid; e < wb * wa; e += CS_NT) {
      const int q = e / wa, i = e % wa, col = b * wb + q;
      B[e] = (col < wa) ? ld_cg(AS + i + (size_t)col * wa) : dfloat(0.0f, 0.0f);
      B[(size_t)wb * wa + e] = dfloat((col < wa && i == col) ? 1.0f : 0.0f, 0.0f);
    }
  }
  __syncthreads();
  bool ok = cluster_jacobi<dfloat>(cl, cs, base, cur, wa, wb, 40, true, 1e-4, tiny_abs);
  broadcast_sigma(cl, base, cur, wa, wb, sig);
  sort_sigma(wa, sig, perm);
  if (tid == 0) {
    r_new = decide_rank(wa, R, a.rmin, a.tol, sig, perm);
    const double sv = (r_new > 0) ? (double)sig[perm[r_new - 1]] : 0.0;
    redo = (r_new > 0 && sv * sv <= 4.0 * tiny_abs);  // the minimum rank keeps skipped columns
  }
  __syncthreads();
  double tiny_left = tiny_abs;
  if (redo) {
    // continue the sweeps without the truncation-level skip
    ok = cluster_jacobi<dfloat>(cl, cs, base, cur, wa, wb, 40, true, 1e-4, 0.0);
    broadcast_sigma(cl, base, cur, wa, wb, sig);
    sort_sigma(wa, sig, perm);
    if (tid == 0) r_new = decide_rank(wa, R, a.rmin, a.tol, sig, perm);
    tiny_left = 0.0;
    __syncthreads();
  }
  // rotated columns to AF, right rotations V_p to Xn (free), then V = X V_p
  dfloat* VP = Xn;
  for (int slot = 0; slot < 2; ++slot) {
    const int b = slot ? blk_second(cr, 0) : blk_first(cr, 0);
    const dfloat* B = base + (size_t)(cur * 2 + slot) * bstride;
    for (int e = tid; e < wb * wa; e += CS_NT) {
      const int col = b * wb + e / wa;
      if (col < wa) {
        AF[(size_t)col * wa + e % wa] = B[e];
        VP[(size_t)col * wa + e % wa] = B[(size_t)wb * wa + e];
      }
    }
  }
  __threadfence();
  cl.sync();
  prod_cols(wa, X, nullptr, false, VP, j0, j1, VF, false, smem);
  __threadfence();
  cl.sync();  // no distributed access after this point
  if (cr != 0) return;

  // ---- CTA 0: truncation, left vectors, outputs ----
  const int r1 = r_new;
  if (tid == 0) {
    if (!ok) atomicOr(a.status, a.st_noconv);
    *a.rank = r1;
  }
  // left vectors AS_j / sigma_j in place (P1 as scratch before it is written)
  complete_left<dfloat, CS_NT>(wa, r1, AF, sig, perm, reinterpret_cast<dfloat*>(a.P1), tiny_left);
  __syncthreads();
  for (int o = tid; o < w * R; o += CS_NT) a.P1[o] = a.Q1[o] = 0.0;
  __syncthreads();
  auto idx = [&](int i) { return (i < r) ? i : R + (i - r); };
  for (int o = tid; o < wa * r1; o += CS_NT) {
    const int i = o % wa, j = o / wa;
    const int pj = perm[j];
    a.P1[idx(i) + (size_t)j * w] = (double)AF[i + (size_t)pj * wa];
    a.Q1[idx(i) + (size_t)j * w] = (double)VF[i + (size_t)pj * wa];
  }
  for (int o = tid; o < R * R; o += CS_NT) {
    const int i = o % R, j = o / R;
    a.S0[o] = (i == j && i < r1) ? (float)(double)sig[perm[i]] : 0.0f;
  }
  __syncthreads();
  bool bad = false;
  for (int o = tid; o < R * R; o += CS_NT) bad |= !isfinite(a.S0[o]);
  if (__syncthreads_or(bad) && tid == 0) atomicOr(a.status, a.st_nonfinite);
}

}  // namespace

cudaError_t core_svd_cluster(const CoreSvdArgs& a, cudaStream_t st) {
  if (a.R < 1 || 2 * a.R > CORE_SVD_MAX_WA) return cudaErrorInvalidValue;
  static std::atomic<uint64_t> attr_done{0};
  cudaError_t e = set_smem_limit(core_svd_kernel, CS_SMEM, attr_done);
  if (e != cudaSuccess) return e;
  core_svd_kernel<<<CS_C, CS_NT, CS_SMEM, st>>>(a);
  return cudaGetLastError();
}

}  // namespace lri
