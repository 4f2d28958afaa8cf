// engine.cu - the instance engine: one CTA advances one DLRA instance by one
// integrator step (BUG, rank-adaptive BUG, or KSL), for a whole batch of
// independent instances per launch.
//
// Reference correspondence (paths within LowRankIntegrators.jl):
//   bug_step      src/integrators/unconventional.jl:133-157
//   ra_bug_step   src/integrators/rank_adaptive_unconventional.jl:194-233
//   ksl_primal    src/integrators/projector_splitting.jl:129-152
//   ksl_dual      src/integrators/projector_splitting.jl:166-189
//   Strang        src/integrators/projector_splitting.jl:205-211
//   greedy_step   src/integrators/greedy_integrator.jl:73-104
//   data substeps src/integrators/data_integrator.jl:13-16 (u += sign*left'*Δy*right)
//   K/L/S rhs     src/integrators/unconventional.jl:52-54,62-64,72-74
#pragma once
#include <cooperative_groups.h>

#include <type_traits>

#include "engine.cuh"
#include "engine_api.h"

namespace lri {

// Workspace layout of one side (rows N): five panels.
template <typename T>
struct Side {
  int N;
  T* X;            // caller's basis (U or V), ld N
  const T* tri;    // tridiagonal coefficients of this side's operator (3N)
  T* PY;           // N x W : substep state / QR panel
  T* PQ;           // N x W : explicit Q
  T* PA;           // N x rcap : RK accumulator
  T* PZ0;          // N x rcap : RK stage input (ping)
  T* PZ1;          // N x rcap : RK stage input (pong)
};

template <typename T>
struct Inst {
  int n, m, rcap, W, inst;
  T* U;
  T* S;
  T* V;
  Side<T> k, l;
  T* small;   // B_COUNT blocks of W*W elements, each block 16-byte aligned
  const T* Yp;
  const T* Yn;
  T* Ypw;     // writable previous snapshot
  // block stride: W*W rounded up to 4 elements, so a block can also hold
  // double-float values in a float batch (8-byte aligned)
  __device__ int64_t bstride() const { return ((int64_t)W * W + 3) & ~int64_t(3); }
  __device__ T* blk(int i) const { return small + (int64_t)i * bstride(); }
};

// small-scratch block indices
// (B_DM .. B_DPV: double-float matrices of the FP32 class, two blocks each)
enum : int { B_GU = 0, B_GV = 2, B_M = 4, B_N = 5, B_ST = 6, B_SA = 7, B_SZ0 = 8, B_SZ1 = 9, B_SK = 10,
             B_T1 = 11, B_T2 = 12, B_RK = 13, B_RL = 14, B_DM = 15, B_DN = 17, B_DPU = 19, B_DPV = 21,
             B_COUNT = 23 };
static_assert(B_COUNT == kSmallBlocks, "small-scratch layout and allocation disagree");

// Projections of a basis X (N x w) needed by the Sylvester rhs:
//   G = X^T X  (at dst, ld W),  P = X^T (T X)  (at dst + w*W, ld W).
// (The fast forms take G = I and compute P only.)
template <typename T>
__device__ __noinline__ void projections(const Inst<T>& I, const T* X, int N, int w, const T* tri, T* dst, Smem<T>& sm) {
  if (AssumeOrthonormal<T>::value) {
    tile_gram<T>(N, w, w, sm.stage, RowLoadPanel<T>{X, N, w}, RowLoadStencil<T>{X, N, N, w, tri},
                 dst + (int64_t)w * I.W, I.W, T(1), T(0));
  } else {
    tile_gram<T>(N, w, 2 * w, sm.stage, RowLoadPanel<T>{X, N, w}, RowLoadStencilAug<T>{X, N, N, w, tri}, dst, I.W,
                 T(1), T(0));
  }
}

// Orthonormalises the N x W panel Kp (global): the explicit Q goes to Qdst
// (ld N) and, when R is given, the triangular factor to R (ld ldr).  The
// panel is factored in shared memory when it fits in the staging area
// (which the QR does not otherwise use), else in place in global memory.
template <typename T>
__device__ __noinline__ void qr_panel(T* Kp, int N, int W, T* Qdst, T* R, int ldr, Smem<T>& sm) {
  const int off = NW * WMAX;  // hh_* keep their reduction scratch below this offset
  if ((int64_t)N * W <= (int64_t)(Stage<T>::ELEMS - off)) {
    T* A = sm.stage + off;
    for (int j = 0; j < W; ++j)
      for (int i = threadIdx.x; i < N; i += NT) A[i + j * N] = Kp[i + (int64_t)j * N];
    __syncthreads();
    hh_factor<T>(A, N, N, W, sm);
    if (R) extract_r<T>(A, N, W, R, ldr);
    hh_form_q_inplace<T>(A, N, N, W, sm);
    for (int j = 0; j < W; ++j)
      for (int i = threadIdx.x; i < N; i += NT) Qdst[i + (int64_t)j * N] = A[i + j * N];
    __syncthreads();
  } else {
    hh_factor<T>(Kp, N, N, W, sm);
    if (R) extract_r<T>(Kp, N, W, R, ldr);
    hh_form_q<T>(Kp, N, N, W, Qdst, N, sm);
  }
}

// CholeskyQR orthonormalisation of the fast forms: two passes for FP32 (the
// Gram accumulated in double-float from exact products keeps
// kappa^2 * u far below 1 for the FP32 class), three for double-float with
// the first pass shifted (Fukaya, Kannan, Nakatsukasa, Zhang, Yamamoto,
// SIAM J. Sci. Comput. 2020), stable up to kappa(K) ~ 1e11.  K <- K R^{-1} is
// a row-wise triangular solve, so the residual stays O(u ||K||).  Returns
// false (K unchanged, or restored) on a Cholesky breakdown; the caller then
// falls back to Householder.
template <typename T>
__device__ __noinline__ bool cholqr_panel(const Inst<T>& I, T* K, int N, int W, T* Qdst, T* R, int ldr,
                                          Smem<T>& sm) {
  dfloat* G = reinterpret_cast<dfloat*>(I.blk(B_SA));
  dfloat* Racc = reinterpret_cast<dfloat*>(I.blk(B_SZ1));
  dfloat* Rtmp = reinterpret_cast<dfloat*>(I.blk(B_T1));
  const bool shiftable = sizeof(T) != sizeof(float);
  int npass = 2;
  // 11 (N W + W (W+1)) u with u = 2^-44 for the double-float arithmetic
  const double shift = shiftable ? 11.0 * ((double)N * W + (double)W * (W + 1)) * 5.7e-14 : 0.0;
  if (R) copy_mat<T>(N, W, K, N, Qdst, N);  // backup of K for a late fallback
  for (int pass = 0; pass < npass; ++pass) {
    gram_df<T>(N, W, K, N, G, W, sm.stage);
    bool ok;
    if (pass == 0 && shiftable) {
      // plain CholeskyQR2 suffices while kappa(K)^2 u << 1; the spread of the
      // Cholesky diagonal bounds kappa(K) from below.  Beyond 1e6 (or on a
      // breakdown) restart from the saved Gram with the shift, three passes.
      for (int e = threadIdx.x; e < W * W; e += NT) Rtmp[e] = G[e];
      __syncthreads();
      ok = chol_df(W, G, W, 0.0, reinterpret_cast<dfloat*>(sm.stage));
      float dmax = 0.0f, dmin = 3.0e38f;
      for (int j = 0; j < W; ++j) {
        const float d = G[j + (int64_t)j * W].hi;
        dmax = fmaxf(dmax, d);
        dmin = fminf(dmin, d);
      }
      if (!ok || !(dmin > 0.0f) || dmax > 1.0e6f * dmin) {
        __syncthreads();
        for (int e = threadIdx.x; e < W * W; e += NT) G[e] = Rtmp[e];
        __syncthreads();
        ok = chol_df(W, G, W, shift, reinterpret_cast<dfloat*>(sm.stage));
        npass = 3;
      }
    } else {
      ok = chol_df(W, G, W, 0.0, reinterpret_cast<dfloat*>(sm.stage));
    }
    if (!ok) {
      if (pass > 0 && R) copy_mat<T>(N, W, Qdst, N, K, N);
      return false;
    }
    trsm_rows<T>(N, W, K, G, W, sm.stage, sm.vec);
    if (R) {
      if (pass == 0) {
        for (int e = threadIdx.x; e < W * W; e += NT) Racc[e] = ((e % W) <= (e / W)) ? G[e] : dfloat(0.0f, 0.0f);
        __syncthreads();
      } else {
        tri_mul_df(W, G, Racc, Rtmp);
        for (int e = threadIdx.x; e < W * W; e += NT) Racc[e] = Rtmp[e];
        __syncthreads();
      }
    }
  }
  copy_mat<T>(N, W, K, N, Qdst, N);
  if (R) {
    for (int e = threadIdx.x; e < W * W; e += NT) {
      const int i = e % W, j = e / W;
      T v;
      from_df(Racc[e], v);
      R[i + (int64_t)j * ldr] = v;
    }
    __syncthreads();
  }
  return true;
}

// Orthonormal basis of an N x W panel for BUG and KSL: shifted CholeskyQR3 in
// double-float, Householder QR (the reference's LAPACK algorithm) in FP32,
// plain FP64 and as the fallback.  (FP32 keeps Householder: the FP32 step's
// error budget is set by its reductions, and Householder's orthogonality
// error is the smaller of the two.)
template <typename T>
__device__ __noinline__ void orth_panel(const Inst<T>& I, T* Kp, int N, int W, T* Qdst, T* R, int ldr,
                                        Smem<T>& sm) {
  if constexpr (AssumeOrthonormal<T>::value && sizeof(T) == 8) {
    if (cholqr_panel<T>(I, Kp, N, W, Qdst, R, ldr, sm)) return;
  }
  qr_panel<T>(Kp, N, W, Qdst, R, ldr, sm);
}

// The registered local flow of the batch: the Burgers operator is flow 0.
template <typename T>
__device__ __forceinline__ int flow_id(const StepArgs<T>& g) {
  return g.op == OP_BURGERS ? 0 : g.flow;
}

// Local-flow (Burgers or registered) K (side 0) or L (side 1) substep on the panel Y (N x r, ld N):
// the scheme's stages one by one (the flow is nonlinear), each stage
// derivative k_s = F(Z_s V^T) V (K) or F(U Z_s^T)^T U (L) formed by
// flow_contract into the free QR panel; Xo is the other side's basis.
template <typename T>
__device__ __noinline__ void burgers_panel_rk(const StepArgs<T>& g, const Inst<T>& I, const Side<T>& sd, int side,
                                              T* Y, int r, const T* Xo, const Scheme& sc, double dt, Smem<T>& sm) {
  const int N = sd.N;
  const T* nu = I.l.tri;  // operator B: per-column viscosities (m)
  T* Kst = sd.PQ;
  T* A = sd.PA;
  T* Zb[2] = {sd.PZ0, sd.PZ1};
  const int ns = sc.nstages;
  const T h = T(dt / sc.nsub);
  const int64_t NR = (int64_t)N * r;
  for (int sub = 0; sub < sc.nsub; ++sub) {
    for (int s = 0; s < ns; ++s) {
      const T* Z = (s == 0) ? Y : Zb[(s - 1) & 1];
      with_local_flow(flow_id(g), [&](auto flow) {
        using Flow = decltype(flow);
        if (side == 0)
          flow_contract<T, Flow>(BURG_K, I.n, I.m, r, Z, Xo, nullptr, 0, nu, g.bh, g.balpha, g.bbeta, T(1), Kst,
                                 N, sm.stage);
        else
          flow_contract<T, Flow>(BURG_L, I.n, I.m, r, Xo, Z, nullptr, 0, nu, g.bh, g.balpha, g.bbeta, T(1), Kst,
                                 N, sm.stage);
      });
      const T bs = T(sc.b[s]);
      const T an = (s + 1 < ns) ? T(sc.a[s + 1]) : T(0);
      T* Zout = Zb[s & 1];
      for (int64_t o = threadIdx.x; o < NR; o += NT) {
        const T kv = Kst[o];
        if (ns == 1) {
          Y[o] = fma(h * bs, kv, Y[o]);
        } else if (s == 0) {
          A[o] = bs * kv;
          Zout[o] = fma(h * an, kv, Y[o]);
        } else if (s + 1 < ns) {
          A[o] = fma(bs, kv, A[o]);
          Zout[o] = fma(h * an, kv, Y[o]);
        } else {
          Y[o] = fma(h, fma(bs, kv, A[o]), Y[o]);
        }
      }
      __syncthreads();
    }
  }
}

// One substep of side `sd` on the panel Y (N x r, ld N), in place.
//   Sylvester: Y' = T Y G + Y P^T  with (G, P) the projections of the other
//              side's basis (K: V^T V, V^T B V; L: U^T U, U^T A U).
//   Data:      Y += Δy Xo (K side) or Δy^T Xo (L side).
//   Zero:      nothing.
template <typename T>
__device__ void substep_side(const StepArgs<T>& g, const Inst<T>& I, const Side<T>& sd, int side, T* Y, int r,
                             const T* Gp, const T* Xo, const Scheme& sc, double dt, Smem<T>& sm) {
  const int N = sd.N;
  if (g.op == OP_ZERO) return;
  if (g.op == OP_BURGERS || g.op == OP_LOCAL) {
    burgers_panel_rk<T>(g, I, sd, side, Y, r, Xo, sc, dt, sm);
    return;
  }
  if (g.op == OP_DATA) {
    const int a = (side == 0) ? I.m : I.n;
    const int ldo = (side == 0) ? I.m : I.n;
    tile_gemm<T>(N, a, r, sm.stage, LoadDelta<T>{I.Yn, I.Yp, I.n, side == 1}, LoadSmall<T>{Xo, ldo, false},
                 EpiAdd<T>{Y, N});
    return;
  }
  // Sylvester tridiagonal: the rhs L(Y) = T Y G + Y P^T is linear and
  // autonomous, so any explicit RK scheme with a sub-diagonal tableau maps
  // y -> R(hL) y with the stability polynomial R(z) = 1 + sum_j gamma_j z^j,
  //   gamma_{j+1} = sum_{s>=j} b_s * a_s a_{s-1} ... a_{s-j+1}.
  // Horner: w = gamma_ns y;  w = gamma_j y + h L(w) (j = ns-1..1);
  // y1 = y + h L(w): ns applications of L, as many as the stages, without
  // an accumulator panel.  (Equal to the stage-by-stage scheme up to
  // rounding.)
  const T* G = Gp;
  const T* P = Gp + (int64_t)r * I.W;
  const int ns = sc.nstages;
  constexpr bool ortho = AssumeOrthonormal<T>::value;
  double gam[5];
  horner_coeffs(sc, gam);
  const T h = T(dt / sc.nsub);
  // short panels: the whole substep interval with the rows in registers
  if (reg_substep<T, ortho>(N, r, Y, sd.tri, G, P, I.W, gam, ns, sc.nsub, h, sm.stage)) return;
  T* Zb[2] = {sd.PZ0, sd.PZ1};
  for (int sub = 0; sub < sc.nsub; ++sub) {
    // the first application acts on gamma_ns * y: fold gamma_ns into h
    const T* win = Y;
    T hw = h * T(gam[ns]);
    for (int j = ns - 1; j >= 0; --j) {
      T* wout = (j == 0) ? ((ns == 1) ? Zb[0] : Y) : Zb[(ns - 1 - j) & 1];
      const T gj = (j == 0) ? T(1) : T(gam[j]);
      if constexpr (ortho) {
        tile_sylv<T>(N, r, win, sd.tri, P, I.W, wout, Y, gj, hw, sm.stage);
      } else {
        tile_gemm<T>(N, 2 * r, r, sm.stage, LoadStencilAug<T>{win, N, N, r, sd.tri}, LoadGP<T>{G, P, I.W, r},
                     EpiAxpby<T>{wout, Y, N, gj, hw});
      }
      win = wout;
      hw = h;
    }
    if (ns == 1) copy_mat<T>(N, r, Zb[0], N, Y, N);
  }
}

// S-substep on the p x q core St (ld W):
//   Sylvester: S' = sign * (P_U S G_V + G_U S P_V^T)
//   Data:      S += sign * U^T Δy V   (exact flow)
template <typename T>
__device__ __noinline__ void substep_core(const StepArgs<T>& g, const Inst<T>& I, T* St, int p, int q, T sign, const T* GUp,
                             const T* GVp, const T* Ub, const T* Vb, const Scheme& sc, double dt, Smem<T>& sm) {
  const int W = I.W;
  if (g.op == OP_ZERO) return;
  if (g.op == OP_DATA) {
    // Z = Δy V (n x q) into the K-side QR panel (free at this point), then St += sign * U^T Z
    T* Z = I.k.PY;
    const int n = I.n;
    tile_gemm<T>(n, I.m, q, sm.stage, LoadDelta<T>{I.Yn, I.Yp, n, false}, LoadSmall<T>{Vb, I.m, false},
                 EpiStore<T>{Z, n});
    tile_gram<T>(n, p, q, sm.stage, RowLoadPanel<T>{Ub, n, p}, RowLoadPanel<T>{Z, n, q}, St, W, sign, T(1));
    return;
  }
  if (g.op == OP_BURGERS || g.op == OP_LOCAL) {
    // k_s = sign * U^T F(U Z_s V^T) V with U Z_s formed in the free K-side
    // QR panel (n x q), stages one by one
    T* XLp = I.k.PY;
    T* SAb = I.blk(B_SA);
    T* SZb[2] = {I.blk(B_SZ0), I.blk(B_SZ1)};
    T* SKb = I.blk(B_SK);
    const int ns = sc.nstages;
    const T h = T(dt / sc.nsub);
    for (int sub = 0; sub < sc.nsub; ++sub) {
      for (int s = 0; s < ns; ++s) {
        const T* Z = (s == 0) ? St : SZb[(s - 1) & 1];
        tile_gemm<T>(I.n, p, q, sm.stage, LoadPanel<T>{Ub, I.n}, LoadSmall<T>{Z, W, false}, EpiStore<T>{XLp, I.n});
        with_local_flow(flow_id(g), [&](auto flow) {
          flow_contract<T, decltype(flow)>(BURG_S, I.n, I.m, q, XLp, Vb, Ub, p, I.l.tri, g.bh, g.balpha, g.bbeta,
                                           sign, SKb, W, sm.stage);
        });
        const T bs = T(sc.b[s]);
        const T an = (s + 1 < ns) ? T(sc.a[s + 1]) : T(0);
        T* Zout = SZb[s & 1];
        for (int o = threadIdx.x; o < p * q; o += NT) {
          const int64_t idx = (o % p) + (int64_t)(o / p) * W;
          const T kv = SKb[idx];
          if (ns == 1) {
            St[idx] = fma(h * bs, kv, St[idx]);
          } else if (s == 0) {
            SAb[idx] = bs * kv;
            Zout[idx] = fma(h * an, kv, St[idx]);
          } else if (s + 1 < ns) {
            SAb[idx] = fma(bs, kv, SAb[idx]);
            Zout[idx] = fma(h * an, kv, St[idx]);
          } else {
            St[idx] = fma(h, fma(bs, kv, SAb[idx]), St[idx]);
          }
        }
        __syncthreads();
      }
    }
    return;
  }
  if (p * q <= NT && p <= 16 && q <= 16) {
    // small cores: state in registers, one or two barriers per stage
    core_small<T, AssumeOrthonormal<T>::value>(p, q, W, St, sign, GUp, GUp + (int64_t)p * W, GVp,
                                               GVp + (int64_t)q * W, sc, T(dt / sc.nsub), sm.stage);
    return;
  }
  const T* GU = GUp;
  const T* PU = GUp + (int64_t)p * W;
  const T* GV = GVp;
  const T* PV = GVp + (int64_t)q * W;
  T* SA = I.blk(B_SA);
  T* SZ[2] = {I.blk(B_SZ0), I.blk(B_SZ1)};
  T* SK = I.blk(B_SK);
  T* T1 = I.blk(B_T1);
  T* T2 = I.blk(B_T2);
  // Orthonormal forms: stage P_U, P_V, the state and the four work
  // matrices in shared memory when they fit (the products then read shared
  // memory instead of L1/L2).
  T* Sg = St;
  if (AssumeOrthonormal<T>::value && 7 * W * W <= Stage<T>::ELEMS) {
    T* base = sm.stage;
    T* PUs = base;
    T* PVs = base + W * W;
    T* Ss = base + 2 * W * W;
    copy_mat<T>(p, p, PU, W, PUs, W);
    copy_mat<T>(q, q, PV, W, PVs, W);
    copy_mat<T>(p, q, St, W, Ss, W);
    PU = PUs;
    PV = PVs;
    St = Ss;
    SZ[0] = base + 3 * W * W;
    SZ[1] = base + 4 * W * W;
    SK = base + 5 * W * W;
    SA = base + 6 * W * W;
  }
  const int ns = sc.nstages;
  const T h = T(dt / sc.nsub);
  for (int sub = 0; sub < sc.nsub; ++sub) {
    for (int s = 0; s < ns; ++s) {
      const T* Z = (s == 0) ? St : SZ[(s - 1) & 1];
      if (AssumeOrthonormal<T>::value) {
        // SK = sign * (PU Z + Z PV^T)
        small_gemm<T>(p, p, q, sign, PU, W, false, Z, W, false, T(0), SK, W);
        small_gemm<T>(p, q, q, sign, Z, W, false, PV, W, true, T(1), SK, W);
      } else {
        // SK = sign * (PU (Z GV) + GU (Z PV^T))
        small_gemm<T>(p, q, q, T(1), Z, W, false, GV, W, false, T(0), T1, W);
        small_gemm<T>(p, q, q, T(1), Z, W, false, PV, W, true, T(0), T2, W);
        small_gemm<T>(p, p, q, sign, PU, W, false, T1, W, false, T(0), SK, W);
        small_gemm<T>(p, p, q, sign, GU, W, false, T2, W, false, T(1), SK, W);
      }
      const T bs = T(sc.b[s]);
      const T an = (s + 1 < ns) ? T(sc.a[s + 1]) : T(0);
      T* Zout = SZ[s & 1];
      for (int o = threadIdx.x; o < p * q; o += NT) {
        const int i = o % p, j = o / p;
        const int64_t idx = i + (int64_t)j * W;
        const T kv = SK[idx];
        if (ns == 1) {
          St[idx] = fma(h * bs, kv, St[idx]);
        } else if (s == 0) {
          SA[idx] = bs * kv;
          Zout[idx] = fma(h * an, kv, St[idx]);
        } else if (s + 1 < ns) {
          SA[idx] = fma(bs, kv, SA[idx]);
          Zout[idx] = fma(h * an, kv, St[idx]);
        } else {
          St[idx] = fma(h, fma(bs, kv, SA[idx]), St[idx]);
        }
      }
      __syncthreads();
    }
  }
  if (St != Sg) copy_mat<T>(p, q, St, W, Sg, W);
}

// K0 = X * C (C = S, or S^T when trans) into panel Y (N x r).
template <typename T>
__device__ void form_k0(const Inst<T>& I, const T* X, int N, const T* C, int ldc, bool trans, T* Y, int r,
                        Smem<T>& sm) {
  tile_gemm<T>(N, r, r, sm.stage, LoadPanel<T>{X, N}, LoadSmall<T>{C, ldc, trans}, EpiStore<T>{Y, N});
}

// K0 = X C followed by the substep, into the panel Y (N x r): fused in
// shared memory for the orthonormal-basis Sylvester flow when the tile fits,
// else the panel product and the panel-by-panel substep.
template <typename T>
__device__ __noinline__ void k_step(const StepArgs<T>& g, const Inst<T>& I, const Side<T>& sd, int side,
                                    const T* X, const T* C, int ldc, bool transC, T* Y, int r, const T* Gp,
                                    const T* Xo, const Scheme& sc, double dt, Smem<T>& sm) {
  const int N = sd.N;
  // (float only: for double-float the halo recomputation costs more
  // arithmetic than the saved panel passes are worth)
  if constexpr (AssumeOrthonormal<T>::value && sizeof(T) == 4) {
    if (g.op == OP_SYLVESTER && sc.nstages * sc.nsub <= 8) {
      double gam[5];
      horner_coeffs(sc, gam);
      const T* P = Gp + (int64_t)r * I.W;
      if (fused_substep<T>(N, r, X, N, C, ldc, transC, sd.tri, P, I.W, gam, sc.nstages, sc.nsub,
                           T(dt / sc.nsub), Y, sm.stage))
        return;
    }
  }
  form_k0<T>(I, X, N, C, ldc, transC, Y, r, sm);
  substep_side<T>(g, I, sd, side, Y, r, Gp, Xo, sc, dt, sm);
}

template <typename T>
__device__ void check_finite(const StepArgs<T>& g, const T* S, int r, int ld) {
  __shared__ int bad;
  if (threadIdx.x == 0) bad = 0;
  __syncthreads();
  for (int o = threadIdx.x; o < r * r; o += NT)
    if (!is_finite_val(S[(o % r) + (int64_t)(o / r) * ld])) bad = 1;
  __syncthreads();
  if (threadIdx.x == 0 && bad) atomicOr(g.status, ST_NONFINITE);
  __syncthreads();
}

// non-finite entries of an N x r panel (ld N) -> status
template <typename T>
__device__ void check_finite_panel(const StepArgs<T>& g, const T* X, int N, int r) {
  const int64_t len = (int64_t)N * r;
  bool bad = false;
  for (int64_t o = threadIdx.x; o < len; o += NT) bad |= !is_finite_val(X[o]);
  if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(g.status, ST_NONFINITE);
}

// S-step of the FP32 class in double-float (Sylvester flow, orthonormal
// bases): S0 = M S N^T from the FP32 core and the double-float basis
// changes, then the substeps of S' = P_U S + S P_V^T in Horner form (the
// K/L substeps' form) on double-float P_U, P_V; the result is rounded into
// the FP32 core.  Everything is staged in shared memory (5 r^2 double-float
// values).  The FP32 step's rounding error is otherwise dominated by these
// r x r reductions and the core update, not by the panel arithmetic.
static __device__ __noinline__ void core_bug_acc(const Inst<float>& I, int r, const dfloat* Md, const dfloat* Nd,
                                          const dfloat* PUd, const dfloat* PVd, const Scheme& sc, double dt,
                                          Smem<float>& sm) {
  const int W = I.W, rr = r * r;
  dfloat* PUs = reinterpret_cast<dfloat*>(sm.stage);
  dfloat* PVs = PUs + rr;
  dfloat* Ss = PUs + 2 * rr;
  dfloat* Wa = PUs + 3 * rr;
  dfloat* Wb = PUs + 4 * rr;
  for (int o = threadIdx.x; o < rr; o += NT) {
    const int i = o % r, j = o / r;
    PUs[o] = PUd[i + (int64_t)j * W];
    PVs[o] = PVd[i + (int64_t)j * W];
    Wb[o] = dfloat(I.S[i + (int64_t)j * I.rcap]);
  }
  __syncthreads();
  // Wa = S N^T
  for (int o = threadIdx.x; o < rr; o += NT) {
    const int i = o % r, j = o / r;
    dfloat acc(0.0f, 0.0f);
    for (int k = 0; k < r; ++k) acc = fma_acc(Wb[i + k * r], Nd[j + (int64_t)k * W], acc);
    Wa[o] = renorm(acc);
  }
  __syncthreads();
  // Ss = M Wa
  for (int o = threadIdx.x; o < rr; o += NT) {
    const int i = o % r, j = o / r;
    dfloat acc(0.0f, 0.0f);
    for (int k = 0; k < r; ++k) acc = fma_acc(Md[i + (int64_t)k * W], Wa[k + j * r], acc);
    Ss[o] = renorm(acc);
  }
  __syncthreads();
  double gam[5];
  horner_coeffs(sc, gam);
  const int ns = sc.nstages;
  const dfloat h(dt / sc.nsub);
  for (int sub = 0; sub < sc.nsub; ++sub) {
    // w = gam_ns S;  w <- gam_j S + h L(w) (j = ns-1 .. 0, gam_0 = 1)
    const dfloat* win = Ss;
    dfloat hw = h * dfloat(gam[ns]);
    for (int j = ns - 1; j >= 0; --j) {
      dfloat* wout = (win == Wa) ? Wb : Wa;
      const dfloat gj = (j == 0) ? dfloat(1.0f, 0.0f) : dfloat(gam[j]);
      for (int o = threadIdx.x; o < rr; o += NT) {
        const int i = o % r, c = o / r;
        dfloat l(0.0f, 0.0f);
        for (int k = 0; k < r; ++k) {
          l = fma_acc(PUs[i + k * r], win[k + c * r], l);
          l = fma_acc(win[i + k * r], PVs[c + k * r], l);
        }
        wout[o] = fma(hw, renorm(l), gj * Ss[o]);
      }
      __syncthreads();
      win = wout;
      hw = h;
    }
    for (int o = threadIdx.x; o < rr; o += NT) Ss[o] = win[o];
    __syncthreads();
  }
  for (int o = threadIdx.x; o < rr; o += NT) {
    const int i = o % r, j = o / r;
    I.S[i + (int64_t)j * I.rcap] = Ss[o].hi + Ss[o].lo;
  }
  __syncthreads();
}

// ---------------------------------------------------------------------------
// BUG (unconventional integrator) step
// ---------------------------------------------------------------------------
template <typename T>
__device__ __noinline__ void bug_step(const StepArgs<T>& g, Inst<T>& I, int r, Smem<T>& sm) {
  const int n = I.n, m = I.m, W = I.W;
  T* GU = I.blk(B_GU);
  T* GV = I.blk(B_GV);
  T* Mm = I.blk(B_M);
  T* Nm = I.blk(B_N);
  T* St = I.blk(B_ST);
  T* T1 = I.blk(B_T1);
  const bool sylv = (g.op == OP_SYLVESTER);
  // fast forms: fuse the basis change M (resp. N) with the projection of the
  // new basis, written to the otherwise unused KSL blocks until the swap
  const bool fuse = sylv && AssumeOrthonormal<T>::value && 2 * r <= 128;
  T* PUn = I.blk(B_RK);
  T* PVn = I.blk(B_RL);
  // FP32 class: the basis changes, the new projections and the S-step in
  // double-float (their FP32 rounding errors dominate the FP32 step's)
  bool acc = false;
  if constexpr (sizeof(T) == 4) acc = fuse && ((r + 3) >> 2) * ((2 * r + 3) >> 2) <= NT &&
                                      5 * r * r * 2 <= Stage<T>::ELEMS;
  dfloat* DM = reinterpret_cast<dfloat*>(I.blk(B_DM));
  dfloat* DN = reinterpret_cast<dfloat*>(I.blk(B_DN));
  dfloat* DPU = reinterpret_cast<dfloat*>(I.blk(B_DPU));
  dfloat* DPV = reinterpret_cast<dfloat*>(I.blk(B_DPV));
  if (sylv && g.proj_valid[I.inst] == 0) {
    projections<T>(I, I.U, n, r, I.k.tri, GU, sm);
    projections<T>(I, I.V, m, r, I.l.tri, GV, sm);
  }
  // K step (unconventional.jl:136-142)
  k_step<T>(g, I, I.k, 0, I.U, I.S, I.rcap, false, I.k.PY, r, GV, I.V, g.sK, g.dt, sm);
  orth_panel<T>(I, I.k.PY, n, r, I.k.PQ, nullptr, 0, sm);
  bool done = false;
  if constexpr (sizeof(T) == 4) {
    if (acc) {
      tile_gram_acc(n, r, 2 * r, sm.stage, RowLoadPanel<T>{I.k.PQ, n, r},
                    RowLoadPanelStencil<T>{I.U, n, I.k.PQ, n, n, r, I.k.tri}, DM, DPU, nullptr, PUn, W, r);
      done = true;
    }
  }
  if (done) {
  } else if (fuse) {
    // one pass over Q_K: [M | P_U(new)] = Q_K^T [U0 | A Q_K]
    tile_gram<T>(n, r, 2 * r, sm.stage, RowLoadPanel<T>{I.k.PQ, n, r},
                 RowLoadPanelStencil<T>{I.U, n, I.k.PQ, n, n, r, I.k.tri}, Mm, W, T(1), T(0), PUn, r);
  } else {
    tile_gram<T>(n, r, r, sm.stage, RowLoadPanel<T>{I.k.PQ, n, r}, RowLoadPanel<T>{I.U, n, r}, Mm, W, T(1), T(0));
  }
  // L step (unconventional.jl:144-150), still with the old U
  k_step<T>(g, I, I.l, 1, I.V, I.S, I.rcap, true, I.l.PY, r, GU, I.U, g.sL, g.dt, sm);
  orth_panel<T>(I, I.l.PY, m, r, I.l.PQ, nullptr, 0, sm);
  if constexpr (sizeof(T) == 4) {
    if (acc) {
      tile_gram_acc(m, r, 2 * r, sm.stage, RowLoadPanel<T>{I.l.PQ, m, r},
                    RowLoadPanelStencil<T>{I.V, m, I.l.PQ, m, m, r, I.l.tri}, DN, DPV, nullptr, PVn, W, r);
    }
  }
  if (done) {
  } else if (fuse) {
    tile_gram<T>(m, r, 2 * r, sm.stage, RowLoadPanel<T>{I.l.PQ, m, r},
                 RowLoadPanelStencil<T>{I.V, m, I.l.PQ, m, m, r, I.l.tri}, Nm, W, T(1), T(0), PVn, r);
  } else {
    tile_gram<T>(m, r, r, sm.stage, RowLoadPanel<T>{I.l.PQ, m, r}, RowLoadPanel<T>{I.V, m, r}, Nm, W, T(1), T(0));
  }
  // basis swap (unconventional.jl:151-152)
  copy_mat<T>(n, r, I.k.PQ, n, I.U, n);
  copy_mat<T>(m, r, I.l.PQ, m, I.V, m);
  if (fuse) {
    copy_mat<T>(r, r, PUn, W, GU + (int64_t)r * W, W);
    copy_mat<T>(r, r, PVn, W, GV + (int64_t)r * W, W);
    if (threadIdx.x == 0) g.proj_valid[I.inst] = 1;
  } else if (sylv) {
    projections<T>(I, I.U, n, r, I.k.tri, GU, sm);
    projections<T>(I, I.V, m, r, I.l.tri, GV, sm);
    if (threadIdx.x == 0) g.proj_valid[I.inst] = 1;
  }
  // S step on the new bases (unconventional.jl:154-156): S0 = M S N^T
  if constexpr (sizeof(T) == 4) {
    if (acc) {
      core_bug_acc(I, r, DM, DN, DPU, DPV, g.sS, g.dt, sm);
      check_finite<T>(g, I.S, r, I.rcap);
      return;
    }
  }
  small_gemm<T>(r, r, r, T(1), I.S, I.rcap, false, Nm, W, true, T(0), T1, W);
  small_gemm<T>(r, r, r, T(1), Mm, W, false, T1, W, false, T(0), St, W);
  substep_core<T>(g, I, St, r, r, T(1), GU, GV, I.U, I.V, g.sS, g.dt, sm);
  copy_mat<T>(r, r, St, W, I.S, I.rcap);
  check_finite<T>(g, I.S, r, I.rcap);
}

// BUG step of one FP64 Sylvester instance on a 2-CTA thread-block cluster
// (batches small enough for two SMs per instance): the K and L steps read
// only the old factors, so CTA 0 runs the K step and CTA 1 the L step; then
// each swaps in its new basis and its projections; then CTA 0 runs the S
// step.  The same operations as bug_step's literal (FP64) form.  Cluster
// barriers (each after a __threadfence) separate the three phases, and both
// CTAs reach both barriers.
template <typename T>
__device__ __noinline__ void bug_step_pair(const StepArgs<T>& g, Inst<T>& I, int r, Smem<T>& sm) {
  namespace cg = cooperative_groups;
  const int n = I.n, m = I.m, W = I.W;
  const bool kside = cg::this_cluster().block_rank() == 0;
  T* GU = I.blk(B_GU);
  T* GV = I.blk(B_GV);
  T* Mm = I.blk(B_M);
  T* Nm = I.blk(B_N);
  T* St = I.blk(B_ST);
  T* T1 = I.blk(B_T1);
  // both CTAs read the flag before the first barrier; CTA 0 sets it after
  const bool fresh = g.proj_valid[I.inst] == 0;
  if (kside) {
    // K step (unconventional.jl:136-142) with the projections of the old V
    if (fresh) projections<T>(I, I.V, m, r, I.l.tri, GV, sm);
    k_step<T>(g, I, I.k, 0, I.U, I.S, I.rcap, false, I.k.PY, r, GV, I.V, g.sK, g.dt, sm);
    orth_panel<T>(I, I.k.PY, n, r, I.k.PQ, nullptr, 0, sm);
    tile_gram<T>(n, r, r, sm.stage, RowLoadPanel<T>{I.k.PQ, n, r}, RowLoadPanel<T>{I.U, n, r}, Mm, W, T(1), T(0));
  } else {
    // L step (unconventional.jl:144-150) with the projections of the old U
    if (fresh) projections<T>(I, I.U, n, r, I.k.tri, GU, sm);
    k_step<T>(g, I, I.l, 1, I.V, I.S, I.rcap, true, I.l.PY, r, GU, I.U, g.sL, g.dt, sm);
    orth_panel<T>(I, I.l.PY, m, r, I.l.PQ, nullptr, 0, sm);
    tile_gram<T>(m, r, r, sm.stage, RowLoadPanel<T>{I.l.PQ, m, r}, RowLoadPanel<T>{I.V, m, r}, Nm, W, T(1), T(0));
  }
  __threadfence();
  cg::this_cluster().sync();
  // basis swap (unconventional.jl:151-152) and the new bases' projections
  if (kside) {
    copy_mat<T>(n, r, I.k.PQ, n, I.U, n);
    projections<T>(I, I.U, n, r, I.k.tri, GU, sm);
    if (threadIdx.x == 0) g.proj_valid[I.inst] = 1;
  } else {
    copy_mat<T>(m, r, I.l.PQ, m, I.V, m);
    projections<T>(I, I.V, m, r, I.l.tri, GV, sm);
  }
  __threadfence();
  cg::this_cluster().sync();
  // S step on the new bases (unconventional.jl:154-156): S0 = M S N^T
  if (kside) {
    small_gemm<T>(r, r, r, T(1), I.S, I.rcap, false, Nm, W, true, T(0), T1, W);
    small_gemm<T>(r, r, r, T(1), Mm, W, false, T1, W, false, T(0), St, W);
    substep_core<T>(g, I, St, r, r, T(1), GU, GV, I.U, I.V, g.sS, g.dt, sm);
    copy_mat<T>(r, r, St, W, I.S, I.rcap);
    check_finite<T>(g, I.S, r, I.rcap);
  }
}

// ---------------------------------------------------------------------------
// Rank-adaptive BUG step
// ---------------------------------------------------------------------------
template <typename T>
__device__ __noinline__ void ra_bug_step(const StepArgs<T>& g, Inst<T>& I, int r, Smem<T>& sm) {
  const int n = I.n, m = I.m, W = I.W;
  const int w2 = 2 * r;
  T* GU = I.blk(B_GU);
  T* GV = I.blk(B_GV);
  T* Mm = I.blk(B_M);
  T* Nm = I.blk(B_N);
  T* St = I.blk(B_ST);
  T* T1 = I.blk(B_T1);
  T* T2 = I.blk(B_T2);
  const bool sylv = (g.op == OP_SYLVESTER);
  if (sylv) {
    projections<T>(I, I.U, n, r, I.k.tri, GU, sm);
    projections<T>(I, I.V, m, r, I.l.tri, GV, sm);
  }
  // K step: Uhat = orth([K1 | U0]) (rank_adaptive_unconventional.jl:197-206)
  k_step<T>(g, I, I.k, 0, I.U, I.S, I.rcap, false, I.k.PY, r, GV, I.V, g.sK, g.dt, sm);
  copy_mat<T>(n, r, I.U, n, I.k.PY + (int64_t)r * n, n);
  qr_panel<T>(I.k.PY, n, w2, I.k.PQ, nullptr, 0, sm);
  tile_gram<T>(n, w2, r, sm.stage, RowLoadPanel<T>{I.k.PQ, n, w2}, RowLoadPanel<T>{I.U, n, r}, Mm, W, T(1), T(0));
  // L step (:208-217)
  k_step<T>(g, I, I.l, 1, I.V, I.S, I.rcap, true, I.l.PY, r, GU, I.U, g.sL, g.dt, sm);
  copy_mat<T>(m, r, I.V, m, I.l.PY + (int64_t)r * m, m);
  qr_panel<T>(I.l.PY, m, w2, I.l.PQ, nullptr, 0, sm);
  tile_gram<T>(m, w2, r, sm.stage, RowLoadPanel<T>{I.l.PQ, m, w2}, RowLoadPanel<T>{I.V, m, r}, Nm, W, T(1), T(0));
  // S step on the augmented bases (:219-220)
  if (sylv) {
    projections<T>(I, I.k.PQ, n, w2, I.k.tri, GU, sm);
    projections<T>(I, I.l.PQ, m, w2, I.l.tri, GV, sm);
  }
  small_gemm<T>(r, r, w2, T(1), I.S, I.rcap, false, Nm, W, true, T(0), T1, W);   // S N^T  (r x 2r)
  small_gemm<T>(w2, r, w2, T(1), Mm, W, false, T1, W, false, T(0), St, W);       // M S N^T (2r x 2r)
  substep_core<T>(g, I, St, w2, w2, T(1), GU, GV, I.k.PQ, I.l.PQ, g.sS, g.dt, sm);
  // SVD of the core and truncation (:222-231)
  T* a = sm.stage;
  T* v = sm.stage + w2 * w2;
  int* perm = reinterpret_cast<int*>(sm.stage + 2 * w2 * w2);
  int* flag = perm + w2 + 1;
  T* sigma = sm.vec;
  for (int o = threadIdx.x; o < w2 * w2; o += NT) a[o] = St[(o % w2) + (int64_t)(o / w2) * W];
  __syncthreads();
  const bool ok = jacobi_svd<T>(w2, a, v, sigma, perm, flag);
  __shared__ int r_new_s;
  if (threadIdx.x == 0) {
    if (!ok) atomicOr(g.status, ST_SVD_NOCONV);
    // truncate_to_tolerance: smallest r1 with sum_{j>r1} s_j^2 < tol^2 (at least 1)
    const double tol2 = g.tol * g.tol;
    double acc = 0.0;
    int rr = w2;
    while (acc < tol2 && rr > 0) {
      const double s = (double)sigma[perm[rr - 1]];
      acc += s * s;
      --rr;
    }
    int r1 = rr + 1;
    if (r1 > I.rcap) r1 = I.rcap;   // min(r_max, .)
    if (r1 < g.r_min) r1 = g.r_min;
    if (r1 > w2) r1 = w2;
    r_new_s = r1;
  }
  __syncthreads();
  const int r1 = r_new_s;
  // left vectors a_j / sigma_j in place (T1 as scratch)
  complete_left<T>(w2, r1, a, sigma, perm, T1);
  // P1 = left vectors (2r x r1) into T1, Q1 = right vectors into T2; sorted
  // singular values into sm.vec[WMAX..] (the staging area is reused below)
  T* sig_sorted = sm.vec + WMAX;
  for (int o = threadIdx.x; o < w2 * r1; o += NT) {
    const int i = o % w2, j = o / w2;
    const int pj = perm[j];
    T1[i + (int64_t)j * W] = a[i + pj * w2];
    T2[i + (int64_t)j * W] = v[i + pj * w2];
  }
  for (int j = threadIdx.x; j < r1; j += NT) sig_sorted[j] = sigma[perm[j]];
  __syncthreads();
  // new factors: U = Uhat P1, V = Vhat Q1, S = diag(sigma) (:224-231)
  tile_gemm<T>(n, w2, r1, sm.stage, LoadPanel<T>{I.k.PQ, n}, LoadSmall<T>{T1, W, false}, EpiStore<T>{I.U, n});
  tile_gemm<T>(m, w2, r1, sm.stage, LoadPanel<T>{I.l.PQ, m}, LoadSmall<T>{T2, W, false}, EpiStore<T>{I.V, m});
  // sig_sorted lives in sm.vec, which the products above do not touch
  for (int o = threadIdx.x; o < I.rcap * I.rcap; o += NT) {
    const int i = o % I.rcap, j = o / I.rcap;
    I.S[o] = (i == j && i < r1) ? sig_sorted[i] : T(0);
  }
  if (threadIdx.x == 0) g.rank[I.inst] = r1;
  __syncthreads();
  check_finite<T>(g, I.S, r1, I.rcap);
}

// ---------------------------------------------------------------------------
// Projector-splitting (KSL) half steps
// ---------------------------------------------------------------------------
template <typename T>
__device__ __noinline__ void ksl_primal(const StepArgs<T>& g, Inst<T>& I, int r, double dt, Smem<T>& sm) {
  const int n = I.n, m = I.m, W = I.W;
  T* GU = I.blk(B_GU);
  T* GV = I.blk(B_GV);
  T* St = I.blk(B_ST);
  T* RK = I.blk(B_RK);
  T* RL = I.blk(B_RL);
  const bool sylv = (g.op == OP_SYLVESTER);
  if (sylv) projections<T>(I, I.V, m, r, I.l.tri, GV, sm);
  // K step (projector_splitting.jl:133-138)
  k_step<T>(g, I, I.k, 0, I.U, I.S, I.rcap, false, I.k.PY, r, GV, I.V, g.sK, dt, sm);
  orth_panel<T>(I, I.k.PY, n, r, I.k.PQ, RK, W, sm);
  copy_mat<T>(n, r, I.k.PQ, n, I.U, n);
  if (sylv) projections<T>(I, I.U, n, r, I.k.tri, GU, sm);
  // S step, backward in time (:141-142; rhs negated at :64)
  copy_mat<T>(r, r, RK, W, St, W);
  substep_core<T>(g, I, St, r, r, T(-1), GU, GV, I.U, I.V, g.sS, dt, sm);
  // L step (:145-151)
  k_step<T>(g, I, I.l, 1, I.V, St, W, true, I.l.PY, r, GU, I.U, g.sL, dt, sm);
  orth_panel<T>(I, I.l.PY, m, r, I.l.PQ, RL, W, sm);
  copy_mat<T>(m, r, I.l.PQ, m, I.V, m);
  // S = R^T
  for (int o = threadIdx.x; o < r * r; o += NT) {
    const int i = o % r, j = o / r;
    I.S[i + (int64_t)j * I.rcap] = RL[j + (int64_t)i * W];
  }
  __syncthreads();
}

template <typename T>
__device__ __noinline__ void ksl_dual(const StepArgs<T>& g, Inst<T>& I, int r, double dt, Smem<T>& sm) {
  const int n = I.n, m = I.m, W = I.W;
  T* GU = I.blk(B_GU);
  T* GV = I.blk(B_GV);
  T* St = I.blk(B_ST);
  T* RK = I.blk(B_RK);
  T* RL = I.blk(B_RL);
  const bool sylv = (g.op == OP_SYLVESTER);
  if (sylv) projections<T>(I, I.U, n, r, I.k.tri, GU, sm);
  // L step (projector_splitting.jl:170-175)
  k_step<T>(g, I, I.l, 1, I.V, I.S, I.rcap, true, I.l.PY, r, GU, I.U, g.sL, dt, sm);
  orth_panel<T>(I, I.l.PY, m, r, I.l.PQ, RL, W, sm);
  copy_mat<T>(m, r, I.l.PQ, m, I.V, m);
  if (sylv) projections<T>(I, I.V, m, r, I.l.tri, GV, sm);
  // S step backward from R^T (:178-179)
  for (int o = threadIdx.x; o < r * r; o += NT) {
    const int i = o % r, j = o / r;
    St[i + (int64_t)j * W] = RL[j + (int64_t)i * W];
  }
  __syncthreads();
  substep_core<T>(g, I, St, r, r, T(-1), GU, GV, I.U, I.V, g.sS, dt, sm);
  // K step (:182-188)
  k_step<T>(g, I, I.k, 0, I.U, St, W, false, I.k.PY, r, GV, I.V, g.sK, dt, sm);
  orth_panel<T>(I, I.k.PY, n, r, I.k.PQ, RK, W, sm);
  copy_mat<T>(n, r, I.k.PQ, n, I.U, n);
  copy_mat<T>(r, r, RK, W, I.S, I.rcap);
}

// ---------------------------------------------------------------------------
// Greedy basis fitting (GreedyIntegrator, src/integrators/greedy_integrator.jl)
// ---------------------------------------------------------------------------
// dst (N x r) = the orthonormal polar factor of X (N x r, ld N): the Q P^T of
// svd(X) = Q Sigma P^T (greedy_integrator.jl:80-81,92-93), formed as
// X = Q_X R (QR), R = A Sigma B^T (one-sided Jacobi), dst = Q_X (A B^T).
// A rank-deficient X keeps directions completed by complete_left.  Uses the
// side's QR panel and the small blocks B_RK, B_T2; X may be sd.PY.
template <typename T>
__device__ void polar_panel(const StepArgs<T>& g, const Inst<T>& I, const Side<T>& sd, T* X, int N, int r, T* dst,
                            Smem<T>& sm) {
  const int W = I.W;
  T* R = I.blk(B_RK);
  T* C = I.blk(B_T2);
  orth_panel<T>(I, X, N, r, sd.PQ, R, W, sm);
  T* a = sm.stage;
  T* v = sm.stage + r * r;
  int* perm = reinterpret_cast<int*>(sm.stage + 2 * r * r);
  int* flag = perm + r + 1;
  T* sigma = sm.vec;
  for (int o = threadIdx.x; o < r * r; o += NT) a[o] = R[(o % r) + (int64_t)(o / r) * W];
  __syncthreads();
  const bool ok = jacobi_svd<T>(r, a, v, sigma, perm, flag);
  if (threadIdx.x == 0 && !ok) atomicOr(g.status, ST_SVD_NOCONV);
  complete_left<T>(r, r, a, sigma, perm, R);  // R is free once copied
  // C = A B^T (the polar factor of R)
  for (int o = threadIdx.x; o < r * r; o += NT) {
    const int i = o % r, j = o / r;
    T acc = T(0);
    for (int k = 0; k < r; ++k) acc = fma_acc(a[i + perm[k] * r], v[j + perm[k] * r], acc);
    C[i + (int64_t)j * W] = renorm(acc);
  }
  __syncthreads();
  tile_gemm<T>(N, r, r, sm.stage, LoadPanel<T>{sd.PQ, N}, LoadSmall<T>{C, W, false}, EpiStore<T>{dst, N});
}

// One greedy step with the snapshot X = y(t + dt) (update_data!,
// data_integrator.jl:22-28):
//   SVD-like factors (greedy_integrator.jl:96-104): U = Q of qr(X V),
//     V = Q of qr(X^T U), S = U^T X V with the new U, V;
//   two factors u = U Z^T, Z kept in the V buffer (S unused):
//     data problem (:84-94): Z = X^T U, U = polar(X Z);
//     hybrid problem (:73-82): Z advanced over [t, t + dt] by the flow's
//     L substep, Z' = F(U Z^T)^T U with U fixed (the reference's coefficient
//     ODE f(Z, U, t) for a flow map F), then U = polar(X Z).
template <typename T>
__device__ __noinline__ void greedy_step(const StepArgs<T>& g, Inst<T>& I, int r, Smem<T>& sm) {
  const int n = I.n, m = I.m, W = I.W;
  const LoadDelta<T> Xn{I.Yn, nullptr, n, false};
  const LoadDelta<T> Xt{I.Yn, nullptr, n, true};
  if (!g.two_factor) {
    tile_gemm<T>(n, m, r, sm.stage, Xn, LoadSmall<T>{I.V, m, false}, EpiStore<T>{I.k.PY, n});  // X V
    tile_gemm<T>(m, n, r, sm.stage, Xt, LoadSmall<T>{I.U, n, false}, EpiStore<T>{I.l.PY, m});  // X^T U
    orth_panel<T>(I, I.k.PY, n, r, I.k.PQ, nullptr, 0, sm);
    orth_panel<T>(I, I.l.PY, m, r, I.l.PQ, nullptr, 0, sm);
    copy_mat<T>(n, r, I.k.PQ, n, I.U, n);
    copy_mat<T>(m, r, I.l.PQ, m, I.V, m);
    tile_gemm<T>(n, m, r, sm.stage, Xn, LoadSmall<T>{I.V, m, false}, EpiStore<T>{I.k.PY, n});  // X V (new V)
    T* St = I.blk(B_ST);
    tile_gram<T>(n, r, r, sm.stage, RowLoadPanel<T>{I.U, n, r}, RowLoadPanel<T>{I.k.PY, n, r}, St, W, T(1), T(0));
    copy_mat<T>(r, r, St, W, I.S, I.rcap);
    check_finite<T>(g, I.S, r, I.rcap);
    return;
  }
  T* Z = I.V;
  if (g.op == OP_DATA) {
    tile_gemm<T>(m, n, r, sm.stage, Xt, LoadSmall<T>{I.U, n, false}, EpiStore<T>{Z, m});  // Z = X^T U
  } else {
    T* GU = I.blk(B_GU);
    if (g.op == OP_SYLVESTER) projections<T>(I, I.U, n, r, I.k.tri, GU, sm);
    substep_side<T>(g, I, I.l, 1, Z, r, GU, I.U, g.sL, g.dt, sm);
  }
  tile_gemm<T>(n, m, r, sm.stage, Xn, LoadSmall<T>{Z, m, false}, EpiStore<T>{I.k.PY, n});  // X Z
  polar_panel<T>(g, I, I.k, I.k.PY, n, r, I.U, sm);
  check_finite_panel<T>(g, I.U, n, r);
  check_finite_panel<T>(g, Z, m, r);
}

// ---------------------------------------------------------------------------
// The step kernel
// ---------------------------------------------------------------------------
// MINB: CTAs per SM the register allocation is sized for (3: at most 80
// registers per thread; 2: at most 128); the autotuner picks per precision.
template <typename T, int MINB>
__global__ void __launch_bounds__(NT, MINB) step_kernel(StepArgs<T> g) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Smem<T>& sm = *reinterpret_cast<Smem<T>*>(smem_raw);
  const int inst = g.order[g.split ? (blockIdx.x >> 1) : blockIdx.x];
  const InstDesc d = g.inst[inst];
  Inst<T> I;
  I.n = d.n; I.m = d.m; I.rcap = d.rcap; I.W = d.wcap; I.inst = inst;
  I.U = g.U + d.offU;
  I.S = g.S + d.offS;
  I.V = g.V + d.offV;
  T* wk = g.work + d.offWK;
  T* wl = g.work + d.offWL;
  const int W = d.wcap, rc = d.rcap;
  I.k = Side<T>{d.n, I.U, g.opA ? g.opA + d.offA : nullptr, wk, wk + (int64_t)d.n * W,
                wk + (int64_t)d.n * 2 * W, wk + (int64_t)d.n * (2 * W + rc), wk + (int64_t)d.n * (2 * W + 2 * rc)};
  I.l = Side<T>{d.m, I.V, g.opB ? g.opB + d.offB : nullptr, wl, wl + (int64_t)d.m * W,
                wl + (int64_t)d.m * 2 * W, wl + (int64_t)d.m * (2 * W + rc), wl + (int64_t)d.m * (2 * W + 2 * rc)};
  I.small = g.small + d.offSmall;
  // data problems read A(t + dt) and A(t); the greedy steps read y(t + dt) only
  const bool prev = (g.op == OP_DATA) && (g.alg != ALG_GREEDY);
  I.Yp = prev ? g.Yprev + d.offY : nullptr;
  I.Ypw = prev ? g.Yprev + d.offY : nullptr;
  I.Yn = (g.op == OP_DATA || g.alg == ALG_GREEDY) ? g.Ynext + d.offY : nullptr;
  const int r = g.rank[inst];
  if (r < 1 || r > d.rcap || (g.alg == ALG_RA_BUG && (2 * r > d.wcap || 2 * r > d.n || 2 * r > d.m))) {
    if (threadIdx.x == 0) atomicOr(g.status, ST_BAD_SHAPE);
    return;
  }
  if (g.alg == ALG_BUG) {
    if constexpr (std::is_same<T, double>::value) {
      if (g.split) {
        bug_step_pair<T>(g, I, r, sm);
      } else {
        bug_step<T>(g, I, r, sm);
      }
    } else {
      bug_step<T>(g, I, r, sm);
    }
  } else if (g.alg == ALG_GREEDY) {
    greedy_step<T>(g, I, r, sm);
  } else if (g.alg == ALG_RA_BUG) {
    ra_bug_step<T>(g, I, r, sm);
  } else {
    if (g.ksl_order == KSL_PRIMAL) {
      ksl_primal<T>(g, I, r, g.dt, sm);
    } else if (g.ksl_order == KSL_DUAL) {
      ksl_dual<T>(g, I, r, g.dt, sm);
    } else {
      ksl_primal<T>(g, I, r, 0.5 * g.dt, sm);
      ksl_dual<T>(g, I, r, 0.5 * g.dt, sm);
    }
    check_finite<T>(g, I.S, r, I.rcap);
  }
  // data problems: yprev <- ycurr (unconventional.jl:125)
  if (prev) {
    const int64_t nm = (int64_t)d.n * d.m;
    for (int64_t o = threadIdx.x; o < nm; o += NT) I.Ypw[o] = I.Yn[o];
  }
}

template <typename T>
size_t step_smem_bytes() {
  return sizeof(Smem<T>);
}

// FP64 BUG steps of the Sylvester flow in batches small enough that every
// instance can have two SMs run as one 2-CTA cluster per instance
// (bug_step_pair).  The pair's CTAs ask for more shared memory than two CTAs
// of an SM can hold, so the K and L steps run on two SMs, each with its own
// FP64 units.
constexpr int kPairSmem = 120 * 1024;

template <typename T, int MINB>
cudaError_t launch_step_occ(const StepArgs<T>& g, int count, cudaStream_t stream) {
  const size_t smem = sizeof(Smem<T>);
  constexpr bool f64 = std::is_same<T, double>::value;
  static_assert(sizeof(Smem<T>) <= kPairSmem, "pair launch smem below the kernel's");
  static std::atomic<uint64_t> attr_done{0};
  cudaError_t e = set_smem_limit(step_kernel<T, MINB>, f64 ? kPairSmem : (int)smem, attr_done);
  if (e != cudaSuccess) return e;
  if (f64 && g.alg == ALG_BUG && g.op == OP_SYLVESTER) {
    int dev = 0, sms = 0;
    e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    if (2 * count <= sms) {
      StepArgs<T> gp = g;
      gp.split = 1;
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3(2 * count, 1, 1);
      cfg.blockDim = dim3(NT, 1, 1);
      cfg.dynamicSmemBytes = kPairSmem;
      cfg.stream = stream;
      cudaLaunchAttribute attr[1];
      attr[0].id = cudaLaunchAttributeClusterDimension;
      attr[0].val.clusterDim.x = 2;
      attr[0].val.clusterDim.y = 1;
      attr[0].val.clusterDim.z = 1;
      cfg.attrs = attr;
      cfg.numAttrs = 1;
      e = cudaLaunchKernelEx(&cfg, step_kernel<T, MINB>, gp);
      if (e != cudaSuccess) return e;
      return cudaGetLastError();
    }
  }
  step_kernel<T, MINB><<<count, NT, smem, stream>>>(g);
  return cudaGetLastError();
}


}  // namespace lri
