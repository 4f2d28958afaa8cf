// adjoint.cu - discrete adjoint of the BUG step (FP64, Sylvester flow).
//
// One CTA per instance (or, for small batches, one 2-CTA cluster: the K side
// on one SM, the L side on another) reverses one BUG step: given the step's input factors
// (U0, S0, V0) and the adjoints of its outputs (U1_bar, S1_bar, V1_bar), it
// recomputes the step in stage form keeping every intermediate (RK stage
// inputs, Q and R of both QRs, M, N, the projections, the S-stage inputs)
// and sweeps back through it, producing (U0_bar, S0_bar, V0_bar) in place and
// accumulating theta_bar for a diagonal shift theta of the left operator A.
// Forward step (src/integrators/unconventional.jl:133-157), F = A X + X B^T:
//   K' = A K G_V + K P_V^T   from K0 = U0 S0      U1 = Q(K1), M = U1^T U0
//   L' = B L G_U + L P_U^T   from L0 = V0 S0^T    V1 = Q(L1), N = V1^T V0
//   S' = Pu S Gv + Gu S Pv^T from M S0 N^T on (U1, V1)
// with G_X = X^T X and P_X = X^T T X.  The reference has no derivative; the
// reverse sweep is the exact adjoint of this discrete map (RK stages in
// reverse, thin-QR adjoint A_bar = (Q_bar + Q copyltu(-Q_bar^T Q)) R^{-T}).
#include <cooperative_groups.h>

#include "engine_impl.cuh"

namespace cg = cooperative_groups;

namespace lri {
namespace {

constexpr int kAdjMaxStages = 16;  // nstages * nsub of any substep scheme

// small-block indices (W x W doubles each, ld W)
enum : int {
  A_GV = 0, A_PV = 1, A_GU = 2, A_PU = 3, A_GU1 = 4, A_PU1 = 5, A_GV1 = 6, A_PV1 = 7, A_M = 8, A_N = 9, A_RK = 10,
  A_RL = 11, A_CPU = 12, A_CGV = 13, A_CGU = 14, A_CPV = 15, A_KG = 16, A_KP = 17, A_LG = 18, A_LP = 19, A_MB = 20,
  A_NB = 21, A_S0B = 22, A_SB = 23, A_SYB = 24, A_SKB = 25, A_SZB = 26, A_T1 = 27, A_T2 = 28, A_T3 = 29,
  A_ZERO = 30, A_X1 = 31, A_X2 = 32, A_SACC = 33, A_SK = 34, A_SST = 35,  // A_SST .. A_SST + 15: S stage inputs
  A_COUNT = A_SST + kAdjMaxStages
};
// panels per side: stage inputs, then
enum : int { P_Y1 = 0, P_Q = 1, P_YB = 2, P_KB = 3, P_ZB = 4, P_T1 = 5, P_T2 = 6, P_XB = 7, P_COUNT = 8 };

struct AdjArgs {
  const InstDesc* inst;
  const int64_t* adj_off;  // per-instance adjoint workspace offset
  const int64_t* th_off;   // per-instance theta_bar offset
  const double* U0;
  const double* S0;
  const double* V0;
  double* Ub;
  double* Sb;
  double* Vb;
  double* thb;
  const double* opA;
  const double* opB;
  double* work;
  Scheme sK, sL, sS;
  double dt;
  int split;  // 1: one 2-CTA cluster per instance (K side on CTA 0, L side on CTA 1)
};

struct AdjSide {
  int N;
  const double* X0;   // the side's input basis (U0 or V0), ld N
  const double* tri;  // its operator (A or B)
  double* triT;       // transposed operator coefficients (3N)
  double* Z;          // stage inputs, ns*nsub panels N x r
  double* P[P_COUNT];
};

__device__ __forceinline__ double* blkp(double* small, int W, int i) { return small + (int64_t)i * W * W; }

// T^T of a tridiagonal T = [sub | dia | sup]: sub'[i] = sup[i-1], sup'[i] = sub[i+1].
__device__ void tri_transpose(int N, const double* tri, double* triT) {
  for (int i = threadIdx.x; i < N; i += NT) {
    triT[i] = (i > 0) ? tri[2 * N + i - 1] : 0.0;
    triT[N + i] = tri[N + i];
    triT[2 * N + i] = (i + 1 < N) ? tri[i + 1] : 0.0;
  }
  __syncthreads();
}

__device__ void panel_copy(int64_t len, const double* x, double* y) {
  for (int64_t o = threadIdx.x; o < len; o += NT) y[o] = x[o];
  __syncthreads();
}

// y = a * x (+ b * z when z != nullptr)
__device__ void panel_axpby(int64_t len, double a, const double* x, double b, const double* z, double* y) {
  for (int64_t o = threadIdx.x; o < len; o += NT) y[o] = z ? fma(b, z[o], a * x[o]) : a * x[o];
  __syncthreads();
}

// y += a * x
__device__ void panel_add(int64_t len, double a, const double* x, double* y) {
  for (int64_t o = threadIdx.x; o < len; o += NT) y[o] = fma(a, x[o], y[o]);
  __syncthreads();
}

// out[i] += sum_j X(i, j) Y(i, j)   (N x r panels, ld N)
__device__ void rowdot_add(int N, int r, const double* X, const double* Y, double* out) {
  for (int i = threadIdx.x; i < N; i += NT) {
    double s = 0.0;
    for (int j = 0; j < r; ++j) s = fma(X[i + (int64_t)j * N], Y[i + (int64_t)j * N], s);
    out[i] += s;
  }
  __syncthreads();
}

// C <- C R^{-T} row by row (back substitution; R upper triangular, ld ldr)
__device__ void solve_rt_rows(int N, int r, double* C, const double* R, int ldr) {
  for (int i = threadIdx.x; i < N; i += NT) {
    for (int k = r - 1; k >= 0; --k) {
      double s = C[i + (int64_t)k * N];
      for (int j = k + 1; j < r; ++j) s = fma(-C[i + (int64_t)j * N], R[k + (int64_t)j * ldr], s);
      C[i + (int64_t)k * N] = s / R[k + (int64_t)k * ldr];
    }
  }
  __syncthreads();
}

__device__ void small_transpose(int r, const double* X, int W, double* Y) {
  for (int o = threadIdx.x; o < r * r; o += NT) {
    const int i = o % r, j = o / r;
    Y[j + (int64_t)i * W] = X[i + (int64_t)j * W];
  }
  __syncthreads();
}

// Y = X + X^T
__device__ void small_sym(int r, const double* X, int W, double* Y) {
  for (int o = threadIdx.x; o < r * r; o += NT) {
    const int i = o % r, j = o / r;
    Y[i + (int64_t)j * W] = X[i + (int64_t)j * W] + X[j + (int64_t)i * W];
  }
  __syncthreads();
}

// out (N x r) = L(z) = T z G + z P^T     (Gm = G, Pm = P; pass transposes for L^T)
__device__ void apply_op(int N, int r, const double* z, const double* tri, const double* Gm, const double* Pm, int W,
                         double* out, Smem<double>& sm) {
  tile_gemm<double>(N, 2 * r, r, sm.stage, LoadStencilAug<double>{z, N, N, r, tri}, LoadGP<double>{Gm, Pm, W, r},
                    EpiStore<double>{out, N});
}

// Xb += [T X | X] [C1^T ; C2] + [T^T X | X] [C1 ; 0] with C2 symmetric:
// the adjoint of G = X^T X (C2 = Gbar + Gbar^T) and P = X^T T X (C1 = Pbar).
__device__ void proj_adjoint(int N, int r, const double* X, const double* tri, const double* triT, const double* C1,
                             const double* C2, double* small, int W, double* Xb, Smem<double>& sm) {
  double* C1t = blkp(small, W, A_X1);
  small_transpose(r, C1, W, C1t);
  tile_gemm<double>(N, 2 * r, r, sm.stage, LoadStencilAug<double>{X, N, N, r, tri}, LoadGP<double>{C1t, C2, W, r},
                    EpiAdd<double>{Xb, N});
  tile_gemm<double>(N, 2 * r, r, sm.stage, LoadStencilAug<double>{X, N, N, r, triT},
                    LoadGP<double>{C1, blkp(small, W, A_ZERO), W, r}, EpiAdd<double>{Xb, N});
}

// Stage-form RK of y' = T y G + y P^T from y0 (panel Z[0]); the stage
// inputs stay in Z[sub*ns + s]; the result goes to out.
__device__ void rk_forward(const AdjSide& sd, int r, const double* Gm, const double* Pm, int W, const Scheme& sc,
                           double dt, double* out, Smem<double>& sm) {
  const int N = sd.N, ns = sc.nstages;
  const int64_t len = (int64_t)N * r;
  const double h = dt / sc.nsub;
  double* k = sd.P[P_T1];
  double* acc = sd.P[P_T2];
  for (int sub = 0; sub < sc.nsub; ++sub) {
    const double* y = sd.Z + (int64_t)(sub * ns) * len;
    for (int s = 0; s < ns; ++s) {
      const double* z = sd.Z + (int64_t)(sub * ns + s) * len;
      apply_op(N, r, z, sd.tri, Gm, Pm, W, k, sm);
      if (s == 0) panel_axpby(len, sc.b[0], k, 0.0, nullptr, acc);
      else panel_add(len, sc.b[s], k, acc);
      if (s + 1 < ns) panel_axpby(len, 1.0, y, h * sc.a[s + 1], k, sd.Z + (int64_t)(sub * ns + s + 1) * len);
    }
    double* ynext = (sub + 1 < sc.nsub) ? sd.Z + (int64_t)((sub + 1) * ns) * len : out;
    panel_axpby(len, 1.0, y, h, acc, ynext);
  }
}

// Reverse of rk_forward: on entry P[P_YB] holds y1_bar, on exit y0_bar.
// Accumulates Gbar += (T z)^T kbar, Pbar += kbar^T z per stage, and
// theta_bar[i] += kbar(i,:) . (z G)(i,:) when thb != nullptr.
__device__ void rk_reverse(const AdjSide& sd, int r, const double* Gm, const double* GmT, const double* PmT, int W,
                           const Scheme& sc, double dt, double* Gbar, double* Pbar, double* thb, Smem<double>& sm) {
  const int N = sd.N, ns = sc.nstages;
  const int64_t len = (int64_t)N * r;
  const double h = dt / sc.nsub;
  double* yb = sd.P[P_YB];
  double* kb = sd.P[P_KB];
  double* zb = sd.P[P_ZB];
  double* ybn = sd.P[P_T2];
  double* tmp = sd.P[P_T1];
  for (int sub = sc.nsub - 1; sub >= 0; --sub) {
    panel_copy(len, yb, ybn);
    for (int s = ns - 1; s >= 0; --s) {
      const double* z = sd.Z + (int64_t)(sub * ns + s) * len;
      // kbar_s = h b_s ybar' + h a_{s+1} zbar_{s+1}
      panel_axpby(len, h * sc.b[s], ybn, h * ((s + 1 < ns) ? sc.a[s + 1] : 0.0), (s + 1 < ns) ? zb : nullptr, kb);
      tile_gram<double>(N, r, r, sm.stage, RowLoadStencil<double>{z, N, N, r, sd.tri}, RowLoadPanel<double>{kb, N, r},
                        Gbar, W, 1.0, 1.0);
      tile_gram<double>(N, r, r, sm.stage, RowLoadPanel<double>{kb, N, r}, RowLoadPanel<double>{z, N, r}, Pbar, W,
                        1.0, 1.0);
      if (thb) {
        tile_gemm<double>(N, r, r, sm.stage, LoadPanel<double>{z, N}, LoadSmall<double>{Gm, W, false},
                          EpiStore<double>{tmp, N});
        rowdot_add(N, r, kb, tmp, thb);
      }
      // zbar_s = T^T kbar G^T + kbar P
      apply_op(N, r, kb, sd.triT, GmT, PmT, W, zb, sm);
      panel_add(len, 1.0, zb, yb);
    }
  }
}

// Thin-QR adjoint in place: Xb <- (Xb + Q copyltu(-Xb^T Q)) R^{-T}.
__device__ void qr_adjoint(int N, int r, const double* Q, const double* R, double* Xb, double* small, int W,
                           Smem<double>& sm) {
  double* Mx = blkp(small, W, A_T1);
  double* Cl = blkp(small, W, A_T2);
  tile_gram<double>(N, r, r, sm.stage, RowLoadPanel<double>{Xb, N, r}, RowLoadPanel<double>{Q, N, r}, Mx, W, -1.0,
                    0.0);
  for (int o = threadIdx.x; o < r * r; o += NT) {
    const int i = o % r, j = o / r;
    Cl[i + (int64_t)j * W] = (i >= j) ? Mx[i + (int64_t)j * W] : Mx[j + (int64_t)i * W];
  }
  __syncthreads();
  tile_gemm<double>(N, r, r, sm.stage, LoadPanel<double>{Q, N}, LoadSmall<double>{Cl, W, false},
                    EpiAdd<double>{Xb, N});
  solve_rt_rows(N, r, Xb, R, W);
}

__device__ void small_zero(int r, double* X, int W) {
  for (int o = threadIdx.x; o < r * r; o += NT) X[(o % r) + (int64_t)(o / r) * W] = 0.0;
  __syncthreads();
}

// S-step stage derivative: out = Pu z Gv + Gu z Pv^T
__device__ void s_op(int r, const double* z, double* small, int W, double* out) {
  double* t1 = blkp(small, W, A_T3);
  small_gemm<double>(r, r, r, 1.0, blkp(small, W, A_PU1), W, false, z, W, false, 0.0, t1, W);
  small_gemm<double>(r, r, r, 1.0, t1, W, false, blkp(small, W, A_GV1), W, false, 0.0, out, W);
  small_gemm<double>(r, r, r, 1.0, blkp(small, W, A_GU1), W, false, z, W, false, 0.0, t1, W);
  small_gemm<double>(r, r, r, 1.0, t1, W, false, blkp(small, W, A_PV1), W, true, 1.0, out, W);
}

// One instance per CTA, or (split) per 2-CTA thread-block cluster: CTA 0
// takes the K side (U), CTA 1 the L side (V), in four phases separated by
// cluster barriers (every thread of both CTAs reaches all three):
//   1. forward recomputation of each side's substep, QR, basis change and
//      projections;
//   2. (CTA 0) the S step forward and reversed, Mbar, Nbar, S0bar;
//   3. each side's QR adjoint and RK reversal (the gradients of its
//      projection coefficients, its part of S0bar);
//   4. each side adds the adjoint of the other side's projections of its own
//      basis (K step -> G_V, P_V; L step -> G_U, P_U) and writes its output;
//      CTA 1 sums S0bar.
// Scratch blocks: the K side uses `small`, the L side `small1` (disjoint),
// so the halves never write the same block.  Without a cluster the same
// phases run one after the other in one CTA.
__global__ void __launch_bounds__(NT, 3) adjoint_step_kernel(AdjArgs g) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Smem<double>& sm = *reinterpret_cast<Smem<double>*>(smem_raw);
  const bool split = g.split != 0;
  const int inst = split ? (int)(blockIdx.x >> 1) : (int)blockIdx.x;
  const int crank = split ? (int)cg::this_cluster().block_rank() : 0;
  const bool doK = !split || crank == 0;
  const bool doL = !split || crank == 1;
  auto phase_end = [&]() {
    if (split) {
      __threadfence();
      cg::this_cluster().sync();
    }
  };
  const InstDesc d = g.inst[inst];
  const int n = d.n, m = d.m, r = d.rcap, W = d.rcap, ldS = d.rcap;
  const double* U0 = g.U0 + d.offU;
  const double* S0 = g.S0 + d.offS;
  const double* V0 = g.V0 + d.offV;
  double* Ub = g.Ub + d.offU;
  double* Sb = g.Sb + d.offS;
  double* Vb = g.Vb + d.offV;
  double* thb = g.thb + g.th_off[inst];
  double* w = g.work + g.adj_off[inst];
  // workspace: small blocks | L-side scratch blocks | K side (triT, stage panels, panels) | L side
  double* small = w;
  w += (int64_t)A_COUNT * W * W;
  double* small1 = w;
  w += (int64_t)A_COUNT * W * W;
  AdjSide K, L;
  K.N = n;
  K.X0 = U0;
  K.tri = g.opA + d.offA;
  K.triT = w;
  w += 3 * (int64_t)n;
  K.Z = w;
  w += (int64_t)(g.sK.nstages * g.sK.nsub) * n * r;
  for (int p = 0; p < P_COUNT; ++p) {
    K.P[p] = w;
    w += (int64_t)n * r;
  }
  L.N = m;
  L.X0 = V0;
  L.tri = g.opB + d.offB;
  L.triT = w;
  w += 3 * (int64_t)m;
  L.Z = w;
  w += (int64_t)(g.sL.nstages * g.sL.nsub) * m * r;
  for (int p = 0; p < P_COUNT; ++p) {
    L.P[p] = w;
    w += (int64_t)m * r;
  }
  Inst<double> I;
  I.n = n;
  I.m = m;
  I.rcap = r;
  I.W = W;
  I.inst = inst;
  const double* U1 = K.P[P_Q];
  const double* V1 = L.P[P_Q];
  double* T1s = blkp(small, W, A_T1);
  double* T2s = blkp(small, W, A_T2);

  // ---------------- phase 1: forward recomputation of both sides ----------------
  if (doK) {
    tri_transpose(n, K.tri, K.triT);
    small_zero(r, blkp(small, W, A_ZERO), W);
    projections<double>(I, V0, m, r, L.tri, blkp(small, W, A_GV), sm);  // G_V, P_V (adjacent blocks)
    // K step: K0 = U0 S0 -> K1 -> U1 = Q, RK
    tile_gemm<double>(n, r, r, sm.stage, LoadPanel<double>{U0, n}, LoadSmall<double>{S0, ldS, false},
                      EpiStore<double>{K.Z, n});
    rk_forward(K, r, blkp(small, W, A_GV), blkp(small, W, A_PV), W, g.sK, g.dt, K.P[P_Y1], sm);
    qr_panel<double>(K.P[P_Y1], n, r, K.P[P_Q], blkp(small, W, A_RK), W, sm);
    tile_gram<double>(n, r, r, sm.stage, RowLoadPanel<double>{K.P[P_Q], n, r}, RowLoadPanel<double>{U0, n, r},
                      blkp(small, W, A_M), W, 1.0, 0.0);
    projections<double>(I, U1, n, r, K.tri, blkp(small, W, A_GU1), sm);  // Gu1, Pu1
  }
  if (doL) {
    tri_transpose(m, L.tri, L.triT);
    small_zero(r, blkp(small1, W, A_ZERO), W);
    projections<double>(I, U0, n, r, K.tri, blkp(small, W, A_GU), sm);  // G_U, P_U
    // L step: L0 = V0 S0^T -> L1 -> V1, RL
    tile_gemm<double>(m, r, r, sm.stage, LoadPanel<double>{V0, m}, LoadSmall<double>{S0, ldS, true},
                      EpiStore<double>{L.Z, m});
    rk_forward(L, r, blkp(small, W, A_GU), blkp(small, W, A_PU), W, g.sL, g.dt, L.P[P_Y1], sm);
    qr_panel<double>(L.P[P_Y1], m, r, L.P[P_Q], blkp(small, W, A_RL), W, sm);
    tile_gram<double>(m, r, r, sm.stage, RowLoadPanel<double>{L.P[P_Q], m, r}, RowLoadPanel<double>{V0, m, r},
                      blkp(small, W, A_N), W, 1.0, 0.0);
    projections<double>(I, V1, m, r, L.tri, blkp(small, W, A_GV1), sm);  // Gv1, Pv1
  }
  phase_end();

  // ---------------- phase 2: the S step, forward and reversed ----------------
  double* Mb = blkp(small, W, A_MB);
  double* Nb = blkp(small, W, A_NB);
  double* S0b = blkp(small, W, A_S0B);
  if (doK) {
    // S~0 = M S0 N^T into the first stage input
    small_gemm<double>(r, r, r, 1.0, S0, ldS, false, blkp(small, W, A_N), W, true, 0.0, T1s, W);
    small_gemm<double>(r, r, r, 1.0, blkp(small, W, A_M), W, false, T1s, W, false, 0.0, blkp(small, W, A_SST), W);
    {
      const int ns = g.sS.nstages;
      const double h = g.dt / g.sS.nsub;
      double* kS = blkp(small, W, A_SK);
      double* acc = blkp(small, W, A_SACC);
      for (int sub = 0; sub < g.sS.nsub; ++sub) {
        const double* y = blkp(small, W, A_SST + sub * ns);
        for (int s = 0; s < ns; ++s) {
          s_op(r, blkp(small, W, A_SST + sub * ns + s), small, W, kS);
          for (int o = threadIdx.x; o < r * r; o += NT) {
            const int64_t e = (o % r) + (int64_t)(o / r) * W;
            acc[e] = (s == 0) ? g.sS.b[0] * kS[e] : fma(g.sS.b[s], kS[e], acc[e]);
            if (s + 1 < ns) blkp(small, W, A_SST + sub * ns + s + 1)[e] = fma(h * g.sS.a[s + 1], kS[e], y[e]);
          }
          __syncthreads();
        }
        if (sub + 1 < g.sS.nsub) {
          double* yn = blkp(small, W, A_SST + (sub + 1) * ns);
          for (int o = threadIdx.x; o < r * r; o += NT) {
            const int64_t e = (o % r) + (int64_t)(o / r) * W;
            yn[e] = fma(h, acc[e], y[e]);
          }
          __syncthreads();
        }
      }
    }
    // S step reversed: Sbar = S1_bar -> S~0_bar; coefficient gradients cPu, cGv, cGu, cPv
    double* Sbar = blkp(small, W, A_SB);
    for (int o = threadIdx.x; o < r * r; o += NT)
      Sbar[(o % r) + (int64_t)(o / r) * W] = Sb[(o % r) + (int64_t)(o / r) * ldS];
    for (int b = A_CPU; b <= A_LP; ++b) small_zero(r, blkp(small, W, b), W);
    {
      const int ns = g.sS.nstages;
      const double h = g.dt / g.sS.nsub;
      double* ybn = blkp(small, W, A_SYB);
      double* kb = blkp(small, W, A_SKB);
      double* zb = blkp(small, W, A_SZB);
      double* t3 = blkp(small, W, A_T3);
      for (int sub = g.sS.nsub - 1; sub >= 0; --sub) {
        copy_mat<double>(r, r, Sbar, W, ybn, W);
        for (int s = ns - 1; s >= 0; --s) {
          const double* z = blkp(small, W, A_SST + sub * ns + s);
          for (int o = threadIdx.x; o < r * r; o += NT) {
            const int64_t e = (o % r) + (int64_t)(o / r) * W;
            kb[e] = h * g.sS.b[s] * ybn[e] + ((s + 1 < ns) ? h * g.sS.a[s + 1] * zb[e] : 0.0);
          }
          __syncthreads();
          // cPu += kb Gv1^T z^T ; cGv += (Pu1 z)^T kb ; cGu += kb Pv1 z^T ; cPv += kb^T Gu1 z
          small_gemm<double>(r, r, r, 1.0, kb, W, false, blkp(small, W, A_GV1), W, true, 0.0, t3, W);
          small_gemm<double>(r, r, r, 1.0, t3, W, false, z, W, true, 1.0, blkp(small, W, A_CPU), W);
          small_gemm<double>(r, r, r, 1.0, blkp(small, W, A_PU1), W, false, z, W, false, 0.0, t3, W);
          small_gemm<double>(r, r, r, 1.0, t3, W, true, kb, W, false, 1.0, blkp(small, W, A_CGV), W);
          small_gemm<double>(r, r, r, 1.0, kb, W, false, blkp(small, W, A_PV1), W, false, 0.0, t3, W);
          small_gemm<double>(r, r, r, 1.0, t3, W, false, z, W, true, 1.0, blkp(small, W, A_CGU), W);
          small_gemm<double>(r, r, r, 1.0, blkp(small, W, A_GU1), W, false, z, W, false, 0.0, t3, W);
          small_gemm<double>(r, r, r, 1.0, kb, W, true, t3, W, false, 1.0, blkp(small, W, A_CPV), W);
          // zb = Pu1^T kb Gv1^T + Gu1^T kb Pv1
          small_gemm<double>(r, r, r, 1.0, blkp(small, W, A_PU1), W, true, kb, W, false, 0.0, t3, W);
          small_gemm<double>(r, r, r, 1.0, t3, W, false, blkp(small, W, A_GV1), W, true, 0.0, zb, W);
          small_gemm<double>(r, r, r, 1.0, blkp(small, W, A_GU1), W, true, kb, W, false, 0.0, t3, W);
          small_gemm<double>(r, r, r, 1.0, t3, W, false, blkp(small, W, A_PV1), W, false, 1.0, zb, W);
          for (int o = threadIdx.x; o < r * r; o += NT) {
            const int64_t e = (o % r) + (int64_t)(o / r) * W;
            Sbar[e] += zb[e];
          }
          __syncthreads();
        }
      }
    }
    // S~0 = M S0 N^T:  Mb = St0b N S0^T, Nb = St0b^T M S0, S0b = M^T St0b N
    small_gemm<double>(r, r, r, 1.0, blkp(small, W, A_N), W, false, S0, ldS, true, 0.0, T1s, W);
    small_gemm<double>(r, r, r, 1.0, Sbar, W, false, T1s, W, false, 0.0, Mb, W);
    small_gemm<double>(r, r, r, 1.0, blkp(small, W, A_M), W, false, S0, ldS, false, 0.0, T1s, W);
    small_gemm<double>(r, r, r, 1.0, Sbar, W, true, T1s, W, false, 0.0, Nb, W);
    small_gemm<double>(r, r, r, 1.0, Sbar, W, false, blkp(small, W, A_N), W, false, 0.0, T1s, W);
    small_gemm<double>(r, r, r, 1.0, blkp(small, W, A_M), W, true, T1s, W, false, 0.0, S0b, W);
  }
  phase_end();

  // ---------------- phase 3: QR adjoints and RK reversals of both sides ----------------
  const int64_t lenK = (int64_t)n * r, lenL = (int64_t)m * r;
  if (doK) {
    // U1_bar (panel K.P[P_YB]) = U1_bar(out) + U0 Mb^T + adjoint of Gu1, Pu1; theta_bar from Pu1
    for (int64_t o = threadIdx.x; o < lenK; o += NT) K.P[P_YB][o] = Ub[o];
    __syncthreads();
    tile_gemm<double>(n, r, r, sm.stage, LoadPanel<double>{U0, n}, LoadSmall<double>{Mb, W, true},
                      EpiAdd<double>{K.P[P_YB], n});
    small_sym(r, blkp(small, W, A_CGU), W, T2s);
    proj_adjoint(n, r, U1, K.tri, K.triT, blkp(small, W, A_CPU), T2s, small, W, K.P[P_YB], sm);
    tile_gemm<double>(n, r, r, sm.stage, LoadPanel<double>{U1, n},
                      LoadSmall<double>{blkp(small, W, A_CPU), W, true}, EpiStore<double>{K.P[P_T1], n});
    rowdot_add(n, r, K.P[P_T1], U1, thb);
    // U0_bar accumulator (panel P_XB): U1 Mb
    tile_gemm<double>(n, r, r, sm.stage, LoadPanel<double>{U1, n}, LoadSmall<double>{Mb, W, false},
                      EpiStore<double>{K.P[P_XB], n});
    // K step: K1_bar = qr_adjoint(U1_bar); RK reverse -> K0_bar
    qr_adjoint(n, r, U1, blkp(small, W, A_RK), K.P[P_YB], small, W, sm);
    small_transpose(r, blkp(small, W, A_GV), W, blkp(small, W, A_T1));
    small_transpose(r, blkp(small, W, A_PV), W, blkp(small, W, A_T2));
    // L^T(X) = A^T X G_V^T + X P_V : apply_op with (G^T, P^T) gives [G^T ; P]
    rk_reverse(K, r, blkp(small, W, A_GV), blkp(small, W, A_T1), blkp(small, W, A_T2), W, g.sK, g.dt,
               blkp(small, W, A_KG), blkp(small, W, A_KP), thb, sm);
    // U0_bar += K0_bar S0^T ; S0_bar += U0^T K0_bar
    tile_gemm<double>(n, r, r, sm.stage, LoadPanel<double>{K.P[P_YB], n}, LoadSmall<double>{S0, ldS, true},
                      EpiAdd<double>{K.P[P_XB], n});
    tile_gram<double>(n, r, r, sm.stage, RowLoadPanel<double>{U0, n, r}, RowLoadPanel<double>{K.P[P_YB], n, r}, S0b,
                      W, 1.0, 1.0);
  }
  if (doL) {
    double* T2l = blkp(small1, W, A_T2);
    // V1_bar (panel L.P[P_YB]) = V1_bar(out) + V0 Nb^T + adjoint of Gv1, Pv1
    for (int64_t o = threadIdx.x; o < lenL; o += NT) L.P[P_YB][o] = Vb[o];
    __syncthreads();
    tile_gemm<double>(m, r, r, sm.stage, LoadPanel<double>{V0, m}, LoadSmall<double>{Nb, W, true},
                      EpiAdd<double>{L.P[P_YB], m});
    small_sym(r, blkp(small, W, A_CGV), W, T2l);
    proj_adjoint(m, r, V1, L.tri, L.triT, blkp(small, W, A_CPV), T2l, small1, W, L.P[P_YB], sm);
    // V0_bar accumulator: V1 Nb
    tile_gemm<double>(m, r, r, sm.stage, LoadPanel<double>{V1, m}, LoadSmall<double>{Nb, W, false},
                      EpiStore<double>{L.P[P_XB], m});
    // L step: L1_bar = qr_adjoint(V1_bar); RK reverse -> L0_bar
    qr_adjoint(m, r, V1, blkp(small, W, A_RL), L.P[P_YB], small1, W, sm);
    small_transpose(r, blkp(small, W, A_GU), W, blkp(small1, W, A_T1));
    small_transpose(r, blkp(small, W, A_PU), W, blkp(small1, W, A_T2));
    rk_reverse(L, r, blkp(small, W, A_GU), blkp(small1, W, A_T1), blkp(small1, W, A_T2), W, g.sL, g.dt,
               blkp(small, W, A_LG), blkp(small, W, A_LP), nullptr, sm);
    // V0_bar += L0_bar S0 ; this side's part of S0_bar: L0_bar^T V0
    tile_gemm<double>(m, r, r, sm.stage, LoadPanel<double>{L.P[P_YB], m}, LoadSmall<double>{S0, ldS, false},
                      EpiAdd<double>{L.P[P_XB], m});
    tile_gram<double>(m, r, r, sm.stage, RowLoadPanel<double>{L.P[P_YB], m, r}, RowLoadPanel<double>{V0, m, r},
                      blkp(small1, W, A_S0B), W, 1.0, 0.0);
  }
  phase_end();

  // ---------------- phase 4: cross-side projection adjoints, outputs ----------------
  if (doK) {
    // U0_bar += adjoint of G_U, P_U (L step) ; theta_bar from P_U
    small_sym(r, blkp(small, W, A_LG), W, T2s);
    proj_adjoint(n, r, U0, K.tri, K.triT, blkp(small, W, A_LP), T2s, small, W, K.P[P_XB], sm);
    tile_gemm<double>(n, r, r, sm.stage, LoadPanel<double>{U0, n}, LoadSmall<double>{blkp(small, W, A_LP), W, true},
                      EpiStore<double>{K.P[P_T1], n});
    rowdot_add(n, r, K.P[P_T1], U0, thb);
    for (int64_t o = threadIdx.x; o < lenK; o += NT) Ub[o] = K.P[P_XB][o];
  }
  if (doL) {
    // V0_bar += adjoint of G_V, P_V (K step)
    double* T2l = blkp(small1, W, A_T2);
    small_sym(r, blkp(small, W, A_KG), W, T2l);
    proj_adjoint(m, r, V0, L.tri, L.triT, blkp(small, W, A_KP), T2l, small1, W, L.P[P_XB], sm);
    for (int64_t o = threadIdx.x; o < lenL; o += NT) Vb[o] = L.P[P_XB][o];
    const double* S0bl = blkp(small1, W, A_S0B);
    for (int o = threadIdx.x; o < r * r; o += NT) {
      const int64_t e = (o % r) + (int64_t)(o / r) * W;
      Sb[(o % r) + (int64_t)(o / r) * ldS] = S0b[e] + S0bl[e];
    }
  }
}

}  // namespace

size_t adjoint_work_elems(int64_t n, int64_t m, int64_t r, int ns_k, int ns_l) {
  return 2 * (size_t)A_COUNT * r * r + 3 * (size_t)(n + m) + (size_t)(ns_k + P_COUNT) * n * r +
         (size_t)(ns_l + P_COUNT) * m * r;
}

int adjoint_max_stages() { return kAdjMaxStages; }

cudaError_t launch_adjoint_step(const InstDesc* inst, const int64_t* adj_off, const int64_t* th_off, int count,
                                const double* U0, const double* S0, const double* V0, double* Ub, double* Sb,
                                double* Vb, double* thb, const double* opA, const double* opB, double* work,
                                const Scheme& sK, const Scheme& sL, const Scheme& sS, double dt, cudaStream_t st) {
  AdjArgs g{inst, adj_off, th_off, U0, S0, V0, Ub, Sb, Vb, thb, opA, opB, work, sK, sL, sS, dt, 0};
  const size_t smem = sizeof(Smem<double>);
  // Batches small enough that every instance can have two SMs run the K and
  // L sides on a 2-CTA cluster each.  Its CTAs ask for more shared memory
  // than two CTAs of an SM can hold, so the pair runs on two SMs (a CTA pair
  // on one SM would share its FP64 units).
  constexpr int kSplitSmem = 120 * 1024;
  static_assert(sizeof(Smem<double>) <= kSplitSmem, "split launch smem below the kernel's");
  static std::atomic<uint64_t> attr_done{0};
  cudaError_t e = set_smem_limit(adjoint_step_kernel, kSplitSmem, attr_done);
  if (e != cudaSuccess) return e;
  int dev = 0, sms = 0;
  e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return e;
  if (2 * count <= sms) {
    g.split = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(2 * count, 1, 1);
    cfg.blockDim = dim3(NT, 1, 1);
    cfg.dynamicSmemBytes = kSplitSmem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = 2;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    e = cudaLaunchKernelEx(&cfg, adjoint_step_kernel, g);
    if (e != cudaSuccess) return e;
    return cudaGetLastError();
  }
  adjoint_step_kernel<<<count, NT, smem, st>>>(g);
  return cudaGetLastError();
}

}  // namespace lri
