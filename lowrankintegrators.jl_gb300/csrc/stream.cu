// stream.cu - rank-adaptive BUG for one large instance spread over the whole
// GPU: a data stream (MatrixDataProblem whose snapshots are too large for the
// one-CTA instance engine, lri_stream_*) or a periodic Burgers flow
// (MatrixDEProblem, lri_burgers_*).
//
// One data step A(t) -> A(t+1) (src/integrators/rank_adaptive_unconventional.jl:
// 182-233 with the data substeps of data_integrator.jl:13-16):
//   K1 = U0 S0 + dY V0,  L1 = V0 S0^T + dY^T U0          dY = A(t+1) - A(t)
//   Uhat = orth[K1 | U0], Vhat = orth[L1 | V0]
//   S~ = (Uhat^T U0) S0 (Vhat^T V0)^T + Uhat^T dY Vhat
//   S~ = P Sigma Q^T, r1 = truncation, U1 = Uhat P1, V1 = Vhat Q1, S1 = Sigma1.
// span[K1 | U0] = span[U0 | (I - U0 U0^T) dY V0], so Uhat is formed as
// [U0 | Q] with Q an orthonormal basis of the part of dY V0 orthogonal to U0
// (orth_against: projections, a rank-revealing pivoted Cholesky pass whose
// dependent directions become zero columns, one more projection, then
// Newton-Schulz or CholeskyQR).  The step's result depends only on
// span(Uhat), span(Vhat).  The Burgers step has the same bases and core with
// RK substeps whose flows use the exact low-rank structure of F (no n x m
// matrix; see the flow kernels below).
//
// Kernels: streaming passes over the snapshot pair (dY V0, dY^T U0, dY Vhat;
// dY is formed in the loader and never stored), tall-skinny Gram products
// X^T Y reduced in FP64 through per-block partials, row-parallel panel
// products X B, the Burgers flow kernels, and single-CTA kernels (double-float
// for FP32 panels) for the r x r / 2r x 2r factorisations and the core SVD.
// Panel widths are fixed at r_max (Uhat, Vhat: 2 r_max) with zero columns
// beyond the current rank, which stays on the device; kernels that read it
// work on the active columns only.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <type_traits>
#include <vector>

#include "../../include/lri.h"
#include "core_svd.h"
#include "engine.cuh"
#include "tc_kr.h"
#include "tc_pass.h"

namespace lri {
namespace {

constexpr int SMAX = 96;      // largest r_max

// active column j (0 <= j < ka) -> panel column: the first r of each half
__device__ __forceinline__ int act_col(int j, int r, int R) { return (j < r) ? j : R + (j - r); }

// ---------------------------------------------------------------------------
// Streaming pass A: out (n x cols) = dY B, dY = A1 - A0 (n x m, col-major),
// B (m x cols, ld ldb) with cols = R (aug = 0) or 2R (aug = 1), on the active
// columns only (the first r of each half; r read on the device): the
// multiply-adds run for ceil(ka / 32) groups of 32 columns, inactive output
// columns are written as zeros.  CTA = 32 rows, loops over all columns of dY.
// ---------------------------------------------------------------------------
template <typename T, int CGN>
__device__ __forceinline__ void pass_rows_tile(const T (*ds)[33], const T (*bs)[2 * SMAX + 1], int BJ, int rg,
                                               int cg, T (&acc)[4][6]) {
#pragma unroll 4
  for (int jj = 0; jj < BJ; ++jj) {
    T x[4], w[CGN];
#pragma unroll
    for (int p = 0; p < 4; ++p) x[p] = ds[jj][4 * rg + p];
#pragma unroll
    for (int u = 0; u < CGN; ++u) w[u] = bs[jj][cg + 32 * u];
#pragma unroll
    for (int p = 0; p < 4; ++p)
#pragma unroll
      for (int u = 0; u < CGN; ++u) acc[p][u] = fma(x[p], w[u], acc[p][u]);
  }
}

template <typename T>
__global__ void __launch_bounds__(256) pass_rows(int n, int m, int R, int aug, const int32_t* __restrict__ rank,
                                                 const T* __restrict__ A1, const T* __restrict__ A0,
                                                 const T* __restrict__ B, int ldb, T* __restrict__ out) {
  // 4 rows x up to 6 column groups per thread (ka <= 192); BJ keeps the
  // static shared memory under 48 KB for both types
  constexpr int BI = 32, BJ = sizeof(T) == 8 ? 16 : 32;
  __shared__ T ds[BJ][BI + 1];             // dY tile, column-major
  __shared__ T bs[BJ][2 * SMAX + 1];       // B rows of the tile (active columns)
  const int r = min(R, (int)*rank), ka = aug ? 2 * r : r, cols = aug ? 2 * R : R;
  const int ncg = (ka + 31) / 32;
  const int tid = threadIdx.x;
  const int i0 = blockIdx.x * BI;
  const int rg = tid & 7, cg = tid >> 3;   // rows 4rg.., columns cg + 32u
  T acc[4][6];
#pragma unroll
  for (int p = 0; p < 4; ++p)
#pragma unroll
    for (int u = 0; u < 6; ++u) acc[p][u] = T(0);
  for (int j0 = 0; j0 < m; j0 += BJ) {
    for (int e = tid; e < BI * BJ; e += 256) {
      const int ii = e % BI, jj = e / BI;
      const int i = i0 + ii, j = j0 + jj;
      T v = T(0);
      if (i < n && j < m) {
        const int64_t o = (int64_t)i + (int64_t)j * n;
        v = A0 ? A1[o] - A0[o] : A1[o];  // no A0: the snapshot itself
      }
      ds[jj][ii] = v;
    }
    for (int e = tid; e < BJ * 32 * ncg; e += 256) {
      const int jj = e % BJ, k = e / BJ;
      const int j = j0 + jj;
      bs[jj][k] = (j < m && k < ka) ? B[j + (int64_t)act_col(k, r, R) * ldb] : T(0);
    }
    __syncthreads();
    switch (ncg) {
      case 1: pass_rows_tile<T, 1>(ds, bs, BJ, rg, cg, acc); break;
      case 2: pass_rows_tile<T, 2>(ds, bs, BJ, rg, cg, acc); break;
      case 3: pass_rows_tile<T, 3>(ds, bs, BJ, rg, cg, acc); break;
      case 4: pass_rows_tile<T, 4>(ds, bs, BJ, rg, cg, acc); break;
      case 5: pass_rows_tile<T, 5>(ds, bs, BJ, rg, cg, acc); break;
      default: pass_rows_tile<T, 6>(ds, bs, BJ, rg, cg, acc); break;
    }
    __syncthreads();
  }
#pragma unroll
  for (int p = 0; p < 4; ++p) {
    const int i = i0 + 4 * rg + p;
    if (i >= n) continue;
#pragma unroll
    for (int u = 0; u < 6; ++u) {
      const int k = cg + 32 * u;
      if (k < ka) out[i + (int64_t)act_col(k, r, R) * n] = acc[p][u];
    }
  }
  // inactive columns of this CTA's rows
  for (int e = tid; e < BI * cols; e += 256) {
    const int ii = e % BI, col = e / BI;
    const int i = i0 + ii;
    if (i < n && (col % R) >= r) out[i + (int64_t)col * n] = T(0);
  }
}

// ---------------------------------------------------------------------------
// Streaming pass B: out (m x R) = dY^T X, X (n x R, ld ldx), on the first r
// columns (r read on the device; the others are written as zeros), r <=
// SMAX.  CTA = 16 columns of dY, loops over all rows.
// ---------------------------------------------------------------------------
template <typename T, int NW>
__device__ __forceinline__ void pass_cols_tile(const T (*ds)[65], const T (*xs)[129], int BI, int jg, int cg,
                                               T (&acc)[4][2]) {
#pragma unroll 4
  for (int ii = 0; ii < BI; ++ii) {
    T x[4], w[NW];
#pragma unroll
    for (int p = 0; p < 4; ++p) x[p] = ds[4 * jg + p][ii];
#pragma unroll
    for (int u = 0; u < NW; ++u) w[u] = xs[ii][cg + 64 * u];
#pragma unroll
    for (int p = 0; p < 4; ++p)
#pragma unroll
      for (int u = 0; u < NW; ++u) acc[p][u] = fma(x[p], w[u], acc[p][u]);
  }
}

template <typename T>
__global__ void __launch_bounds__(256) pass_cols(int n, int m, int R, const int32_t* __restrict__ rank,
                                                 const T* __restrict__ A1, const T* __restrict__ A0,
                                                 const T* __restrict__ X, int ldx, T* __restrict__ out) {
  constexpr int BJ = 16, BI = sizeof(T) == 8 ? 32 : 64;
  __shared__ T ds[BJ][64 + 1];
  __shared__ T xs[BI][129];  // columns cg + 64u < 128 of X (zero beyond r)
  const int c = min(R, (int)*rank);
  const int tid = threadIdx.x;
  const int j0 = blockIdx.x * BJ;
  const int jg = tid & 3, cg = tid >> 2;   // columns 4jg.., outputs cg + 64u
  T acc[4][2];
#pragma unroll
  for (int p = 0; p < 4; ++p) acc[p][0] = acc[p][1] = T(0);
  for (int i0 = 0; i0 < n; i0 += BI) {
    for (int e = tid; e < BI * BJ; e += 256) {
      const int ii = e % BI, jj = e / BI;
      const int i = i0 + ii, j = j0 + jj;
      T v = T(0);
      if (i < n && j < m) {
        const int64_t o = (int64_t)i + (int64_t)j * n;
        v = A0 ? A1[o] - A0[o] : A1[o];  // no A0: the snapshot itself
      }
      ds[jj][ii] = v;
    }
    for (int e = tid; e < BI * 128; e += 256) {
      const int ii = e % BI, k = e / BI;
      const int i = i0 + ii;
      xs[ii][k] = (i < n && k < c) ? X[i + (int64_t)k * ldx] : T(0);
    }
    __syncthreads();
    if (c <= 64) pass_cols_tile<T, 1>(ds, xs, BI, jg, cg, acc);
    else pass_cols_tile<T, 2>(ds, xs, BI, jg, cg, acc);
    __syncthreads();
  }
#pragma unroll
  for (int p = 0; p < 4; ++p) {
    const int j = j0 + 4 * jg + p;
    if (j >= m) continue;
    if (cg < R) out[j + (int64_t)cg * m] = (cg < c) ? acc[p][0] : T(0);
    if (cg + 64 < R) out[j + (int64_t)(cg + 64) * m] = (cg + 64 < c) ? acc[p][1] : T(0);
  }
}

// ---------------------------------------------------------------------------
// Gram products out = X^T Y on the active columns, X (N x a, ld ldx), Y
// (N x c, ld ldy); a, c <= 2*SMAX.  A panel of 2R columns has the first r of
// each half active, one of R (or fewer) columns the first r (r = *rank, read
// on the device; the other columns are zero).  The active block is cut into
// 64 x 64 tiles (ntile of them) and the rows into nrb blocks, nrb =
// max(1, ctas / ntile) rounded to whole 32-row slabs, so every rank keeps
// about `ctas` CTAs busy.  Work item (row block, tile) writes its 64 x 64
// partial at part[item * 4096]; gram_reduce sums the row blocks in order
// (deterministic).
// ---------------------------------------------------------------------------
// FP32 panels: exact products, double-float sums (the FP64 pipe of GB300
// runs at 1/64 of the FP32 rate); FP64 panels: FP64.
template <typename T> struct GramAcc { using type = double; };
template <> struct GramAcc<float> { using type = dfloat; };
__device__ __forceinline__ double gacc_mul(double acc, double x, double y) { return fma(x, y, acc); }
__device__ __forceinline__ dfloat gacc_mul(dfloat acc, float x, float y) { return acc_mul_acc(acc, x, y); }
__device__ __forceinline__ double gacc_val(double a) { return a; }
__device__ __forceinline__ double gacc_val(dfloat a) { return (double)a.hi + (double)a.lo; }

constexpr int GRAM_TILE = 64;
constexpr int GRAM_TILE_MAX = 9;  // (2 SMAX / 64)^2 tiles

// active width of a panel of `a` columns (2R: both halves)
__device__ __forceinline__ int panel_active(int a, int r, int R) { return (a == 2 * R) ? 2 * r : min(a, r); }
// panel column of active index j
__device__ __forceinline__ int panel_col(int a, int j, int r, int R) { return (a == 2 * R) ? act_col(j, r, R) : j; }
// active index of panel column p, or -1
__device__ __forceinline__ int panel_act_index(int a, int p, int r, int R) {
  if (a == 2 * R) return (p < R) ? (p < r ? p : -1) : (p - R < r ? r + (p - R) : -1);
  return (p < r) ? p : -1;
}

// the split of a Gram product: tiles of the active block, row blocks
struct GramSplit {
  int ka, kc, ta, ntile, rows, nrb;
};
__device__ __forceinline__ GramSplit gram_split(int N, int a, int c, int R, int r, int ctas) {
  GramSplit g;
  g.ka = panel_active(a, r, R);
  g.kc = panel_active(c, r, R);
  g.ta = (g.ka + GRAM_TILE - 1) / GRAM_TILE;
  g.ntile = g.ta * ((g.kc + GRAM_TILE - 1) / GRAM_TILE);
  const int want = max(1, ctas / max(1, g.ntile));
  g.rows = max(32, (((N + want - 1) / want) + 31) / 32 * 32);
  g.nrb = (N + g.rows - 1) / g.rows;
  return g;
}

template <typename T>
__global__ void __launch_bounds__(256) gram_part(int N, int a, int c, int R, const int32_t* __restrict__ rank,
                                                 const T* __restrict__ X, int ldx, const T* __restrict__ Y, int ldy,
                                                 double* __restrict__ part) {
  using A = typename GramAcc<T>::type;
  constexpr int TI = 32;
  __shared__ T xs[TI][GRAM_TILE + 1];
  __shared__ T ys[TI][GRAM_TILE + 1];
  const int tid = threadIdx.x;
  const int r = min(R, (int)*rank);
  const GramSplit g = gram_split(N, a, c, R, r, (int)gridDim.x);
  const int pa = tid & 15, pc = tid >> 4;  // 4 x 4 outputs: a0 + 4pa.., c0 + 4pc..
  for (int item = blockIdx.x; item < g.nrb * g.ntile; item += gridDim.x) {
    const int rb = item / g.ntile, tile = item % g.ntile;
    const int a0 = (tile % g.ta) * GRAM_TILE, c0 = (tile / g.ta) * GRAM_TILE;
    const int r0 = rb * g.rows, r1 = min(N, r0 + g.rows);
    A acc[4][4];
#pragma unroll
    for (int p = 0; p < 4; ++p)
#pragma unroll
      for (int q = 0; q < 4; ++q) acc[p][q] = A(0.0);
    for (int i0 = r0; i0 < r1; i0 += TI) {
      __syncthreads();  // the previous slab (or item) is consumed
      for (int e = tid; e < TI * GRAM_TILE; e += 256) {
        const int ii = e % TI, k = e / TI;
        const int i = i0 + ii;
        const bool ok = i < r1;
        xs[ii][k] = (ok && a0 + k < g.ka) ? X[i + (int64_t)panel_col(a, a0 + k, r, R) * ldx] : T(0);
        ys[ii][k] = (ok && c0 + k < g.kc) ? Y[i + (int64_t)panel_col(c, c0 + k, r, R) * ldy] : T(0);
      }
      __syncthreads();
#pragma unroll 4
      for (int ii = 0; ii < TI; ++ii) {
        T xv[4], yv[4];
#pragma unroll
        for (int p = 0; p < 4; ++p) xv[p] = xs[ii][4 * pa + p];
#pragma unroll
        for (int q = 0; q < 4; ++q) yv[q] = ys[ii][4 * pc + q];
#pragma unroll
        for (int p = 0; p < 4; ++p)
#pragma unroll
          for (int q = 0; q < 4; ++q) acc[p][q] = gacc_mul(acc[p][q], xv[p], yv[q]);
      }
#pragma unroll
      for (int p = 0; p < 4; ++p)
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[p][q] = renorm(acc[p][q]);
    }
    double* dst = part + (int64_t)item * GRAM_TILE * GRAM_TILE;
#pragma unroll
    for (int p = 0; p < 4; ++p)
#pragma unroll
      for (int q = 0; q < 4; ++q) dst[(4 * pa + p) + (4 * pc + q) * GRAM_TILE] = gacc_val(acc[p][q]);
  }
}

// out (a x c, ld ldo) = alpha * sum of the row blocks' partials + beta * out
// on the active entries, beta * out elsewhere (the Gram of zero columns);
// `ctas` as in gram_part's launch.  One warp per entry: the lanes stride over
// the row blocks, a fixed shuffle tree adds them (deterministic).
__global__ void __launch_bounds__(256) gram_reduce(int N, int a, int c, int R, const int32_t* __restrict__ rank,
                                                   int ctas, const double* __restrict__ part, double alpha,
                                                   double beta, double* __restrict__ out, int ldo) {
  const int lane = threadIdx.x & 31;
  const int o = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
  if (o >= a * c) return;  // warp-uniform
  const int r = min(R, (int)*rank);
  const GramSplit g = gram_split(N, a, c, R, r, ctas);
  const int i = o % a, j = o / a;
  const int ia = panel_act_index(a, i, r, R), jc = panel_act_index(c, j, r, R);
  double s = 0.0;
  if (ia >= 0 && jc >= 0) {
    const int tile = (ia / GRAM_TILE) + (jc / GRAM_TILE) * g.ta;
    const int64_t off = (ia % GRAM_TILE) + (int64_t)(jc % GRAM_TILE) * GRAM_TILE;
    for (int b = lane; b < g.nrb; b += 32) s += part[((int64_t)b * g.ntile + tile) * GRAM_TILE * GRAM_TILE + off];
  }
  for (int x = 16; x > 0; x >>= 1) s += __shfl_xor_sync(0xffffffffu, s, x);
  if (lane == 0) {
    double* d = out + i + (int64_t)j * ldo;
    *d = (beta == 0.0) ? alpha * s : fma(alpha, s, beta * *d);
  }
}

// ---------------------------------------------------------------------------
// Panel product: out (N x c, ld ldo) = X (N x a, ld ldx) B (a x c, FP64,
// ld ldb) + beta * out.  Grid (row blocks of 32) x (column tiles of 64);
// a <= 2*SMAX.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(256) panel_mul(int N, int a, int c, const T* __restrict__ X, int ldx,
                                                 const double* __restrict__ B, int ldb, T beta, T* __restrict__ out,
                                                 int ldo) {
  constexpr int KC2 = 32;
  __shared__ T xs[32][KC2 + 1];
  __shared__ T bs[KC2][65];
  const int tid = threadIdx.x;
  const int i0 = blockIdx.x * 32, c0 = blockIdx.y * 64;
  const int ri = tid & 15, cj = tid >> 4;  // rows ri, ri+16; columns cj + 16q
  T acc[2][4];
#pragma unroll
  for (int p = 0; p < 2; ++p)
#pragma unroll
    for (int q = 0; q < 4; ++q) acc[p][q] = T(0);
  for (int k0 = 0; k0 < a; k0 += KC2) {
    const int kc = min(KC2, a - k0);
    for (int e = tid; e < 32 * KC2; e += 256) {
      const int ii = e % 32, k = e / 32;
      const int i = i0 + ii;
      xs[ii][k] = (i < N && k < kc) ? X[i + (int64_t)(k0 + k) * ldx] : T(0);
    }
    for (int e = tid; e < KC2 * 64; e += 256) {
      const int k = e % KC2, cc = e / KC2;
      bs[k][cc] = (k < kc && c0 + cc < c) ? T(B[(k0 + k) + (int64_t)(c0 + cc) * ldb]) : T(0);
    }
    __syncthreads();
#pragma unroll 8
    for (int k = 0; k < KC2; ++k) {
      const T x0 = xs[ri][k], x1 = xs[ri + 16][k];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const T w = bs[k][cj + 16 * q];
        acc[0][q] = fma(x0, w, acc[0][q]);
        acc[1][q] = fma(x1, w, acc[1][q]);
      }
    }
    __syncthreads();
  }
#pragma unroll
  for (int p = 0; p < 2; ++p) {
    const int i = i0 + ri + 16 * p;
    if (i >= N) continue;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int j = c0 + cj + 16 * q;
      if (j >= c) continue;
      T* d = out + i + (int64_t)j * ldo;
      *d = (beta == T(0)) ? acc[p][q] : fma(beta, *d, acc[p][q]);
    }
  }
}

// out = X B for FP32 panels with double-float sums: B = Bh + Bl split into
// floats, X Bh accumulated from exact products (TwoProduct), X Bl added to
// the low part.  For orthonormalisation factors B whose entries are far
// larger than the entries of X B (the inverse Cholesky factor of a nearly
// dependent panel): FP32 sums would lose u32 * |X| |B| to cancellation.
__global__ void __launch_bounds__(256) panel_mul_df(int N, int a, int c, const float* __restrict__ X, int ldx,
                                                    const double* __restrict__ B, int ldb, float* __restrict__ out,
                                                    int ldo) {
  constexpr int KC2 = 32;
  __shared__ float xs[32][KC2 + 1];
  __shared__ float bh[KC2][65];
  __shared__ float bl[KC2][65];
  const int tid = threadIdx.x;
  const int i0 = blockIdx.x * 32, c0 = blockIdx.y * 64;
  const int ri = tid & 15, cj = tid >> 4;
  dfloat acc[2][4];
#pragma unroll
  for (int p = 0; p < 2; ++p)
#pragma unroll
    for (int q = 0; q < 4; ++q) acc[p][q] = dfloat(0.0f, 0.0f);
  for (int k0 = 0; k0 < a; k0 += KC2) {
    const int kc = min(KC2, a - k0);
    for (int e = tid; e < 32 * KC2; e += 256) {
      const int ii = e % 32, k = e / 32;
      const int i = i0 + ii;
      xs[ii][k] = (i < N && k < kc) ? X[i + (int64_t)(k0 + k) * ldx] : 0.0f;
    }
    for (int e = tid; e < KC2 * 64; e += 256) {
      const int k = e % KC2, cc = e / KC2;
      const double b = (k < kc && c0 + cc < c) ? B[(k0 + k) + (int64_t)(c0 + cc) * ldb] : 0.0;
      const float h = (float)b;
      bh[k][cc] = h;
      bl[k][cc] = (float)(b - (double)h);
    }
    __syncthreads();
    for (int k = 0; k < KC2; ++k) {
      const float x0 = xs[ri][k], x1 = xs[ri + 16][k];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const float wh = bh[k][cj + 16 * q], wl = bl[k][cj + 16 * q];
        acc[0][q] = acc_mul_acc(acc[0][q], x0, wh);
        acc[0][q].lo = fmaf(x0, wl, acc[0][q].lo);
        acc[1][q] = acc_mul_acc(acc[1][q], x1, wh);
        acc[1][q].lo = fmaf(x1, wl, acc[1][q].lo);
      }
    }
    __syncthreads();
  }
#pragma unroll
  for (int p = 0; p < 2; ++p) {
    const int i = i0 + ri + 16 * p;
    if (i >= N) continue;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int j = c0 + cj + 16 * q;
      if (j < c) out[i + (int64_t)j * ldo] = renorm(acc[p][q]).hi;
    }
  }
}

// B = (3I - G) / 2 (R x R): one Newton-Schulz step X <- X B for G = X^T X
__global__ void ns_factor(int R, const double* __restrict__ G, double* __restrict__ B) {
  const int o = blockIdx.x * blockDim.x + threadIdx.x;
  if (o < R * R) B[o] = ((o % R == o / R) ? 1.5 : 0.0) - 0.5 * G[o];
}

__global__ void negate(int k, double* x) {
  const int o = blockIdx.x * blockDim.x + threadIdx.x;
  if (o < k) x[o] = -x[o];
}

template <typename T>
__global__ void copy_cols(int N, int c, const T* __restrict__ X, int ldx, T* __restrict__ Y, int ldy) {
  const int64_t total = (int64_t)N * c;
  for (int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; o < total; o += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = o % N, j = o / N;
    Y[i + j * ldy] = X[i + j * ldx];
  }
}

// ---------------------------------------------------------------------------
// Single-CTA FP64 kernels (dynamic shared memory).
// ---------------------------------------------------------------------------

// Small-matrix arithmetic of the single-CTA kernels: double-float for FP32
// panels (the FP64 pipe of GB300 runs at 1/64 of the FP32 rate), FP64 for
// FP64 panels.
template <typename T> struct SmallT { using type = double; };
template <> struct SmallT<float> { using type = dfloat; };
__device__ __forceinline__ double to_d(double x) { return x; }
__device__ __forceinline__ double to_d(dfloat x) { return (double)x; }

constexpr int NTS = 1024;  // threads of the single-CTA kernels
constexpr size_t CORE_MAT = 160 * 1024;  // core_step's shared-memory matrix area (+ 40 KB of tiles)


// One CholeskyQR factor: G + shift_rel * trace(G) I = R^T R (a x a, ld a),
// Bout = R^{-1}; columns with G_jj <= tol_rel * max G_jj are decoupled
// (R_jj = 1, zero off-diagonal), so zero columns of the panel stay zero.
// R and R^{-1} in shared memory.
template <typename ST>
__global__ void __launch_bounds__(NTS) chol_inv_factor(int a, const double* __restrict__ G, double tol_rel,
                                                       double shift_rel, double* __restrict__ Bout) {
  extern __shared__ __align__(16) unsigned char smraw[];
  ST* R = reinterpret_cast<ST*>(smraw);  // a x a
  ST* Ri = R + a * a;                     // a x a
  __shared__ int keep[2 * SMAX];
  const int tid = threadIdx.x;
  double gmax = 0.0;
  for (int j = 0; j < a; ++j) gmax = fmax(gmax, G[j + (int64_t)j * a]);
  for (int j = tid; j < a; j += NTS) keep[j] = G[j + (int64_t)j * a] > tol_rel * gmax;
  __syncthreads();
  double tr = 0.0;
  for (int j = 0; j < a; ++j) tr += keep[j] ? G[j + (int64_t)j * a] : 0.0;
  for (int o = tid; o < a * a; o += NTS) {
    const int i = o % a, j = o / a;
    const bool kk = keep[i] && keep[j];
    R[o] = kk ? ST(G[o] + ((i == j) ? shift_rel * tr : 0.0)) : ST((i == j) ? 1.0 : 0.0);
  }
  __syncthreads();
  // right-looking Cholesky, upper factor in R (two barriers per column)
  for (int k = 0; k < a; ++k) {
    ST dk = R[k + k * a];
    if (!(to_d(dk) > 0.0)) dk = ST(1.0);
    const ST rkk = sqrt(dk);
    const ST inv = ST(1.0) / rkk;
    for (int j = k + 1 + tid; j < a; j += NTS) R[k + j * a] = R[k + j * a] * inv;
    __syncthreads();
    if (tid == 0) R[k + k * a] = rkk;
    const int cnt = a - k - 1;
    for (int e = tid; e < cnt * cnt; e += NTS) {
      const int i = k + 1 + e % cnt, j = k + 1 + e / cnt;
      if (i <= j) R[i + j * a] = R[i + j * a] - R[k + i * a] * R[k + j * a];
    }
    __syncthreads();
  }
  // R^{-1} row by row from the bottom: row i needs rows i+1.. (one barrier per row)
  for (int o = tid; o < a * a; o += NTS) Ri[o] = ST(0.0);
  __syncthreads();
  for (int i = a - 1; i >= 0; --i) {
    const ST rii = ST(1.0) / R[i + i * a];
    for (int j = i + tid; j < a; j += NTS) {
      ST sacc = (i == j) ? ST(1.0) : ST(0.0);
      for (int k = i + 1; k <= j; ++k) sacc = sacc - R[i + k * a] * Ri[k + j * a];
      Ri[i + j * a] = sacc * rii;
    }
    __syncthreads();
  }
  for (int o = tid; o < a * a; o += NTS) Bout[o] = to_d(Ri[o]);
}

// C (P x P, ld P) = op(A) B with op(A) = A or A^T, all in ST, NTS = 1024
// threads: 32 x 32 output tiles (one entry per thread) over 32-wide k
// chunks staged in shared memory (tile: 2 * 32 * 33 ST).  C must not alias
// A or B.
template <typename ST>
__device__ void sq_mul(int P, const ST* A, bool ta, const ST* B, ST* C, ST* tile) {
  static_assert(NTS == 1024, "one 32 x 32 tile per pass");
  ST* As = tile;
  ST* Bs = tile + 32 * 33;
  const int tid = threadIdx.x, ti = tid & 31, tj = tid >> 5;
  const int nt = (P + 31) / 32;
  for (int tI = 0; tI < nt; ++tI)
    for (int tJ = 0; tJ < nt; ++tJ) {
      ST acc(0.0);
      for (int k0 = 0; k0 < P; k0 += 32) {
        {
          const int i = tI * 32 + ti, k = k0 + tj;
          As[ti * 33 + tj] = (i < P && k < P) ? (ta ? A[k + i * P] : A[i + k * P]) : ST(0.0);
          const int kk = k0 + ti, j = tJ * 32 + tj;
          Bs[ti * 33 + tj] = (kk < P && j < P) ? B[kk + j * P] : ST(0.0);
        }
        __syncthreads();
#pragma unroll 8
        for (int k = 0; k < 32; ++k) acc = fma_acc(As[ti * 33 + k], Bs[k * 33 + tj], acc);
        __syncthreads();
      }
      const int i = tI * 32 + ti, j = tJ * 32 + tj;
      if (i < P && j < P) C[i + j * P] = renorm(acc);
    }
  __syncthreads();
}

// SVD of the P x P double-float matrix a (global, read only; right vectors
// to v): the Jacobi sweeps run in FP32 (a32, v32: P*P floats each, shared
// memory when they fit), the FP32 right vectors are made orthonormal to
// double-float precision by two Newton-Schulz steps X <- X (3I - X^T X) / 2,
// as = a X, and double-float sweeps polish the rotated matrix as (shared
// memory when it fits; it may overlay a32/v32, which are dead by then).  The
// columns of a X are orthogonal to FP32 precision, so one sweep squares that
// for well-separated singular values; directions whose singular values FP32
// cannot resolve need more sweeps.  t1, t2: P*P double-float scratch
// (global); tile: sq_mul's shared-memory tiles.
__device__ bool jacobi_svd_mixed(int P, const dfloat* a, dfloat* as, dfloat* v, dfloat* sig, int* perm, int* flag,
                                 float* a32, float* v32, float* sig32, dfloat* t1, dfloat* t2, dfloat* tile,
                                 int polish_sweeps, double tiny_abs = 0.0) {
  for (int o = threadIdx.x; o < P * P; o += NTS) a32[o] = a[o].hi + a[o].lo;
  __syncthreads();
  // FP32 sweeps as a preconditioner: near FP32's resolution limit they need
  // not converge (rotations between columns of very different size keep
  // re-creating rounding-level products), so at most 12
  jacobi_svd<float, NTS>(P, a32, v32, sig32, perm, flag, 12, false);
  for (int o = threadIdx.x; o < P * P; o += NTS) t1[o] = dfloat(v32[o], 0.0f);  // X0 = V32
  __syncthreads();
  for (int it = 0; it < 2; ++it) {
    sq_mul<dfloat>(P, t1, true, t1, t2, tile);                                       // X^T X
    for (int o = threadIdx.x; o < P * P; o += NTS) {
      const int i = o % P, j = o / P;
      t2[o] = ((i == j) ? dfloat(1.5f, 0.0f) : dfloat(0.0f, 0.0f)) - dfloat(0.5f, 0.0f) * t2[o];
    }
    __syncthreads();
    sq_mul<dfloat>(P, t1, false, t2, v, tile);                                       // X (3I - X^T X)/2
    for (int o = threadIdx.x; o < P * P; o += NTS) t1[o] = v[o];
    __syncthreads();
  }
  sq_mul<dfloat>(P, a, false, t1, t2, tile);                                         // a X
  for (int o = threadIdx.x; o < P * P; o += NTS) as[o] = t2[o];
  __syncthreads();
  // polish: a = U S, V_p, until the rotations are below 1e-4 (left vectors
  // orthogonal to ~P 1e-8, singular values to ~1e-8 relative: the FP32
  // panels' level; the factors' Newton-Schulz refresh absorbs the rest)
  const bool ok = jacobi_svd<dfloat, NTS>(P, as, v, sig, perm, flag, polish_sweeps, true, 1e-4, tiny_abs);
  sq_mul<dfloat>(P, t1, false, v, t2, tile);                                         // V = X V_p
  for (int o = threadIdx.x; o < P * P; o += NTS) v[o] = t2[o];
  __syncthreads();
  return ok;
}

// Rank-revealing orthonormalisation factor of a Gram matrix G (a x a, ld a)
// restricted to its leading r x r block (r = *rank: the panel's columns
// beyond the rank are zero): Cholesky with diagonal pivoting of the scaled
// Gram D G D (D = diag(G)^{-1/2}), D G D = Pi R^T R Pi^T, stopped when the
// largest remaining diagonal entry (the squared distance of a unit column
// from the span of those chosen) is <= tol_rel.  Bout (a x a, zero outside
// the leading k x k block, k the revealed rank) = D Pi R^{-1}, so X Bout has
// k orthonormal columns up to about (error of G) / tol_rel and zero columns
// after them.  Columns whose squared norm is <= tol_rel of the largest are
// rounding noise of the panel and are dropped before the scaling (which
// would hide that).  Factor and inverse in shared memory (2 r (r + 1) ST); one CTA
// of NTP threads: the pivot steps are a chain of barriers, so few warps.
// R^{-1} by 16 x 16 blocks: the diagonal blocks by back substitution (one
// warp each, a lane per column), then the block diagonals d = 1, 2, ... as
// Ri_IJ = -Ri_II sum_{K = I+1..J} R_IK Ri_KJ (one thread per entry).
constexpr int NTP = 256;
constexpr int PCB = 16;  // block size of the triangular inverse
static_assert(NTP == PCB * PCB, "one thread per entry of a 16 x 16 block");
template <typename ST>
__global__ void __launch_bounds__(NTP) pchol_factor(int a, const double* __restrict__ G, const int32_t* rank,
                                                    double tol_rel, double* __restrict__ Bout) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int r = min(a, (int)*rank);
  const int ld = r + 1;                   // odd: rows of A read across lanes hit distinct banks
  ST* A = reinterpret_cast<ST*>(smraw);  // r x r, column-major, ld
  ST* Ri = A + r * ld;                    // r x r, ld
  __shared__ double d[SMAX];
  __shared__ int piv[SMAX];
  __shared__ double red[NTP / 32];
  __shared__ __align__(16) unsigned char tb_raw[PCB * PCB * sizeof(ST)];
  ST* Tb = reinterpret_cast<ST*>(tb_raw);
  __shared__ int pk_s, kk_s;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  constexpr int NWP = NTP / 32;
  double gm = 0.0;
  for (int j = tid; j < r; j += NTP) gm = fmax(gm, G[j + (int64_t)j * a]);
  for (int o = 16; o > 0; o >>= 1) gm = fmax(gm, __shfl_xor_sync(0xffffffffu, gm, o));
  if (lane == 0) red[warp] = gm;
  __syncthreads();
  double gmax = 0.0;
  for (int w = 0; w < NWP; ++w) gmax = fmax(gmax, red[w]);
  for (int j = tid; j < r; j += NTP) {
    const double g = G[j + (int64_t)j * a];
    d[j] = (g > tol_rel * gmax && g > 0.0) ? 1.0 / sqrt(g) : 0.0;
    piv[j] = j;
  }
  __syncthreads();
  for (int o = tid; o < r * r; o += NTP) {
    const int i = o % r, j = o / r;
    A[i + j * ld] = ST(d[i] * G[i + (int64_t)j * a] * d[j]);
  }
  if (tid == 0) kk_s = r;
  __syncthreads();
  for (int k = 0; k < r; ++k) {
    if (warp == 0) {  // pivot: the largest remaining diagonal entry (first on ties), compared in ST
      ST best = ST(-1.0);
      int bi = k;
      for (int j = k + lane; j < r; j += 32) {
        const ST v = A[j + j * ld];
        if (v > best) { best = v; bi = j; }
      }
      for (int o = 16; o > 0; o >>= 1) {
        const ST ob = shfl_xor(best, o);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
      }
      if (lane == 0) {
        pk_s = bi;
        if (!(best > ST(tol_rel))) kk_s = k;
      }
    }
    __syncthreads();
    if (kk_s == k) break;
    const int p = pk_s;
    if (p != k) {
      // symmetric swap of rows and columns k < p in one pass: R's rows above
      // k swap columns only, the trailing symmetric block rows and columns,
      // the diagonal entries trade places and A[k, p] = A[p, k] stays
      for (int i = tid; i < r; i += NTP) {
        if (i == k) {
          const ST t = A[k + k * ld];
          A[k + k * ld] = A[p + p * ld];
          A[p + p * ld] = t;
          const int tp = piv[k];
          piv[k] = piv[p];
          piv[p] = tp;
        } else if (i != p) {
          const ST t = A[i + k * ld];
          A[i + k * ld] = A[i + p * ld];
          A[i + p * ld] = t;
          if (i > k) {
            const ST u = A[k + i * ld];
            A[k + i * ld] = A[p + i * ld];
            A[p + i * ld] = u;
          }
        }
      }
      __syncthreads();
    }
    const ST rkk = sqrt(A[k + k * ld]);
    const ST inv = ST(1.0) / rkk;
    for (int j = k + 1 + tid; j < r; j += NTP) A[k + j * ld] = A[k + j * ld] * inv;
    __syncthreads();
    if (tid == 0) A[k + k * ld] = rkk;
    // trailing update of the full symmetric block (rows and columns > k):
    // a warp per column, lanes down the rows
    for (int j = k + 1 + warp; j < r; j += NWP) {
      const ST akj = A[k + j * ld];
      for (int i = k + 1 + lane; i < r; i += 32) A[i + j * ld] = A[i + j * ld] - A[k + i * ld] * akj;
    }
    __syncthreads();
  }
  const int kk = kk_s;
  // R^{-1} (kk x kk, upper triangular; R in the upper triangle of A)
  for (int o = tid; o < r * ld; o += NTP) Ri[o] = ST(0.0);
  __syncthreads();
  const int nb = (kk + PCB - 1) / PCB;
  for (int b = warp; b < nb; b += NWP) {  // diagonal blocks: lane = column
    const int b0 = b * PCB, mb = min(PCB, kk - b0);
    if (lane < mb) {
      const int j = b0 + lane;
      Ri[j + j * ld] = ST(1.0) / A[j + j * ld];
      for (int i = j - 1; i >= b0; --i) {
        ST sacc = ST(0.0);
        for (int q = i + 1; q <= j; ++q) sacc = sacc + A[i + q * ld] * Ri[q + j * ld];
        Ri[i + j * ld] = -(sacc / A[i + i * ld]);
      }
    }
  }
  __syncthreads();
  for (int dd = 1; dd < nb; ++dd)
    for (int I = 0; I + dd < nb; ++I) {
      const int i0 = I * PCB, j0 = (I + dd) * PCB;
      const int mi = min(PCB, kk - i0), mj = min(PCB, kk - j0);
      const int ii = tid % PCB, jj = tid / PCB;  // NTP = PCB^2 entries
      const int i = i0 + ii, j = j0 + jj;
      const bool ok = ii < mi && jj < mj;
      if (ok) {  // T = sum_{K = I+1..J} R_IK Ri_KJ (Ri_KJ is zero below row j)
        ST sacc = ST(0.0);
        for (int q = i0 + PCB; q <= j; ++q) sacc = sacc + A[i + q * ld] * Ri[q + j * ld];
        Tb[ii + jj * PCB] = sacc;
      }
      __syncthreads();
      if (ok) {  // Ri_IJ = -Ri_II T
        ST sacc = ST(0.0);
        for (int q = i; q < i0 + mi; ++q) sacc = sacc + Ri[i + q * ld] * Tb[(q - i0) + jj * PCB];
        Ri[i + j * ld] = -sacc;
      }
      __syncthreads();
    }
  for (int o = tid; o < a * a; o += NTP) Bout[o] = 0.0;
  __syncthreads();
  for (int o = tid; o < kk * kk; o += NTP) {
    const int i = o % kk, j = o / kk;
    const int pi = piv[i];
    Bout[pi + (int64_t)j * a] = d[pi] * to_d(Ri[i + j * ld]);
  }
}

// The active block of S~ = Mh S0 Nh^T + D (FP64, compact wa x wa, ld wa),
// wa = 2r, for core_step: form_t1 (T1 = S0 Nh^T, r x wa, ld r), then
// form_core; one thread per entry over the whole GPU (the products are
// r^2 wa + r wa^2 FP64 multiply-adds, far too slow on one SM).
template <typename T>
__global__ void form_t1(int R, const int32_t* __restrict__ rank, const T* __restrict__ S0,
                        const double* __restrict__ Nh, double* __restrict__ T1) {
  const int r = min(R, (int)*rank), wa = 2 * r, w = 2 * R;
  const int64_t len = (int64_t)r * wa;
  for (int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; o < len; o += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(o % r), j = (int)(o / r);
    const int jj = act_col(j, r, R);
    double sacc = 0.0;
#pragma unroll 8
    for (int k = 0; k < r; ++k) sacc = fma((double)S0[i + (int64_t)k * R], Nh[jj + (int64_t)k * w], sacc);
    T1[o] = sacc;
  }
}
__global__ void form_core(int R, const int32_t* __restrict__ rank, const double* __restrict__ Mh,
                          const double* __restrict__ T1, const double* __restrict__ D, double* __restrict__ F) {
  const int r = min(R, (int)*rank), wa = 2 * r, w = 2 * R;
  const int64_t len = (int64_t)wa * wa;
  for (int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; o < len; o += (int64_t)gridDim.x * blockDim.x) {
    const int i = act_col((int)(o % wa), r, R), j = (int)(o / wa);
    double sacc = D[i + (int64_t)act_col(j, r, R) * w];
#pragma unroll 8
    for (int k = 0; k < r; ++k) sacc = fma(Mh[i + (int64_t)k * w], T1[k + (int64_t)j * r], sacc);
    F[o] = sacc;
  }
}

// S-step core and truncation.  In: Mh = Uhat^T U0 (w x R), Nh = Vhat^T V0
// (w x R), D = Uhat^T dY Vhat (w x w), S0 (R x R, T), rank (device).  Out:
// P1, Q1 (w x R FP64: the kept left / right singular vectors, zero beyond
// the new rank), S (R x R, diag), rank.  The SVD runs in ST (double-float
// for FP32 panels: an FP32 Jacobi SVD of a w x w matrix accumulates
// O(w u) rotation error per sweep) with the w x w matrix in shared memory
// when it fits, else in the global scratch ag; the right vectors in vg.
template <typename T, typename ST>
__global__ void __launch_bounds__(NTS) core_step(int R, const double* __restrict__ F, T* S0, int32_t* rank,
                                                 double tol, int rmin, ST* __restrict__ ag, ST* __restrict__ vg,
                                                 double* __restrict__ P1, double* __restrict__ Q1, uint32_t* status,
                                                 double* __restrict__ mx) {
  extern __shared__ __align__(16) unsigned char smraw[];
  __shared__ __align__(16) unsigned char sig_raw[2 * SMAX * sizeof(ST)];
  ST* sig = reinterpret_cast<ST*>(sig_raw);
  __shared__ int perm[2 * SMAX + 1];
  __shared__ int flag;
  __shared__ int r_new;
  const int tid = threadIdx.x;
  const int w = 2 * R;
  // active rows / columns: the first r of each half of [U0 | Q] ([V0 | Q])
  const int r = min(R, (int)*rank), wa = 2 * r;
  auto idx = [&](int i) { return (i < r) ? i : R + (i - r); };
  // shared memory: [0, CORE_MAT) the wa x wa matrix being rotated (or the
  // two FP32 matrices of the mixed SVD) when it fits, then sq_mul's tiles
  const bool a_in_smem = (size_t)wa * wa * sizeof(ST) <= CORE_MAT;
  ST* tile = reinterpret_cast<ST*>(smraw + CORE_MAT);
  ST* a = ag;  // wa x wa; the rotated matrix of the polish, below
  ST* v = vg;  // wa x wa
  for (int o = tid; o < wa * wa; o += NTS) a[o] = ST(F[o]);
  __syncthreads();
  // FP32 panels: the sweeps leave alone pairs whose columns both have squared
  // norm <= tol^2 / (4 wa).  Such columns together hold less than tol^2 / 4
  // and are rotated against every larger column, so the kept singular
  // directions are those of the exact SVD.  FP64 panels exist for parity with
  // the reference: no truncation-level skip there.
  const double tiny_abs = std::is_same<ST, double>::value ? 0.0 : tol * tol / (4.0 * wa);
  bool ok;
  if constexpr (sizeof(ST) == 8 && !std::is_same<ST, double>::value) {
    // double-float: FP32 sweeps, double-float polish; the FP32 pair and
    // then the polished matrix in shared memory when they fit (same bytes)
    float* a32 = a_in_smem ? reinterpret_cast<float*>(smraw) : reinterpret_cast<float*>(mx);
    float* v32 = a32 + wa * wa;
    __shared__ float sig32[2 * SMAX];
    ST* as = a_in_smem ? reinterpret_cast<ST*>(smraw) : ag;
    // (double-float sweeps to convergence: kept singular values far below the
    // largest are beyond what the FP32 sweeps resolve, and their left vectors
    // a_j / sigma_j need the double-float accuracy)
    ok = jacobi_svd_mixed(wa, ag, as, v, sig, perm, &flag, a32, v32, sig32,
                          reinterpret_cast<ST*>(mx) + wa * wa, reinterpret_cast<ST*>(mx) + 2 * wa * wa, tile, 40,
                          tiny_abs);
    a = as;
  } else {
    if (a_in_smem) {
      ST* as = reinterpret_cast<ST*>(smraw);
      for (int o = tid; o < wa * wa; o += NTS) as[o] = a[o];
      __syncthreads();
      a = as;
    }
    ok = jacobi_svd<ST, NTS>(wa, a, v, sig, perm, &flag, 40, true, -1.0, tiny_abs);
  }
  // smallest r1 with sum_{j > r1} sigma_j^2 < tol^2, then [rmin, R] (thread 0)
  auto decide_rank = [&]() {
    const double tol2 = tol * tol;
    double acc = 0.0;
    int rr = wa;
    while (acc < tol2 && rr > 0) {
      const double sv = to_d(sig[perm[rr - 1]]);
      acc += sv * sv;
      --rr;
    }
    int r1 = rr + 1;
    if (r1 > R) r1 = R;
    if (r1 < rmin) r1 = rmin;
    if (r1 > wa) r1 = wa;
    return r1;
  };
  __shared__ int redo;
  if (tid == 0) {
    r_new = decide_rank();
    const double sv = to_d(sig[perm[r_new - 1]]);
    redo = (tiny_abs > 0.0 && sv * sv <= 4.0 * tiny_abs);  // the minimum rank keeps skipped columns
  }
  __syncthreads();
  double tiny_left = tiny_abs;
  if (redo) {
    // continue the sweeps without the truncation-level skip (v <- v v2)
    ST* v2 = reinterpret_cast<ST*>(mx) + (size_t)wa * wa;
    ST* t2 = reinterpret_cast<ST*>(mx) + (size_t)2 * wa * wa;
    const double conv = std::is_same<ST, double>::value ? -1.0 : 1e-4;
    ok = jacobi_svd<ST, NTS>(wa, a, v2, sig, perm, &flag, 40, true, conv, 0.0);
    sq_mul<ST>(wa, v, false, v2, t2, tile);
    for (int o = tid; o < wa * wa; o += NTS) v[o] = t2[o];
    __syncthreads();
    if (tid == 0) r_new = decide_rank();
    tiny_left = 0.0;
    __syncthreads();
  }
  if (tid == 0) {
    if (!ok) atomicOr(status, ST_SVD_NOCONV);
    *rank = r_new;
  }
  __syncthreads();
  const int r1 = r_new;
  // left vectors a_j / sigma_j in place (P1 as scratch before it is written)
  complete_left<ST, NTS>(wa, r1, a, sig, perm, reinterpret_cast<ST*>(P1), tiny_left);
  for (int o = tid; o < w * R; o += NTS) P1[o] = Q1[o] = 0.0;
  __syncthreads();
  for (int o = tid; o < wa * r1; o += NTS) {
    const int i = o % wa, j = o / wa;
    const int pj = perm[j];
    P1[idx(i) + (int64_t)j * w] = to_d(a[i + (int64_t)pj * wa]);
    Q1[idx(i) + (int64_t)j * w] = to_d(v[i + (int64_t)pj * wa]);
  }
  for (int o = tid; o < R * R; o += NTS) {
    const int i = o % R, j = o / R;
    S0[o] = (i == j && i < r1) ? T(to_d(sig[perm[i]])) : T(0);
  }
  __syncthreads();
  bool bad = false;
  for (int o = tid; o < R * R; o += NTS) bad |= !isfinite((double)S0[o]);
  if (__syncthreads_or(bad) && tid == 0) atomicOr(status, ST_NONFINITE);
}

// ---------------------------------------------------------------------------
// Periodic Burgers flow on one large instance, spread over the GPU:
//   F(Y) = (Dxx Y) diag(nu) + alpha (Dx Y).*Y + beta Dx(Y.*Y),
// periodic central differences Dx = tridiag(-1, 0, 1) / 2h (Dx^T = -Dx),
// Dxx = tridiag(1, -2, 1) / h^2 (symmetric), one column per sample.
// The substep flows never form the N x M matrix Y.  With Y = K V^T:
//   (Dxx Y) diag(nu) V      = (Dxx K) (V^T diag(nu) V)
//   ((Dx Y).*Y) V, row i    = sum_{a,b} (Dx K)_ia K_ib T_V[a,b,:]
//   (Y.*Y) V, row i         = sum_{a,b} K_ia K_ib T_V[a,b,:]
// with the symmetric tensor T_V[a,b,c] = sum_j V_ja V_jb V_jc, formed once
// per step.  The L and S substeps have the same structure (their tensors
// below).  Per RK stage this costs O((N + M) r^3 / 2) against O(N M r) for
// the dense tiles; the tensors cost O(M r^3 / 2) once per step.
// Tensors are stored over packed pairs a <= b of the active columns (ka of
// them: r, or 2r for the augmented bases, whose active columns are the first
// r of each half), with the off-diagonal pairs counted twice:
//   T'[p(a,b), c] = c_ab T[a,b,c],  c_ab = 1 (a = b), 2 (a < b),
// and the Khatri-Rao rows KR(P,Q)_i,p(a,b) = (P_ia Q_ib + P_ib Q_ia) / 2, so
// sum_{a,b} P_ia Q_ib T[a,b,c] = sum_p KR(P,Q)_ip T'[p,c] for T symmetric
// in (a,b).  All launch shapes depend on r_max only; the active rank is read
// on the device, so a step is one fixed launch sequence.
// ---------------------------------------------------------------------------
constexpr int KR_ROWS = 1024;  // rows per split of the tensor sums

__device__ __forceinline__ int active_cols(const int32_t* rank, int R, int aug) {
  const int r = min(R, (int)*rank);
  return aug ? 2 * r : r;
}
// packed pair p (0 <= p < ka (ka + 1) / 2) -> (a, b), a <= b < ka, row-wise:
// pairs of a start at a ka - a (a - 1) / 2
__device__ __forceinline__ void pair_ab(int p, int ka, int& a, int& b) {
  const double q = 2.0 * ka + 1.0;
  int x = (int)((q - sqrt(q * q - 8.0 * p)) * 0.5);
  x = max(0, min(x, ka - 1));
  while (x > 0 && x * ka - x * (x - 1) / 2 > p) --x;
  while (x + 1 < ka && (x + 1) * ka - (x + 1) * x / 2 <= p) ++x;
  a = x;
  b = a + (p - (a * ka - a * (a - 1) / 2));
}

// part[s] (pairs x ka, ld PP) = sum over the rows of split s of
// KR(P,Q)^T Y (active columns of Y).  Grid (pair tiles of 64, column tiles
// of 64, row splits of KR_ROWS rows); tiles beyond the active sizes exit.
template <typename T>
__global__ void __launch_bounds__(256) kr_gram_part(int N, int R, int aug, const int32_t* __restrict__ rank,
                                                    const T* __restrict__ P, const T* __restrict__ Q,
                                                    const T* __restrict__ Y, int PP, T* __restrict__ part) {
  const int ka = active_cols(rank, R, aug), r = min(R, (int)*rank);
  const int np = ka * (ka + 1) / 2;
  const int p0 = blockIdx.x * 64, c0 = blockIdx.y * 64;
  if (p0 >= np || c0 >= ka) return;
  __shared__ int pa[64], pb[64];
  __shared__ __align__(16) T krs[32][64];
  __shared__ __align__(16) T ys[32][64];
  const int tid = threadIdx.x;
  if (tid < 64) {
    int a = 0, b = 0;
    if (p0 + tid < np) pair_ab(p0 + tid, ka, a, b);
    pa[tid] = act_col(a, r, R);
    pb[tid] = act_col(b, r, R);
  }
  const int tp = tid & 15, tc = tid >> 4;  // pairs 4 tp.., columns 4 tc..
  T acc[4][4];
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) acc[u][v] = T(0);
  const int j_lo = blockIdx.z * KR_ROWS, j_hi = min(N, j_lo + KR_ROWS);
  __syncthreads();
  for (int j0 = j_lo; j0 < j_hi; j0 += 32) {
    for (int e = tid; e < 32 * 64; e += 256) {
      const int jj = e & 31, pp = e >> 5;
      const int j = j0 + jj;
      T kv = T(0), yv = T(0);
      if (j < j_hi) {
        if (p0 + pp < np) {
          const T pa_ = P[j + (int64_t)pa[pp] * N], pb_ = P[j + (int64_t)pb[pp] * N];
          const T qa_ = Q[j + (int64_t)pa[pp] * N], qb_ = Q[j + (int64_t)pb[pp] * N];
          kv = T(0.5) * (pa_ * qb_ + pb_ * qa_);
        }
        if (c0 + pp < ka) yv = Y[j + (int64_t)act_col(c0 + pp, r, R) * N];
      }
      krs[jj][pp] = kv;
      ys[jj][pp] = yv;
    }
    __syncthreads();
#pragma unroll 4
    for (int jj = 0; jj < 32; ++jj) {
      T kv[4], yv[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) kv[u] = krs[jj][tp * 4 + u];
#pragma unroll
      for (int v = 0; v < 4; ++v) yv[v] = ys[jj][tc * 4 + v];
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) acc[u][v] = fma(kv[u], yv[v], acc[u][v]);
    }
    __syncthreads();
  }
  T* dst = part + (int64_t)blockIdx.z * PP * (2 * R);
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    const int p = p0 + tp * 4 + u;
    if (p >= np) continue;
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const int c = c0 + tc * 4 + v;
      if (c < ka) dst[p + (int64_t)c * PP] = acc[u][v];
    }
  }
}

// Tout[p, c] = (acc ? Tout[p, c] : 0) + coef c_ab sum_s part[s][p, c] (FP64
// sums of the split partials), over the active pairs and columns.
template <typename T>
__global__ void kr_reduce(int R, int aug, const int32_t* __restrict__ rank, int nsplit, int PP,
                          const T* __restrict__ part, double coef, int acc, T* __restrict__ Tout) {
  const int ka = active_cols(rank, R, aug);
  const int np = ka * (ka + 1) / 2;
  const int64_t len = (int64_t)np * ka;
  for (int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; o < len; o += (int64_t)gridDim.x * blockDim.x) {
    const int p = (int)(o % np), c = (int)(o / np);
    int a, b;
    pair_ab(p, ka, a, b);
    double sum = 0.0;
    for (int s = 0; s < nsplit; ++s) sum += (double)part[(int64_t)s * PP * (2 * R) + p + (int64_t)c * PP];
    const double v = coef * ((a == b) ? 1.0 : 2.0) * sum;
    T* d = Tout + p + (int64_t)c * PP;
    *d = acc ? T((double)*d + v) : T(v);
  }
}

// part[z] (N x 2R panel, active columns) = scale * sum_{a in split z}
// diag(X[:, a]) Y[:, a:ka] T'[p(a, a..ka-1), :] -- the packed Khatri-Rao
// product KR(X,X) T' for Y = X; for X != Y the symmetrised one needs the
// sum of (X, Y) and (Y, X) at scale 1/2.  The pairs of a are contiguous rows
// of T', so the inner loop is a plain GEMM of the staged rows of Y with
// 32-row chunks of T' (double-buffered through registers), and the
// Khatri-Rao products are never formed.  Grid (row tiles of BM, column tiles
// of 64, splits of the a range with about equal pair counts); 256 threads,
// 8 x 4 (FP32) or 4 x 4 (FP64) outputs per thread.  Dynamic shared memory:
// the active columns of the tile's rows of Y (and of X when distinct),
// ka x BM each.
template <typename T>
struct KrTile {
  static constexpr int BM = (sizeof(T) == 4) ? 128 : 64;
  static constexpr int TM = BM / 16;  // rows per thread
};
constexpr int KR_KB = 32;

// n consecutive values from 16-byte aligned shared memory (n a multiple of 4)
template <int n>
__device__ __forceinline__ void ld_vec(const float* p, float* out) {
#pragma unroll
  for (int q = 0; q < n / 4; ++q) {
    const float4 v = reinterpret_cast<const float4*>(p)[q];
    out[4 * q] = v.x;
    out[4 * q + 1] = v.y;
    out[4 * q + 2] = v.z;
    out[4 * q + 3] = v.w;
  }
}
template <int n>
__device__ __forceinline__ void ld_vec(const double* p, double* out) {
#pragma unroll
  for (int q = 0; q < n / 2; ++q) {
    const double2 v = reinterpret_cast<const double2*>(p)[q];
    out[2 * q] = v.x;
    out[2 * q + 1] = v.y;
  }
}

template <typename T, bool SAME>
__global__ void __launch_bounds__(256) kr_apply_part(int N, int R, int aug, const int32_t* __restrict__ rank,
                                                     const T* __restrict__ X, const T* __restrict__ Y,
                                                     const T* __restrict__ Tp, int PP, double scale, int accum,
                                                     T* __restrict__ part) {
  constexpr int BM = KrTile<T>::BM, TM = KrTile<T>::TM;
  extern __shared__ __align__(16) unsigned char smraw[];
  const int ka = active_cols(rank, R, aug), r = min(R, (int)*rank);
  const int np = ka * (ka + 1) / 2;
  const int i0 = blockIdx.x * BM, c0 = blockIdx.y * 64;
  if (c0 >= ka) return;
  // a range of this split: the a whose pair rows start in [z np / Z, (z+1) np / Z)
  auto start = [&](int a) { return a * ka - a * (a - 1) / 2; };
  auto first_a = [&](int64_t pb) {
    int x = 0;
    while (x < ka && start(x) < pb) ++x;
    return x;
  };
  const int a_lo = first_a((int64_t)blockIdx.z * np / gridDim.z);
  const int a_hi = first_a((int64_t)(blockIdx.z + 1) * np / gridDim.z);
  T* ys = reinterpret_cast<T*>(smraw);        // ka x BM (column b: the tile's rows)
  T* xs = SAME ? ys : ys + (size_t)ka * BM;   // ka x BM
  __shared__ __align__(16) T ts[2][KR_KB][64];
  const int tid = threadIdx.x;
  const int rows = min(BM, N - i0);
  for (int e = tid; e < BM * ka; e += 256) {
    const int ii = e % BM, b = e / BM;
    const int64_t off = (int64_t)act_col(b, r, R) * N + i0 + ii;
    ys[e] = (ii < rows) ? Y[off] : T(0);
    if (!SAME) xs[e] = (ii < rows) ? X[off] : T(0);
  }
  const int tr = tid >> 4, tc = tid & 15;  // rows TM tr.., columns 4 tc..
  T acc[TM][4];
#pragma unroll
  for (int u = 0; u < TM; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) acc[u][v] = T(0);
  // chunk sequence: for a in [a_lo, a_hi), b0 = a, a + KB, ... < ka
  int a = a_lo, b0 = a_lo;
  T pre[KR_KB * 64 / 256];
  auto load_chunk = [&](int ca, int cb0) {
#pragma unroll
    for (int q = 0; q < KR_KB * 64 / 256; ++q) {
      const int e = tid + q * 256;
      const int bb = e >> 6, cc = e & 63;
      const int b = cb0 + bb;
      pre[q] = (ca < a_hi && b < ka && c0 + cc < ka) ? Tp[(start(ca) + (b - ca)) + (int64_t)(c0 + cc) * PP] : T(0);
    }
  };
  auto store_chunk = [&](int buf) {
#pragma unroll
    for (int q = 0; q < KR_KB * 64 / 256; ++q) {
      const int e = tid + q * 256;
      ts[buf][e >> 6][e & 63] = pre[q];
    }
  };
  if (a < a_hi) load_chunk(a, b0);
  __syncthreads();
  store_chunk(0);
  __syncthreads();
  int buf = 0;
  T g[TM][4];
#pragma unroll
  for (int u = 0; u < TM; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) g[u][v] = T(0);
  while (a < a_hi) {
    // next chunk position, prefetched into registers during this one
    int na = a, nb0 = b0 + KR_KB;
    if (nb0 >= ka) { ++na; nb0 = na; }
    if (na < a_hi) load_chunk(na, nb0);
    const int kc = min(KR_KB, ka - b0);
    for (int bb = 0; bb < kc; ++bb) {
      T yv[TM], tv[4];
      ld_vec<TM>(ys + (size_t)(b0 + bb) * BM + tr * TM, yv);
      ld_vec<4>(&ts[buf][bb][tc * 4], tv);
#pragma unroll
      for (int u = 0; u < TM; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) g[u][v] = fma(yv[u], tv[v], g[u][v]);
    }
    if (na != a) {  // a done: acc += X[:, a] g
      const T* xrow = xs + (size_t)a * BM + tr * TM;
#pragma unroll
      for (int u = 0; u < TM; ++u) {
        const T xv = xrow[u];
#pragma unroll
        for (int v = 0; v < 4; ++v) {
          acc[u][v] = fma(xv, g[u][v], acc[u][v]);
          g[u][v] = T(0);
        }
      }
    }
    a = na;
    b0 = nb0;
    if (a < a_hi) {
      store_chunk(buf ^ 1);
      __syncthreads();
      buf ^= 1;
    }
  }
  T* dst = part + (int64_t)blockIdx.z * N * (2 * R);
#pragma unroll
  for (int u = 0; u < TM; ++u) {
    const int i = i0 + tr * TM + u;
    if (i >= N) continue;
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const int c = c0 + tc * 4 + v;
      if (c < ka) {
        T* d = dst + i + (int64_t)act_col(c, r, R) * N;
        *d = accum ? fma(T(scale), acc[u][v], *d) : T(scale) * acc[u][v];
      }
    }
  }
}

// Dxx X and Dx X (periodic) on the active columns: d2 = c2 Dxx X, d1 = c1 Dx X
// (either may be null); the other columns are set to zero.
template <typename T>
__global__ void stencil_panel(int N, int R, int aug, const int32_t* __restrict__ rank, const T* __restrict__ X,
                              double c2, T* __restrict__ d2, double c1, T* __restrict__ d1) {
  const int r = min(R, (int)*rank);
  const int wcols = aug ? 2 * R : R;
  const int64_t len = (int64_t)N * wcols;
  for (int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; o < len; o += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(o % N), col = (int)(o / N);
    const bool act = (col % R) < r;
    const T* x = X + (int64_t)col * N;
    const T xm = act ? x[(i == 0) ? N - 1 : i - 1] : T(0), xp = act ? x[(i == N - 1) ? 0 : i + 1] : T(0);
    if (d2) d2[o] = act ? T(c2) * ((xm + xp) - T(2) * x[i]) : T(0);
    if (d1) d1[o] = act ? T(c1) * (xp - xm) : T(0);
  }
}

// One explicit RK stage update fused into the kernel that assembles the
// stage derivative v (tableau with sub-diagonal a only, as lri_scheme):
// acc = (first ? 0 : acc) + b v; before the last stage the next stage input
// z = y + h a_{s+1} v, at the last stage y += h acc.
template <typename T>
struct RkStage {
  T b, ha, h;
  int first, last;
  T* y;
  T* z;
  T* acc;
};
template <typename T>
__device__ __forceinline__ void rk_apply(const RkStage<T>& c, int64_t o, T v) {
  const T a = c.first ? c.b * v : fma(c.b, v, c.acc[o]);
  if (c.last) {
    c.y[o] = fma(c.h, a, c.y[o]);
  } else {
    c.acc[o] = a;
    c.z[o] = fma(c.ha, v, c.y[o]);
  }
}

// out = lin + alpha sum_z part1[z] + beta Dx(sum_z part2[z]) on the active
// columns (lin, part1, part2 may be null), zero elsewhere; ihx = 1 / 2h.
template <typename T>
__global__ void flow_combine(int N, int R, int aug, const int32_t* __restrict__ rank, const T* __restrict__ lin,
                             const T* __restrict__ part1, const T* __restrict__ part2, int nz, double alpha,
                             double beta, double ihx, T* __restrict__ out, RkStage<T> rk) {
  const int r = min(R, (int)*rank);
  const int wcols = aug ? 2 * R : R;
  const int64_t len = (int64_t)N * wcols, zs = (int64_t)N * 2 * R;
  for (int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; o < len; o += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(o % N), col = (int)(o / N);
    T v = T(0);
    if ((col % R) < r) {
      v = lin ? lin[o] : T(0);
      if (part1) {
        T sacc = T(0);
        for (int z = 0; z < nz; ++z) sacc += part1[z * zs + o];
        v = fma(T(alpha), sacc, v);
      }
      if (part2) {
        const int64_t om = o - i + ((i == 0) ? N - 1 : i - 1), op = o - i + ((i == N - 1) ? 0 : i + 1);
        T sm = T(0), sp = T(0);
        for (int z = 0; z < nz; ++z) {
          sm += part2[z * zs + om];
          sp += part2[z * zs + op];
        }
        v = fma(T(beta * ihx), sp - sm, v);
      }
    }
    if (rk.y) rk_apply(rk, o, v);
    else out[o] = v;
  }
}

// v[j, c] = nu_j lin[j, c] + sum_z part[z][j, c] (L substep: F(U L^T)^T U =
// diag(nu) L (U^T Dxx U) + KR(L, L) T'_L) on the active columns, zero
// elsewhere, fused with the RK stage update.
template <typename T>
__global__ void flow_combine_rows(int M, int R, const int32_t* __restrict__ rank, const T* __restrict__ nu,
                                  const T* __restrict__ lin, const T* __restrict__ part, int nz, RkStage<T> rk) {
  const int r = min(R, (int)*rank);
  const int64_t len = (int64_t)M * R, zs = (int64_t)M * 2 * R;
  for (int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; o < len; o += (int64_t)gridDim.x * blockDim.x) {
    const int j = (int)(o % M), col = (int)(o / M);
    T v = T(0);
    if (col < r) {
      v = nu[j] * lin[o];
      if (part)
        for (int z = 0; z < nz; ++z) v += part[z * zs + o];
    }
    rk_apply(rk, o, v);
  }
}

// Y (N x cols) = diag(w) X
template <typename T>
__global__ void scale_rows(int N, int cols, const T* __restrict__ X, const T* __restrict__ w, T* __restrict__ Y) {
  const int64_t len = (int64_t)N * cols;
  for (int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; o < len; o += (int64_t)gridDim.x * blockDim.x)
    Y[o] = w[o % N] * X[o];
}

// C = A B on the active block of w x w FP64 matrices (ld w = 2R; active
// indices: the first r of each half), products summed in T (the S flow's
// A_xx S N_nu, a stage derivative: FP32 sums for FP32 panels); one CTA per
// 32 x 32 tile of the active block.  The other entries of C are left alone.
template <typename T>
__global__ void __launch_bounds__(256) small_gemm_act(int R, const int32_t* __restrict__ rank,
                                                      const double* __restrict__ A, const double* __restrict__ B,
                                                      double* __restrict__ C) {
  const int r = min(R, (int)*rank), ka = 2 * r, w = 2 * R;
  const int i0 = blockIdx.x * 32, j0 = blockIdx.y * 32;
  if (i0 >= ka || j0 >= ka) return;
  __shared__ T as[32][33];
  __shared__ T bs[32][33];
  const int tid = threadIdx.x, ti = tid & 31, tj = tid >> 5;
  T acc[4] = {T(0), T(0), T(0), T(0)};
  for (int k0 = 0; k0 < ka; k0 += 32) {
    for (int e = tid; e < 32 * 32; e += 256) {
      const int x = e & 31, y = e >> 5;
      as[x][y] = (i0 + x < ka && k0 + y < ka)
                     ? T(A[act_col(i0 + x, r, R) + (int64_t)act_col(k0 + y, r, R) * w]) : T(0);
      bs[x][y] = (k0 + x < ka && j0 + y < ka)
                     ? T(B[act_col(k0 + x, r, R) + (int64_t)act_col(j0 + y, r, R) * w]) : T(0);
    }
    __syncthreads();
#pragma unroll 8
    for (int k = 0; k < 32; ++k) {
      const T a = as[ti][k];
#pragma unroll
      for (int q = 0; q < 4; ++q) acc[q] = fma(a, bs[k][tj + 8 * q], acc[q]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int i = i0 + ti, j = j0 + tj + 8 * q;
    if (i < ka && j < ka) C[act_col(i, r, R) + (int64_t)act_col(j, r, R) * w] = (double)acc[q];
  }
}

// out[:, c] = sum_{k active} X[:, k] B[k, c] for the active columns c of an N
// x R (aug = 0) or N x 2R (aug = 1) panel; B FP64 with ld ldb.  Grid (row
// blocks of 32, column tiles of 64); tiles beyond the active columns exit,
// inactive output columns are left alone.
template <typename T>
__global__ void __launch_bounds__(256) panel_mul_act(int N, int R, int aug, const int32_t* __restrict__ rank,
                                                     const T* __restrict__ X, const double* __restrict__ B,
                                                     int ldb, T* __restrict__ out) {
  const int ka = active_cols(rank, R, aug), r = min(R, (int)*rank);
  const int i0 = blockIdx.x * 32, c0 = blockIdx.y * 64;
  if (c0 >= ka) return;
  __shared__ T xs[32][33];
  __shared__ T bs[32][65];
  const int tid = threadIdx.x;
  const int ri = tid & 15, cj = tid >> 4;
  T acc[2][4];
#pragma unroll
  for (int p = 0; p < 2; ++p)
#pragma unroll
    for (int q = 0; q < 4; ++q) acc[p][q] = T(0);
  for (int k0 = 0; k0 < ka; k0 += 32) {
    const int kc = min(32, ka - k0);
    for (int e = tid; e < 32 * 32; e += 256) {
      const int ii = e % 32, k = e / 32;
      const int i = i0 + ii;
      xs[ii][k] = (i < N && k < kc) ? X[i + (int64_t)act_col(k0 + k, r, R) * N] : T(0);
    }
    for (int e = tid; e < 32 * 64; e += 256) {
      const int k = e % 32, cc = e / 32;
      bs[k][cc] = (k < kc && c0 + cc < ka)
                      ? T(B[act_col(k0 + k, r, R) + (int64_t)act_col(c0 + cc, r, R) * ldb])
                      : T(0);
    }
    __syncthreads();
#pragma unroll 8
    for (int k = 0; k < 32; ++k) {
      const T x0 = xs[ri][k], x1 = xs[ri + 16][k];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const T wv = bs[k][cj + 16 * q];
        acc[0][q] = fma(x0, wv, acc[0][q]);
        acc[1][q] = fma(x1, wv, acc[1][q]);
      }
    }
    __syncthreads();
  }
#pragma unroll
  for (int p = 0; p < 2; ++p) {
    const int i = i0 + ri + 16 * p;
    if (i >= N) continue;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int c = c0 + cj + 16 * q;
      if (c < ka) out[i + (int64_t)act_col(c, r, R) * N] = acc[p][q];
    }
  }
}

// part[z][a, c] = X[:, a]^T Y[:, c] over the rows of split z, on the active
// w x w block (aug panels N x 2R; part ld 2R), one CTA per 32 x 32 tile of
// active entries and split of GA_ROWS rows: sums of 32-row chunks in T,
// added up in FP64 (an RK stage derivative: FP32 chunk sums are well inside
// the FP32 step's accuracy).  s_stage_finish adds the splits in a fixed order.
constexpr int GA_ROWS = 128;
template <typename T>
__global__ void __launch_bounds__(256) gram_act(int N, int R, const int32_t* __restrict__ rank,
                                                const T* __restrict__ X, const T* __restrict__ Y,
                                                double* __restrict__ part) {
  const int r = min(R, (int)*rank), ka = 2 * r, w = 2 * R;
  const int a0 = blockIdx.x * 32, c0 = blockIdx.y * 32;
  if (a0 >= ka || c0 >= ka) return;
  __shared__ T xs[32][33];
  __shared__ T ys[32][33];
  const int tid = threadIdx.x;
  const int ta = tid & 31, tcb = tid >> 5;  // entry (ta, tcb + 8 q)
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  const int i_lo = blockIdx.z * GA_ROWS, i_hi = min(N, i_lo + GA_ROWS);
  for (int i0 = i_lo; i0 < i_hi; i0 += 32) {
    for (int e = tid; e < 32 * 32; e += 256) {
      const int ii = e % 32, k = e / 32;
      const int i = i0 + ii;
      xs[k][ii] = (i < i_hi && a0 + k < ka) ? X[i + (int64_t)act_col(a0 + k, r, R) * N] : T(0);
      ys[k][ii] = (i < i_hi && c0 + k < ka) ? Y[i + (int64_t)act_col(c0 + k, r, R) * N] : T(0);
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      T sacc = T(0);
#pragma unroll 8
      for (int ii = 0; ii < 32; ++ii) sacc = fma(xs[ta][ii], ys[tcb + 8 * q][ii], sacc);
      acc[q] += (double)sacc;
    }
    __syncthreads();
  }
  double* dst = part + (int64_t)blockIdx.z * w * w;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int a = a0 + ta, c = c0 + tcb + 8 * q;
    if (a < ka && c < ka) dst[act_col(a, r, R) + (int64_t)act_col(c, r, R) * w] = acc[q];
  }
}

// S-flow stage: v[a, c] = C[a, c] + sum_z part[z][a, c] (fixed order; C holds
// A_xx S N_nu) on the active block, then the RK stage update of the FP64
// w x w stage arrays.
__global__ void s_stage_finish(int R, const int32_t* __restrict__ rank, int nz, const double* __restrict__ part,
                               const double* __restrict__ C, RkStage<double> rk) {
  const int r = min(R, (int)*rank), ka = 2 * r, w = 2 * R;
  const int64_t len = (int64_t)ka * ka;
  for (int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; o < len; o += (int64_t)gridDim.x * blockDim.x) {
    const int64_t idx = act_col((int)(o % ka), r, R) + (int64_t)act_col((int)(o / ka), r, R) * w;
    double v = C[idx];
    for (int z = 0; z < nz; ++z) v += part[z * (int64_t)w * w + idx];
    rk_apply(rk, idx, v);
  }
}

// ---------------------------------------------------------------------------
// Fused RK stages of the Burgers flows for small active widths (ka <= 32).
// At low rank each stage of the K, L and S substep flows is row-local work
// on an n x ka panel plus small matrices (N_nu, A_xx, Z) and the packed flow
// tensor T' (np x ka, np = ka (ka + 1) / 2 pairs), all of which fit in shared
// memory; one kernel per stage replaces the stencil, panel product,
// Khatri-Rao and combine launches above (same arithmetic per entry, sums in
// a different order).  One CTA per FUSED_BMH rows (K and S flows, with one
// periodic halo row on each side for the stencils and the Dx of the
// quadratic term: 32 rows of Khatri-Rao work, one per thread and column
// group) or FUSED_BML rows (L flow).  The tensor sits pair-major in shared
// memory, tpt[p kpp + c] with kpp = ka rounded up to 4, plus 4: one 16-byte
// load (a broadcast across the warp) serves four columns.
// ---------------------------------------------------------------------------
constexpr int FUSED_BMH = 30;
constexpr int FUSED_BML = 64;
constexpr int FUSED_KMAX = 32;

// Four consecutive columns c0 .. c0 + 3 of one row of
//   sum_{a <= b} KR(P, Q)_ab T'[p(a,b), c],  KR(P, Q)_ab = (P_a Q_b + P_b Q_a) / 2
// (SAME: P == Q, KR = P_a P_b); P, Q: the row's ka <= 32 values; T'
// pair-major in shared memory, tpt[p kpp + c], zero beyond the active
// columns.  Each 16-byte tensor load serves 4 (8) multiply-adds and is the
// loop's only shared-memory read; a warp's threads share c0, so the tensor
// reads are broadcasts.
template <typename T, int KMAX, bool SAME>
__device__ __forceinline__ void kr_row4_k(int ka, int kpp, const T* P, const T* Q, const T* tpt, int c0,
                                          T (&acc)[4]) {
  // the row's values in registers (zero beyond ka); loops unrolled over the
  // KMAX x KMAX triangle, pairs beyond ka skipped (ka is uniform)
  T qv[KMAX], pv[SAME ? 1 : KMAX];
#pragma unroll
  for (int k = 0; k < KMAX; ++k) {
    qv[k] = (k < ka) ? Q[k] : T(0);
    if (!SAME) pv[SAME ? 0 : k] = (k < ka) ? P[k] : T(0);
  }
  const T* tp = tpt + c0;
#pragma unroll
  for (int a = 0; a < KMAX; ++a) {
    if (a < ka) {
      T g1[4] = {T(0), T(0), T(0), T(0)}, g2[4] = {T(0), T(0), T(0), T(0)};
#pragma unroll
      for (int b = a; b < KMAX; ++b) {
        if (b < ka) {
          T t[4];
          ld_vec<4>(tp, t);
          tp += kpp;
#pragma unroll
          for (int v = 0; v < 4; ++v) {
            g1[v] = fma(qv[b], t[v], g1[v]);
            if (!SAME) g2[v] = fma(pv[SAME ? 0 : b], t[v], g2[v]);
          }
        }
      }
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        if (SAME) acc[v] = fma(qv[a], g1[v], acc[v]);
        else acc[v] = fma(T(0.5), fma(pv[SAME ? 0 : a], g1[v], qv[a] * g2[v]), acc[v]);
      }
    }
  }
}
template <typename T, bool SAME>
__device__ __forceinline__ void kr_row4(int ka, int kpp, const T* P, const T* Q, const T* tpt, int c0, T (&acc)[4]) {
  if (ka <= 16) kr_row4_k<T, 16, SAME>(ka, kpp, P, Q, tpt, c0, acc);
  else kr_row4_k<T, 32, SAME>(ka, kpp, P, Q, tpt, c0, acc);
}

// row stride of the pair-major tensor in shared memory
__host__ __device__ constexpr int tensor_kpp(int kap) { return kap + 4; }

// the packed tensor's active block, pair-major: tpt[p kpp + c] = Tp[p + c PP]
// for c < ka, zero for ka <= c < kpp (kap = ka rounded up to 4); global
// reads run along the pairs (coalesced)
template <typename T>
__device__ __forceinline__ void load_tensor(int ka, int kap, const T* __restrict__ Tp, int PP, T* tpt) {
  const int np = ka * (ka + 1) / 2, kpp = tensor_kpp(kap), total = np * kpp;
  constexpr int U = 8;  // loads in flight per thread
  for (int e0 = threadIdx.x; e0 < total; e0 += U * blockDim.x) {
    T v[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int e = e0 + u * blockDim.x;
      const int pp = e % np, c = e / np;
      v[u] = (e < total && c < ka) ? Tp[pp + (int64_t)c * PP] : T(0);
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int e = e0 + u * blockDim.x;
      if (e < total) tpt[(e % np) * kpp + e / np] = v[u];
    }
  }
}

// Per-row arrays in shared memory have an odd row stride (ka | 1), and
// threads run along the rows, so a warp touches 32 distinct banks and its
// global accesses to a column are coalesced.

// K substep stage: v = (ih2 Dxx Z) N_nu + alpha KR(Dx Z, Z) T'_V + beta Dx(KR(Z, Z) T'_V),
// Dx = ihx (shift - shift) on the active columns (zero elsewhere), then the RK update.
template <typename T>
__global__ void __launch_bounds__(256) burgers_k_stage(int N, int R, const int32_t* __restrict__ rank,
                                                       const T* __restrict__ Z, const double* __restrict__ Nnu,
                                                       const T* __restrict__ Tp, int PP, double ih2, double ihx,
                                                       double alpha, double beta, uint32_t* status, RkStage<T> rk) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int ka = min(R, (int)*rank);
  if (ka > FUSED_KMAX) {
    if (threadIdx.x == 0 && blockIdx.x == 0) atomicOr(status, ST_BAD_SHAPE);
    return;
  }
  const int np = ka * (ka + 1) / 2, ld = ka | 1, kap = (ka + 3) & ~3, ncg = kap / 4;
  const bool nonlin = (alpha != 0.0 || beta != 0.0);
  T* tpt = reinterpret_cast<T*>(smraw);            // np x kpp
  T* zs = tpt + (nonlin ? np * tensor_kpp(kap) : 0);  // (BM + 2) x ld: rows i0 - 1 .. i0 + BM
  T* ks = zs + (FUSED_BMH + 2) * ld;                 // (BM + 2) x ld: KR(Z, Z) T' (kap columns used)
  T* ns = ks + (FUSED_BMH + 2) * (kap | 1);          // ka x ka: N_nu
  T* d1 = ns + ka * ka;                             // BM x ld: Dx Z
  const int ldk = kap | 1;
  const int i0 = blockIdx.x * FUSED_BMH;
  if (nonlin) load_tensor(ka, kap, Tp, PP, tpt);
  for (int e = threadIdx.x; e < (FUSED_BMH + 2) * ka; e += blockDim.x) {
    const int ii = e % (FUSED_BMH + 2), a = e / (FUSED_BMH + 2);
    int g = i0 - 1 + ii;
    g = (g < 0) ? g + N : ((g >= N) ? g - N : g);
    zs[ii * ld + a] = Z[g + (int64_t)a * N];
  }
  for (int e = threadIdx.x; e < ka * ka; e += blockDim.x) ns[e] = T(Nnu[(e % ka) + (int64_t)(e / ka) * R]);
  __syncthreads();
  if (beta != 0.0)
    for (int e = threadIdx.x; e < (FUSED_BMH + 2) * ncg; e += blockDim.x) {
      const int ii = e % (FUSED_BMH + 2), c0 = 4 * (e / (FUSED_BMH + 2));
      T acc[4] = {T(0), T(0), T(0), T(0)};
      kr_row4<T, true>(ka, tensor_kpp(kap), zs + ii * ld, zs + ii * ld, tpt, c0, acc);
#pragma unroll
      for (int v = 0; v < 4; ++v) ks[ii * ldk + c0 + v] = acc[v];
    }
  for (int e = threadIdx.x; e < FUSED_BMH * ka; e += blockDim.x) {
    const int ii = e % FUSED_BMH, a = e / FUSED_BMH;
    d1[ii * ld + a] = T(ihx) * (zs[(ii + 2) * ld + a] - zs[ii * ld + a]);
  }
  __syncthreads();
  const int rows = min(FUSED_BMH, N - i0);
  for (int e = threadIdx.x; e < FUSED_BMH * ncg; e += blockDim.x) {  // active column groups
    const int ii = e % FUSED_BMH, c0 = 4 * (e / FUSED_BMH);
    if (ii >= rows) continue;
    T v[4] = {T(0), T(0), T(0), T(0)};
    const T* zm = zs + ii * ld;
    const T* z0 = zm + ld;
    const T* zp = z0 + ld;
    for (int a = 0; a < ka; ++a) {
      const T d2 = T(ih2) * ((zm[a] + zp[a]) - T(2) * z0[a]);
#pragma unroll
      for (int q = 0; q < 4; ++q)
        if (c0 + q < ka) v[q] = fma(d2, ns[a + (c0 + q) * ka], v[q]);
    }
    if (alpha != 0.0) {
      T k1[4] = {T(0), T(0), T(0), T(0)};
      kr_row4<T, false>(ka, tensor_kpp(kap), d1 + ii * ld, z0, tpt, c0, k1);
#pragma unroll
      for (int q = 0; q < 4; ++q) v[q] = fma(T(alpha), k1[q], v[q]);
    }
    if (beta != 0.0)
#pragma unroll
      for (int q = 0; q < 4; ++q) v[q] = fma(T(beta * ihx), ks[(ii + 2) * ldk + c0 + q] - ks[ii * ldk + c0 + q], v[q]);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int c = c0 + q;
      if (c < R) rk_apply(rk, (int64_t)(i0 + ii) + (int64_t)c * N, (c < ka) ? v[q] : T(0));
    }
  }
  for (int e = threadIdx.x; e < FUSED_BMH * (R - kap); e += blockDim.x) {  // inactive columns: zero rate
    const int ii = e % FUSED_BMH, c = kap + e / FUSED_BMH;
    if (ii < rows) rk_apply(rk, (int64_t)(i0 + ii) + (int64_t)c * N, T(0));
  }
}

// L substep stage: v[j, c] = nu_j (Z A_xx)[j, c] + KR(Z, Z)_j T'_L[:, c], then the RK update.
template <typename T>
__global__ void __launch_bounds__(256) burgers_l_stage(int M, int R, const int32_t* __restrict__ rank,
                                                       const T* __restrict__ Z, const T* __restrict__ nu,
                                                       const double* __restrict__ Axx, const T* __restrict__ Tp,
                                                       int PP, int nonlin, uint32_t* status, RkStage<T> rk) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int ka = min(R, (int)*rank);
  if (ka > FUSED_KMAX) {
    if (threadIdx.x == 0 && blockIdx.x == 0) atomicOr(status, ST_BAD_SHAPE);
    return;
  }
  const int np = ka * (ka + 1) / 2, ld = ka | 1, kap = (ka + 3) & ~3;
  T* tpt = reinterpret_cast<T*>(smraw);
  T* zs = tpt + (nonlin ? np * tensor_kpp(kap) : 0);  // BM x ld
  T* as = zs + FUSED_BML * ld;              // ka x ka: A_xx
  const int j0 = blockIdx.x * FUSED_BML;
  const int rows = min(FUSED_BML, M - j0);
  if (nonlin) load_tensor(ka, kap, Tp, PP, tpt);
  for (int e = threadIdx.x; e < FUSED_BML * ka; e += blockDim.x) {
    const int jj = e % FUSED_BML, a = e / FUSED_BML;
    zs[jj * ld + a] = (jj < rows) ? Z[(j0 + jj) + (int64_t)a * M] : T(0);
  }
  for (int e = threadIdx.x; e < ka * ka; e += blockDim.x) as[e] = T(Axx[(e % ka) + (int64_t)(e / ka) * R]);
  __syncthreads();
  const int ncg = kap / 4;
  for (int e = threadIdx.x; e < FUSED_BML * ncg; e += blockDim.x) {  // active column groups
    const int jj = e % FUSED_BML, c0 = 4 * (e / FUSED_BML);
    if (jj >= rows) continue;
    T v[4] = {T(0), T(0), T(0), T(0)};
    const T* z = zs + jj * ld;
    T lin[4] = {T(0), T(0), T(0), T(0)};
    for (int a = 0; a < ka; ++a)
#pragma unroll
      for (int q = 0; q < 4; ++q)
        if (c0 + q < ka) lin[q] = fma(z[a], as[a + (c0 + q) * ka], lin[q]);
    const T nj = nu[j0 + jj];
#pragma unroll
    for (int q = 0; q < 4; ++q) v[q] = nj * lin[q];
    if (nonlin) {
      T k[4] = {T(0), T(0), T(0), T(0)};
      kr_row4<T, true>(ka, tensor_kpp(kap), z, z, tpt, c0, k);
#pragma unroll
      for (int q = 0; q < 4; ++q) v[q] += k[q];
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int c = c0 + q;
      if (c < R) rk_apply(rk, (int64_t)(j0 + jj) + (int64_t)c * M, (c < ka) ? v[q] : T(0));
    }
  }
  for (int e = threadIdx.x; e < FUSED_BML * (R - kap); e += blockDim.x) {  // inactive columns: zero rate
    const int jj = e % FUSED_BML, c = kap + e / FUSED_BML;
    if (jj < rows) rk_apply(rk, (int64_t)(j0 + jj) + (int64_t)c * M, T(0));
  }
}

// S substep stage, row part: with A = Uhat Z (N x ka on the active columns
// of the augmented panel), P2 = alpha KR(Dx A, A) T'_h + beta Dx(KR(A, A) T'_h)
// and this CTA's partial of Uhat^T P2 (ka x ka, FP64 at the active indices
// of part[blockIdx.x], ld 2R).  s_stage_finish_warp adds the partials.
template <typename T>
__global__ void __launch_bounds__(256) burgers_s_rows(int N, int R, const int32_t* __restrict__ rank,
                                                      const T* __restrict__ Uh, const double* __restrict__ Zs,
                                                      const T* __restrict__ Tp, int PP, double ihx, double alpha,
                                                      double beta, uint32_t* status, double* __restrict__ part,
                                                      const double* __restrict__ Nnu, const double* __restrict__ Axx,
                                                      double* __restrict__ C) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int r = min(R, (int)*rank), ka = 2 * r, w = 2 * R;
  if (ka > FUSED_KMAX) {
    if (threadIdx.x == 0 && blockIdx.x == 0) atomicOr(status, ST_BAD_SHAPE);
    return;
  }
  const int np = ka * (ka + 1) / 2, ld = ka | 1, kap = (ka + 3) & ~3, ncg = kap / 4, ldk = kap | 1;
  T* tpt = reinterpret_cast<T*>(smraw);        // np x kpp
  T* us = tpt + np * tensor_kpp(kap);          // (BM + 2) x ld: Uhat rows i0 - 1 .. i0 + BM
  T* zm = us + (FUSED_BMH + 2) * ld;            // ka x ka: Z, row-major (zm[k ka + c] = Z[k, c])
  T* as = zm + ka * ka;                        // (BM + 2) x ld: A rows
  T* ks = as + (FUSED_BMH + 2) * ld;            // (BM + 2) x ldk: KR(A, A) T'
  T* d1 = ks + (FUSED_BMH + 2) * ldk;           // BM x ld: Dx A
  T* p2 = d1 + FUSED_BMH * ld;                  // BM x ldk: P2
  const int i0 = blockIdx.x * FUSED_BMH;
  const int rows = min(FUSED_BMH, N - i0);
  load_tensor(ka, kap, Tp, PP, tpt);
  for (int e = threadIdx.x; e < (FUSED_BMH + 2) * ka; e += blockDim.x) {
    const int ii = e % (FUSED_BMH + 2), a = e / (FUSED_BMH + 2);
    int g = i0 - 1 + ii;
    g = (g < 0) ? g + N : ((g >= N) ? g - N : g);
    us[ii * ld + a] = Uh[g + (int64_t)act_col(a, r, R) * N];
  }
  for (int e = threadIdx.x; e < ka * ka; e += blockDim.x) {
    const int k = e % ka, c = e / ka;
    zm[k * ka + c] = T(Zs[act_col(k, r, R) + (int64_t)act_col(c, r, R) * w]);
  }
  __syncthreads();
  for (int e = threadIdx.x; e < (FUSED_BMH + 2) * ka; e += blockDim.x) {  // A = Uhat Z
    const int ii = e % (FUSED_BMH + 2), c = e / (FUSED_BMH + 2);
    T acc = T(0);
    for (int k = 0; k < ka; ++k) acc = fma(us[ii * ld + k], zm[k * ka + c], acc);
    as[ii * ld + c] = acc;
  }
  __syncthreads();
  if (beta != 0.0)
    for (int e = threadIdx.x; e < (FUSED_BMH + 2) * ncg; e += blockDim.x) {
      const int ii = e % (FUSED_BMH + 2), c0 = 4 * (e / (FUSED_BMH + 2));
      T acc[4] = {T(0), T(0), T(0), T(0)};
      kr_row4<T, true>(ka, tensor_kpp(kap), as + ii * ld, as + ii * ld, tpt, c0, acc);
#pragma unroll
      for (int v = 0; v < 4; ++v) ks[ii * ldk + c0 + v] = acc[v];
    }
  for (int e = threadIdx.x; e < FUSED_BMH * ka; e += blockDim.x) {
    const int ii = e % FUSED_BMH, c = e / FUSED_BMH;
    d1[ii * ld + c] = T(ihx) * (as[(ii + 2) * ld + c] - as[ii * ld + c]);
  }
  __syncthreads();
  for (int e = threadIdx.x; e < FUSED_BMH * ncg; e += blockDim.x) {
    const int ii = e % FUSED_BMH, c0 = 4 * (e / FUSED_BMH);
    T v[4] = {T(0), T(0), T(0), T(0)};
    if (ii < rows) {
      if (alpha != 0.0) {
        T k1[4] = {T(0), T(0), T(0), T(0)};
        kr_row4<T, false>(ka, tensor_kpp(kap), d1 + ii * ld, as + (ii + 1) * ld, tpt, c0, k1);
#pragma unroll
        for (int q = 0; q < 4; ++q) v[q] = fma(T(alpha), k1[q], v[q]);
      }
      if (beta != 0.0)
#pragma unroll
        for (int q = 0; q < 4; ++q) v[q] = fma(T(beta * ihx), ks[(ii + 2) * ldk + c0 + q] - ks[ii * ldk + c0 + q], v[q]);
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) p2[ii * ldk + c0 + q] = v[q];
  }
  __syncthreads();
  double* dst = part + (int64_t)blockIdx.x * w * w;
  for (int e = threadIdx.x; e < ka * ka; e += blockDim.x) {  // Uhat^T P2 over the tile's rows
    const int a = e % ka, c = e / ka;
    T acc = T(0);
    for (int ii = 0; ii < rows; ++ii) acc = fma(us[(ii + 1) * ld + a], p2[ii * ldk + c], acc);
    dst[act_col(a, r, R) + (int64_t)act_col(c, r, R) * w] = (double)acc;
  }
  if (blockIdx.x == 0) {
    // the linear part of the stage, C = A_xx Z N_nu on the active block
    // (T1 = Z N_nu first), in the tensor's area once every thread is past it
    __syncthreads();
    T* nn = tpt;           // N_nu, row-major
    T* ax = nn + ka * ka;  // A_xx, row-major
    T* t1 = ax + ka * ka;  // Z N_nu, row-major
    for (int e = threadIdx.x; e < ka * ka; e += blockDim.x) {
      const int k = e / ka, c = e % ka;
      const int64_t g = act_col(k, r, R) + (int64_t)act_col(c, r, R) * w;
      nn[e] = T(Nnu[g]);
      ax[e] = T(Axx[g]);
    }
    __syncthreads();
    for (int e = threadIdx.x; e < ka * ka; e += blockDim.x) {
      const int i = e / ka, c = e % ka;
      T acc = T(0);
      for (int k = 0; k < ka; ++k) acc = fma(zm[i * ka + k], nn[k * ka + c], acc);
      t1[e] = acc;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < ka * ka; e += blockDim.x) {
      const int i = e % ka, c = e / ka;
      T acc = T(0);
      for (int k = 0; k < ka; ++k) acc = fma(ax[i * ka + k], t1[k * ka + c], acc);
      C[act_col(i, r, R) + (int64_t)act_col(c, r, R) * w] = (double)acc;
    }
  }
}

// S-flow stage of the fused path: v[a, c] = C[a, c] + sum_z part[z][a, c] on
// the active block, one warp per entry (lane-strided partials, a fixed
// shuffle tree: deterministic), then the RK update of the FP64 stage arrays.
__global__ void __launch_bounds__(256) s_stage_finish_warp(int R, const int32_t* __restrict__ rank, int nz,
                                                           const double* __restrict__ part,
                                                           const double* __restrict__ C, RkStage<double> rk) {
  const int r = min(R, (int)*rank), ka = 2 * r, w = 2 * R;
  const int lane = threadIdx.x & 31;
  const int64_t len = (int64_t)ka * ka;
  for (int64_t o = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; o < len;
       o += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    const int64_t idx = act_col((int)(o % ka), r, R) + (int64_t)act_col((int)(o / ka), r, R) * w;
    double v = 0.0;
    for (int z = lane; z < nz; z += 32) v += part[z * (int64_t)w * w + idx];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    if (lane == 0) rk_apply(rk, idx, C[idx] + v);
  }
}

// dynamic shared memory of the fused stages at the largest width (FUSED_KMAX)
template <typename T>
size_t fused_smem(int which) {
  const size_t K = FUSED_KMAX, np = K * (K + 1) / 2, KP = tensor_kpp(FUSED_KMAX);
  const size_t L = K | 1;  // padded row stride
  if (which == 0) return sizeof(T) * (np * KP + 2 * (FUSED_BMH + 2) * L + K * K + FUSED_BMH * L);
  if (which == 1) return sizeof(T) * (np * KP + FUSED_BML * L + K * K);
  return sizeof(T) * (np * KP + 3 * (FUSED_BMH + 2) * L + K * K + 2 * FUSED_BMH * L);
}

// small FP64 helpers of the S step: X (R x R, T, ld R) -> Y (FP64, ld R), optionally transposed
template <typename T>
__global__ void small_to_f64(int R, const T* __restrict__ X, int trans, double* __restrict__ Y) {
  for (int o = blockIdx.x * blockDim.x + threadIdx.x; o < R * R; o += gridDim.x * blockDim.x) {
    const int i = o % R, j = o / R;
    Y[o] = (double)(trans ? X[j + (int64_t)i * R] : X[o]);
  }
}

// S (R x R, T) = the active r x r block of B (FP64, ld R), zeros elsewhere
template <typename T>
__global__ void store_core(int R, const int32_t* __restrict__ rank, const double* __restrict__ B, T* __restrict__ S) {
  const int r = min(R, (int)*rank);
  for (int o = blockIdx.x * blockDim.x + threadIdx.x; o < R * R; o += gridDim.x * blockDim.x) {
    const int i = o % R, j = o / R;
    S[o] = (i < r && j < r) ? T(B[o]) : T(0);
  }
}

// S~0 (w x w) = Mh S0 Nh^T with Mh, Nh (w x R), S0 (R x R, FP64)
__global__ void small_msn(int w, int R, const double* __restrict__ Mh, const double* __restrict__ S0,
                          const double* __restrict__ Nh, double* __restrict__ tmp, double* __restrict__ out) {
  for (int o = threadIdx.x; o < R * w; o += blockDim.x) {
    const int i = o % R, j = o / R;
    double s = 0.0;
    for (int kk = 0; kk < R; ++kk) s = fma(S0[i + (int64_t)kk * R], Nh[j + (int64_t)kk * w], s);
    tmp[i + (int64_t)j * R] = s;
  }
  __syncthreads();
  for (int o = threadIdx.x; o < w * w; o += blockDim.x) {
    const int i = o % w, j = o / w;
    double s = 0.0;
    for (int kk = 0; kk < R; ++kk) s = fma(Mh[i + (int64_t)kk * w], tmp[kk + (int64_t)j * R], s);
    out[o] = s;
  }
}

// One Newton-Schulz step towards orthonormal factors without changing
// Y = U S V^T: with Gu = U^T U = I + Eu (and Gv likewise) on the active
// r x r block, Xu = (3I - Gu) / 2 (U <- U Xu has U^T U = I + O(Eu^2)) and
// S <- (I + Eu/2) S (I + Ev/2)^T, the inverse of Xu to first order.
// Identity outside the active block.  Eu and Ev are at the rounding level
// of FP32 panels, so the corrections Eu S and S Ev^T are accumulated in
// FP32 (relative error u32 of a u32-sized term) from shared-memory copies;
// S is updated in FP64 before its final rounding.  One CTA; dynamic shared
// memory 3 r^2 floats.
__global__ void ns_refresh(int R, const int32_t* __restrict__ rank, const double* __restrict__ Gu,
                           const double* __restrict__ Gv, double* __restrict__ Xu, double* __restrict__ Xv,
                           float* __restrict__ S, double* __restrict__ tmp) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int r = min(R, (int)*rank);
  float* E = reinterpret_cast<float*>(smraw);  // r x r: Eu / 2, then Ev / 2
  float* Sf = E + r * r;                        // r x r: S, then tmp
  for (int o = threadIdx.x; o < R * R; o += blockDim.x) {
    const int i = o % R, j = o / R;
    const bool act = i < r && j < r;
    const double id = (i == j) ? 1.0 : 0.0;
    Xu[o] = act ? 0.5 * (3.0 * id - Gu[o]) : id;
    Xv[o] = act ? 0.5 * (3.0 * id - Gv[o]) : id;
  }
  for (int o = threadIdx.x; o < r * r; o += blockDim.x) {
    const int i = o % r, j = o / r;
    E[o] = (float)(0.5 * (Gu[i + (int64_t)j * R] - ((i == j) ? 1.0 : 0.0)));
    Sf[o] = S[i + (int64_t)j * R];
  }
  __syncthreads();
  // tmp = S + (Eu/2) S
  for (int o = threadIdx.x; o < r * r; o += blockDim.x) {
    const int i = o % r, j = o / r;
    float c = 0.0f;
    for (int k = 0; k < r; ++k) c = fmaf(E[i + k * r], Sf[k + j * r], c);
    tmp[i + (int64_t)j * R] = (double)Sf[o] + (double)c;
  }
  __syncthreads();
  for (int o = threadIdx.x; o < r * r; o += blockDim.x) {
    const int i = o % r, j = o / r;
    E[o] = (float)(0.5 * (Gv[i + (int64_t)j * R] - ((i == j) ? 1.0 : 0.0)));
    Sf[o] = (float)tmp[i + (int64_t)j * R];
  }
  __syncthreads();
  // S = tmp + tmp (Ev/2)^T
  for (int o = threadIdx.x; o < r * r; o += blockDim.x) {
    const int i = o % r, j = o / r;
    float c = 0.0f;
    for (int k = 0; k < r; ++k) c = fmaf(Sf[i + k * r], E[j + k * r], c);
    S[i + (int64_t)j * R] = (float)(tmp[i + (int64_t)j * R] + (double)c);
  }
}

}  // namespace
}  // namespace lri

using namespace lri;

struct lri_stream {
  int32_t dtype;
  int64_t n, m, R;
  int sms = 0;  // streaming multiprocessors of the device (Gram launches: two CTAs per SM)
  double tol;
  int32_t rmin;
  size_t es;
  void* U = nullptr;
  void* S = nullptr;
  void* V = nullptr;
  bool bound = false;
  // device workspace
  int32_t* d_rank = nullptr;
  uint32_t* d_status = nullptr;
  void* Uh = nullptr;   // n x 2R: [U0 | Q]
  void* Vh = nullptr;   // m x 2R
  void* Xk = nullptr;   // n x R (dY V0, then its orthonormalised part)
  void* Xl = nullptr;   // m x R
  void* Zp = nullptr;   // max(n, m) x 2R (dY Vhat; scratch of the orthonormalisation)
  double* part = nullptr;
  double* small = nullptr;
  // FP32 data streams: snapshot passes on the tensor cores (tc_pass.cu)
  bool tc_ok = false;   // shapes and device allow them
  bool use_tc = false;  // selected (lri_stream_set_tensor_cores)
  lri::TcPass tc;
  void* Kd = nullptr;   // n x R: dY V0 of the step, reused as the first half of dY Vhat
  int32_t* d_ncols = nullptr;  // column count of lri_stream_data_product on the CUDA-core passes
  // Burgers flow (lri_burgers_create): parameters and RK work panels
  bool burgers = false;
  double bh = 0.0, balpha = 0.0, bbeta = 0.0, bh_dt = 0.0;
  lri::Scheme sc{};
  const void* nu = nullptr;
  void* Kp = nullptr;   // n x R x 4: y, stage input, stage derivative, accumulator
  void* Lp = nullptr;   // m x R x 4
  void* tv = nullptr;   // flow tensors T'_V, T'_L, T'_Vhat: PP x 2R each (PP = 2R (2R + 1) / 2 pairs)
  void* tl = nullptr;
  void* th = nullptr;
  void* kgp = nullptr;  // split partials of the tensor sums (ceil(max(n, m) / KR_ROWS) x PP x 2R) and of gram_act
  void* kap = nullptr;  // pair-split partials of the Khatri-Rao products: 2 x kZmax x max(n, m) x 2R
  void* pw = nullptr;   // 3 work panels of max(n, m) x 2R
  void* pw2 = nullptr;     // the side stream's L-flow product panel, max(n, m) x 2R
  void* kap2nd = nullptr;  // the side stream's L-flow Khatri-Rao partials, kZmax x max(n, m) x 2R
  // one captured Burgers step (launch shapes depend on r_max only; the rank
  // is read on the device), replayed while dt and the bound factors stay
  cudaStream_t cap = nullptr;
  // independent halves of a step run on a second stream, forked from and
  // joined to the step's stream by these events: the V-side
  // orthonormalisation (with the second scratch set below) and the fused
  // L substep flow
  cudaStream_t side = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  double* part2 = nullptr;   // Gram partials of the side stream
  double* small2 = nullptr;  // three (2R)^2 FP64 scratch blocks of the side stream
  void* zp2 = nullptr;       // max(n, m) x R panel product of the side stream
  cudaGraphExec_t step_exec[3] = {nullptr, nullptr, nullptr};  // one per fused class
  double graph_dt[3] = {0.0, 0.0, 0.0};
  bool class_seen[3] = {false, false, false};
  double last_dt[3] = {0.0, 0.0, 0.0};  // dt of the class's previous step (a repeat of it is captured)
  // fused RK-stage kernels for the current rank: 0 none (rank > 32), 1 the K
  // and L stages (rank <= 32), 2 also the S stage (rank <= 16)
  int fused = 0;
  // FP32 Burgers engines: the Khatri-Rao products of the unfused flows
  // (active width above 32) on the tensor cores (tc_kr.cu)
  bool kr_ok = false, use_kr = false;
  lri::TcKr kr;
  double* fgp = nullptr;  // the fused S stage's per-tile partials: ceil(n / FUSED_BMH) x (2R)^2 FP64
};


namespace lri {
namespace {

constexpr int kBlocksSmall = 24;  // FP64 scratch of (2R)^2 each (14, 15, 23: refresh; 13..23: the Burgers step)
constexpr int kZmax = 8;          // pair splits of the Khatri-Rao products (fill the GPU for short panels)

int gram_ctas(const lri_stream* s) { return 2 * std::max(1, s->sms); }

template <typename T>
struct StreamOps {
  lri_stream* s;
  cudaStream_t st;
  int sid = 0;  // scratch set: 0 the step's stream, 1 the side stream
  double* blk(int i) const { return s->small + (int64_t)i * 4 * s->R * s->R; }
  T* tp(void* p) const { return static_cast<T*>(p); }
  // the scratch of the Grams and of the orthonormalisation (per scratch set)
  double* gpart() const { return sid ? s->part2 : s->part; }
  double* sblk(int i) const { return sid ? s->small2 + (int64_t)i * 4 * s->R * s->R : blk(i); }
  T* zpan() const { return tp(sid ? s->zp2 : s->Zp); }

  cudaError_t gram(int N, int a, int c, const T* X, int ldx, const T* Y, int ldy, double alpha, double beta,
                   double* out, int ldo) const {
    const int ctas = gram_ctas(s);
    gram_part<T><<<ctas, 256, 0, st>>>(N, a, c, (int)s->R, s->d_rank, X, ldx, Y, ldy, gpart());
    gram_reduce<<<(a * c + 7) / 8, 256, 0, st>>>(N, a, c, (int)s->R, s->d_rank, ctas, gpart(), alpha, beta, out,
                                                 ldo);
    return cudaGetLastError();
  }
  cudaError_t mul(int N, int a, int c, const T* X, int ldx, const double* B, int ldb, T beta, T* out,
                  int ldo) const {
    dim3 grid((N + 31) / 32, (c + 63) / 64);
    panel_mul<T><<<grid, 256, 0, st>>>(N, a, c, X, ldx, B, ldb, beta, out, ldo);
    return cudaGetLastError();
  }
  // X B for factors with large entries: double-float sums for FP32 panels
  cudaError_t mul_precise(int N, int a, int c, const T* X, int ldx, const double* B, int ldb, T* out,
                          int ldo) const {
    if constexpr (std::is_same<T, float>::value) {
      dim3 grid((N + 31) / 32, (c + 63) / 64);
      panel_mul_df<<<grid, 256, 0, st>>>(N, a, c, X, ldx, B, ldb, out, ldo);
      return cudaGetLastError();
    } else {
      return mul(N, a, c, X, ldx, B, ldb, T(0), out, ldo);
    }
  }
  // the tensor-core passes: FP32 streams whose shapes they take, when selected
  bool tc_selected() const { return std::is_same<T, float>::value && s->use_tc; }
  cudaError_t tc_run(int trans, const T* A1, const T* A0, const T* X, int64_t ldx, T* out, int64_t ldo, T* kd,
                     int ncols = -1) const {
    if constexpr (std::is_same<T, float>::value)
      return tc_pass_run(&s->tc, trans, A1, A0, X, ldx, s->d_rank, ncols, out, ldo, kd, s->d_status, ST_TIMEOUT, st);
    return cudaErrorNotSupported;
  }
  using ST = typename SmallT<T>::type;
  cudaError_t pchol(int a, const double* G, double* B) const {
    static std::atomic<uint64_t> attr_done{0};
    cudaError_t e = set_smem_limit(pchol_factor<ST>, (int)(2 * SMAX * (SMAX + 1) * sizeof(ST)), attr_done);
    if (e != cudaSuccess) return e;
    // directions whose squared distance from the span of the others (unit
    // columns) is below tol_rel are treated as dependent.  The columns of
    // X B are orthonormal up to about (error of G) / tol_rel: about 1e-3 for
    // FP32 panels (Gram and factor in double-float, ~1e-14; X B with
    // double-float sums) and for FP64 panels (~1e-16), so that one
    // CholeskyQR pass afterwards is well conditioned.
    const double tol_rel = sizeof(T) == 4 ? 1e-11 : 1e-13;
    pchol_factor<ST><<<1, NTP, 2 * (size_t)a * (a + 1) * sizeof(ST), st>>>(a, G, s->d_rank, tol_rel, B);
    return cudaGetLastError();
  }
  cudaError_t cholinv(int a, const double* G, double* B, double shift_rel) const {
    static std::atomic<uint64_t> attr_done{0};
    const size_t smem = 2 * (size_t)a * a * sizeof(ST);
    cudaError_t e = set_smem_limit(chol_inv_factor<ST>, (int)(2 * SMAX * SMAX * sizeof(ST)), attr_done);
    if (e != cudaSuccess) return e;
    chol_inv_factor<ST><<<1, NTS, smem, st>>>(a, G, 1e-20, shift_rel, B);
    return cudaGetLastError();
  }
  // X <- X - Y0 (Y0^T X) for the orthonormal columns of Y0 (N x R)
  cudaError_t project_out(int N, T* X, const T* Y0) const {
    const int R = (int)s->R;
    cudaError_t e = gram(N, R, R, Y0, N, X, N, 1.0, 0.0, sblk(0), R);  // C = Y0^T X
    if (e != cudaSuccess) return e;
    // panel_mul computes Y0 (-C) + X
    negate<<<(R * R + 255) / 256, 256, 0, st>>>(R * R, sblk(0));
    return mul(N, R, R, Y0, N, sblk(0), R, T(1), X, N);
  }
  // X (N x R) <- orthonormal basis of the part of X orthogonal to the
  // orthonormal columns of Y0 (N x R); blocks 0..2 are scratch.  Block
  // Gram-Schmidt with re-orthogonalisation: two projections, a
  // rank-revealing pivoted Cholesky pass (dependent directions become zero
  // columns), one more projection (the pivoted pass combines nearly
  // dependent columns with large coefficients, which magnifies what is left
  // of their Y0 components), then X^T X = I + E with |E| ~ 1e-3: for FP32
  // panels two Newton-Schulz steps X <- X (3I - X^T X) / 2 (E -> ~E^2, below
  // FP32 rounding after two; whole-GPU Grams and products only), for FP64
  // panels one CholeskyQR pass.  Zero columns stay zero either way.
  // (Y0 null: a plain orthonormal basis of X, no projections)
  cudaError_t orth_against(int N, T* X, const T* Y0) const {
    const int R = (int)s->R;
    cudaError_t e = Y0 ? project_out(N, X, Y0) : cudaSuccess;
    if (e == cudaSuccess && Y0) e = project_out(N, X, Y0);
    const int npass = std::is_same<T, float>::value ? 3 : 2;
    for (int pass = 0; pass < npass && e == cudaSuccess; ++pass) {
      if (pass == 1 && Y0) e = project_out(N, X, Y0);
      if (e == cudaSuccess) e = gram(N, R, R, X, N, X, N, 1.0, 0.0, sblk(1), R);        // G = X^T X
      if (e == cudaSuccess) {
        if (pass == 0) e = pchol(R, sblk(1), sblk(2));
        else if (std::is_same<T, float>::value) {
          ns_factor<<<(R * R + 255) / 256, 256, 0, st>>>(R, sblk(1), sblk(2));
          e = cudaGetLastError();
        } else e = cholinv(R, sblk(1), sblk(2), 0.0);
      }
      if (e == cudaSuccess)
        e = (pass == 0) ? mul_precise(N, R, R, X, N, sblk(2), R, zpan(), N)              // Z = X B
                        : mul(N, R, R, X, N, sblk(2), R, T(0), zpan(), N);
      if (e == cudaSuccess) {
        copy_cols<T><<<304, 256, 0, st>>>(N, R, zpan(), N, X, N);
        e = cudaGetLastError();
      }
    }
    return e;
  }

  // Burgers flow helpers (see the kernels' notes)
  int64_t pairs_max() const { return (2 * s->R) * (2 * s->R + 1) / 2; }
  // Tout (+)= coef * (packed tensor of KR(P,Q)^T Y over N rows)
  cudaError_t tensor(int N, int aug, const T* P, const T* Q, const T* Y, double coef, int acc, T* Tout) const {
    const int R = (int)s->R, ka = aug ? 2 * R : R;
    const int np = ka * (ka + 1) / 2;
    dim3 grid((np + 63) / 64, (ka + 63) / 64, (N + KR_ROWS - 1) / KR_ROWS);
    kr_gram_part<T><<<grid, 256, 0, st>>>(N, R, aug, s->d_rank, P, Q, Y, (int)pairs_max(), tp(s->kgp));
    kr_reduce<T><<<304, 256, 0, st>>>(R, aug, s->d_rank, (int)grid.z, (int)pairs_max(), tp(s->kgp), coef, acc,
                                       Tout);
    return cudaGetLastError();
  }
  // the tensor-core Khatri-Rao products (FP32 Burgers engines, X == Y)
  bool kr_tc() const { return std::is_same<T, float>::value && s->use_kr; }
  int kz(int N, int aug) const {
    const int R = (int)s->R, ka = aug ? 2 * R : R;
    if (kr_tc()) return tc_kr_splits(N, R, aug, std::max(1, s->sms), kZmax);
    const int tiles = ((N + KrTile<T>::BM - 1) / KrTile<T>::BM) * ((ka + 63) / 64);
    return std::max(1, std::min(kZmax, (2 * 152 + tiles - 1) / tiles));
  }
  // part[z] (=, or += with accum) scale * sum_{a in split z} diag(X[:, a]) Y[:, a:] T'_a
  // (z < kz(N, aug)): KR(X, X) T' for Y = X
  cudaError_t apply(int N, int aug, const T* X, const T* Y, const T* Tp, T* part, double scale = 1.0,
                    int accum = 0) const {
    const int R = (int)s->R, ka = aug ? 2 * R : R;
    if constexpr (std::is_same<T, float>::value) {
      const int k = (Tp == tp(s->tv)) ? 0 : (Tp == tp(s->tl)) ? 1 : (Tp == tp(s->th)) ? 2 : -1;
      if (kr_tc() && X == Y && k >= 0)
        return tc_kr_apply(&s->kr, k, N, aug, s->d_rank, X, part, kz(N, aug), scale, accum, s->d_status, ST_TIMEOUT,
                           st);
    }
    constexpr int BM = KrTile<T>::BM;
    static std::atomic<uint64_t> attr_same{0}, attr_diff{0};
    const int mx = (int)(2 * (2 * 64) * BM * sizeof(T));
    cudaError_t ea = set_smem_limit(kr_apply_part<T, true>, mx, attr_same);
    if (ea == cudaSuccess) ea = set_smem_limit(kr_apply_part<T, false>, mx, attr_diff);
    if (ea != cudaSuccess) return ea;
    dim3 grid((N + BM - 1) / BM, (ka + 63) / 64, kz(N, aug));
    const size_t smem = (size_t)ka * BM * sizeof(T) * (X == Y ? 1 : 2);
    if (X == Y)
      kr_apply_part<T, true><<<grid, 256, smem, st>>>(N, R, aug, s->d_rank, X, Y, Tp, (int)pairs_max(), scale,
                                                      accum, part);
    else
      kr_apply_part<T, false><<<grid, 256, smem, st>>>(N, R, aug, s->d_rank, X, Y, Tp, (int)pairs_max(), scale,
                                                       accum, part);
    return cudaGetLastError();
  }
  // one RK substep sequence of a panel flow y' = f(y) (N x R): y in P[0],
  // stage input P[1], accumulator P[3]; f(stage input, RkStage) launches
  // the kernels of one stage, the last of which applies the stage update.
  template <class F>
  cudaError_t rk_panel(int64_t len, T* P, const F& f) const {
    const Scheme& sc = s->sc;
    const T h = T(s->bh_dt / sc.nsub);
    T* y = P;
    T* z = P + len;
    T* acc = P + 3 * len;
    cudaError_t e = cudaSuccess;
    for (int sub = 0; sub < sc.nsub && e == cudaSuccess; ++sub)
      for (int st_ = 0; st_ < sc.nstages && e == cudaSuccess; ++st_) {
        const bool last = (st_ + 1 == sc.nstages);
        const RkStage<T> c{T(sc.b[st_]), last ? T(0) : T(h * T(sc.a[st_ + 1])), h, st_ == 0, last, y, z, acc};
        e = f(st_ == 0 ? y : z, c);
      }
    return e;
  }

  // FP32 panels: U and V are reused from step to step as the first half of
  // the augmented bases, so their rounding-level loss of orthogonality
  // (~u32 per step) would accumulate; one Newton-Schulz step per step keeps
  // it at u32.  (FP64 panels: u64 per step, left alone.)
  cudaError_t refresh() const {
    if constexpr (!std::is_same<T, float>::value) return cudaSuccess;
    const int n = (int)s->n, m = (int)s->m, R = (int)s->R;
    T* U = tp(s->U);
    T* V = tp(s->V);
    double* Gu = blk(14);
    double* Gv = blk(15);
    double* Xu = Gu + (int64_t)R * R;
    double* Xv = Gv + (int64_t)R * R;
    cudaError_t e = fork_join([&](const StreamOps<T>& o) { return o.gram(n, R, R, U, n, U, n, 1.0, 0.0, Gu, R); },
                              [&](const StreamOps<T>& o) { return o.gram(m, R, R, V, m, V, m, 1.0, 0.0, Gv, R); });
    if (e != cudaSuccess) return e;
    static std::atomic<uint64_t> attr_done{0};
    e = set_smem_limit(ns_refresh, (int)(2 * SMAX * SMAX * sizeof(float)), attr_done);
    if (e != cudaSuccess) return e;
    ns_refresh<<<1, 1024, 2 * (size_t)R * R * sizeof(float), st>>>(R, s->d_rank, Gu, Gv, Xu, Xv,
                                                                  reinterpret_cast<float*>(s->S), blk(23));
    auto apply = [&](const StreamOps<T>& o, int N, T* Y, const double* X) -> cudaError_t {
      cudaError_t e2 = o.mul(N, R, R, Y, N, X, R, T(0), o.zpan(), N);
      if (e2 != cudaSuccess) return e2;
      copy_cols<T><<<304, 256, 0, o.st>>>(N, R, o.zpan(), N, Y, N);
      return cudaGetLastError();
    };
    return fork_join([&](const StreamOps<T>& o) { return apply(o, n, U, Xu); },
                     [&](const StreamOps<T>& o) { return apply(o, m, V, Xv); });
  }

  // a(ops on the step's stream) and b(ops on the side stream, second scratch
  // set) run concurrently: b forked after the work queued so far, joined
  // before anything queued later (a capture must end with the side stream
  // joined, so the join happens even when a or b fails)
  template <class FA, class FB>
  cudaError_t fork_join(const FA& a, const FB& b) const {
    if (!s->side) {
      const cudaError_t e = a(*this);
      return e != cudaSuccess ? e : b(*this);
    }
    cudaError_t e = cudaEventRecord(s->ev_fork, st);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s->side, s->ev_fork, 0);
    if (e != cudaSuccess) return e;
    cudaError_t eb = b(StreamOps<T>{s, s->side, 1});
    const cudaError_t ej = cudaEventRecord(s->ev_join, s->side);
    if (eb == cudaSuccess) eb = ej;
    e = a(*this);
    const cudaError_t ew = cudaStreamWaitEvent(st, s->ev_join, 0);
    if (e == cudaSuccess) e = (eb != cudaSuccess) ? eb : ew;
    return e;
  }

  // Uhat = [U0 | orth((I - U0 U0^T) Xk)] (K side: n rows), Vhat likewise
  // from Xl (V side: m rows), Mh = Uhat^T U0 into block 3, Nh = Vhat^T V0
  // into block 4.  The two sides are independent: the V side runs on the
  // side stream with the second scratch set, forked and joined by events.
  cudaError_t bases() const {
    const int n = (int)s->n, m = (int)s->m, R = (int)s->R, w = 2 * R;
    auto side = [&](const StreamOps<T>& o, int N, T* X, const T* Y0, T* H, double* Mout) -> cudaError_t {
      cudaError_t e = o.orth_against(N, X, Y0);
      if (e != cudaSuccess) return e;
      copy_cols<T><<<304, 256, 0, o.st>>>(N, R, Y0, N, H, N);
      copy_cols<T><<<304, 256, 0, o.st>>>(N, R, X, N, H + (int64_t)R * N, N);
      if ((e = cudaGetLastError()) != cudaSuccess) return e;
      return o.gram(N, w, R, H, N, Y0, N, 1.0, 0.0, Mout, w);
    };
    T* U = tp(s->U);
    T* V = tp(s->V);
    return fork_join([&](const StreamOps<T>& o) { return side(o, n, tp(s->Xk), U, tp(s->Uh), blk(3)); },
                     [&](const StreamOps<T>& o) { return side(o, m, tp(s->Xl), V, tp(s->Vh), blk(4)); });
  }

  // TF32 split of flow tensor k for the tensor-core products
  cudaError_t kr_split(int k, const T* Tp, int aug) const {
    if constexpr (std::is_same<T, float>::value) return tc_kr_split(&s->kr, k, Tp, s->d_rank, aug, st);
    return cudaSuccess;
  }

  // one fused L-flow stage on this object's stream
  cudaError_t l_stage_fused(const T* Z, const double* Axx, bool nonlin, const RkStage<T>& rk) const {
    const int m = (int)s->m, R = (int)s->R;
    burgers_l_stage<T><<<(m + FUSED_BML - 1) / FUSED_BML, 256, fused_smem<T>(1), st>>>(
        m, R, s->d_rank, Z, static_cast<const T*>(s->nu), Axx, tp(s->tl), (int)pairs_max(), nonlin ? 1 : 0,
        s->d_status, rk);
    return cudaGetLastError();
  }
  // the whole L substep flow (Lp holds L0 and its RK panels): the fused
  // stages, or the product panel, the Khatri-Rao partials and the combine
  // (with the side stream's own panel and partials for scratch set 1)
  cudaError_t l_flow(T* Lp, const double* Axx, bool nonlin) const {
    if (s->fused >= 1)
      return rk_panel((int64_t)s->m * s->R, Lp,
                      [&](const T* Z, const RkStage<T>& rk) { return l_stage_fused(Z, Axx, nonlin, rk); });
    const int m = (int)s->m, R = (int)s->R, w = 2 * R;
    const int64_t nm = std::max(s->n, s->m);
    T* P2 = sid ? tp(s->pw2) : tp(s->pw) + 2 * nm * w;
    T* kap1 = tp(sid ? s->kap2nd : s->kap);
    const T* nu = static_cast<const T*>(s->nu);
    const int zl = kz(m, 0);
    return rk_panel((int64_t)m * R, Lp, [&](const T* Z, const RkStage<T>& rk) {
      panel_mul_act<T><<<dim3((m + 31) / 32, (R + 63) / 64), 256, 0, st>>>(m, R, 0, s->d_rank, Z, Axx, R, P2);
      cudaError_t e2 = cudaGetLastError();
      if (e2 == cudaSuccess && nonlin) e2 = apply(m, 0, Z, Z, tp(s->tl), kap1);
      if (e2 != cudaSuccess) return e2;
      flow_combine_rows<T><<<304, 256, 0, st>>>(m, R, s->d_rank, nu, P2, nonlin ? kap1 : nullptr, zl, rk);
      return cudaGetLastError();
    });
  }

  cudaError_t burgers_step() const {
    const int n = (int)s->n, m = (int)s->m, R = (int)s->R, w = 2 * R;
    const int64_t nm = std::max(n, m);
    T* U = tp(s->U);
    T* V = tp(s->V);
    T* S = tp(s->S);
    T* Uh = tp(s->Uh);
    T* Vh = tp(s->Vh);
    T* Xk = tp(s->Xk);
    T* Xl = tp(s->Xl);
    const T* nu = static_cast<const T*>(s->nu);
    const double bh = s->bh, ba = s->balpha, bb = s->bbeta;
    const double ih2 = 1.0 / (bh * bh), ihx = 0.5 / bh;
    const bool nonlin = (ba != 0.0 || bb != 0.0);
    T* P0 = tp(s->pw);
    T* P1 = P0 + nm * w;
    T* P2 = P1 + nm * w;
    T* kap1 = tp(s->kap);
    T* kap2 = kap1 + (int64_t)kZmax * nm * w;
    const int g = 304;
    cudaError_t e = refresh();
    if (e != cudaSuccess) return e;
    if (s->fused) {
      static std::atomic<uint64_t> a0{0}, a1{0}, a2{0};
      if ((e = set_smem_limit(burgers_k_stage<T>, (int)fused_smem<T>(0), a0)) != cudaSuccess) return e;
      if ((e = set_smem_limit(burgers_l_stage<T>, (int)fused_smem<T>(1), a1)) != cudaSuccess) return e;
      if ((e = set_smem_limit(burgers_s_rows<T>, (int)fused_smem<T>(2), a2)) != cudaSuccess) return e;
    }
    small_to_f64<T><<<16, 256, 0, st>>>(R, S, 0, blk(16));
    small_to_f64<T><<<16, 256, 0, st>>>(R, S, 1, blk(17));
    // operators of the K substep (V0 fixed): N_nu = V0^T diag(nu) V0, T'_V
    double* Nnu = blk(13);
    scale_rows<T><<<g, 256, 0, st>>>(m, R, V, nu, P0);
    if ((e = gram(m, R, R, V, m, P0, m, 1.0, 0.0, Nnu, R)) != cudaSuccess) return e;
    if (nonlin && (e = tensor(m, 0, V, V, V, 1.0, 0, tp(s->tv))) != cudaSuccess) return e;
    if (nonlin && kr_tc() && (e = kr_split(0, tp(s->tv), 0)) != cudaSuccess) return e;
    // operators of the L substep (U0 fixed): A_xx = U0^T Dxx U0,
    // T_L = alpha sym(KR(Dx U0, U0))^T U0 - beta KR(U0, U0)^T Dx U0
    double* Axx = blk(14);
    stencil_panel<T><<<g, 256, 0, st>>>(n, R, 0, s->d_rank, U, ih2, P0, ihx, P1);
    if ((e = gram(n, R, R, U, n, P0, n, 1.0, 0.0, Axx, R)) != cudaSuccess) return e;
    if (ba != 0.0 && (e = tensor(n, 0, P1, U, U, ba, 0, tp(s->tl))) != cudaSuccess) return e;
    if (bb != 0.0 && (e = tensor(n, 0, U, U, P1, -bb, ba != 0.0, tp(s->tl))) != cudaSuccess) return e;
    if (nonlin && kr_tc() && (e = kr_split(1, tp(s->tl), 0)) != cudaSuccess) return e;
    // K step: K0 = U0 S0, K' = (Dxx K) N_nu + alpha KR(Dx K, K) T'_V + beta Dx(KR(K, K) T'_V);
    // L step: L0 = V0 S0^T, L' = diag(nu) L A_xx + KR(L, L) T'_L.  The two
    // flows are independent (both start from the old factors): with the
    // fused stages the L flow runs on the side stream beside the K flow.
    T* Kp = tp(s->Kp);
    T* Lp = tp(s->Lp);
    if ((e = mul(n, R, R, U, n, blk(16), R, T(0), Kp, n)) != cudaSuccess) return e;
    if ((e = mul(m, R, R, V, m, blk(17), R, T(0), Lp, m)) != cudaSuccess) return e;
    const bool fork = s->side != nullptr && (s->fused >= 1 || s->pw2 != nullptr);
    cudaError_t el = cudaSuccess;
    if (fork) {
      if ((e = cudaEventRecord(s->ev_fork, st)) != cudaSuccess) return e;
      if ((e = cudaStreamWaitEvent(s->side, s->ev_fork, 0)) != cudaSuccess) return e;
      el = StreamOps<T>{s, s->side, 1}.l_flow(Lp, Axx, nonlin);
      const cudaError_t ej = cudaEventRecord(s->ev_join, s->side);
      if (el == cudaSuccess) el = ej;
    }
    const int zk = kz(n, 0);
    e = rk_panel((int64_t)n * R, Kp, [&](const T* Z, const RkStage<T>& rk) {
      if (s->fused >= 1) {
        burgers_k_stage<T><<<(n + FUSED_BMH - 1) / FUSED_BMH, 256, fused_smem<T>(0), st>>>(
            n, R, s->d_rank, Z, Nnu, tp(s->tv), (int)pairs_max(), ih2, ihx, ba, bb, s->d_status, rk);
        return cudaGetLastError();
      }
      stencil_panel<T><<<g, 256, 0, st>>>(n, R, 0, s->d_rank, Z, ih2, P0, ihx, ba != 0.0 ? P1 : nullptr);
      panel_mul_act<T><<<dim3((n + 31) / 32, (R + 63) / 64), 256, 0, st>>>(n, R, 0, s->d_rank, P0, Nnu, R, P2);
      cudaError_t e2 = cudaGetLastError();
      if (e2 == cudaSuccess && ba != 0.0) e2 = apply(n, 0, P1, Z, tp(s->tv), kap1, 0.5, 0);
      if (e2 == cudaSuccess && ba != 0.0) e2 = apply(n, 0, Z, P1, tp(s->tv), kap1, 0.5, 1);
      if (e2 == cudaSuccess && bb != 0.0) e2 = apply(n, 0, Z, Z, tp(s->tv), kap2);
      if (e2 != cudaSuccess) return e2;
      flow_combine<T><<<g, 256, 0, st>>>(n, R, 0, s->d_rank, P2, ba != 0.0 ? kap1 : nullptr,
                                         bb != 0.0 ? kap2 : nullptr, zk, ba, bb, ihx, nullptr, rk);
      return cudaGetLastError();
    });
    if (fork) {  // join before anything can return (a capture must end with the side stream joined)
      const cudaError_t ew = cudaStreamWaitEvent(st, s->ev_join, 0);
      if (e == cudaSuccess) e = (el != cudaSuccess) ? el : ew;
    }
    if (e != cudaSuccess) return e;
    if (!fork && (e = l_flow(Lp, Axx, nonlin)) != cudaSuccess) return e;
    // augmented bases Uhat = [U0 | orth((I - U0 U0^T) K1)], Vhat likewise; Mh, Nh
    copy_cols<T><<<304, 256, 0, st>>>(n, R, Kp, n, Xk, n);
    copy_cols<T><<<304, 256, 0, st>>>(m, R, Lp, m, Xl, m);
    if ((e = bases()) != cudaSuccess) return e;
    // operators of the S substep: A_xx = Uhat^T Dxx Uhat, N_nu = Vhat^T diag(nu) Vhat, T'_Vhat
    double* Axxh = blk(15);
    double* Nnuh = blk(23);
    double* Stmp = blk(22);
    stencil_panel<T><<<g, 256, 0, st>>>(n, R, 1, s->d_rank, Uh, ih2, P0, 0.0, nullptr);
    if ((e = gram(n, w, w, Uh, n, P0, n, 1.0, 0.0, Axxh, w)) != cudaSuccess) return e;
    scale_rows<T><<<g, 256, 0, st>>>(m, w, Vh, nu, P0);
    if ((e = gram(m, w, w, Vh, m, P0, m, 1.0, 0.0, Nnuh, w)) != cudaSuccess) return e;
    if (nonlin && (e = tensor(m, 1, Vh, Vh, Vh, 1.0, 0, tp(s->th))) != cudaSuccess) return e;
    if (nonlin && kr_tc() && (e = kr_split(2, tp(s->th), 1)) != cudaSuccess) return e;
    // S step on the augmented bases from S~0 = Mh S0 Nh^T (FP64 w x w):
    // S' = A_xx S N_nu + Uhat^T [alpha KR(Dx A, A) T'_Vhat + beta Dx(KR(A, A) T'_Vhat)], A = Uhat S
    small_msn<<<1, 1024, 0, st>>>(w, R, blk(3), blk(16), blk(4), Stmp, blk(18));
    {
      const Scheme& sc = s->sc;
      const double h = s->bh_dt / sc.nsub;
      double* Sy = blk(18);
      double* Sz = blk(19);
      double* Sk = blk(20);
      double* Sa = blk(21);
      const int zs = kz(n, 1);
      const int nzg = (n + GA_ROWS - 1) / GA_ROWS;
      double* gpart = reinterpret_cast<double*>(s->kgp);  // free during the S substep
      const dim3 gsm((w + 31) / 32, (w + 31) / 32);
      for (int sub = 0; sub < sc.nsub && e == cudaSuccess; ++sub) {
        for (int st_ = 0; st_ < sc.nstages && e == cudaSuccess; ++st_) {
          const double* Z = (st_ == 0) ? Sy : Sz;
          const bool last = (st_ + 1 == sc.nstages);
          const RkStage<double> rk{sc.b[st_], last ? 0.0 : h * sc.a[st_ + 1], h, st_ == 0, last, Sy, Sz, Sa};
          if (nonlin && s->fused >= 2) {
            // burgers_s_rows also forms C = A_xx Z N_nu (its first CTA)
            const int nzf = (n + FUSED_BMH - 1) / FUSED_BMH;
            burgers_s_rows<T><<<nzf, 256, fused_smem<T>(2), st>>>(n, R, s->d_rank, Uh, Z, tp(s->th),
                                                                   (int)pairs_max(), ihx, ba, bb, s->d_status, s->fgp,
                                                                   Nnuh, Axxh, Sk);
            s_stage_finish_warp<<<128, 256, 0, st>>>(R, s->d_rank, nzf, s->fgp, Sk, rk);
            e = cudaGetLastError();
            continue;
          }
          small_gemm_act<T><<<gsm, 256, 0, st>>>(R, s->d_rank, Z, Nnuh, Stmp);
          small_gemm_act<T><<<gsm, 256, 0, st>>>(R, s->d_rank, Axxh, Stmp, Sk);
          if (nonlin) {
            panel_mul_act<T><<<dim3((n + 31) / 32, (w + 63) / 64), 256, 0, st>>>(n, R, 1, s->d_rank, Uh, Z, w, P0);
            if (ba != 0.0) {
              stencil_panel<T><<<g, 256, 0, st>>>(n, R, 1, s->d_rank, P0, 0.0, nullptr, ihx, P1);
              if ((e = apply(n, 1, P1, P0, tp(s->th), kap1, 0.5, 0)) != cudaSuccess) break;
              if ((e = apply(n, 1, P0, P1, tp(s->th), kap1, 0.5, 1)) != cudaSuccess) break;
            }
            if (bb != 0.0 && (e = apply(n, 1, P0, P0, tp(s->th), kap2)) != cudaSuccess) break;
            flow_combine<T><<<g, 256, 0, st>>>(n, R, 1, s->d_rank, nullptr, ba != 0.0 ? kap1 : nullptr,
                                               bb != 0.0 ? kap2 : nullptr, zs, ba, bb, ihx, P2, RkStage<T>{});
            gram_act<T><<<dim3((w + 31) / 32, (w + 31) / 32, nzg), 256, 0, st>>>(n, R, s->d_rank, Uh, P2, gpart);
          }
          s_stage_finish<<<64, 256, 0, st>>>(R, s->d_rank, nonlin ? nzg : 0, gpart, Sk, rk);
          e = cudaGetLastError();
        }
      }
      if (e != cudaSuccess) return e;
    }
    // SVD and truncation of S~1 (core_step with Mh = Nh = 0 and D = S~1)
    cudaMemsetAsync(blk(3), 0, sizeof(double) * (size_t)w * R, st);
    cudaMemsetAsync(blk(4), 0, sizeof(double) * (size_t)w * R, st);
    cudaMemcpyAsync(blk(5), blk(18), sizeof(double) * (size_t)w * w, cudaMemcpyDeviceToDevice, st);
    if ((e = core(w)) != cudaSuccess) return e;
    return fork_join([&](const StreamOps<T>& o) { return o.mul(n, w, R, Uh, n, blk(8), w, T(0), U, n); },
                     [&](const StreamOps<T>& o) { return o.mul(m, w, R, Vh, m, blk(9), w, T(0), V, m); });
  }

  cudaError_t core(int w) const {
    const int R = (int)s->R;
    T* S = tp(s->S);
    cudaError_t e;
    // S~ = Mh S0 Nh^T + D on the active block, over the whole GPU (T1 in block 14, S~ in block 13)
    form_t1<T><<<64, 256, 0, st>>>(R, s->d_rank, S, blk(4), blk(14));
    form_core<<<128, 256, 0, st>>>(R, s->d_rank, blk(3), blk(14), blk(5), blk(13));
    if constexpr (std::is_same<T, float>::value) {
      // FP32 panels: the SVD on a thread-block cluster (blocks 6, 7, 10..12 as scratch)
      CoreSvdArgs ca{};
      ca.R = R;
      ca.F = blk(13);
      ca.S0 = S;
      ca.rank = s->d_rank;
      ca.tol = s->tol;
      ca.rmin = s->rmin;
      ca.scr[0] = blk(6);
      ca.scr[1] = blk(7);
      ca.scr[2] = blk(10);
      ca.scr[3] = blk(11);
      ca.scr[4] = blk(12);
      ca.P1 = blk(8);
      ca.Q1 = blk(9);
      ca.status = s->d_status;
      ca.st_noconv = ST_SVD_NOCONV;
      ca.st_nonfinite = ST_NONFINITE;
      return core_svd_cluster(ca, st);
    }
    const int abytes = 200 * 1024;  // CORE_MAT + tiles
    static std::atomic<uint64_t> attr_done{0};
    if ((e = set_smem_limit(core_step<T, ST>, abytes, attr_done)) != cudaSuccess) return e;
    ST* scr = reinterpret_cast<ST*>(blk(6));  // blocks 6 and 7: 2 w^2 values
    // blocks 10..12: FP32 copies and double-float products of the mixed-precision SVD
    core_step<T, ST><<<1, NTS, abytes, st>>>(R, blk(13), S, s->d_rank, s->tol, s->rmin, scr, scr + (int64_t)w * w,
                                             blk(8), blk(9), s->d_status, blk(10));
    return cudaGetLastError();
  }

  // GreedyIntegrator on the snapshot A = y(t + dt) (greedy_integrator.jl:
  // 96-104): U = orth(A V), V = orth(A^T U), S = U^T A V with the new bases;
  // three single-snapshot passes, the rank is kept.
  cudaError_t greedy_step(const T* A) const {
    const int n = (int)s->n, m = (int)s->m, R = (int)s->R;
    T* U = tp(s->U);
    T* V = tp(s->V);
    T* Xk = tp(s->Xk);
    T* Xl = tp(s->Xl);
    T* Z = tp(s->Zp);
    const bool tc = tc_selected();
    cudaError_t e = cudaSuccess;
    auto prod = [&](int trans, const T* X, T* out) {
      if (tc) return tc_run(trans, A, nullptr, X, trans ? n : m, out, trans ? m : n, nullptr);
      if (trans)
        pass_cols<T><<<(m + 15) / 16, 256, 0, st>>>(n, m, R, s->d_rank, A, nullptr, X, n, out);
      else
        pass_rows<T><<<(n + 31) / 32, 256, 0, st>>>(n, m, R, 0, s->d_rank, A, nullptr, X, m, out);
      return cudaGetLastError();
    };
    if ((e = prod(0, V, Xk)) != cudaSuccess) return e;   // A V
    if ((e = prod(1, U, Xl)) != cudaSuccess) return e;   // A^T U
    if ((e = orth_against(n, Xk, nullptr)) != cudaSuccess) return e;
    if ((e = orth_against(m, Xl, nullptr)) != cudaSuccess) return e;
    copy_cols<T><<<304, 256, 0, st>>>(n, R, Xk, n, U, n);
    copy_cols<T><<<304, 256, 0, st>>>(m, R, Xl, m, V, m);
    if ((e = prod(0, V, Z)) != cudaSuccess) return e;    // A V with the new V
    if ((e = gram(n, R, R, U, n, Z, n, 1.0, 0.0, blk(0), R)) != cudaSuccess) return e;
    store_core<T><<<16, 256, 0, st>>>(R, s->d_rank, blk(0), tp(s->S));
    return cudaGetLastError();
  }

  cudaError_t step(const T* A0, const T* A1) const {
    const int n = (int)s->n, m = (int)s->m, R = (int)s->R, w = 2 * R;
    T* U = tp(s->U);
    T* V = tp(s->V);
    T* S = tp(s->S);
    T* Uh = tp(s->Uh);
    T* Vh = tp(s->Vh);
    T* Xk = tp(s->Xk);
    T* Xl = tp(s->Xl);
    cudaError_t e = refresh();
    if (e != cudaSuccess) return e;
    // data passes 1 and 2: dY V0, dY^T U0
    const bool tc = tc_selected();
    if (tc) {
      e = tc_run(0, A1, A0, V, m, Xk, n, tp(s->Kd));
      if (e == cudaSuccess) e = tc_run(1, A1, A0, U, n, Xl, m, nullptr);
    } else {
      pass_rows<T><<<(n + 31) / 32, 256, 0, st>>>(n, m, R, 0, s->d_rank, A1, A0, V, m, Xk);
      pass_cols<T><<<(m + 15) / 16, 256, 0, st>>>(n, m, R, s->d_rank, A1, A0, U, n, Xl);
      e = cudaGetLastError();
    }
    if (e != cudaSuccess) return e;
    // Uhat = [U0 | orth((I - U0 U0^T) dY V0)], Vhat likewise; Mh = Uhat^T U0,
    // Nh = Vhat^T V0 (w x R)
    if ((e = bases()) != cudaSuccess) return e;
    // data pass 3: Z = dY Vhat; D = Uhat^T Z.  On the tensor cores only
    // dY Q_V is new (Vhat = [V0 | Q_V]): dY V0 is the copy kept by pass 1.
    if (tc) {
      copy_cols<T><<<304, 256, 0, st>>>(n, R, tp(s->Kd), n, tp(s->Zp), n);
      if ((e = tc_run(0, A1, A0, Vh + (int64_t)R * m, m, tp(s->Zp) + (int64_t)R * n, n, nullptr)) != cudaSuccess)
        return e;
    } else {
      pass_rows<T><<<(n + 31) / 32, 256, 0, st>>>(n, m, R, 1, s->d_rank, A1, A0, Vh, m, tp(s->Zp));
    }
    if ((e = gram(n, w, w, Uh, n, tp(s->Zp), n, 1.0, 0.0, blk(5), w)) != cudaSuccess) return e;
    if ((e = core(w)) != cudaSuccess) return e;
    // U1 = Uhat P1, V1 = Vhat Q1
    return fork_join([&](const StreamOps<T>& o) { return o.mul(n, w, R, Uh, n, blk(8), w, T(0), U, n); },
                     [&](const StreamOps<T>& o) { return o.mul(m, w, R, Vh, m, blk(9), w, T(0), V, m); });
  }
};

}  // namespace
}  // namespace lri

static cudaError_t burgers_step_on(lri_stream* s, cudaStream_t st) {
  return (s->dtype == LRI_F32) ? StreamOps<float>{s, st}.burgers_step() : StreamOps<double>{s, st}.burgers_step();
}

static void drop_graph(lri_stream* s) {
  for (int c = 0; c < 3; ++c) {
    if (s->step_exec[c]) cudaGraphExecDestroy(s->step_exec[c]);
    s->step_exec[c] = nullptr;
  }
}

// Capture one step of the current fused class on the private stream (nothing
// runs); on any failure the steps of that class run eagerly.
static void capture_step(lri_stream* s) {
  const int c = s->fused;
  if (s->step_exec[c]) cudaGraphExecDestroy(s->step_exec[c]);
  s->step_exec[c] = nullptr;
  if (!s->cap && cudaStreamCreateWithFlags(&s->cap, cudaStreamNonBlocking) != cudaSuccess) {
    s->cap = nullptr;
    return;
  }
  cudaGraph_t g = nullptr;
  if (cudaStreamBeginCapture(s->cap, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return;
  const cudaError_t e = burgers_step_on(s, s->cap);
  const cudaError_t ec = cudaStreamEndCapture(s->cap, &g);
  if (e == cudaSuccess && ec == cudaSuccess && g) {
    if (cudaGraphInstantiate(&s->step_exec[c], g, 0) != cudaSuccess) s->step_exec[c] = nullptr;
    else s->graph_dt[c] = s->bh_dt;
  }
  if (g) cudaGraphDestroy(g);
  cudaGetLastError();  // a failed capture leaves no sticky error; clear the last one
}

// The fused class of the next step from the device rank (synchronises st).
static cudaError_t fused_class(lri_stream* s, cudaStream_t st, int* cls) {
  int32_t r = 0;
  cudaError_t e = cudaMemcpyAsync(&r, s->d_rank, sizeof(r), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return e;
  const int ra = std::min<int>((int)s->R, r);
  *cls = (2 * ra <= lri::FUSED_KMAX) ? 2 : (ra <= lri::FUSED_KMAX ? 1 : 0);
  return cudaSuccess;
}

extern "C" {

lri_status lri_stream_create(lri_stream** out, int32_t dtype, int64_t n, int64_t m, int64_t r0, int64_t r_max,
                             double tol, int32_t r_min) {
  if (!out) return LRI_ERR_ARG;
  *out = nullptr;
  if (dtype != LRI_F32 && dtype != LRI_F64) return LRI_ERR_UNSUPPORTED;
  if (r_max < 1 || r_max > SMAX || r0 < 1 || r0 > r_max || r_min < 1 || r_min > r_max) return LRI_ERR_ARG;
  if (n < 2 * r_max || m < 2 * r_max || n >= (1LL << 31) / 4 || m >= (1LL << 31) / 4) return LRI_ERR_ARG;
  if (!(tol >= 0.0)) return LRI_ERR_ARG;
  lri_stream* s = new lri_stream();
  s->dtype = dtype;
  s->n = n;
  s->m = m;
  s->R = r_max;
  s->tol = tol;
  s->rmin = r_min;
  s->es = dtype == LRI_F32 ? 4 : 8;
  const int64_t R = r_max;
  cudaError_t e = cudaSuccess;
  {
    int dev = 0;
    e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&s->sms, cudaDevAttrMultiProcessorCount, dev);
  }
  auto alloc = [&](void** p, size_t bytes) {
    if (e == cudaSuccess) e = cudaMalloc(p, bytes < 16 ? 16 : bytes);
  };
  alloc((void**)&s->d_rank, sizeof(int32_t));
  alloc((void**)&s->d_status, sizeof(uint32_t));
  alloc(&s->Uh, s->es * n * 2 * R);
  alloc(&s->Vh, s->es * m * 2 * R);
  alloc(&s->Xk, s->es * n * R);
  alloc(&s->Xl, s->es * m * R);
  alloc(&s->Zp, s->es * std::max(n, m) * 2 * R);
  // Gram partials: at most max(ctas, tiles) 64 x 64 work items
  alloc((void**)&s->part, sizeof(double) * (size_t)(lri::gram_ctas(s) + lri::GRAM_TILE_MAX) * lri::GRAM_TILE *
                              lri::GRAM_TILE);
  alloc((void**)&s->small, sizeof(double) * kBlocksSmall * 4 * R * R);
  alloc((void**)&s->part2, sizeof(double) * (size_t)(lri::gram_ctas(s) + lri::GRAM_TILE_MAX) * lri::GRAM_TILE *
                               lri::GRAM_TILE);
  alloc((void**)&s->small2, sizeof(double) * 3 * 4 * R * R);
  alloc(&s->zp2, s->es * std::max(n, m) * R);
  alloc((void**)&s->d_ncols, sizeof(int32_t));
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->side, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->ev_fork, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->ev_join, cudaEventDisableTiming);
  if (e == cudaSuccess && dtype == LRI_F32 && lri::tc_pass_supported(n, m, (int)R)) {
    alloc(&s->Kd, s->es * n * R);
    if (e == cudaSuccess) e = lri::tc_pass_init(&s->tc, n, m, (int)R);
    s->tc_ok = s->use_tc = (e == cudaSuccess);
  }
  const int32_t r32 = (int32_t)r0;
  if (e == cudaSuccess) e = cudaMemcpy(s->d_rank, &r32, sizeof(r32), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(s->d_status, 0, sizeof(uint32_t));
  if (e == cudaSuccess) e = cudaMemset(s->small, 0, sizeof(double) * kBlocksSmall * 4 * R * R);
  if (e != cudaSuccess) {
    lri_stream_destroy(s);
    return LRI_ERR_CUDA;
  }
  *out = s;
  return LRI_OK;
}

lri_status lri_burgers_create(lri_stream** out, int32_t dtype, int64_t n, int64_t m, int64_t r0, int64_t r_max,
                              double tol, int32_t r_min, double h, double alpha, double beta,
                              const lri_scheme* scheme) {
  if (!out || !scheme) return LRI_ERR_ARG;
  *out = nullptr;
  if (r_max > 64) return LRI_ERR_ARG;  // the flow tiles take panels of at most 2 r_max = 128 columns
  if (!(h > 0.0) || !std::isfinite(h) || !std::isfinite(alpha) || !std::isfinite(beta)) return LRI_ERR_ARG;
  if (scheme->nstages < 1 || scheme->nstages > 4 || scheme->nsub < 1) return LRI_ERR_ARG;
  lri_status st = lri_stream_create(out, dtype, n, m, r0, r_max, tol, r_min);
  if (st != LRI_OK) return st;
  lri_stream* s = *out;
  s->burgers = true;
  s->bh = h;
  s->balpha = alpha;
  s->bbeta = beta;
  s->sc.nstages = scheme->nstages;
  s->sc.nsub = scheme->nsub;
  for (int i = 0; i < 4; ++i) {
    s->sc.a[i] = scheme->a[i];
    s->sc.b[i] = scheme->b[i];
    s->sc.c[i] = scheme->c[i];
  }
  const int64_t R = r_max, nm = std::max(n, m), PP = (2 * R) * (2 * R + 1) / 2;
  cudaError_t e = cudaSuccess;
  auto alloc = [&](void** p, size_t bytes) {
    if (e == cudaSuccess) e = cudaMalloc(p, bytes < 16 ? 16 : bytes);
  };
  alloc(&s->Kp, s->es * n * R * 4);
  alloc(&s->Lp, s->es * m * R * 4);
  alloc(&s->tv, s->es * PP * 2 * R);
  alloc(&s->tl, s->es * PP * 2 * R);
  alloc(&s->th, s->es * PP * 2 * R);
  // (also the split partials of the S substep's Gram: ceil(n / GA_ROWS) x (2R)^2 FP64)
  alloc(&s->kgp, std::max<int64_t>(s->es * ((nm + KR_ROWS - 1) / KR_ROWS) * PP * 2 * R,
                                   (int64_t)sizeof(double) * ((n + GA_ROWS - 1) / GA_ROWS) * 4 * R * R));
  alloc(&s->kap, s->es * 2 * kZmax * nm * 2 * R);
  alloc(&s->pw, s->es * 3 * nm * 2 * R);
  alloc(&s->pw2, s->es * nm * 2 * R);
  alloc(&s->kap2nd, s->es * kZmax * nm * 2 * R);
  alloc((void**)&s->fgp, sizeof(double) * ((n + lri::FUSED_BMH - 1) / lri::FUSED_BMH) * 4 * R * R);
  if (e == cudaSuccess && dtype == LRI_F32 && lri::tc_kr_supported((int)R)) {
    e = lri::tc_kr_init(&s->kr, (int)R);
    s->kr_ok = s->use_kr = (e == cudaSuccess);
  }
  if (e != cudaSuccess) {
    lri_stream_destroy(s);
    *out = nullptr;
    return LRI_ERR_CUDA;
  }
  return LRI_OK;
}

lri_status lri_burgers_bind(lri_stream* s, void* U, void* S, void* V, const void* nu) {
  if (!s || !s->burgers || !nu) return LRI_ERR_ARG;
  drop_graph(s);
  s->nu = nu;
  return lri_stream_bind(s, U, S, V);
}

lri_status lri_burgers_step(lri_stream* s, double dt, int32_t nsteps, void* stream) {
  if (!s || !s->burgers || nsteps < 0 || !std::isfinite(dt)) return LRI_ERR_ARG;
  if (!s->bound || !s->nu) return LRI_ERR_STATE;
  s->bh_dt = dt;
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e = cudaSuccess;
  // Each step takes the launch sequence of its rank class (fused RK-stage
  // kernels up to rank 32): one captured graph per class, replayed while dt
  // and the binding stay; a class's first step runs eagerly, and the graph
  // is captured at its next step with the same dt (also across calls of one
  // step each, as a solve that reads every step back makes).
  for (int k = 0; k < nsteps && e == cudaSuccess; ++k) {
    int cls = 0;
    if ((e = fused_class(s, st, &cls)) != cudaSuccess) break;
    s->fused = cls;
    if (s->step_exec[cls] && s->graph_dt[cls] != dt) {
      cudaGraphExecDestroy(s->step_exec[cls]);
      s->step_exec[cls] = nullptr;
    }
    if (!s->step_exec[cls] && s->class_seen[cls] && (nsteps > 1 || s->last_dt[cls] == dt)) capture_step(s);
    if (s->step_exec[cls]) {
      e = cudaGraphLaunch(s->step_exec[cls], st);
    } else {
      e = burgers_step_on(s, st);
      s->class_seen[cls] = true;
    }
    s->last_dt[cls] = dt;
  }
  return e == cudaSuccess ? LRI_OK : LRI_ERR_CUDA;
}

lri_status lri_stream_destroy(lri_stream* s) {
  if (!s) return LRI_ERR_ARG;
  drop_graph(s);
  if (s->cap) cudaStreamDestroy(s->cap);
  if (s->side) cudaStreamDestroy(s->side);
  if (s->ev_fork) cudaEventDestroy(s->ev_fork);
  if (s->ev_join) cudaEventDestroy(s->ev_join);
  cudaFree(s->Kp);
  cudaFree(s->Lp);
  cudaFree(s->tv);
  cudaFree(s->tl);
  cudaFree(s->th);
  cudaFree(s->kgp);
  cudaFree(s->kap);
  cudaFree(s->pw);
  cudaFree(s->pw2);
  cudaFree(s->kap2nd);
  cudaFree(s->fgp);
  cudaFree(s->d_rank);
  cudaFree(s->d_status);
  cudaFree(s->Uh);
  cudaFree(s->Vh);
  cudaFree(s->Xk);
  cudaFree(s->Xl);
  cudaFree(s->Zp);
  lri::tc_kr_free(&s->kr);
  cudaFree(s->part);
  cudaFree(s->part2);
  cudaFree(s->small2);
  cudaFree(s->zp2);
  cudaFree(s->small);
  cudaFree(s->Kd);
  cudaFree(s->d_ncols);
  lri::tc_pass_free(&s->tc);
  delete s;
  return LRI_OK;
}

lri_status lri_stream_bind(lri_stream* s, void* U, void* S, void* V) {
  if (!s || !U || !S || !V) return LRI_ERR_ARG;
  drop_graph(s);  // the captured step holds the factor pointers
  s->U = U;
  s->S = S;
  s->V = V;
  s->bound = true;
  return LRI_OK;
}

lri_status lri_stream_step(lri_stream* s, const void* A_prev, const void* A_next, void* stream) {
  if (!s || !A_prev || !A_next) return LRI_ERR_ARG;
  if (!s->bound) return LRI_ERR_STATE;
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e;
  if (s->dtype == LRI_F32)
    e = StreamOps<float>{s, st}.step(static_cast<const float*>(A_prev), static_cast<const float*>(A_next));
  else
    e = StreamOps<double>{s, st}.step(static_cast<const double*>(A_prev), static_cast<const double*>(A_next));
  return e == cudaSuccess ? LRI_OK : LRI_ERR_CUDA;
}

lri_status lri_stream_greedy_step(lri_stream* s, const void* A_next, void* stream) {
  if (!s || s->burgers || !A_next) return LRI_ERR_ARG;
  if (!s->bound) return LRI_ERR_STATE;
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e;
  if (s->dtype == LRI_F32)
    e = StreamOps<float>{s, st}.greedy_step(static_cast<const float*>(A_next));
  else
    e = StreamOps<double>{s, st}.greedy_step(static_cast<const double*>(A_next));
  return e == cudaSuccess ? LRI_OK : LRI_ERR_CUDA;
}

lri_status lri_stream_rank(lri_stream* s, int64_t* r_out, void* stream) {
  if (!s || !r_out) return LRI_ERR_ARG;
  int32_t r = 0;
  if (cudaMemcpyAsync(&r, s->d_rank, sizeof(r), cudaMemcpyDeviceToHost, (cudaStream_t)stream) != cudaSuccess ||
      cudaStreamSynchronize((cudaStream_t)stream) != cudaSuccess)
    return LRI_ERR_CUDA;
  *r_out = r;
  return LRI_OK;
}

lri_status lri_stream_status(lri_stream* s, void* stream) {
  if (!s) return LRI_ERR_ARG;
  uint32_t w = 0;
  if (cudaMemcpyAsync(&w, s->d_status, sizeof(w), cudaMemcpyDeviceToHost, (cudaStream_t)stream) != cudaSuccess ||
      cudaStreamSynchronize((cudaStream_t)stream) != cudaSuccess)
    return LRI_ERR_CUDA;
  if (w) cudaMemsetAsync(s->d_status, 0, sizeof(uint32_t), (cudaStream_t)stream);
  if (w & ST_TIMEOUT) return LRI_ERR_TIMEOUT;
  if (w & ST_NONFINITE) return LRI_ERR_NONFINITE;
  if (w & ST_SVD_NOCONV) return LRI_ERR_BREAKDOWN;
  return w ? LRI_ERR_ARG : LRI_OK;
}

lri_status lri_stream_set_tensor_cores(lri_stream* s, int32_t enable) {
  if (!s || s->burgers) return LRI_ERR_ARG;
  if (enable && !s->tc_ok) return LRI_ERR_UNSUPPORTED;
  s->use_tc = enable != 0;
  return LRI_OK;
}

lri_status lri_stream_set_pass_tiles(lri_stream* s, int32_t splits_rows, int32_t splits_cols, int32_t stages) {
  if (!s || s->burgers) return LRI_ERR_ARG;
  if (!s->tc_ok) return LRI_ERR_UNSUPPORTED;
  const cudaError_t e = lri::tc_pass_set_tiles(&s->tc, splits_rows, splits_cols, stages);
  if (e == cudaErrorInvalidValue) return LRI_ERR_ARG;
  return e == cudaSuccess ? LRI_OK : LRI_ERR_CUDA;
}

lri_status lri_stream_uses_tensor_cores(const lri_stream* s, int32_t* out) {
  if (!s || !out) return LRI_ERR_ARG;
  *out = s->use_tc ? 1 : 0;
  return LRI_OK;
}

lri_status lri_stream_data_product(lri_stream* s, int32_t trans, const void* A_prev, const void* A_next,
                                   const void* X, int64_t ldx, int64_t ncols, void* out, int64_t ldo, void* stream) {
  if (!s || s->burgers || !A_prev || !A_next || !X || !out) return LRI_ERR_ARG;
  if (trans != 0 && trans != 1) return LRI_ERR_ARG;
  const int64_t rows_x = trans ? s->n : s->m, rows_o = trans ? s->m : s->n;
  if (ncols < 1 || ncols > s->R || ldx < rows_x || ldo < rows_o) return LRI_ERR_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  const int R = (int)s->R, n = (int)s->n, m = (int)s->m;
  cudaError_t e;
  if (s->dtype == LRI_F32 && s->use_tc) {
    e = StreamOps<float>{s, st}.tc_run(trans, static_cast<const float*>(A_next), static_cast<const float*>(A_prev),
                                        static_cast<const float*>(X), ldx, static_cast<float*>(out), ldo, nullptr,
                                        (int)ncols);
    return e == cudaSuccess ? LRI_OK : LRI_ERR_CUDA;
  }
  // CUDA-core passes: the column count goes through a device word
  const int32_t c32 = (int32_t)ncols;
  if (cudaMemcpyAsync(s->d_ncols, &c32, sizeof(c32), cudaMemcpyHostToDevice, st) != cudaSuccess) return LRI_ERR_CUDA;
  if (ldo != rows_o) return LRI_ERR_UNSUPPORTED;  // the CUDA-core passes write a packed panel
  if (s->dtype == LRI_F32) {
    auto A1 = static_cast<const float*>(A_next);
    auto A0 = static_cast<const float*>(A_prev);
    if (trans == 0)
      pass_rows<float><<<(n + 31) / 32, 256, 0, st>>>(n, m, R, 0, s->d_ncols, A1, A0, static_cast<const float*>(X),
                                                      (int)ldx, static_cast<float*>(out));
    else
      pass_cols<float><<<(m + 15) / 16, 256, 0, st>>>(n, m, R, s->d_ncols, A1, A0, static_cast<const float*>(X),
                                                      (int)ldx, static_cast<float*>(out));
  } else {
    auto A1 = static_cast<const double*>(A_next);
    auto A0 = static_cast<const double*>(A_prev);
    if (trans == 0)
      pass_rows<double><<<(n + 31) / 32, 256, 0, st>>>(n, m, R, 0, s->d_ncols, A1, A0,
                                                       static_cast<const double*>(X), (int)ldx,
                                                       static_cast<double*>(out));
    else
      pass_cols<double><<<(m + 15) / 16, 256, 0, st>>>(n, m, R, s->d_ncols, A1, A0,
                                                       static_cast<const double*>(X), (int)ldx,
                                                       static_cast<double*>(out));
  }
  e = cudaGetLastError();
  return e == cudaSuccess ? LRI_OK : LRI_ERR_CUDA;
}

}  // extern "C"
