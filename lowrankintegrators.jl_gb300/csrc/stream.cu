// stream.cu - rank-adaptive BUG for one large data stream (MatrixDataProblem
// whose snapshots are too large for the one-CTA instance engine), spread
// over the whole GPU.
//
// One step A(t) -> A(t+1) (src/integrators/rank_adaptive_unconventional.jl:
// 182-233 with the data substeps of data_integrator.jl:13-16):
//   K1 = U0 S0 + dY V0,  L1 = V0 S0^T + dY^T U0          dY = A(t+1) - A(t)
//   Uhat = orth[K1 | U0], Vhat = orth[L1 | V0]
//   S~ = (Uhat^T U0) S0 (Vhat^T V0)^T + Uhat^T dY Vhat
//   S~ = P Sigma Q^T, r1 = truncation, U1 = Uhat P1, V1 = Vhat Q1, S1 = Sigma1.
// span[K1 | U0] = span[U0 | (I - U0 U0^T) dY V0], so Uhat is formed as
// [U0 | Q] with Q an orthonormal basis of the part of dY V0 orthogonal to U0
// (two classical Gram-Schmidt passes, then two eigenvalue-based
// orthonormalisations X <- X D W Lambda^{-1/2}; directions with eigenvalues
// below the rounding level become zero columns).  The step's result depends
// only on span(Uhat), span(Vhat) as long as [K1 | U0] has full column rank.
//
// Kernels: three streaming passes over the snapshot pair (dY V0, dY^T U0,
// dY Vhat; dY is formed in the loader and never stored), tall-skinny Gram
// products X^T Y reduced in FP64 through per-block partials, row-parallel
// panel products X B, and single-CTA FP64 kernels for the r x r / 2r x 2r
// work.  Panel widths are fixed at r_max (Uhat, Vhat: 2 r_max) with zero
// columns beyond the current rank, which stays on the device.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <type_traits>
#include <vector>

#include "../../include/lri.h"
#include "engine.cuh"

namespace lri {
namespace {

constexpr int SMAX = 96;      // largest r_max
constexpr int GROWS = 512;    // rows per Gram partial block

// ---------------------------------------------------------------------------
// Streaming pass A: out (n x c) = dY B,  dY = A1 - A0 (n x m, col-major),
// B (m x c, ld ldb), c <= 2*SMAX.  CTA = 32 rows, loops over all columns.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(256) pass_rows(int n, int m, int c, const T* __restrict__ A1,
                                                 const T* __restrict__ A0, const T* __restrict__ B, int ldb,
                                                 T* __restrict__ out) {
  // 4 rows x CG columns per thread (c <= 192); BJ keeps the static shared
  // memory under 48 KB for both types
  constexpr int BI = 32, BJ = sizeof(T) == 8 ? 16 : 32, CG = 6;
  __shared__ T ds[BJ][BI + 1];             // dY tile, column-major
  __shared__ T bs[BJ][2 * SMAX + 1];       // B rows of the tile
  const int tid = threadIdx.x;
  const int i0 = blockIdx.x * BI;
  const int rg = tid & 7, cg = tid >> 3;   // rows 4rg.., columns cg + 32u
  T acc[4][CG];
#pragma unroll
  for (int p = 0; p < 4; ++p)
#pragma unroll
    for (int u = 0; u < CG; ++u) acc[p][u] = T(0);
  for (int j0 = 0; j0 < m; j0 += BJ) {
    for (int e = tid; e < BI * BJ; e += 256) {
      const int ii = e % BI, jj = e / BI;
      const int i = i0 + ii, j = j0 + jj;
      T v = T(0);
      if (i < n && j < m) {
        const int64_t o = (int64_t)i + (int64_t)j * n;
        v = A1[o] - A0[o];
      }
      ds[jj][ii] = v;
    }
    for (int e = tid; e < BJ * c; e += 256) {
      const int jj = e % BJ, k = e / BJ;
      const int j = j0 + jj;
      bs[jj][k] = (j < m) ? B[j + (int64_t)k * ldb] : T(0);
    }
    __syncthreads();
#pragma unroll 4
    for (int jj = 0; jj < BJ; ++jj) {
      T x[4], w[CG];
#pragma unroll
      for (int p = 0; p < 4; ++p) x[p] = ds[jj][4 * rg + p];
#pragma unroll
      for (int u = 0; u < CG; ++u) w[u] = (cg + 32 * u < c) ? bs[jj][cg + 32 * u] : T(0);
#pragma unroll
      for (int p = 0; p < 4; ++p)
#pragma unroll
        for (int u = 0; u < CG; ++u) acc[p][u] = fma(x[p], w[u], acc[p][u]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int p = 0; p < 4; ++p) {
    const int i = i0 + 4 * rg + p;
    if (i >= n) continue;
#pragma unroll
    for (int u = 0; u < CG; ++u) {
      const int k = cg + 32 * u;
      if (k < c) out[i + (int64_t)k * n] = acc[p][u];
    }
  }
}

// ---------------------------------------------------------------------------
// Streaming pass B: out (m x c) = dY^T X, X (n x c, ld ldx), c <= SMAX.
// CTA = 16 columns of dY, loops over all rows.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(256) pass_cols(int n, int m, int c, const T* __restrict__ A1,
                                                 const T* __restrict__ A0, const T* __restrict__ X, int ldx,
                                                 T* __restrict__ out) {
  constexpr int BJ = 16, BI = sizeof(T) == 8 ? 32 : 64;
  __shared__ T ds[BJ][BI + 1];
  __shared__ T xs[BI][SMAX + 1];
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
        v = A1[o] - A0[o];
      }
      ds[jj][ii] = v;
    }
    for (int e = tid; e < BI * c; e += 256) {
      const int ii = e % BI, k = e / BI;
      const int i = i0 + ii;
      xs[ii][k] = (i < n) ? X[i + (int64_t)k * ldx] : T(0);
    }
    __syncthreads();
#pragma unroll 4
    for (int ii = 0; ii < BI; ++ii) {
      T x[4], w[2];
#pragma unroll
      for (int p = 0; p < 4; ++p) x[p] = ds[4 * jg + p][ii];
      w[0] = (cg < c) ? xs[ii][cg] : T(0);
      w[1] = (cg + 64 < c) ? xs[ii][cg + 64] : T(0);
#pragma unroll
      for (int p = 0; p < 4; ++p) {
        acc[p][0] = fma(x[p], w[0], acc[p][0]);
        acc[p][1] = fma(x[p], w[1], acc[p][1]);
      }
    }
    __syncthreads();
  }
#pragma unroll
  for (int p = 0; p < 4; ++p) {
    const int j = j0 + 4 * jg + p;
    if (j >= m) continue;
    if (cg < c) out[j + (int64_t)cg * m] = acc[p][0];
    if (cg + 64 < c) out[j + (int64_t)(cg + 64) * m] = acc[p][1];
  }
}

// ---------------------------------------------------------------------------
// Gram partials: part[blk] (a x c, FP64, ld a) = X(rows of blk)^T Y(rows),
// X (N x a, ld ldx), Y (N x c, ld ldy); a, c <= 2*SMAX.  Grid
// (row blocks of GROWS) x (64 x 64 output tiles).  Then gram_reduce.
// ---------------------------------------------------------------------------
// FP32 panels: exact products, double-float sums (the FP64 pipe of GB300
// runs at 1/64 of the FP32 rate); FP64 panels: FP64.
template <typename T> struct GramAcc { using type = double; };
template <> struct GramAcc<float> { using type = dfloat; };
__device__ __forceinline__ double gacc_mul(double acc, double x, double y) { return fma(x, y, acc); }
__device__ __forceinline__ dfloat gacc_mul(dfloat acc, float x, float y) { return acc_mul_acc(acc, x, y); }
__device__ __forceinline__ double gacc_val(double a) { return a; }
__device__ __forceinline__ double gacc_val(dfloat a) { return (double)a.hi + (double)a.lo; }

template <typename T>
__global__ void __launch_bounds__(256) gram_part(int N, int a, int c, const T* __restrict__ X, int ldx,
                                                 const T* __restrict__ Y, int ldy, double* __restrict__ part) {
  using A = typename GramAcc<T>::type;
  constexpr int TI = 32;
  __shared__ T xs[TI][65];
  __shared__ T ys[TI][65];
  const int tid = threadIdx.x;
  const int blk = blockIdx.x;
  const int ta = blockIdx.y % ((a + 63) / 64), tc = blockIdx.y / ((a + 63) / 64);
  const int a0 = ta * 64, c0 = tc * 64;
  const int r0 = blk * GROWS, r1 = min(N, r0 + GROWS);
  const int pa = tid & 15, pc = tid >> 4;  // 4 x 4 outputs: a0 + 4pa.., c0 + 4pc..
  A acc[4][4];
#pragma unroll
  for (int p = 0; p < 4; ++p)
#pragma unroll
    for (int q = 0; q < 4; ++q) acc[p][q] = A(0.0);
  for (int i0 = r0; i0 < r1; i0 += TI) {
    for (int e = tid; e < TI * 64; e += 256) {
      const int ii = e % TI, k = e / TI;
      const int i = i0 + ii;
      const bool ok = i < r1;
      xs[ii][k] = (ok && a0 + k < a) ? X[i + (int64_t)(a0 + k) * ldx] : T(0);
      ys[ii][k] = (ok && c0 + k < c) ? Y[i + (int64_t)(c0 + k) * ldy] : T(0);
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
    __syncthreads();
  }
  double* dst = part + (int64_t)blk * a * c;
#pragma unroll
  for (int p = 0; p < 4; ++p)
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int ia = a0 + 4 * pa + p, jc = c0 + 4 * pc + q;
      if (ia < a && jc < c) dst[ia + (int64_t)jc * a] = gacc_val(acc[p][q]);
    }
}

// out (a x c, ld ldo) = alpha * sum_blk part[blk] + beta * out
__global__ void gram_reduce(int nblk, int a, int c, const double* __restrict__ part, double alpha, double beta,
                            double* __restrict__ out, int ldo) {
  const int o = blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= a * c) return;
  double s = 0.0;
  for (int b = 0; b < nblk; ++b) s += part[(int64_t)b * a * c + o];
  const int i = o % a, j = o / a;
  double* d = out + i + (int64_t)j * ldo;
  *d = (beta == 0.0) ? alpha * s : fma(alpha, s, beta * *d);
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

// Eigenvalue-based orthonormalisation factor of a Gram matrix G (a x a, ld a)
// restricted to its leading r x r block (r = *rank: the panel's columns
// beyond the rank are zero): Bout (a x a, ld a, zero outside that block) =
// D W Lambda^{-1/2} with D = diag(G)^{-1/2} and D G D = W Lambda W^T, so
// X Bout has orthonormal columns; eigenvalues below tol_rel * max
// eigenvalue (and zero diagonal entries) give zero columns.
template <typename ST>
__global__ void __launch_bounds__(NTS) svqb_factor(int a, const double* __restrict__ G, const int32_t* rank,
                                                   double tol_rel, double* __restrict__ Bout) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int r = min(a, (int)*rank);
  ST* M = reinterpret_cast<ST*>(smraw);  // r x r
  ST* W = M + r * r;                      // r x r
  ST* lam = W + r * r;                    // r
  double* d = reinterpret_cast<double*>(lam + r);
  int* perm = reinterpret_cast<int*>(d + r);
  int* flag = perm + r + 1;
  const int tid = threadIdx.x;
  for (int j = tid; j < r; j += NTS) {
    const double g = G[j + (int64_t)j * a];
    d[j] = (g > 0.0) ? 1.0 / sqrt(g) : 0.0;
  }
  __syncthreads();
  for (int o = tid; o < r * r; o += NTS) {
    const int i = o % r, j = o / r;
    M[o] = ST(d[i] * G[i + (int64_t)j * a] * d[j]);
  }
  __syncthreads();
  // symmetric PSD: the one-sided Jacobi SVD gives eigenvectors (v) and eigenvalues (sigma)
  jacobi_svd<ST, NTS>(r, M, W, lam, perm, flag);
  double lmax = 0.0;
  for (int j = 0; j < r; ++j) lmax = fmax(lmax, to_d(lam[j]));
  for (int o = tid; o < a * a; o += NTS) {
    const int i = o % a, j = o / a;
    double bv = 0.0;
    if (i < r && j < r) {
      const double l = to_d(lam[j]);
      bv = (l > tol_rel * lmax && l > 0.0) ? d[i] * to_d(W[i + j * r]) / sqrt(l) : 0.0;
    }
    Bout[o] = bv;
  }
}

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

// C (P x P, ld P) = op(A) B with op(A) = A or A^T, all in ST, NTS threads.
template <typename ST>
__device__ void sq_mul(int P, const ST* A, bool ta, const ST* B, ST* C) {
  for (int o = threadIdx.x; o < P * P; o += NTS) {
    const int i = o % P, j = o / P;
    ST acc(0.0);
    for (int k = 0; k < P; ++k) acc = fma_acc(ta ? A[k + i * P] : A[i + k * P], B[k + j * P], acc);
    C[o] = renorm(acc);
  }
  __syncthreads();
}

// SVD of the P x P double-float matrix a (in place; right vectors to v): the
// Jacobi sweeps run in FP32 (a32, v32: P*P floats each), the FP32 right
// vectors are made orthonormal to double-float precision by two Newton-Schulz
// steps X <- X (3I - X^T X) / 2, a <- a X, and one double-float sweep
// polishes the rotated matrix (its columns are then orthogonal to FP32
// precision, so one sweep squares that).  t1, t2: P*P double-float scratch.
__device__ bool jacobi_svd_mixed(int P, dfloat* a, dfloat* v, dfloat* sig, int* perm, int* flag, float* a32,
                                 float* v32, float* sig32, dfloat* t1, dfloat* t2) {
  for (int o = threadIdx.x; o < P * P; o += NTS) a32[o] = a[o].hi + a[o].lo;
  __syncthreads();
  const bool ok = jacobi_svd<float, NTS>(P, a32, v32, sig32, perm, flag);
  for (int o = threadIdx.x; o < P * P; o += NTS) t1[o] = dfloat(v32[o], 0.0f);  // X0 = V32
  __syncthreads();
  for (int it = 0; it < 2; ++it) {
    sq_mul<dfloat>(P, t1, true, t1, t2);                                             // X^T X
    for (int o = threadIdx.x; o < P * P; o += NTS) {
      const int i = o % P, j = o / P;
      t2[o] = ((i == j) ? dfloat(1.5f, 0.0f) : dfloat(0.0f, 0.0f)) - dfloat(0.5f, 0.0f) * t2[o];
    }
    __syncthreads();
    sq_mul<dfloat>(P, t1, false, t2, v);                                             // X (3I - X^T X)/2
    for (int o = threadIdx.x; o < P * P; o += NTS) t1[o] = v[o];
    __syncthreads();
  }
  sq_mul<dfloat>(P, a, false, t1, t2);                                               // a X
  for (int o = threadIdx.x; o < P * P; o += NTS) a[o] = t2[o];
  __syncthreads();
  jacobi_svd<dfloat, NTS>(P, a, v, sig, perm, flag, 1);                              // polish: a = U S, V_p
  sq_mul<dfloat>(P, t1, false, v, t2);                                               // V = X V_p
  for (int o = threadIdx.x; o < P * P; o += NTS) v[o] = t2[o];
  __syncthreads();
  return ok;
}

// S-step core and truncation.  In: Mh = Uhat^T U0 (w x R), Nh = Vhat^T V0
// (w x R), D = Uhat^T dY Vhat (w x w), S0 (R x R, T), rank (device).  Out:
// P1, Q1 (w x R FP64: the kept left / right singular vectors, zero beyond
// the new rank), S (R x R, diag), rank.  The SVD runs in ST (double-float
// for FP32 panels: an FP32 Jacobi SVD of a w x w matrix accumulates
// O(w u) rotation error per sweep) with the w x w matrix in shared memory
// when it fits, else in the global scratch ag; the right vectors in vg.
template <typename T, typename ST>
__global__ void __launch_bounds__(NTS) core_step(int R, const double* __restrict__ Mh, const double* __restrict__ Nh,
                                                 const double* __restrict__ D, T* S0, int32_t* rank, double tol,
                                                 int rmin, ST* __restrict__ ag, ST* __restrict__ vg,
                                                 double* __restrict__ P1, double* __restrict__ Q1, uint32_t* status,
                                                 int smem_bytes, double* __restrict__ mx) {
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
  const bool a_in_smem = (size_t)wa * wa * sizeof(ST) <= (size_t)smem_bytes;
  ST* a = a_in_smem ? reinterpret_cast<ST*>(smraw) : ag;  // wa x wa
  ST* v = vg;                                              // wa x wa
  // T1 = S0 N^T (r x wa) into v; a = M T1 + D on the active block (FP64 products)
  for (int o = tid; o < r * wa; o += NTS) {
    const int i = o % r, j = o / r;
    double sacc = 0.0;
    for (int k = 0; k < r; ++k) sacc = fma((double)S0[i + (int64_t)k * R], Nh[idx(j) + (int64_t)k * w], sacc);
    v[i + (int64_t)j * r] = ST(sacc);
  }
  __syncthreads();
  for (int o = tid; o < wa * wa; o += NTS) {
    const int i = o % wa, j = o / wa;
    double sacc = D[idx(i) + (int64_t)idx(j) * w];
    for (int k = 0; k < r; ++k) sacc = fma(Mh[idx(i) + (int64_t)k * w], to_d(v[k + (int64_t)j * r]), sacc);
    a[o] = ST(sacc);
  }
  __syncthreads();
  bool ok;
  if constexpr (sizeof(ST) == 8 && !std::is_same<ST, double>::value) {
    // double-float: FP32 sweeps, double-float polish (scratch after a in
    // shared memory when it fits, else in the global scratch mx)
    float* a32 = reinterpret_cast<float*>(mx);
    float* v32 = a32 + wa * wa;
    __shared__ float sig32[2 * SMAX];
    ok = jacobi_svd_mixed(wa, a, v, sig, perm, &flag, a32, v32, sig32,
                          reinterpret_cast<ST*>(mx) + wa * wa, reinterpret_cast<ST*>(mx) + 2 * wa * wa);
  } else {
    ok = jacobi_svd<ST, NTS>(wa, a, v, sig, perm, &flag);
  }
  if (tid == 0) {
    if (!ok) atomicOr(status, ST_SVD_NOCONV);
    // smallest r1 with sum_{j > r1} sigma_j^2 < tol^2, then [rmin, R]
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
    r_new = r1;
    *rank = r1;
  }
  __syncthreads();
  const int r1 = r_new;
  for (int o = tid; o < w * R; o += NTS) P1[o] = Q1[o] = 0.0;
  __syncthreads();
  for (int o = tid; o < wa * r1; o += NTS) {
    const int i = o % wa, j = o / wa;
    const int pj = perm[j];
    const double sg = to_d(sig[pj]);
    P1[idx(i) + (int64_t)j * w] = (sg > 0.0) ? to_d(a[i + (int64_t)pj * wa]) / sg : 0.0;
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

}  // namespace
}  // namespace lri

using namespace lri;

struct lri_stream {
  int32_t dtype;
  int64_t n, m, R;
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
};


namespace lri {
namespace {

constexpr int kBlocksSmall = 16;  // FP64 scratch of (2R)^2 each

template <typename T>
struct StreamOps {
  lri_stream* s;
  cudaStream_t st;
  double* blk(int i) const { return s->small + (int64_t)i * 4 * s->R * s->R; }
  T* tp(void* p) const { return static_cast<T*>(p); }

  cudaError_t gram(int N, int a, int c, const T* X, int ldx, const T* Y, int ldy, double alpha, double beta,
                   double* out, int ldo) const {
    const int nblk = (N + GROWS - 1) / GROWS;
    dim3 grid(nblk, ((a + 63) / 64) * ((c + 63) / 64));
    gram_part<T><<<grid, 256, 0, st>>>(N, a, c, X, ldx, Y, ldy, s->part);
    gram_reduce<<<(a * c + 255) / 256, 256, 0, st>>>(nblk, a, c, s->part, alpha, beta, out, ldo);
    return cudaGetLastError();
  }
  cudaError_t mul(int N, int a, int c, const T* X, int ldx, const double* B, int ldb, T beta, T* out,
                  int ldo) const {
    dim3 grid((N + 31) / 32, (c + 63) / 64);
    panel_mul<T><<<grid, 256, 0, st>>>(N, a, c, X, ldx, B, ldb, beta, out, ldo);
    return cudaGetLastError();
  }
  using ST = typename SmallT<T>::type;
  static size_t svqb_smem(int a) {
    return (size_t)(2 * a * a + a) * sizeof(ST) + (size_t)a * sizeof(double) + (size_t)(a + 2) * sizeof(int);
  }
  cudaError_t svqb(int a, const double* G, double* B) const {
    static bool attr_set = false;
    if (!attr_set) {
      cudaError_t e = cudaFuncSetAttribute(svqb_factor<ST>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)svqb_smem(SMAX));
      if (e != cudaSuccess) return e;
      attr_set = true;
    }
    // eigenvalues below 1e-26 of the largest are rounding noise of the Gram
    // (double-float or FP64 sums of exact products)
    svqb_factor<ST><<<1, NTS, svqb_smem(a), st>>>(a, G, s->d_rank, 1e-26, B);
    return cudaGetLastError();
  }
  cudaError_t cholinv(int a, const double* G, double* B, double shift_rel) const {
    static bool attr_set = false;
    const size_t smem = 2 * (size_t)a * a * sizeof(ST);
    if (!attr_set) {
      cudaError_t e = cudaFuncSetAttribute(chol_inv_factor<ST>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)(2 * SMAX * SMAX * sizeof(ST)));
      if (e != cudaSuccess) return e;
      attr_set = true;
    }
    chol_inv_factor<ST><<<1, NTS, smem, st>>>(a, G, 1e-20, shift_rel, B);
    return cudaGetLastError();
  }
  // X (N x R) <- orthonormal basis of the part of X orthogonal to the
  // orthonormal columns of Y0 (N x R); B blocks i0..i0+2 are scratch.
  cudaError_t orth_against(int N, T* X, const T* Y0) const {
    const int R = (int)s->R;
    cudaError_t e = cudaSuccess;
    for (int pass = 0; pass < 2 && e == cudaSuccess; ++pass) {
      e = gram(N, R, R, Y0, N, X, N, 1.0, 0.0, blk(0), R);                                // C = Y0^T X
      if (e == cudaSuccess) {
        // X <- X - Y0 C   (panel_mul computes Y0 (-C) + X)
        negate<<<(R * R + 255) / 256, 256, 0, st>>>(R * R, blk(0));
        e = mul(N, R, R, Y0, N, blk(0), R, T(1), X, N);
      }
    }
    // shifted CholeskyQR3 (Fukaya et al., SIAM J. Sci. Comput. 2020): the
    // first pass shifted by 11 (N a + a (a+1)) u tr(G) with u the Gram's
    // rounding unit (double-float sums of exact FP32 products: 2^-44; FP64:
    // 2^-53), then two plain passes
    const double ug = sizeof(T) == 4 ? 5.7e-14 : 1.1e-16;
    const double shift = 11.0 * ((double)N * R + (double)R * (R + 1)) * ug;
    for (int pass = 0; pass < 3 && e == cudaSuccess; ++pass) {
      e = gram(N, R, R, X, N, X, N, 1.0, 0.0, blk(1), R);                                 // G = X^T X
      if (e == cudaSuccess) e = cholinv(R, blk(1), blk(2), pass == 0 ? shift : 0.0);
      if (e == cudaSuccess) e = mul(N, R, R, X, N, blk(2), R, T(0), tp(s->Zp), N);        // Z = X B
      if (e == cudaSuccess) {
        copy_cols<T><<<304, 256, 0, st>>>(N, R, tp(s->Zp), N, X, N);
        e = cudaGetLastError();
      }
    }
    return e;
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
    cudaError_t e = cudaSuccess;
    // data passes 1 and 2: dY V0, dY^T U0
    pass_rows<T><<<(n + 31) / 32, 256, 0, st>>>(n, m, R, A1, A0, V, m, Xk);
    pass_cols<T><<<(m + 15) / 16, 256, 0, st>>>(n, m, R, A1, A0, U, n, Xl);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    // Uhat = [U0 | orth((I - U0 U0^T) dY V0)], Vhat likewise
    if ((e = orth_against(n, Xk, U)) != cudaSuccess) return e;
    if ((e = orth_against(m, Xl, V)) != cudaSuccess) return e;
    copy_cols<T><<<304, 256, 0, st>>>(n, R, U, n, Uh, n);
    copy_cols<T><<<304, 256, 0, st>>>(n, R, Xk, n, Uh + (int64_t)R * n, n);
    copy_cols<T><<<304, 256, 0, st>>>(m, R, V, m, Vh, m);
    copy_cols<T><<<304, 256, 0, st>>>(m, R, Xl, m, Vh + (int64_t)R * m, m);
    // Mh = Uhat^T U0, Nh = Vhat^T V0 (w x R)
    if ((e = gram(n, w, R, Uh, n, U, n, 1.0, 0.0, blk(3), w)) != cudaSuccess) return e;
    if ((e = gram(m, w, R, Vh, m, V, m, 1.0, 0.0, blk(4), w)) != cudaSuccess) return e;
    // data pass 3: Z = dY Vhat; D = Uhat^T Z
    pass_rows<T><<<(n + 31) / 32, 256, 0, st>>>(n, m, w, A1, A0, Vh, m, tp(s->Zp));
    if ((e = gram(n, w, w, Uh, n, tp(s->Zp), n, 1.0, 0.0, blk(5), w)) != cudaSuccess) return e;
    {
      // the active 2r x 2r matrix in shared memory when it fits (200 KB)
      const int abytes = 200 * 1024;
      static bool attr_set = false;
      if (!attr_set) {
        if ((e = cudaFuncSetAttribute(core_step<T, ST>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024)) !=
            cudaSuccess)
          return e;
        attr_set = true;
      }
      ST* scr = reinterpret_cast<ST*>(blk(6));  // blocks 6 and 7: 2 w^2 values
      // blocks 10..13: FP32 copies and double-float products of the mixed-precision SVD
      core_step<T, ST><<<1, NTS, abytes, st>>>(R, blk(3), blk(4), blk(5), S, s->d_rank, s->tol, s->rmin, scr,
                                               scr + (int64_t)w * w, blk(8), blk(9), s->d_status, abytes, blk(10));
    }
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    // U1 = Uhat P1, V1 = Vhat Q1
    if ((e = mul(n, w, R, Uh, n, blk(8), w, T(0), U, n)) != cudaSuccess) return e;
    return mul(m, w, R, Vh, m, blk(9), w, T(0), V, m);
  }
};

}  // namespace
}  // namespace lri

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
  const int64_t nblk = (std::max(n, m) + GROWS - 1) / GROWS;
  cudaError_t e = cudaSuccess;
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
  alloc((void**)&s->part, sizeof(double) * nblk * 4 * R * R);
  alloc((void**)&s->small, sizeof(double) * kBlocksSmall * 4 * R * R);
  const int32_t r32 = (int32_t)r0;
  if (e == cudaSuccess) e = cudaMemcpy(s->d_rank, &r32, sizeof(r32), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(s->d_status, 0, sizeof(uint32_t));
  if (e != cudaSuccess) {
    lri_stream_destroy(s);
    return LRI_ERR_CUDA;
  }
  *out = s;
  return LRI_OK;
}

lri_status lri_stream_destroy(lri_stream* s) {
  if (!s) return LRI_ERR_ARG;
  cudaFree(s->d_rank);
  cudaFree(s->d_status);
  cudaFree(s->Uh);
  cudaFree(s->Vh);
  cudaFree(s->Xk);
  cudaFree(s->Xl);
  cudaFree(s->Zp);
  cudaFree(s->part);
  cudaFree(s->small);
  delete s;
  return LRI_OK;
}

lri_status lri_stream_bind(lri_stream* s, void* U, void* S, void* V) {
  if (!s || !U || !S || !V) return LRI_ERR_ARG;
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
  if (w & ST_NONFINITE) return LRI_ERR_NONFINITE;
  if (w & ST_SVD_NOCONV) return LRI_ERR_BREAKDOWN;
  return w ? LRI_ERR_ARG : LRI_OK;
}

}  // extern "C"
