// engine.cuh - CTA-level building blocks of the instance engine.
//
// One CTA advances one DLRA instance by one full integrator step: the K-, L-
// and S-substeps, the orthogonalisations and (rank-adaptive) the core SVD
// and truncation.  Everything here is written for a 256-thread CTA; tall
// n x r "panels" live in global scratch (L1/L2 resident while the CTA works
// on them), small r x r matrices in global scratch as well, and every tile
// product is staged through shared memory with 4x4 register micro-tiles.
//
// Matrices are column-major unless stated otherwise.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "dfloat.cuh"
#include "engine_api.h"
#include "flows.cuh"

namespace lri {

constexpr int NT = 256;        // threads per CTA
constexpr int NW = NT / 32;    // warps per CTA
constexpr int KC = 32;         // k-chunk of the tile products
constexpr int WMAX = 64;       // widest panel (columns) handled by the engine

// Shared staging per CTA: 48 KB for 4-byte types, 66 KB for 8-byte types, so
// three CTAs fit on an SM either way.  TRMAX (rows per staged tile) is sized
// so TRMAX*KC + KC*WMAX fits; 8-byte types also hold the 64x64 Jacobi pair.
template <typename T> struct Stage {
  static constexpr int TRMAX = (sizeof(T) == 4) ? 256 : 192;
  static constexpr int ELEMS = (sizeof(T) == 4) ? 12288 : 8448;
};

// ---------------------------------------------------------------------------
// small helpers
// ---------------------------------------------------------------------------

__device__ __forceinline__ float shfl_xor(float v, int o) { return __shfl_xor_sync(0xffffffffu, v, o); }
__device__ __forceinline__ double shfl_xor(double v, int o) { return __shfl_xor_sync(0xffffffffu, v, o); }
__device__ __forceinline__ dfloat shfl_xor(dfloat v, int o) {
  return dfloat(__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o));
}

// The fast forms (FP32 and double-float) take the computed bases as exactly
// orthonormal, so V^T V = I in the substep right-hand sides; the plain FP64
// form keeps the Gram factors, as the reference's algebra does.
template <typename T> struct AssumeOrthonormal { static constexpr bool value = true; };
template <> struct AssumeOrthonormal<double> { static constexpr bool value = false; };

// Relative precision used by convergence tests.
template <typename T> struct Prec;
template <> struct Prec<float> { static constexpr double eps = 1.2e-7; };
template <> struct Prec<double> { static constexpr double eps = 2.3e-16; };
template <> struct Prec<dfloat> { static constexpr double eps = 1.5e-14; };

// Multiply-accumulate of the long inner loops (deferred renormalisation for
// double-float, plain FMA otherwise) and the matching final renormalisation.
__device__ __forceinline__ float fma_acc(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ double fma_acc(double a, double b, double c) { return ::fma(a, b, c); }
__device__ __forceinline__ float renorm(float a) { return a; }
__device__ __forceinline__ double renorm(double a) { return a; }
using lri_df::fma_acc;

// acc + x*y accumulated in double-float: exact FP32 products (TwoProduct)
// for float inputs, double-float FMA for double-float inputs.
__device__ __forceinline__ dfloat acc_mul(dfloat acc, float x, float y) {
  const float p = x * y;
  const float e = fmaf(x, y, -p);
  const dfloat s = lri_df::two_sum(acc.hi, p);
  return lri_df::fast_two_sum(s.hi, s.lo + (acc.lo + e));
}
__device__ __forceinline__ dfloat acc_mul(dfloat acc, dfloat x, dfloat y) { return fma(x, y, acc); }
// the same without the final renormalisation (renorm() before reading)
__device__ __forceinline__ dfloat acc_mul_acc(dfloat acc, float x, float y) {
  const float p = x * y;
  const float e = fmaf(x, y, -p);
  const dfloat s = lri_df::two_sum(acc.hi, p);
  return dfloat(s.hi, acc.lo + (s.lo + e));
}
__device__ __forceinline__ dfloat acc_mul_acc(dfloat acc, dfloat x, dfloat y) { return lri_df::fma_acc(x, y, acc); }
__device__ __forceinline__ dfloat to_df(float x) { return dfloat(x, 0.0f); }
__device__ __forceinline__ dfloat to_df(dfloat x) { return x; }
__device__ __forceinline__ void from_df(dfloat x, float& y) { y = x.hi + x.lo; }
__device__ __forceinline__ void from_df(dfloat x, dfloat& y) { y = x; }
using lri_df::renorm;

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += shfl_xor(v, o);
  return v;
}

// Deterministic block sum: every thread returns the same value.
template <typename T>
__device__ __forceinline__ T block_sum(T v, T* red) {
  v = warp_sum(v);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) red[warp] = v;
  __syncthreads();
  T s = T(0);
#pragma unroll
  for (int w = 0; w < NW; ++w) s += red[w];
  __syncthreads();
  return s;
}

__device__ __forceinline__ void ld4(const float* p, float v[4]) {
  float4 x = *reinterpret_cast<const float4*>(p);
  v[0] = x.x; v[1] = x.y; v[2] = x.z; v[3] = x.w;
}
__device__ __forceinline__ void ld4(const double* p, double v[4]) {
  double2 x = *reinterpret_cast<const double2*>(p);
  double2 y = *reinterpret_cast<const double2*>(p + 2);
  v[0] = x.x; v[1] = x.y; v[2] = y.x; v[3] = y.y;
}

__device__ __forceinline__ void ld4(const dfloat* p, dfloat v[4]) {
  float4 x = *reinterpret_cast<const float4*>(p);
  float4 y = *reinterpret_cast<const float4*>(p + 2);
  v[0] = dfloat(x.x, x.y); v[1] = dfloat(x.z, x.w); v[2] = dfloat(y.x, y.y); v[3] = dfloat(y.z, y.w);
}

__device__ __forceinline__ bool is_finite_val(float x) { return isfinite(x); }
__device__ __forceinline__ bool is_finite_val(double x) { return isfinite(x); }
__device__ __forceinline__ bool is_finite_val(dfloat x) { return lri_df::isfinite(x); }

// Shared-memory workspace of one CTA.
template <typename T>
struct Smem {
  T red[32];
  T vec[2 * WMAX + 8];
  T stage[Stage<T>::ELEMS];
};

// ---------------------------------------------------------------------------
// Tile product  OUT(N x c) = X(N x a) * W(a x c)
//   X is produced row-tile by row-tile by a loader functor:
//     ldx(xs, i0, rows, k0, kc, TR)  fills xs[kk*TR + ii] = X(i0+ii, k0+kk)
//     (ii < TR; rows beyond `rows` must be zero)
//   W by  ldw(ws, k0, kc, ldws, c)    fills ws[kk*ldws + cc] = W(k0+kk, cc)
//     (cc < ldws; columns beyond c zero)
//   The epilogue receives each thread's 4x4 block at once:
//     epi(i, c, acc, nr, nc)  rows i..i+nr-1, columns c..c+nc-1 are valid,
//   so it can issue all of its loads before any store.
// Ends with __syncthreads().
// ---------------------------------------------------------------------------
template <typename T, class LX, class LW, class EPI>
__device__ void tile_gemm(int N, int a, int c, T* stage, const LX& ldx, const LW& ldw, const EPI& epi) {
  const int tid = threadIdx.x;
  const int c4 = (c + 3) >> 2;
  const int ldws = c4 * 4;
  int ng = NT / c4;
  int TR = 4 * ng;
  if (TR > Stage<T>::TRMAX) TR = Stage<T>::TRMAX;
  ng = TR / 4;
  T* xs = stage;
  T* ws = stage + TR * KC;
  const int cg = tid % c4, rg = tid / c4;
  const bool active = rg < ng;
  for (int i0 = 0; i0 < N; i0 += TR) {
    const int rows = min(TR, N - i0);
    T acc[4][4];
#pragma unroll
    for (int p = 0; p < 4; ++p)
#pragma unroll
      for (int q = 0; q < 4; ++q) acc[p][q] = T(0);
    for (int k0 = 0; k0 < a; k0 += KC) {
      const int kc = min(KC, a - k0);
      ldx(xs, i0, rows, k0, kc, TR);
      ldw(ws, k0, kc, ldws, c);
      __syncthreads();
      if (active) {
        for (int kk = 0; kk < kc; ++kk) {
          T xv[4], wv[4];
          ld4(xs + kk * TR + 4 * rg, xv);
          ld4(ws + kk * ldws + 4 * cg, wv);
#pragma unroll
          for (int p = 0; p < 4; ++p)
#pragma unroll
            for (int q = 0; q < 4; ++q) acc[p][q] = fma_acc(xv[p], wv[q], acc[p][q]);
        }
      }
      __syncthreads();
    }
#pragma unroll
    for (int p = 0; p < 4; ++p)
#pragma unroll
      for (int q = 0; q < 4; ++q) acc[p][q] = renorm(acc[p][q]);
    if (active && 4 * rg < rows && 4 * cg < c) epi(i0 + 4 * rg, 4 * cg, acc, min(4, rows - 4 * rg), min(4, c - 4 * cg));
  }
  __syncthreads();
}

// Epilogues for tile_gemm.
template <typename T>
struct EpiStore {  // out(i, c) = acc
  T* out;
  int ld;
  __device__ void operator()(int i, int c, const T (&acc)[4][4], int nr, int nc) const {
#pragma unroll
    for (int q = 0; q < 4; ++q)
#pragma unroll
      for (int p = 0; p < 4; ++p)
        if (p < nr && q < nc) out[(int64_t)(i + p) + (int64_t)(c + q) * ld] = acc[p][q];
  }
};

template <typename T>
struct EpiAdd {  // out(i, c) += acc
  T* out;
  int ld;
  __device__ void operator()(int i, int c, const T (&acc)[4][4], int nr, int nc) const {
    T v[4][4];
#pragma unroll
    for (int q = 0; q < 4; ++q)
#pragma unroll
      for (int p = 0; p < 4; ++p) v[p][q] = (p < nr && q < nc) ? out[(int64_t)(i + p) + (int64_t)(c + q) * ld] : T(0);
#pragma unroll
    for (int q = 0; q < 4; ++q)
#pragma unroll
      for (int p = 0; p < 4; ++p)
        if (p < nr && q < nc) out[(int64_t)(i + p) + (int64_t)(c + q) * ld] = v[p][q] + acc[p][q];
  }
};

// out(i, c) = g * y(i, c) + h * acc   (one Horner step of the substep flow)
template <typename T>
struct EpiAxpby {
  T* out;
  const T* y;
  int ld;
  T g, h;
  __device__ void operator()(int i, int c, const T (&acc)[4][4], int nr, int nc) const {
    T v[4][4];
#pragma unroll
    for (int q = 0; q < 4; ++q)
#pragma unroll
      for (int p = 0; p < 4; ++p) v[p][q] = (p < nr && q < nc) ? y[(int64_t)(i + p) + (int64_t)(c + q) * ld] : T(0);
#pragma unroll
    for (int q = 0; q < 4; ++q)
#pragma unroll
      for (int p = 0; p < 4; ++p)
        if (p < nr && q < nc) out[(int64_t)(i + p) + (int64_t)(c + q) * ld] = fma(h, acc[p][q], g * v[p][q]);
  }
};

// Loaders fill xs[kk*TR + ii] = X(i0+ii, k0+kk) for kk < kc, ii < TR (zero
// beyond `rows`).  Each thread owns rows ii = tid, tid+NT, ... and walks the
// columns in batches of 8 independent loads staged in registers, so a warp
// keeps many L2 requests in flight (consecutive threads = consecutive rows,
// coalesced).

// Loader: plain column-major panel X (ld ldx).
template <typename T>
struct LoadPanel {
  const T* X;
  int ldx;
  __device__ void operator()(T* __restrict__ xs, int i0, int rows, int k0, int kc, int TR) const {
    for (int ii = threadIdx.x; ii < TR; ii += NT) {
      const bool ok = ii < rows;
      const T* src = X + (int64_t)(i0 + ii) + (int64_t)k0 * ldx;
      for (int kb = 0; kb < kc; kb += 8) {
        T v[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) v[u] = (ok && kb + u < kc) ? src[(int64_t)(kb + u) * ldx] : T(0);
#pragma unroll
        for (int u = 0; u < 8; ++u)
          if (kb + u < kc) xs[(kb + u) * TR + ii] = v[u];
      }
    }
  }
};

// Loader: [T z | z] for a tridiagonal T (sub, dia, sup each length N,
// non-periodic: rows -1 and N are zero).  Width 2r.
template <typename T>
struct LoadStencilAug {
  const T* Z;
  int ldz, N, r;
  const T* tri;  // [sub | dia | sup]
  __device__ void operator()(T* __restrict__ xs, int i0, int rows, int k0, int kc, int TR) const {
    for (int ii = threadIdx.x; ii < TR; ii += NT) {
      const bool ok = ii < rows;
      const int i = i0 + ii;
      T cs = T(0), cd = T(0), cp = T(0);
      if (ok) {
        cd = tri[N + i];
        if (i > 0) cs = tri[i];
        if (i + 1 < N) cp = tri[2 * N + i];
      }
      const bool has_m = ok && i > 0, has_p = ok && i + 1 < N;
      for (int kb = 0; kb < kc; kb += 8) {
        T v[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const int k = k0 + kb + u;
          T x = T(0);
          if (ok && kb + u < kc) {
            if (k < r) {
              const T* col = Z + (int64_t)k * ldz;
              const T zm = has_m ? col[i - 1] : T(0);
              const T zc = col[i];
              const T zp = has_p ? col[i + 1] : T(0);
              x = fma(cs, zm, fma(cp, zp, cd * zc));
            } else {
              x = Z[i + (int64_t)(k - r) * ldz];
            }
          }
          v[u] = x;
        }
#pragma unroll
        for (int u = 0; u < 8; ++u)
          if (kb + u < kc) xs[(kb + u) * TR + ii] = v[u];
      }
    }
  }
};

// Loader: Δy = Ynext - Yprev restricted to rows (n x m column-major), or its
// transpose when `trans` (then X is m x n).
template <typename T>
struct LoadDelta {
  const T* Yn;
  const T* Yp;
  int n;      // rows of Y (leading dimension)
  bool trans;
  __device__ void operator()(T* __restrict__ xs, int i0, int rows, int k0, int kc, int TR) const {
    for (int e = threadIdx.x; e < kc * TR; e += NT) {
      int kk, ii;
      if (!trans) { kk = e / TR; ii = e - kk * TR; }
      else { ii = e / kc; kk = e - ii * kc; }  // consecutive threads walk along Y's columns
      T v = T(0);
      if (ii < rows) {
        const int64_t idx = trans ? (int64_t)(k0 + kk) + (int64_t)(i0 + ii) * n
                                  : (int64_t)(i0 + ii) + (int64_t)(k0 + kk) * n;
        v = Yp ? Yn[idx] - Yp[idx] : Yn[idx];  // no previous snapshot: Yn itself
      }
      xs[kk * TR + ii] = v;
    }
  }
};

// ---------------------------------------------------------------------------
// Local flow map (flows.cuh) contracted with low-rank factors (one CTA):
//   Y = XL ZR^T (N x M: rows = grid points, columns = samples),
//   F(Y)_ij = Flow::eval(Y_{i-1,j}, Y_ij, Y_{i+1,j}, nu_j; h, alpha, beta),
//   rows periodic; e.g. the Burgers flow
//   F(Y) = (Dxx Y) diag(nu) + alpha (Dx Y).*Y + beta Dx(Y.*Y),
//   Dxx = tridiag(1,-2,1)/h^2, Dx = tridiag(-1,0,1)/(2h), both periodic;
//   BURG_K: out (N x k, ld ldo) = F ZR
//   BURG_L: out (M x k, ld ldo) = F^T XL
//   BURG_S: out (p x k, ld ldo) = sgn * CL^T F ZR      (CL: N x p, ld N)
// XL: N x k (ld N), ZR: M x k (ld M), k, p <= 64.  Y and F exist only as
// shared-memory tiles (row tiles with one periodic halo row on each side);
// the reference evaluates F on the n x m matrix (unconventional.jl:51-79).
// Ends with __syncthreads().
// ---------------------------------------------------------------------------
enum : int { BURG_K = 0, BURG_L = 1, BURG_S = 2 };

template <typename T, typename Flow>
__device__ __noinline__ void flow_contract(int mode, int N, int M, int k, const T* XL, const T* ZR, const T* CL,
                                              int p, const T* nu, double h, double alpha, double beta, T sgn, T* out,
                                              int ldo, T* stage) {
  const int tid = threadIdx.x;
  const int ldk = k + 1, ldp = p + 1;
  const int TCb = (mode == BURG_S) ? 16 : 32;
  const int ldf = TCb + 1;
  // rows per tile: 32 when the staging area holds it, else 16
  auto need = [&](int tr) {
    int e = (tr + 2) * ldk + TCb * ldk + (tr + 2) * TCb + tr * ldf + TCb;
    if (mode == BURG_S) e += tr * ldp + tr * ldk;
    return e;
  };
  const int TRb = (need(32) <= Stage<T>::ELEMS) ? 32 : 16;
  T* xs = stage;                       // (TRb+2) x ldk: XL rows i0-1 .. i0+TRb (periodic)
  T* zs = xs + (TRb + 2) * ldk;        // TCb x ldk: ZR rows j0 ..
  T* ys = zs + TCb * ldk;              // (TRb+2) x TCb: Y tile
  T* fs = ys + (TRb + 2) * TCb;        // TRb x ldf: F tile
  T* nus = fs + TRb * ldf;             // TCb viscosities
  T* cs = nus + TCb;                   // TRb x ldp: CL rows (BURG_S)
  T* ts = cs + TRb * ldp;              // TRb x ldk: (F ZR) rows (BURG_S)
  const T ih2 = T(1.0 / (h * h)), ihx = T(0.5 / h), al = T(alpha), be = T(beta);
  constexpr int NACC = 8;  // accumulators per thread: TRb * k and TCb * k are <= 2048 = NACC * NT

  auto stage_x = [&](int i0, int rows) {
    for (int e = tid; e < (rows + 2) * k; e += NT) {
      const int ii = e % (rows + 2), a = e / (rows + 2);
      int g = i0 - 1 + ii;
      g = (g < 0) ? g + N : ((g >= N) ? g - N : g);
      xs[ii * ldk + a] = XL[g + (int64_t)a * N];
    }
  };
  auto stage_z = [&](int j0, int cols) {
    for (int e = tid; e < TCb * k; e += NT) {
      const int jj = e % TCb, a = e / TCb;
      zs[jj * ldk + a] = (jj < cols) ? ZR[(j0 + jj) + (int64_t)a * M] : T(0);
    }
    for (int jj = tid; jj < TCb; jj += NT) nus[jj] = (jj < cols) ? nu[j0 + jj] : T(0);
  };
  // Y tile, then F tile (after the caller's barrier over the staged rows)
  auto flow_tile = [&](int rows) {
    for (int o = tid; o < (rows + 2) * TCb; o += NT) {
      const int ii = o / TCb, jj = o - (o / TCb) * TCb;
      T acc = T(0);
      for (int a = 0; a < k; ++a) acc = fma_acc(xs[ii * ldk + a], zs[jj * ldk + a], acc);
      ys[o] = renorm(acc);
    }
    __syncthreads();
    for (int o = tid; o < rows * TCb; o += NT) {
      const int ii = o / TCb, jj = o - (o / TCb) * TCb;
      const T ym = ys[ii * TCb + jj], y0 = ys[(ii + 1) * TCb + jj], yp = ys[(ii + 2) * TCb + jj];
      fs[ii * ldf + jj] = Flow::template eval<T>(ym, y0, yp, nus[jj], ih2, ihx, al, be);
    }
    __syncthreads();
  };

  if (mode == BURG_L) {
    for (int j0 = 0; j0 < M; j0 += TCb) {
      const int cols = min(TCb, M - j0);
      T acc[NACC];
#pragma unroll
      for (int u = 0; u < NACC; ++u) acc[u] = T(0);
      stage_z(j0, cols);
      for (int i0 = 0; i0 < N; i0 += TRb) {
        const int rows = min(TRb, N - i0);
        stage_x(i0, rows);
        __syncthreads();
        flow_tile(rows);
        // acc(jj, c) += sum_ii F(ii, jj) XL(i0+ii, c)
#pragma unroll
        for (int u = 0; u < NACC; ++u) {
          const int o = tid + u * NT;
          if (o < TCb * k) {
            const int jj = o % TCb, c = o / TCb;
            T sacc = acc[u];
            for (int ii = 0; ii < rows; ++ii) sacc = fma_acc(fs[ii * ldf + jj], xs[(ii + 1) * ldk + c], sacc);
            acc[u] = renorm(sacc);
          }
        }
        __syncthreads();
      }
#pragma unroll
      for (int u = 0; u < NACC; ++u) {
        const int o = tid + u * NT;
        if (o < TCb * k) {
          const int jj = o % TCb, c = o / TCb;
          if (jj < cols) out[(j0 + jj) + (int64_t)c * ldo] = acc[u];
        }
      }
    }
    __syncthreads();
    return;
  }

  if (mode == BURG_S) {
    for (int o = tid; o < p * k; o += NT) out[(o % p) + (int64_t)(o / p) * ldo] = T(0);
  }
  for (int i0 = 0; i0 < N; i0 += TRb) {
    const int rows = min(TRb, N - i0);
    T acc[NACC];
#pragma unroll
    for (int u = 0; u < NACC; ++u) acc[u] = T(0);
    stage_x(i0, rows);
    for (int j0 = 0; j0 < M; j0 += TCb) {
      const int cols = min(TCb, M - j0);
      stage_z(j0, cols);
      __syncthreads();
      flow_tile(rows);
      // acc(i, c) += sum_jj F(i, jj) ZR(j0+jj, c)
#pragma unroll
      for (int u = 0; u < NACC; ++u) {
        const int o = tid + u * NT;
        if (o < TRb * k) {
          const int i = o % TRb, c = o / TRb;
          if (i < rows) {
            T sacc = acc[u];
            for (int jj = 0; jj < cols; ++jj) sacc = fma_acc(fs[i * ldf + jj], zs[jj * ldk + c], sacc);
            acc[u] = renorm(sacc);
          }
        }
      }
      __syncthreads();
    }
    if (mode == BURG_K) {
#pragma unroll
      for (int u = 0; u < NACC; ++u) {
        const int o = tid + u * NT;
        if (o < TRb * k) {
          const int i = o % TRb, c = o / TRb;
          if (i < rows) out[(i0 + i) + (int64_t)c * ldo] = acc[u];
        }
      }
    } else {
      // out += sgn * CL(rows)^T (F ZR)(rows)
#pragma unroll
      for (int u = 0; u < NACC; ++u) {
        const int o = tid + u * NT;
        if (o < TRb * k) {
          const int i = o % TRb, c = o / TRb;
          if (i < rows) ts[i * ldk + c] = acc[u];
        }
      }
      for (int e = tid; e < rows * p; e += NT) {
        const int ii = e % rows, a = e / rows;
        cs[ii * ldp + a] = CL[(i0 + ii) + (int64_t)a * N];
      }
      __syncthreads();
      for (int o = tid; o < p * k; o += NT) {
        const int a = o % p, c = o / p;
        T sacc = T(0);
        for (int ii = 0; ii < rows; ++ii) sacc = fma_acc(cs[ii * ldp + a], ts[ii * ldk + c], sacc);
        T* d = out + a + (int64_t)c * ldo;
        *d = fma(sgn, renorm(sacc), *d);
      }
      __syncthreads();
    }
  }
  __syncthreads();
}

// One application of the orthonormal-basis Sylvester substep operator:
//   out = g * y + h * (T z + z P^T)       (N x r, all column-major, ld N)
// T tridiagonal [sub | dia | sup], P (r x r, ld ldp).  Each row tile of z is
// staged once with its two halo rows; the stencil and the z P^T product both
// read shared memory.  out may alias y (never z).  Ends with __syncthreads().
template <typename T>
__device__ void tile_sylv(int N, int r, const T* z, const T* tri, const T* P, int ldp, T* out, const T* y, T g, T h,
                          T* stage) {
  const int tid = threadIdx.x;
  const int c4 = (r + 3) >> 2;
  const int ldw = c4 * 4;
  int TR = 4 * (NT / c4);
  if (TR > Stage<T>::TRMAX) TR = Stage<T>::TRMAX;
  const int ng = TR / 4;
  const int TH = TR + 4;           // staged rows: i0-1 .. i0+TR (padded to a multiple of 4)
  T* zs = stage;                   // [r][TH] column-major, zs[k*TH + 1 + ii] = z(i0+ii, k)
  T* ws = stage + r * TH;          // [r][ldw]  ws[k*ldw + c] = P(c, k) = P^T(k, c)
  for (int e = tid; e < r * ldw; e += NT) {
    const int k = e / ldw, c = e - k * ldw;
    ws[e] = (c < r) ? P[c + (int64_t)k * ldp] : T(0);
  }
  const int cg = tid % c4, rg = tid / c4;
  const bool active = rg < ng;
  for (int i0 = 0; i0 < N; i0 += TR) {
    const int rows = min(TR, N - i0);
    // stage rows i0-1 .. i0+rows (zero outside [0, N))
    for (int ii = tid; ii < rows + 2; ii += NT) {
      const int i = i0 - 1 + ii;
      const bool ok = (i >= 0) && (i < N);
      for (int kb = 0; kb < r; kb += 8) {
        T v[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) v[u] = (ok && kb + u < r) ? z[i + (int64_t)(kb + u) * N] : T(0);
#pragma unroll
        for (int u = 0; u < 8; ++u)
          if (kb + u < r) zs[(kb + u) * TH + ii] = v[u];
      }
    }
    __syncthreads();
    if (active && 4 * rg < rows && 4 * cg < r) {
      T acc[4][4];
#pragma unroll
      for (int p = 0; p < 4; ++p)
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[p][q] = T(0);
      for (int k = 0; k < r; ++k) {
        T xv[4], wv[4];
#pragma unroll
        for (int p = 0; p < 4; ++p) xv[p] = zs[k * TH + 1 + 4 * rg + p];
        ld4(ws + k * ldw + 4 * cg, wv);
#pragma unroll
        for (int p = 0; p < 4; ++p)
#pragma unroll
          for (int q = 0; q < 4; ++q) acc[p][q] = fma_acc(xv[p], wv[q], acc[p][q]);
      }
#pragma unroll
      for (int p = 0; p < 4; ++p)
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[p][q] = renorm(acc[p][q]);
      const int nr = min(4, rows - 4 * rg), nc = min(4, r - 4 * cg);
      T yv[4][4], cs[4], cd[4], cp[4];
#pragma unroll
      for (int p = 0; p < 4; ++p) {
        const int i = i0 + 4 * rg + p;
        const bool okr = p < nr;
        cd[p] = okr ? tri[N + i] : T(0);
        cs[p] = (okr && i > 0) ? tri[i] : T(0);
        cp[p] = (okr && i + 1 < N) ? tri[2 * N + i] : T(0);
#pragma unroll
        for (int q = 0; q < 4; ++q) yv[p][q] = (okr && q < nc) ? y[(int64_t)i + (int64_t)(4 * cg + q) * N] : T(0);
      }
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        if (q < nc) {
          const T* zc = zs + (4 * cg + q) * TH + 4 * rg;  // zc[p] = z(i0+4rg+p-1)
#pragma unroll
          for (int p = 0; p < 4; ++p) {
            if (p < nr) {
              const T tz = fma(cs[p], zc[p], fma(cp[p], zc[p + 2], cd[p] * zc[p + 1]));
              out[(int64_t)(i0 + 4 * rg + p) + (int64_t)(4 * cg + q) * N] = fma(h, tz + acc[p][q], g * yv[p][q]);
            }
          }
        }
      }
    }
    __syncthreads();
  }
}

// acc = sum_{k in [k0,k1)} x(4rg.., k) w(k, 4cg..) with x column-major
// (ld ldx) and w row-major (ld ldw), both in shared memory.
template <typename T>
__device__ __forceinline__ void micro_mm(const T* x, int ldx, const T* w, int ldw, int rg, int cg, int k0, int k1,
                                         T (&acc)[4][4]) {
#pragma unroll
  for (int p = 0; p < 4; ++p)
#pragma unroll
    for (int q = 0; q < 4; ++q) acc[p][q] = T(0);
  for (int k = k0; k < k1; ++k) {
    T xv[4], wv[4];
    ld4(x + k * ldx + 4 * rg, xv);
    ld4(w + k * ldw + 4 * cg, wv);
#pragma unroll
    for (int p = 0; p < 4; ++p)
#pragma unroll
      for (int q = 0; q < 4; ++q) acc[p][q] = fma_acc(xv[p], wv[q], acc[p][q]);
  }
}

// Adds the accumulators of lanes 2j and 2j+1 (both end with the sum).
template <typename T>
__device__ __forceinline__ void pair_sum(T (&acc)[4][4]) {
#pragma unroll
  for (int p = 0; p < 4; ++p)
#pragma unroll
    for (int q = 0; q < 4; ++q) acc[p][q] = acc[p][q] + shfl_xor(acc[p][q], 1);
}

// Coefficients of the stability polynomial R(z) = sum_j gam[j] z^j of an
// explicit RK scheme with a sub-diagonal tableau (gam[0] = 1):
//   gam[j+1] = sum_{s>=j} b_s * a_s a_{s-1} ... a_{s-j+1}.
__device__ inline void horner_coeffs(const Scheme& sc, double gam[5]) {
  gam[0] = 1.0;
  for (int j = 1; j < 5; ++j) gam[j] = 0.0;
  for (int j = 0; j < sc.nstages; ++j) {
    double gsum = 0.0;
    for (int st = j; st < sc.nstages; ++st) {
      double prod = sc.b[st];
      for (int t = st - j + 1; t <= st; ++t) prod *= sc.a[t];
      gsum += prod;
    }
    gam[j + 1] = gsum;
  }
}

// Fused K (or L) substep of the orthonormal-basis Sylvester flow, one row
// tile at a time entirely in shared memory:
//   y = X C  (X = U or V, C = S or S^T),  then H = ns*nsub Horner applications
//   w <- g_j y + h (T w + w P^T),  out = R(hL) y   (rows of this tile)
// The tile is staged with H halo rows on each side (zero outside [0, N), the
// operator's boundary); every application recomputes the halo region, whose
// valid part shrinks by one row per application, so after H applications
// rows [H, H+TR) are exact.  Global traffic: X read once, out written once.
// gam[0..ns] are the Horner coefficients of the stability polynomial.
// Returns false (nothing done) when the tile does not fit the staging area.
template <typename T>
__device__ bool fused_substep(int N, int r, const T* X, int ldx, const T* C, int ldc, bool transC, const T* tri,
                              const T* P, int ldp, const double* gam, int ns, int nsub, T h, T* out, T* stage) {
  const int tid = threadIdx.x;
  const int H = ns * nsub;
  const int c4 = (r + 3) >> 2;
  const int ldw = c4 * 4;
  // three tiles of TH rows (multiple of 4) plus C and P^T fill the staging
  // area; TR = TH - 2H output rows per tile (multiple of 4, <= 256)
  int TH = ((Stage<T>::ELEMS - 2 * r * ldw) / (3 * r)) & ~3;
  if (TH > 256 + 2 * H + 3) TH = (256 + 2 * H + 3) & ~3;
  const int TR = (TH - 2 * H) & ~3;
  if (TR < 16) return false;
  T* bufA = stage;
  T* bufB = bufA + r * TH;
  T* bufC = bufB + r * TH;
  T* Cs = bufC + r * TH;   // Cs[k*ldw + c] = C(k, c)
  T* Ws = Cs + r * ldw;    // Ws[k*ldw + c] = P(c, k)
  for (int e = tid; e < r * ldw; e += NT) {
    const int k = e / ldw, c = e - k * ldw;
    T cv = T(0), wv = T(0);
    if (c < r) {
      cv = transC ? C[c + (int64_t)k * ldc] : C[k + (int64_t)c * ldc];
      wv = P[c + (int64_t)k * ldp];
    }
    Cs[e] = cv;
    Ws[e] = wv;
  }
  const int rg4 = TH / 4;
  const int nmt = rg4 * c4;  // micro-tiles per tile product
  // with at most NT/2 micro-tiles, lane pairs split the k-sum of each one
  // (one pass per product: every thread runs the shuffle of pair_sum)
  const int ks = (2 * nmt <= NT) ? 2 : 1;
  const int kh = (r + ks - 1) / ks;
  for (int i0 = 0; i0 < N; i0 += TR) {
    const int g0 = i0 - H;  // global row of local row 0
    // stage X rows [g0, g0 + TH) into bufA (zero outside [0, N))
    for (int ii = tid; ii < TH; ii += NT) {
      const int i = g0 + ii;
      const bool ok = (i >= 0) && (i < N);
      for (int kb = 0; kb < r; kb += 8) {
        T v[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) v[u] = (ok && kb + u < r) ? X[i + (int64_t)(kb + u) * ldx] : T(0);
#pragma unroll
        for (int u = 0; u < 8; ++u)
          if (kb + u < r) bufA[(kb + u) * TH + ii] = v[u];
      }
    }
    __syncthreads();
    // y = X C into bufB.  With ks == 2 every thread runs exactly one
    // iteration (nmt * 2 <= NT), so all lanes reach the pair shuffle.
    for (int t2 = tid; t2 < ((ks == 2) ? NT : nmt); t2 += NT) {
      const bool act = t2 < nmt * ks;
      const int mt = act ? t2 / ks : 0, half = t2 % ks;
      const int rg = mt / c4, cg = mt - rg * c4;
      T acc[4][4];
      micro_mm<T>(bufA, TH, Cs, ldw, rg, cg, act ? half * kh : 0, act ? min(r, (half + 1) * kh) : 0, acc);
      if (ks == 2) pair_sum(acc);
      if (act && half == 0) {
#pragma unroll
        for (int q = 0; q < 4; ++q)
          if (4 * cg + q < r)
#pragma unroll
            for (int p = 0; p < 4; ++p) bufB[(4 * cg + q) * TH + 4 * rg + p] = renorm(acc[p][q]);
      }
    }
    __syncthreads();
    // Horner applications: win -> wout, y stays in bufB
    const T* y = bufB;
    const T* win = bufB;
    T* wbuf[2] = {bufC, bufA};
    int app = 0;
    for (int sub = 0; sub < nsub; ++sub) {
      T hw = h * T(gam[ns]);
      for (int j = ns - 1; j >= 0; --j, ++app) {
        T* wout = wbuf[app & 1];
        const T gj = (j == 0) ? T(1) : T(gam[j]);
        // the substep's base for later substeps is its own result: y is
        // replaced by wout after each complete substep (below)
        for (int t2 = tid; t2 < ((ks == 2) ? NT : nmt); t2 += NT) {
          const bool act = t2 < nmt * ks;
          const int mt = act ? t2 / ks : 0, half = t2 % ks;
          const int rg = mt / c4, cg = mt - rg * c4;
          T acc[4][4];
          micro_mm<T>(win, TH, Ws, ldw, rg, cg, act ? half * kh : 0, act ? min(r, (half + 1) * kh) : 0, acc);
          if (ks == 2) pair_sum(acc);
          if (!act || half != 0) continue;
#pragma unroll
          for (int p = 0; p < 4; ++p) {
            const int li = 4 * rg + p;
            const int i = g0 + li;
            const bool inside = (i >= 0) && (i < N);
            T cs = T(0), cd = T(0), cp = T(0);
            if (inside) {
              cd = tri[N + i];
              if (i > 0) cs = tri[i];
              if (i + 1 < N) cp = tri[2 * N + i];
            }
#pragma unroll
            for (int q = 0; q < 4; ++q) {
              const int c = 4 * cg + q;
              if (c < r) {
                const T* wc = win + c * TH;
                const T zm = (li > 0) ? wc[li - 1] : T(0);
                const T zp = (li + 1 < TH) ? wc[li + 1] : T(0);
                const T tz = fma(cs, zm, fma(cp, zp, cd * wc[li]));
                const T v = fma(hw, tz + renorm(acc[p][q]), gj * y[c * TH + li]);
                wout[c * TH + li] = inside ? v : T(0);
              }
            }
          }
        }
        __syncthreads();
        win = wout;
        hw = h;
      }
      if (sub + 1 < nsub) {
        // next substep starts from this one's result: copy it into bufB (y)
        T* yb = bufB;
        for (int e = tid; e < r * TH; e += NT) yb[e] = win[e];
        __syncthreads();
        win = bufB;
      }
    }
    // rows [H, H + TR) of the last result are exact
    const int rows = min(TR, N - i0);
    for (int c = 0; c < r; ++c)
      for (int ii = tid; ii < rows; ii += NT) out[(int64_t)(i0 + ii) + (int64_t)c * N] = win[c * TH + H + ii];
    __syncthreads();
  }
  return true;
}

// Register-resident K (or L) substep of the Sylvester flow for short panels
// (N <= NT rows, r <= RR columns): thread i keeps row i of the state in
// registers for the whole substep interval, so the ns*nsub Horner
// applications
//   w <- g_j y + h L(w),   L(w) = (T w) G + w P^T   (G = I: orthonormal form)
// read and write global memory only at the start and the end.  Rows reach
// their neighbours (the tridiagonal T) through a double-buffered
// column-major copy in shared memory with a zero row on each side: one
// barrier per application.  Every thread carries a row, so all eight warps
// feed the arithmetic pipe (in FP64 the SM's few FP64 units are the bound of
// this path; the tiled products leave most warps idle on such panels).
// Literal form (FP64, G = X^T X): G = I + E with E applied in FP32 when
// max|E| <= 2^-36 (the basis is orthonormal to working precision), which
// keeps the E term's FP32 rounding below 2^-54 of T w and removes a third of
// the FP64 multiply-adds; otherwise the full G product.  y stays in shared
// memory (registers go to w and the accumulators).
template <typename T, int RR, bool ORTHO>
__device__ __noinline__ void reg_substep_rr(int N, int r, T* Y, const T* tri, const T* G, const T* P, int ldp, const double* gam,
                               int ns, int nsub, T h, T* stage) {
  const int tid = threadIdx.x;
  const int LDZ = N + 2;
  T* zb0 = stage;                  // zb[k*LDZ + 1 + i] = w(i, k); entries 0 and N+1 stay zero
  T* zb1 = zb0 + RR * LDZ;
  T* ys = zb1 + RR * LDZ;          // ys[k*N + i] = y(i, k)
  T* Ps = ys + RR * N;             // Ps[k*RR + c] = P(c, k)
  T* Gs = Ps + RR * RR;            // Gs[k*RR + c] = G(k, c)
  float* Es = reinterpret_cast<float*>(Gs + RR * RR);  // Es[k*RR + c] = G(k, c) - [k == c]
  int full = 0;
  for (int e = tid; e < RR * RR; e += NT) {
    const int k = e / RR, c = e - k * RR;
    T pv = T(0);
    if (k < r && c < r) pv = P[c + (int64_t)k * ldp];
    Ps[e] = pv;
    if constexpr (!ORTHO) {
      const T gv = (k < r && c < r) ? G[k + (int64_t)c * ldp] : T(0);
      const T ev = gv - ((k == c && k < r) ? T(1) : T(0));
      Gs[e] = gv;
      Es[e] = (float)ev;
      if (!(fabs(ev) <= T(0x1p-36))) full = 1;  // NaN included
    }
  }
  // the zero rows at both ends of both buffers (disjoint from the rows below)
  for (int e = tid; e < 4 * RR; e += NT) {
    const int b = e / (2 * RR), k = (e >> 1) % RR;
    (b ? zb1 : zb0)[k * LDZ + ((e & 1) ? N + 1 : 0)] = T(0);
  }
  const bool own = tid < N;
  T w[RR];
  T cs = T(0), cd = T(0), cp = T(0);
#pragma unroll
  for (int k = 0; k < RR; ++k) w[k] = (own && k < r) ? Y[tid + (int64_t)k * N] : T(0);
  if (own) {
    cd = tri[N + tid];
    if (tid > 0) cs = tri[tid];
    if (tid + 1 < N) cp = tri[2 * N + tid];
#pragma unroll
    for (int k = 0; k < RR; ++k) {
      zb0[k * LDZ + 1 + tid] = w[k];
      ys[k * N + tid] = w[k];
    }
  }
  const bool full_g = __syncthreads_or(full) != 0;
  T* zin = zb0;
  T* zout = zb1;
  for (int sub = 0; sub < nsub; ++sub) {
    T hw = h * T(gam[ns]);
    for (int j = ns - 1; j >= 0; --j) {
      const T gj = (j == 0) ? T(1) : T(gam[j]);
      if (own) {
        T acc[RR];
        if constexpr (ORTHO) {
#pragma unroll
          for (int c = 0; c < RR; ++c) acc[c] = T(0);
#pragma unroll
          for (int k = 0; k < RR; ++k)
#pragma unroll
            for (int c = 0; c < RR; ++c) acc[c] = fma_acc(w[k], Ps[k * RR + c], acc[c]);
#pragma unroll
          for (int c = 0; c < RR; ++c) {
            const T tz = fma(cs, zin[c * LDZ + tid], fma(cp, zin[c * LDZ + tid + 2], cd * w[c]));
            acc[c] = fma(hw, tz + renorm(acc[c]), gj * ys[c * N + tid]);
          }
        } else {
          // acc = T w (the stencil rows), then acc G + w P^T
#pragma unroll
          for (int k = 0; k < RR; ++k)
            acc[k] = fma(cs, zin[k * LDZ + tid], fma(cp, zin[k * LDZ + tid + 2], cd * w[k]));
          bool in_range = true;
#pragma unroll
          for (int k = 0; k < RR; ++k) in_range = in_range && (fabs(acc[k]) < T(0x1p100));
          if (!full_g && in_range) {
            float e[RR];
#pragma unroll
            for (int c = 0; c < RR; ++c) e[c] = 0.0f;
#pragma unroll
            for (int k = 0; k < RR; ++k) {
              const float tk = (float)acc[k];
#pragma unroll
              for (int c = 0; c < RR; ++c) e[c] = fmaf(tk, Es[k * RR + c], e[c]);
            }
#pragma unroll
            for (int c = 0; c < RR; ++c) acc[c] += T(e[c]);
          } else {
            T tz[RR];
#pragma unroll
            for (int k = 0; k < RR; ++k) tz[k] = acc[k];
#pragma unroll
            for (int c = 0; c < RR; ++c) acc[c] = T(0);
#pragma unroll
            for (int k = 0; k < RR; ++k)
#pragma unroll
              for (int c = 0; c < RR; ++c) acc[c] = fma(tz[k], Gs[k * RR + c], acc[c]);
          }
#pragma unroll
          for (int k = 0; k < RR; ++k)
#pragma unroll
            for (int c = 0; c < RR; ++c) acc[c] = fma(w[k], Ps[k * RR + c], acc[c]);
#pragma unroll
          for (int c = 0; c < RR; ++c) acc[c] = fma(hw, acc[c], gj * ys[c * N + tid]);
        }
#pragma unroll
        for (int c = 0; c < RR; ++c) {
          w[c] = acc[c];
          zout[c * LDZ + 1 + tid] = acc[c];
        }
        // the substep's result is the next substep's base (only this
        // thread reads its own row of y)
        if (j == 0 && sub + 1 < nsub) {
#pragma unroll
          for (int c = 0; c < RR; ++c) ys[c * N + tid] = acc[c];
        }
      }
      __syncthreads();
      T* t = zin;
      zin = zout;
      zout = t;
      hw = h;
    }
  }
  if (own) {
    for (int k = 0; k < r; ++k) Y[tid + (int64_t)k * N] = w[k];
  }
  __syncthreads();
}

// Dispatch of reg_substep_rr by panel width; false when the panel does not
// fit the path (more than NT rows or 8 columns, or the staging area).
template <typename T, bool ORTHO>
__device__ bool reg_substep(int N, int r, T* Y, const T* tri, const T* G, const T* P, int ldp, const double* gam,
                            int ns, int nsub, T h, T* stage) {
  if (N > NT || r > 8) return false;
  const int RR = (r <= 4) ? 4 : 8;
  const int64_t need = (int64_t)RR * (2 * (N + 2) + N) + 3 * RR * RR;
  if (need > Stage<T>::ELEMS) return false;
  if (RR == 4)
    reg_substep_rr<T, 4, ORTHO>(N, r, Y, tri, G, P, ldp, gam, ns, nsub, h, stage);
  else
    reg_substep_rr<T, 8, ORTHO>(N, r, Y, tri, G, P, ldp, gam, ns, nsub, h, stage);
  return true;
}

// S substep of the Sylvester flow on a small p x q core (p*q <= NT, p, q <=
// 16): thread i + j*p keeps entry (i, j) of the state and of the RK
// accumulator in registers; the stage inputs alternate between two
// shared-memory copies, so a stage costs one barrier (orthonormal form
//   k = sign (P_U Z + Z P_V^T))
// or two (literal form, k = sign (P_U (Z G_V) + G_U (Z P_V^T)), whose two
// inner products go through shared memory first).  The RK update is the
// stage-by-stage scheme of the panel path (same operations per entry).
// St, G_U, P_U, G_V, P_V: column-major with leading dimension W.
template <typename T, bool ORTHO>
__device__ __noinline__ void core_small(int p, int q, int W, T* St, T sign, const T* GU, const T* PU, const T* GV,
                                        const T* PV, const Scheme& sc, T h, T* stage) {
  const int tid = threadIdx.x;
  const int pq = p * q;
  T* Zb0 = stage;               // Zb[i + k*p] = Z(i, k)
  T* Zb1 = Zb0 + pq;
  T* T1s = Zb1 + pq;            // T1s[k + j*p] = (Z G_V)(k, j)
  T* T2s = T1s + pq;            // T2s[k + j*p] = (Z P_V^T)(k, j)
  T* PUs = T2s + pq;            // PUs[i + k*p] = P_U(i, k)
  T* GUs = PUs + p * p;
  T* PVs = GUs + p * p;         // PVs[j + k*q] = P_V(j, k)
  T* GVs = PVs + q * q;         // GVs[k + j*q] = G_V(k, j)
  for (int e = tid; e < p * p; e += NT) {
    const int i = e % p, k = e / p;
    PUs[e] = PU[i + (int64_t)k * W];
    if constexpr (!ORTHO) GUs[e] = GU[i + (int64_t)k * W];
  }
  for (int e = tid; e < q * q; e += NT) {
    const int a = e % q, b = e / q;
    PVs[e] = PV[a + (int64_t)b * W];
    if constexpr (!ORTHO) GVs[e] = GV[a + (int64_t)b * W];
  }
  const bool own = tid < pq;
  const int i = own ? tid % p : 0, j = own ? tid / p : 0;
  T st = T(0), sa = T(0);
  if (own) {
    st = St[i + (int64_t)j * W];
    Zb0[i + j * p] = st;
  }
  __syncthreads();
  const int ns = sc.nstages;
  int cur = 0;
  for (int sub = 0; sub < sc.nsub; ++sub) {
    for (int s = 0; s < ns; ++s) {
      const T* Z = cur ? Zb1 : Zb0;
      T* Zo = cur ? Zb0 : Zb1;
      T kv = T(0);
      if constexpr (ORTHO) {
        if (own) {
          T a0 = T(0), a1 = T(0);
          for (int k = 0; k < p; ++k) a0 = fma(PUs[i + k * p], Z[k + j * p], a0);
          for (int k = 0; k < q; ++k) a1 = fma(Z[i + k * p], PVs[j + k * q], a1);
          kv = sign * (a0 + a1);
        }
      } else {
        if (own) {
          T t1 = T(0), t2 = T(0);
          for (int k = 0; k < q; ++k) {
            const T z = Z[i + k * p];
            t1 = fma(z, GVs[k + j * q], t1);
            t2 = fma(z, PVs[j + k * q], t2);
          }
          T1s[i + j * p] = t1;
          T2s[i + j * p] = t2;
        }
        __syncthreads();
        if (own) {
          T a0 = T(0), a1 = T(0);
          for (int k = 0; k < p; ++k) {
            a0 = fma(PUs[i + k * p], T1s[k + j * p], a0);
            a1 = fma(GUs[i + k * p], T2s[k + j * p], a1);
          }
          kv = sign * (a0 + a1);
        }
      }
      if (own) {
        const T bs = T(sc.b[s]);
        const T an = (s + 1 < ns) ? T(sc.a[s + 1]) : T(0);
        if (ns == 1) {
          st = fma(h * bs, kv, st);
          Zo[i + j * p] = st;
        } else if (s == 0) {
          sa = bs * kv;
          Zo[i + j * p] = fma(h * an, kv, st);
        } else if (s + 1 < ns) {
          sa = fma(bs, kv, sa);
          Zo[i + j * p] = fma(h * an, kv, st);
        } else {
          st = fma(h, fma(bs, kv, sa), st);
          Zo[i + j * p] = st;
        }
      }
      __syncthreads();
      cur ^= 1;
    }
  }
  if (own) St[i + (int64_t)j * W] = st;
  __syncthreads();
}

// W loader: column-major matrix W (ld ldw0) or its transpose.
template <typename T>
struct LoadSmall {
  const T* W;
  int ld;
  bool trans;  // true: W(k, c) = M[c + k*ld]
  __device__ void operator()(T* ws, int k0, int kc, int ldws, int c) const {
    for (int e = threadIdx.x; e < kc * ldws; e += NT) {
      const int kk = e / ldws, cc = e - kk * ldws;
      T v = T(0);
      if (cc < c) {
        const int k = k0 + kk;
        v = trans ? W[cc + (int64_t)k * ld] : W[k + (int64_t)cc * ld];
      }
      ws[e] = v;
    }
  }
};

// W loader for the Sylvester K/L rhs: W = [G ; P^T]  (2r x r), G and P r x r
// column-major with leading dimension ld.
template <typename T>
struct LoadGP {
  const T* G;
  const T* P;
  int ld, r;
  __device__ void operator()(T* ws, int k0, int kc, int ldws, int c) const {
    for (int e = threadIdx.x; e < kc * ldws; e += NT) {
      const int kk = e / ldws, cc = e - kk * ldws;
      T v = T(0);
      if (cc < c) {
        const int k = k0 + kk;
        v = (k < r) ? G[k + (int64_t)cc * ld] : P[cc + (int64_t)(k - r) * ld];
      }
      ws[e] = v;
    }
  }
};

// ---------------------------------------------------------------------------
// Gram-type reduction  OUT(a x c) = X(N x a)^T * Y(N x c) (a <= 64, c <= 128), written to a
// column-major destination (ld ldo), optionally scaled and accumulated:
//   out = alpha * X^T Y + beta * out.
// X rows come from loader lx(xs, i0, rows, lda_s) writing row-major
// xs[ii*lda_s + k]; Y likewise.  Ends with __syncthreads().
// ---------------------------------------------------------------------------
constexpr int TRG = 32;

// Row-major staging loaders for tile_gram: lane = row (TRG = 32 rows, one
// per lane), warp w takes columns w, w+NW, ... in batches of 4 loads.
template <typename T>
struct RowLoadPanel {  // row-major staging of a column-major panel
  const T* X;
  int ldx, w;
  __device__ void operator()(T* __restrict__ xs, int i0, int rows, int lds) const {
    const int ii = threadIdx.x & 31, wp = threadIdx.x >> 5;
    const bool ok = ii < rows;
    const T* src = X + (int64_t)(i0 + ii);
    for (int kb = wp; kb < w; kb += 4 * NW) {
      T v[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int k = kb + u * NW;
        v[u] = (ok && k < w) ? src[(int64_t)k * ldx] : T(0);
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int k = kb + u * NW;
        if (k < w) xs[ii * lds + k] = v[u];
      }
    }
  }
};

template <typename T>
struct RowLoadStencilAug {  // row-major staging of [Z | T Z] (note order), width 2r
  const T* Z;
  int ldz, N, r;
  const T* tri;
  __device__ void operator()(T* __restrict__ xs, int i0, int rows, int lds) const {
    const int ii = threadIdx.x & 31, wp = threadIdx.x >> 5;
    const bool ok = ii < rows;
    const int i = i0 + ii;
    T cs = T(0), cd = T(0), cp = T(0);
    if (ok) {
      cd = tri[N + i];
      if (i > 0) cs = tri[i];
      if (i + 1 < N) cp = tri[2 * N + i];
    }
    const bool has_m = ok && i > 0, has_p = ok && i + 1 < N;
    for (int kb = wp; kb < r; kb += 4 * NW) {
      T v[4], s[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int k = kb + u * NW;
        T zc = T(0), zm = T(0), zp = T(0);
        if (ok && k < r) {
          const T* col = Z + (int64_t)k * ldz;
          zc = col[i];
          if (has_m) zm = col[i - 1];
          if (has_p) zp = col[i + 1];
        }
        v[u] = zc;
        s[u] = fma(cs, zm, fma(cp, zp, cd * zc));
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int k = kb + u * NW;
        if (k < r) {
          xs[ii * lds + k] = v[u];
          xs[ii * lds + r + k] = s[u];
        }
      }
    }
  }
};

template <typename T>
struct RowLoadPanelStencil {  // row-major staging of [Y | T Z] (Y width r, T Z width r)
  const T* Y;
  int ldy;
  const T* Z;
  int ldz, N, r;
  const T* tri;
  __device__ void operator()(T* __restrict__ xs, int i0, int rows, int lds) const {
    RowLoadPanelShifted(xs, i0, rows, lds);
  }
  __device__ void RowLoadPanelShifted(T* __restrict__ xs, int i0, int rows, int lds) const {
    const int ii = threadIdx.x & 31, wp = threadIdx.x >> 5;
    const bool ok = ii < rows;
    const int i = i0 + ii;
    T cs = T(0), cd = T(0), cp = T(0);
    if (ok) {
      cd = tri[N + i];
      if (i > 0) cs = tri[i];
      if (i + 1 < N) cp = tri[2 * N + i];
    }
    const bool has_m = ok && i > 0, has_p = ok && i + 1 < N;
    for (int kb = wp; kb < r; kb += 4 * NW) {
      T yv[4], s4[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int k = kb + u * NW;
        T zc = T(0), zm = T(0), zp = T(0), y = T(0);
        if (ok && k < r) {
          const T* col = Z + (int64_t)k * ldz;
          zc = col[i];
          if (has_m) zm = col[i - 1];
          if (has_p) zp = col[i + 1];
          y = Y[i + (int64_t)k * ldy];
        }
        yv[u] = y;
        s4[u] = fma(cs, zm, fma(cp, zp, cd * zc));
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int k = kb + u * NW;
        if (k < r) {
          xs[ii * lds + k] = yv[u];
          xs[ii * lds + r + k] = s4[u];
        }
      }
    }
  }
};

template <typename T>
struct RowLoadStencil {  // row-major staging of T Z, width r
  const T* Z;
  int ldz, N, r;
  const T* tri;
  __device__ void operator()(T* __restrict__ xs, int i0, int rows, int lds) const {
    const int ii = threadIdx.x & 31, wp = threadIdx.x >> 5;
    const bool ok = ii < rows;
    const int i = i0 + ii;
    T cs = T(0), cd = T(0), cp = T(0);
    if (ok) {
      cd = tri[N + i];
      if (i > 0) cs = tri[i];
      if (i + 1 < N) cp = tri[2 * N + i];
    }
    const bool has_m = ok && i > 0, has_p = ok && i + 1 < N;
    for (int kb = wp; kb < r; kb += 4 * NW) {
      T s4[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int k = kb + u * NW;
        T zc = T(0), zm = T(0), zp = T(0);
        if (ok && k < r) {
          const T* col = Z + (int64_t)k * ldz;
          zc = col[i];
          if (has_m) zm = col[i - 1];
          if (has_p) zp = col[i + 1];
        }
        s4[u] = fma(cs, zm, fma(cp, zp, cd * zc));
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int k = kb + u * NW;
        if (k < r) xs[ii * lds + k] = s4[u];
      }
    }
  }
};

// Columns [csplit, c) of the result may go to a second destination out2
// (column csplit of the result is column 0 of out2, same ld).
// PER = micro-tiles per thread (1 when a4 * c4 <= NT, else 2); separate
// non-inlined instances so the common one-tile case keeps half the
// accumulators in registers.
template <typename T, int PER, class LXr, class LYr>
__device__ __noinline__ void tile_gram_impl(int N, int a, int c, T* stage, const LXr lx, const LYr ly, T* out,
                                            int ldo, T alpha, T beta, T* out2, int csplit) {
  const int tid = threadIdx.x;
  const int a4 = (a + 3) >> 2, c4 = (c + 3) >> 2;
  const int MT = a4 * c4;
  const int lxs = a4 * 4 + 4, lys = c4 * 4 + 4;
  T* xs = stage;
  T* ys = stage + TRG * lxs;
  const int splits = (MT >= NT) ? 1 : (NT / MT);
  const int per = PER;
  T acc[PER][16];
#pragma unroll
  for (int u = 0; u < PER; ++u)
#pragma unroll
    for (int e = 0; e < 16; ++e) acc[u][e] = T(0);
  const int mt0 = (splits > 1) ? (tid % MT) : tid;
  const int split = (splits > 1) ? (tid / MT) : 0;
  const bool active = (splits > 1) ? (tid < MT * splits) : true;
  for (int i0 = 0; i0 < N; i0 += TRG) {
    const int rows = min(TRG, N - i0);
    lx(xs, i0, rows, lxs);
    ly(ys, i0, rows, lys);
    __syncthreads();
    if (active) {
#pragma unroll
      for (int u = 0; u < PER; ++u) {
        if (u < per) {
          const int mt = mt0 + u * NT;
          if (mt < MT) {
            const int ma = mt / c4, mc = mt - ma * c4;
            for (int ii = split; ii < rows; ii += splits) {
              T xv[4], yv[4];
              ld4(xs + ii * lxs + 4 * ma, xv);
              ld4(ys + ii * lys + 4 * mc, yv);
#pragma unroll
              for (int p = 0; p < 4; ++p)
#pragma unroll
                for (int q = 0; q < 4; ++q) acc[u][p * 4 + q] = fma_acc(xv[p], yv[q], acc[u][p * 4 + q]);
            }
          }
        }
      }
#pragma unroll
      for (int u = 0; u < PER; ++u)
#pragma unroll
        for (int e = 0; e < 16; ++e) acc[u][e] = renorm(acc[u][e]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int u = 0; u < PER; ++u)
#pragma unroll
    for (int e = 0; e < 16; ++e) acc[u][e] = renorm(acc[u][e]);
  // combine splits through shared memory (deterministic order)
  T* part = stage;  // splits * MT * 16 <= NT*16 elements
  if (splits > 1) {
    if (active) {
#pragma unroll
      for (int e = 0; e < 16; ++e) part[(split * MT + mt0) * 16 + e] = acc[0][e];
    }
    __syncthreads();
    for (int o = tid; o < MT * 16; o += NT) {
      const int mt = o >> 4, e = o & 15;
      T s = T(0);
      for (int sp = 0; sp < splits; ++sp) s += part[(sp * MT + mt) * 16 + e];
      const int ma = mt / c4, mc = mt - ma * c4;
      const int ia = 4 * ma + (e >> 2), jc = 4 * mc + (e & 3);
      if (ia < a && jc < c) {
        T* d = (jc < csplit) ? out + ia + (int64_t)jc * ldo : out2 + ia + (int64_t)(jc - csplit) * ldo;
        *d = (beta == T(0)) ? alpha * s : fma(alpha, s, beta * *d);
      }
    }
    __syncthreads();
  } else {
#pragma unroll
    for (int u = 0; u < PER; ++u) {
      if (u < per) {
        const int mt = mt0 + u * NT;
        if (mt < MT) {
          const int ma = mt / c4, mc = mt - ma * c4;
#pragma unroll
          for (int e = 0; e < 16; ++e) {
            const int ia = 4 * ma + (e >> 2), jc = 4 * mc + (e & 3);
            if (ia < a && jc < c) {
              T* d = (jc < csplit) ? out + ia + (int64_t)jc * ldo : out2 + ia + (int64_t)(jc - csplit) * ldo;
              *d = (beta == T(0)) ? alpha * acc[u][e] : fma(alpha, acc[u][e], beta * *d);
            }
          }
        }
      }
    }
    __syncthreads();
  }
}

template <typename T, class LXr, class LYr>
__device__ void tile_gram(int N, int a, int c, T* stage, const LXr& lx, const LYr& ly, T* out, int ldo,
                          T alpha, T beta, T* out2 = nullptr, int csplit = 1 << 30) {
  if (((a + 3) >> 2) * ((c + 3) >> 2) <= NT)
    tile_gram_impl<T, 1, LXr, LYr>(N, a, c, stage, lx, ly, out, ldo, alpha, beta, out2, csplit);
  else
    tile_gram_impl<T, 2, LXr, LYr>(N, a, c, stage, lx, ly, out, ldo, alpha, beta, out2, csplit);
}

// tile_gram for FP32 panels with double-float accumulation (exact FP32
// products, double-float sums; renormalised after every staged row chunk):
// X^T Y (a x c, a4 * c4 <= NT) to the double-float matrices outd (columns
// [0, csplit)) and out2d (columns [csplit, c)), ld ldo, and optionally their
// FP32 roundings to outf / out2f (same ld).  Ends with __syncthreads().
template <class LXr, class LYr>
__device__ __noinline__ void tile_gram_acc(int N, int a, int c, float* stage, const LXr lx, const LYr ly,
                                           dfloat* outd, dfloat* out2d, float* outf, float* out2f, int ldo,
                                           int csplit) {
  const int tid = threadIdx.x;
  const int a4 = (a + 3) >> 2, c4 = (c + 3) >> 2;
  const int MT = a4 * c4;  // <= NT
  const int lxs = a4 * 4 + 4, lys = c4 * 4 + 4;
  float* xs = stage;
  float* ys = stage + TRG * lxs;
  const int splits = NT / MT;
  const int mt = tid % MT, split = tid / MT;
  const bool active = split < splits;
  const int ma = mt / c4, mc = mt - (mt / c4) * c4;
  dfloat acc[16];
#pragma unroll
  for (int e = 0; e < 16; ++e) acc[e] = dfloat(0.0f, 0.0f);
  for (int i0 = 0; i0 < N; i0 += TRG) {
    const int rows = min(TRG, N - i0);
    lx(xs, i0, rows, lxs);
    ly(ys, i0, rows, lys);
    __syncthreads();
    if (active) {
      for (int ii = split; ii < rows; ii += splits) {
        float xv[4], yv[4];
        ld4(xs + ii * lxs + 4 * ma, xv);
        ld4(ys + ii * lys + 4 * mc, yv);
#pragma unroll
        for (int p = 0; p < 4; ++p)
#pragma unroll
          for (int q = 0; q < 4; ++q) acc[p * 4 + q] = acc_mul_acc(acc[p * 4 + q], xv[p], yv[q]);
      }
#pragma unroll
      for (int e = 0; e < 16; ++e) acc[e] = renorm(acc[e]);
    }
    __syncthreads();
  }
  dfloat* part = reinterpret_cast<dfloat*>(stage);  // splits * MT * 16 <= NT * 16 values
  if (active) {
#pragma unroll
    for (int e = 0; e < 16; ++e) part[(split * MT + mt) * 16 + e] = acc[e];
  }
  __syncthreads();
  for (int o = tid; o < MT * 16; o += NT) {
    const int m2 = o >> 4, e = o & 15;
    dfloat sum = part[m2 * 16 + e];
    for (int sp = 1; sp < splits; ++sp) sum += part[(sp * MT + m2) * 16 + e];
    const int a2 = m2 / c4, c2 = m2 - (m2 / c4) * c4;
    const int ia = 4 * a2 + (e >> 2), jc = 4 * c2 + (e & 3);
    if (ia < a && jc < c) {
      const bool first = jc < csplit;
      const int64_t off = ia + (int64_t)(first ? jc : jc - csplit) * ldo;
      (first ? outd : out2d)[off] = sum;
      float* of = first ? outf : out2f;
      if (of) of[off] = sum.hi + sum.lo;
    }
  }
  __syncthreads();
}

// ---------------------------------------------------------------------------
// Small dense products on column-major matrices in global scratch:
//   C(p x s) = alpha * op(A)(p x q) * op(B)(q x s) + beta * C
// ---------------------------------------------------------------------------
template <typename T>
__device__ __noinline__ void small_gemm(int p, int q, int s, T alpha, const T* A, int lda, bool ta, const T* B, int ldb,
                           bool tb, T beta, T* C, int ldc) {
  for (int o = threadIdx.x; o < p * s; o += NT) {
    const int i = o % p, j = o / p;
    T a4[4] = {T(0), T(0), T(0), T(0)};
    int k = 0;
    for (; k + 4 <= q; k += 4) {
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const T av = ta ? A[(k + u) + (int64_t)i * lda] : A[i + (int64_t)(k + u) * lda];
        const T bv = tb ? B[j + (int64_t)(k + u) * ldb] : B[(k + u) + (int64_t)j * ldb];
        a4[u] = fma(av, bv, a4[u]);
      }
    }
    for (; k < q; ++k) {
      const T av = ta ? A[k + (int64_t)i * lda] : A[i + (int64_t)k * lda];
      const T bv = tb ? B[j + (int64_t)k * ldb] : B[k + (int64_t)j * ldb];
      a4[0] = fma(av, bv, a4[0]);
    }
    const T acc = (a4[0] + a4[1]) + (a4[2] + a4[3]);
    T* d = C + i + (int64_t)j * ldc;
    *d = (beta == T(0)) ? alpha * acc : fma(alpha, acc, beta * *d);
  }
  __syncthreads();
}

template <typename T>
__device__ void copy_mat(int p, int q, const T* A, int lda, T* B, int ldb) {
  for (int o = threadIdx.x; o < p * q; o += NT) {
    const int i = o % p, j = o / p;
    B[i + (int64_t)j * ldb] = A[i + (int64_t)j * lda];
  }
  __syncthreads();
}

template <typename T>
__device__ void zero_mat(int p, int q, T* A, int lda) {
  for (int o = threadIdx.x; o < p * q; o += NT) {
    const int i = o % p, j = o / p;
    A[i + (int64_t)j * lda] = T(0);
  }
  __syncthreads();
}

// ---------------------------------------------------------------------------
// Householder QR of the N x W panel A (column-major, ld lda), N >= W, in the
// LAPACK convention (beta = -sign(alpha) * ||x||, v(k) = 1).  hh_factor
// leaves R in the upper triangle, the reflectors below it and tau in
// sm.vec[0..W); hh_form_q writes the explicit thin Q to a separate panel,
// hh_form_q_inplace overwrites A with Q (LAPACK org2r order).  The
// reductions use sm.stage[0 .. NW*WMAX).
// ---------------------------------------------------------------------------
template <typename T>
__device__ __noinline__ void hh_factor(T* A, int lda, int N, int W, Smem<T>& sm) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  T* tau = sm.vec;            // [W]
  T* wv = sm.vec + WMAX;      // [W]
  T* wred = sm.stage;         // [NW * WMAX]
  for (int k = 0; k < W; ++k) {
    T* colk = A + (int64_t)k * lda;
    T loc = T(0);
    for (int i = k + 1 + tid; i < N; i += NT) {
      const T x = colk[i];
      loc = fma(x, x, loc);
    }
    const T xn2 = block_sum(loc, sm.red);
    const T alpha = colk[k];
    T tk = T(0), beta = alpha, scal = T(0);
    if (xn2 > T(0)) {
      beta = -copysign(sqrt(fma(alpha, alpha, xn2)), alpha);
      tk = (beta - alpha) / beta;
      scal = T(1) / (alpha - beta);
    }
    const int nj = W - k - 1;
    if (tk != T(0)) {
      // w_j = A[k,j] + scal * sum_{i>k} x_i A[i,j] with the unscaled x (the
      // reflector v = [1; scal*x] is written back in the update pass below);
      // eight columns at a time so the shuffle reductions overlap.  The same
      // pass accumulates v^T v from the scaled entries, and tau = 2 / v^T v
      // is recomputed from it: H = I - tau v v^T is then orthogonal to working
      // precision even when the squares of a tiny column under- or overflow
      // the exponent range (float and double-float values).
      T pvv = T(0);
      for (int j0 = 0; j0 < max(nj, 1); j0 += 8) {
        T p[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) p[u] = T(0);
        for (int i = k + 1 + tid; i < N; i += NT) {
          const T x = colk[i];
          if (j0 == 0) {
            const T vx = x * scal;
            pvv = fma(vx, vx, pvv);
          }
#pragma unroll
          for (int u = 0; u < 8; ++u)
            if (j0 + u < nj) p[u] = fma(x, A[i + (int64_t)(k + 1 + j0 + u) * lda], p[u]);
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) p[u] = warp_sum(p[u]);
        if (lane == 0) {
#pragma unroll
          for (int u = 0; u < 8; ++u)
            if (j0 + u < nj) wred[warp * WMAX + j0 + u] = p[u];
        }
      }
      pvv = warp_sum(pvv);
      if (lane == 0) wred[warp * WMAX + WMAX - 1] = pvv;
      __syncthreads();
      T vv = T(1);
#pragma unroll
      for (int w = 0; w < NW; ++w) vv += wred[w * WMAX + WMAX - 1];
      tk = T(2) / vv;
      if (tid == 0) tau[k] = tk;
      if (tid < nj) {
        T acc = T(0);
#pragma unroll
        for (int w = 0; w < NW; ++w) acc += wred[w * WMAX + tid];
        wv[tid] = tk * fma(scal, acc, A[k + (int64_t)(k + 1 + tid) * lda]);
      }
      __syncthreads();
      // A[i, k+1:] -= v_i * wv, one row per thread; store v below the diagonal
      for (int i = k + tid; i < N; i += NT) {
        T vi = T(1);
        if (i > k) {
          vi = colk[i] * scal;
          colk[i] = vi;
        }
        T* row = A + i + (int64_t)(k + 1) * lda;
        int j = 0;
        for (; j + 4 <= nj; j += 4) {
          const T a0 = row[(int64_t)j * lda], a1 = row[(int64_t)(j + 1) * lda];
          const T a2 = row[(int64_t)(j + 2) * lda], a3 = row[(int64_t)(j + 3) * lda];
          row[(int64_t)j * lda] = a0 - vi * wv[j];
          row[(int64_t)(j + 1) * lda] = a1 - vi * wv[j + 1];
          row[(int64_t)(j + 2) * lda] = a2 - vi * wv[j + 2];
          row[(int64_t)(j + 3) * lda] = a3 - vi * wv[j + 3];
        }
        for (; j < nj; ++j) row[(int64_t)j * lda] -= vi * wv[j];
      }
    } else if (tid == 0) {
      tau[k] = T(0);
    }
    __syncthreads();
    if (tid == 0) colk[k] = beta;
    __syncthreads();
  }
}

// Explicit thin Q into a separate panel by backward accumulation:
// Q = H_0 ... H_{W-1} [I; 0], reflectors and tau from hh_factor.
template <typename T>
__device__ __noinline__ void hh_form_q(const T* A, int lda, int N, int W, T* Q, int ldq, Smem<T>& sm) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const T* tau = sm.vec;
  T* wv = sm.vec + WMAX;
  T* wred = sm.stage;
  for (int j = 0; j < W; ++j) {
    T* qj = Q + (int64_t)j * ldq;
    for (int i = tid; i < N; i += NT) qj[i] = (i == j) ? T(1) : T(0);
  }
  __syncthreads();
  for (int k = W - 1; k >= 0; --k) {
    const T tk = tau[k];
    if (tk == T(0)) continue;
    const T* colk = A + (int64_t)k * lda;
    const int nj = W - k;
    for (int j0 = 0; j0 < nj; j0 += 8) {
      T p[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) p[u] = (tid == 0 && j0 + u < nj) ? Q[k + (int64_t)(k + j0 + u) * ldq] : T(0);
      for (int i = k + 1 + tid; i < N; i += NT) {
        const T vi = colk[i];
#pragma unroll
        for (int u = 0; u < 8; ++u)
          if (j0 + u < nj) p[u] = fma(vi, Q[i + (int64_t)(k + j0 + u) * ldq], p[u]);
      }
#pragma unroll
      for (int u = 0; u < 8; ++u) p[u] = warp_sum(p[u]);
      if (lane == 0) {
#pragma unroll
        for (int u = 0; u < 8; ++u)
          if (j0 + u < nj) wred[warp * WMAX + j0 + u] = p[u];
      }
    }
    __syncthreads();
    if (tid < nj) {
      T acc = T(0);
#pragma unroll
      for (int w = 0; w < NW; ++w) acc += wred[w * WMAX + tid];
      wv[tid] = tk * acc;
    }
    __syncthreads();
    for (int i = k + tid; i < N; i += NT) {
      const T vi = (i == k) ? T(1) : colk[i];
      T* row = Q + i + (int64_t)k * ldq;
      int j = 0;
      for (; j + 4 <= nj; j += 4) {
        const T q0 = row[(int64_t)j * ldq], q1 = row[(int64_t)(j + 1) * ldq];
        const T q2 = row[(int64_t)(j + 2) * ldq], q3 = row[(int64_t)(j + 3) * ldq];
        row[(int64_t)j * ldq] = q0 - vi * wv[j];
        row[(int64_t)(j + 1) * ldq] = q1 - vi * wv[j + 1];
        row[(int64_t)(j + 2) * ldq] = q2 - vi * wv[j + 2];
        row[(int64_t)(j + 3) * ldq] = q3 - vi * wv[j + 3];
      }
      for (; j < nj; ++j) row[(int64_t)j * ldq] -= vi * wv[j];
    }
    __syncthreads();
  }
}

// Q = H_0 ... H_{W-1} [I; 0] formed in place over the reflectors (org2r):
// for k = W-1..0 apply H_k to A[k:, k+1:] (whose rows < k+1 are already
// zero), then set column k to H_k e_k.
template <typename T>
__device__ __noinline__ void hh_form_q_inplace(T* A, int lda, int N, int W, Smem<T>& sm) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const T* tau = sm.vec;
  T* wv = sm.vec + WMAX;
  T* wred = sm.stage;
  for (int k = W - 1; k >= 0; --k) {
    const T tk = tau[k];
    T* colk = A + (int64_t)k * lda;
    const int nj = W - 1 - k;
    if (nj > 0 && tk != T(0)) {
      // w_j = A[k, j] + sum_{i>k} v_i A[i, j]   (A[k, j] is zero here)
      for (int j0 = 0; j0 < nj; j0 += 8) {
        T p[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) p[u] = T(0);
        for (int i = k + 1 + tid; i < N; i += NT) {
          const T vi = colk[i];
#pragma unroll
          for (int u = 0; u < 8; ++u)
            if (j0 + u < nj) p[u] = fma(vi, A[i + (int64_t)(k + 1 + j0 + u) * lda], p[u]);
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) p[u] = warp_sum(p[u]);
        if (lane == 0) {
#pragma unroll
          for (int u = 0; u < 8; ++u)
            if (j0 + u < nj) wred[warp * WMAX + j0 + u] = p[u];
        }
      }
      __syncthreads();
      if (tid < nj) {
        T acc = T(0);
#pragma unroll
        for (int w = 0; w < NW; ++w) acc += wred[w * WMAX + tid];
        wv[tid] = tk * acc;
      }
      __syncthreads();
      for (int i = k + tid; i < N; i += NT) {
        const T vi = (i == k) ? T(1) : colk[i];
        T* row = A + i + (int64_t)(k + 1) * lda;
        for (int j = 0; j < nj; ++j) row[(int64_t)j * lda] -= vi * wv[j];
      }
      __syncthreads();
    }
    // column k = H_k e_k = e_k - tau v
    for (int i = tid; i < N; i += NT) {
      T x;
      if (i < k) x = T(0);
      else if (i == k) x = T(1) - tk;
      else x = -(tk * colk[i]);
      colk[i] = x;
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// Cholesky-based QR pieces for the fast forms (FP32 and double-float).
// ---------------------------------------------------------------------------


// G = X^T X (W x W, W <= 64) accumulated in double-float; X is N x W
// (column-major, ld ldx, type T), G column-major with ld ldg.  Only the 4x4
// micro-tiles on and above the diagonal are accumulated (the lower ones are
// their transposes), with a renormalisation after every staged row chunk.
template <typename T>
__device__ __noinline__ void gram_df(int N, int W, const T* X, int ldx, dfloat* G, int ldg, T* stage) {
  const int tid = threadIdx.x;
  const int w4 = (W + 3) >> 2;
  const int MT = w4 * (w4 + 1) / 2;       // <= 136 <= NT
  const int splits = NT / MT;
  const int lds = w4 * 4 + 4;
  T* xs = stage;
  const int mt = tid % MT, split = tid / MT;
  const bool active = split < splits;
  // micro-tile mt -> (ma, mc) with ma <= mc, row-major over the upper triangle
  int ma = 0, rem = mt;
  while (rem >= w4 - ma) {
    rem -= w4 - ma;
    ++ma;
  }
  const int mc = ma + rem;
  dfloat acc[16];
#pragma unroll
  for (int e = 0; e < 16; ++e) acc[e] = dfloat(0.0f, 0.0f);
  for (int i0 = 0; i0 < N; i0 += TRG) {
    const int rows = min(TRG, N - i0);
    RowLoadPanel<T>{X, ldx, W}(xs, i0, rows, lds);
    __syncthreads();
    if (active) {
      for (int ii = split; ii < rows; ii += splits) {
        T xa[4], xb[4];
        ld4(xs + ii * lds + 4 * ma, xa);
        ld4(xs + ii * lds + 4 * mc, xb);
#pragma unroll
        for (int p = 0; p < 4; ++p)
#pragma unroll
          for (int q = 0; q < 4; ++q) acc[p * 4 + q] = acc_mul_acc(acc[p * 4 + q], xa[p], xb[q]);
      }
#pragma unroll
      for (int e = 0; e < 16; ++e) acc[e] = renorm(acc[e]);
    }
    __syncthreads();
  }
  dfloat* part = reinterpret_cast<dfloat*>(stage);  // splits * MT * 16 <= 4096 values
  if (active) {
#pragma unroll
    for (int e = 0; e < 16; ++e) part[(split * MT + mt) * 16 + e] = acc[e];
  }
  __syncthreads();
  for (int o = tid; o < MT * 16; o += NT) {
    const int m2 = o >> 4, e = o & 15;
    dfloat sum = part[m2 * 16 + e];
    for (int sp = 1; sp < splits; ++sp) sum += part[(sp * MT + m2) * 16 + e];
    int a2 = 0, r2 = m2;
    while (r2 >= w4 - a2) {
      r2 -= w4 - a2;
      ++a2;
    }
    const int c2 = a2 + r2;
    const int ia = 4 * a2 + (e >> 2), jc = 4 * c2 + (e & 3);
    if (ia < W && jc < W) {
      G[ia + (int64_t)jc * ldg] = sum;
      if (a2 != c2) G[jc + (int64_t)ia * ldg] = sum;
    }
  }
  __syncthreads();
}

// In-place upper Cholesky G = R^T R of a W x W double-float matrix (ld ldg),
// optionally shifted first: G + shift * trace(G) * I.  Returns false on a
// non-positive pivot (G is then unusable).  The factorisation runs in the
// shared buffer gs (W*W values) with two block barriers per column: every
// thread forms the pivot itself (no broadcast), then the trailing update is
// spread over the block.  The lower triangle of G keeps its input values.
static __device__ __noinline__ bool chol_df(int W, dfloat* G, int ldg, double shift_rel, dfloat* gs) {
  const int tid = threadIdx.x;
  __shared__ int bad_s;
  for (int e = tid; e < W * W; e += NT) gs[e] = G[(e % W) + (int64_t)(e / W) * ldg];
  if (tid == 0) bad_s = 0;
  __syncthreads();
  if (shift_rel > 0.0) {
    dfloat tr(0.0f, 0.0f);
    for (int j = 0; j < W; ++j) tr += gs[j + j * W];
    const dfloat sh = tr * dfloat(shift_rel);
    __syncthreads();
    for (int j = tid; j < W; j += NT) gs[j + j * W] += sh;
    __syncthreads();
  }
  for (int k = 0; k < W; ++k) {
    dfloat d = gs[k + k * W];
    const bool bad = !(d.hi > 0.0f);
    if (bad) d = dfloat(1.0f, 0.0f);
    const dfloat rkk = sqrt(d);
    const dfloat inv = dfloat(1.0f, 0.0f) / rkk;
    for (int j = k + 1 + tid; j < W; j += NT) gs[k + j * W] = gs[k + j * W] * inv;
    __syncthreads();
    if (tid == 0) {
      gs[k + k * W] = rkk;
      if (bad) bad_s = 1;
    }
    const int cnt = W - k - 1;
    for (int e = tid; e < cnt * cnt; e += NT) {
      const int i = k + 1 + e % cnt, j = k + 1 + e / cnt;
      if (i <= j) gs[i + j * W] = fma(-gs[k + i * W], gs[k + j * W], gs[i + j * W]);
    }
    __syncthreads();
  }
  for (int e = tid; e < W * W; e += NT) {
    const int i = e % W, j = e / W;
    if (i <= j) G[i + (int64_t)j * ldg] = gs[e];
  }
  const bool ok = (bad_s == 0);
  __syncthreads();
  return ok;
}

// K <- K R^{-1} row by row (forward substitution, backward stable), R upper
// triangular W x W double-float (ld ldr); K is N x W (T, ld N).  Row tiles are
// staged in shared memory with one row per thread; the columns are solved in
// blocks of four, so each staged x_i feeds four accumulators and R is read
// as row segments of four (R kept row-major in shared memory).
template <typename T>
__device__ __noinline__ void trsm_rows(int N, int W, T* K, const dfloat* R, int ldr, T* stage, T* invd) {
  const int tid = threadIdx.x;
  const int Wp = (W + 3) & ~3;
  T* Rt = stage;  // Wp x Wp row-major: Rt[i * Wp + j] = R_ij for i <= j < W, else 0
  for (int e = tid; e < Wp * Wp; e += NT) {
    const int i = e / Wp, j = e - (e / Wp) * Wp;
    T v;
    from_df((i <= j && j < W) ? R[i + (int64_t)j * ldr] : dfloat(0.0f, 0.0f), v);
    Rt[e] = v;
  }
  for (int j = tid; j < Wp; j += NT) {
    T v;
    from_df(j < W ? dfloat(1.0f, 0.0f) / R[j + (int64_t)j * ldr] : dfloat(0.0f, 0.0f), v);
    invd[j] = v;
  }
  int TR = (Stage<T>::ELEMS - Wp * Wp) / Wp;
  if (TR > NT) TR = NT;
  TR &= ~31;
  T* ks = stage + Wp * Wp;  // [Wp][TR]; the padding columns hold zeros
  __syncthreads();
  for (int i0 = 0; i0 < N; i0 += TR) {
    const int rows = min(TR, N - i0);
    for (int ii = tid; ii < rows; ii += NT) {
      const T* src = K + i0 + ii;
      for (int kb = 0; kb < Wp; kb += 8) {
        T v[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) v[u] = (kb + u < W) ? src[(int64_t)(kb + u) * N] : T(0);
#pragma unroll
        for (int u = 0; u < 8; ++u)
          if (kb + u < Wp) ks[(kb + u) * TR + ii] = v[u];
      }
    }
    __syncthreads();
    if (tid < rows) {
      for (int jb = 0; jb < Wp; jb += 4) {
        // x_j = (k_j - sum_{i<j} x_i R_ij) / R_jj for j = jb .. jb+3
        T acc[4] = {T(0), T(0), T(0), T(0)};
        for (int i = 0; i < jb; ++i) {
          const T x = ks[i * TR + tid];
          T rr[4];
          ld4(Rt + i * Wp + jb, rr);
#pragma unroll
          for (int u = 0; u < 4; ++u) acc[u] = fma_acc(x, rr[u], acc[u]);
        }
        T xb[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          T sum = renorm(acc[u]);
#pragma unroll
          for (int v = 0; v < u; ++v) sum = fma_acc(xb[v], Rt[(jb + v) * Wp + jb + u], sum);
          xb[u] = (ks[(jb + u) * TR + tid] - renorm(sum)) * invd[jb + u];
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) ks[(jb + u) * TR + tid] = xb[u];
      }
    }
    __syncthreads();
    for (int ii = tid; ii < rows; ii += NT) {
      T* dst = K + i0 + ii;
      for (int j = 0; j < W; ++j) dst[(int64_t)j * N] = ks[j * TR + ii];
    }
    __syncthreads();
  }
}

// C = A B for upper triangular W x W double-float matrices (ld W each).
static __device__ __noinline__ void tri_mul_df(int W, const dfloat* A, const dfloat* B, dfloat* C) {
  for (int e = threadIdx.x; e < W * W; e += NT) {
    const int i = e % W, j = e / W;
    dfloat acc(0.0f, 0.0f);
    for (int k = i; k <= j; ++k) acc = fma(A[i + k * W], B[k + j * W], acc);
    C[e] = (i <= j) ? acc : dfloat(0.0f, 0.0f);
  }
  __syncthreads();
}

// Copies the upper triangle of the factored panel (R, W x W) to R (ld ldr).
template <typename T>
__device__ void extract_r(const T* A, int lda, int W, T* R, int ldr) {
  for (int o = threadIdx.x; o < W * W; o += NT) {
    const int i = o % W, j = o / W;
    R[i + (int64_t)j * ldr] = (i <= j) ? A[i + (int64_t)j * lda] : T(0);
  }
  __syncthreads();
}

// ---------------------------------------------------------------------------
// One-sided Jacobi SVD of the P x P matrix B (column-major, ld ldb) held in
// shared memory `a` (P x P, ld P) with right vectors in `v` (P x P).
// On exit: sigma[j] (descending), a's columns = left singular vectors,
// v's columns = right singular vectors, both permuted to the sorted order
// through perm[].  Returns false if it did not converge.
// ---------------------------------------------------------------------------
// NTH: threads of the calling block (a multiple of 32); the instance engine
// calls it with its NT threads, the single-CTA kernels of the large-stream
// engine with 1024.
// max_sweeps < 40 runs that many sweeps at most (a polishing pass after a
// lower-precision solve).  skip_noise = false also rotates a noise-level
// column against a larger one (the FP32 preconditioning sweeps of the mixed
// SVD, which stop after a few sweeps anyway and leave the larger columns'
// orthogonality to the polish).
// A sweep whose largest rotation measure |a_p^T a_q| / (|a_p| |a_q|) is
// delta leaves the columns orthogonal to O(P delta^2) (each later rotation of
// the sweep re-creates products of size delta times another delta), so the
// iteration also ends after a sweep with delta <= conv_delta (default
// sqrt(eps): P delta^2 is then the rotation threshold itself) instead of
// spending one more sweep to find nothing to rotate.
// tiny_abs (the caller's truncation level, an absolute squared norm): a pair
// whose columns are BOTH below it is left alone -- together they hold less
// than the truncation drops, and the SVD of the rest is unaffected.  (A rule
// that skipped pairs with EITHER column below it would let a column that
// shrank below the level keep content the exact SVD rotates into the kept
// columns: the truncated result could then differ from the truncated exact
// SVD by up to tol / 2.)
template <typename T, int NTH = NT>
__device__ __noinline__ bool jacobi_svd(int P, T* a, T* v, T* sigma, int* perm, int* flag, int max_sweeps = 40,
                                        bool skip_noise = true, double conv_delta = -1.0, double tiny_abs = 0.0) {
  constexpr int NWJ = NTH / 32;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  // rotation threshold: P ulps (the rounding level of a length-P dot
  // product), so a sweep whose remaining products are rounding noise ends
  const T eps = T(Prec<T>::eps * P);
  for (int o = tid; o < P * P; o += NTH) v[o] = ((o % P) == (o / P)) ? T(1) : T(0);
  // Pairs with a column below eps * ||B||_F are left alone: such a column is
  // rounding noise, and rotating it against several such columns that are
  // not orthogonal among themselves converges only linearly (projection one
  // column at a time).  Their left vectors a_j / sigma_j are therefore not
  // orthogonal to the rest; complete_left below repairs the kept ones.
  __shared__ __align__(16) unsigned char red_raw[NWJ * sizeof(T)];
  T* red = reinterpret_cast<T*>(red_raw);
  T fro2 = T(0);
  for (int o = tid; o < P * P; o += NTH) fro2 = fma(a[o], a[o], fro2);
  fro2 = warp_sum(fro2);
  if (lane == 0) red[warp] = fro2;
  __syncthreads();
  fro2 = T(0);
  for (int wv = 0; wv < NWJ; ++wv) fro2 += red[wv];
  __syncthreads();
  const T tiny = T(Prec<T>::eps) * T(Prec<T>::eps) * fro2;
  const T reach = T(tiny_abs);  // truncation level: a pair is left alone only when both columns are below it
  const int Pe = P + (P & 1);  // even number of players (a dummy when P is odd)
  // lanes per pair G (32, 16, 8 or 4): enough pairs per pass for every warp,
  // so the per-pair reductions and rotation arithmetic are shared by a warp's
  // groups instead of repeated per pair
  const int npair = Pe / 2;
  int G = 32;
  while (G > 4 && NWJ * (32 / G) < npair) G >>= 1;
  const int gpw = 32 / G, gid = lane / G, gl = lane % G;
  const float delta_stop = (float)((conv_delta >= 0.0) ? conv_delta : sqrt(Prec<T>::eps));
  __shared__ unsigned int dmax_bits;  // largest rotation measure of the sweep (non-negative float bits)
  bool converged = false;
  for (int sweep = 0; sweep < max_sweeps && !converged; ++sweep) {
    if (tid == 0) {
      *flag = 0;
      dmax_bits = 0u;
    }
    __syncthreads();
    for (int rnd = 0; rnd < Pe - 1; ++rnd) {
      // warp-uniform loop; each group of G lanes takes one pair
      for (int base = warp * gpw; base < npair; base += NWJ * gpw) {
        const int pr = base + gid;
        int p = 0, q = 0;
        bool valid = pr < npair;
        if (valid) {
          if (pr == 0) { p = rnd % (Pe - 1); q = Pe - 1; }
          else { p = (rnd + pr) % (Pe - 1); q = (rnd - pr + (Pe - 1)) % (Pe - 1); }
          valid = p < P && q < P;
          if (p > q) { int tmp = p; p = q; q = tmp; }
        }
        if (!valid) p = q = 0;
        T* ap = a + p * P;
        T* aq = a + q * P;
        T al = T(0), be = T(0), ga = T(0);
        if (valid)
          for (int i = gl; i < P; i += G) {
            const T x = ap[i], y = aq[i];
            al = fma(x, x, al); be = fma(y, y, be); ga = fma(x, y, ga);
          }
        for (int o = G >> 1; o > 0; o >>= 1) {  // group sums (all lanes take part)
          al += shfl_xor(al, o);
          be += shfl_xor(be, o);
          ga += shfl_xor(ga, o);
        }
        // (sqrt(al) * sqrt(be): al * be can leave the FP32 exponent range)
        const bool live = valid && (skip_noise ? (al > tiny && be > tiny && (al > reach || be > reach))
                                               : (al > tiny || be > tiny));
        if (live && fabs(ga) > eps * sqrt(al) * sqrt(be) && ga != T(0)) {
          const T zeta = (be - al) / (T(2) * ga);
          // for large |zeta| use tan = 1/(2 zeta): zeta^2 would leave the FP32
          // exponent range of float and double-float values
          const T tt = (fabs(zeta) > T(1.0e15)) ? T(0.5) / zeta
                                                 : copysign(T(1), zeta) / (fabs(zeta) + sqrt(T(1) + zeta * zeta));
          const T cs = T(1) / sqrt(T(1) + tt * tt);
          const T sn = cs * tt;
          for (int i = gl; i < P; i += G) {
            const T x = ap[i], y = aq[i];
            ap[i] = cs * x - sn * y;
            aq[i] = sn * x + cs * y;
          }
          T* vp = v + p * P;
          T* vq = v + q * P;
          for (int i = gl; i < P; i += G) {
            const T x = vp[i], y = vq[i];
            vp[i] = cs * x - sn * y;
            vq[i] = sn * x + cs * y;
          }
          if (gl == 0) {
            *flag = 1;
            const float dl = (float)(double)fabs(ga) / ((float)(double)sqrt(al) * (float)(double)sqrt(be));
            atomicMax(&dmax_bits, __float_as_uint(dl));
          }
        }
      }
      __syncthreads();
    }
    converged = (*flag == 0) || (__uint_as_float(dmax_bits) <= delta_stop);
    __syncthreads();
  }
  // singular values = column norms
  for (int j = warp; j < P; j += NWJ) {
    T s = T(0);
    for (int i = lane; i < P; i += 32) s = fma(a[j * P + i], a[j * P + i], s);
    s = warp_sum(s);
    if (lane == 0) sigma[j] = sqrt(s);
  }
  __syncthreads();
  if (tid == 0) {  // selection sort of indices by descending sigma (P <= 128)
    for (int j = 0; j < P; ++j) perm[j] = j;
    for (int j = 0; j < P; ++j) {
      int best = j;
      for (int k = j + 1; k < P; ++k)
        if (sigma[perm[k]] > sigma[perm[best]]) best = k;
      const int tmp = perm[j]; perm[j] = perm[best]; perm[best] = tmp;
    }
  }
  __syncthreads();
  return converged;
}

// Left singular vectors of jacobi_svd's output, in place: the kept columns
// a[:, perm[j]], j < r1 (descending sigma), become a_j / sigma_j.  Those
// whose sigma_j is at the rounding level of the matrix (sigma_j^2 <= 16 eps^2
// ||A||_F^2, where the sweeps leave pairs alone) are not orthogonal to the
// others; the minimum rank can keep them.  Each is re-orthogonalised against
// the kept columns before it (classical Gram-Schmidt, two passes) and
// normalised; when that leaves less than 1 / (2P) of its squared norm (or it
// is zero) a unit vector e_k takes its place (of the P unit vectors, the
// squared residuals sum to P - j >= 1, so one of them passes).  Any unit
// direction orthogonal to the others serves: sigma_j is below rounding.
// scr: P + r1 values of scratch (global or shared).
// tiny_abs: the absolute squared noise level given to jacobi_svd (columns
// below 4 tiny_abs are treated the same way).
template <typename T, int NTH = NT>
__device__ __noinline__ void complete_left(int P, int r1, T* a, const T* sigma, const int* perm, T* scr,
                                           double tiny_abs = 0.0) {
  constexpr int NWJ = NTH / 32;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  __shared__ int j0s;
  __shared__ double nrm_s;
  for (int o = tid; o < P * r1; o += NTH) {
    const int i = o % P, j = o / P;
    const int pj = perm[j];
    const T sg = sigma[pj];
    a[i + pj * P] = (sg > T(0)) ? a[i + pj * P] / sg : T(0);
  }
  if (tid == 0) {
    double fro2 = 0.0;
    for (int j = 0; j < P; ++j) {
      const double sv = (double)sigma[j];
      fro2 += sv * sv;
    }
    const double thr2 = fmax(16.0 * Prec<T>::eps * Prec<T>::eps * fro2, 4.0 * tiny_abs);
    int j0 = r1;
    while (j0 > 0) {
      const double sv = (double)sigma[perm[j0 - 1]];
      if (sv * sv > thr2) break;
      --j0;
    }
    j0s = j0;
  }
  __syncthreads();
  T* cand = scr;
  T* coef = scr + P;
  int next_unit = 0;
  for (int jj = j0s; jj < r1; ++jj) {
    T* col = a + perm[jj] * P;
    bool use_unit = false;
    for (int attempt = 0; attempt <= P; ++attempt) {
      for (int i = tid; i < P; i += NTH) cand[i] = use_unit ? T((i == next_unit) ? 1.0 : 0.0) : col[i];
      __syncthreads();
      double n0 = 0.0;
      if (tid == 0)
        for (int i = 0; i < P; ++i) n0 += (double)cand[i] * (double)cand[i];
      for (int pass = 0; pass < 2; ++pass) {
        for (int c = warp; c < jj; c += NWJ) {
          const T* pc = a + perm[c] * P;
          T d = T(0);
          for (int i = lane; i < P; i += 32) d = fma(pc[i], cand[i], d);
          d = warp_sum(d);
          if (lane == 0) coef[c] = d;
        }
        __syncthreads();
        for (int i = tid; i < P; i += NTH) {
          T x = cand[i];
          for (int c = 0; c < jj; ++c) x = fma(-coef[c], a[i + perm[c] * P], x);
          cand[i] = x;
        }
        __syncthreads();
      }
      if (tid == 0) {
        T q = T(0);
        for (int i = 0; i < P; ++i) q = fma(cand[i], cand[i], q);
        nrm_s = (n0 > 0.0 && (double)q > n0 / (2.0 * P)) ? (double)q : 0.0;
      }
      __syncthreads();
      if (nrm_s > 0.0) break;
      if (use_unit) next_unit = (next_unit + 1) % P;
      use_unit = true;
      __syncthreads();
    }
    if (nrm_s > 0.0) {
      T q = T(0);
      for (int i = 0; i < P; ++i) q = fma(cand[i], cand[i], q);  // every thread: the same sum
      const T inv = T(1) / sqrt(q);
      for (int i = tid; i < P; i += NTH) col[i] = cand[i] * inv;
    } else {
      for (int i = tid; i < P; i += NTH) col[i] = T(0);
    }
    if (use_unit) next_unit = (next_unit + 1) % P;
    __syncthreads();
  }
}

}  // namespace lri
