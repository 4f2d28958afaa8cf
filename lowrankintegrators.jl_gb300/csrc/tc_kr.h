// tc_kr.h - the Khatri-Rao products of the large Burgers engine's flows on the
// tensor cores (tcgen05 + TMA, sm_103a), for active widths above the fused
// stages' 32: part[z] (=, or +=) scale * KR(Y, Y) T' over split z of the
// packed pairs, with KR(Y, Y)_{i, p(a,b)} = Y_ia Y_ib (a <= b) formed per row
// in registers and T' the packed flow tensor (FP32 data split into TF32 hi +
// lo parts: 3xTF32 products, FP32 accumulation drained from tensor memory).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace lri {

// State of the tensor-core Khatri-Rao products of one engine: TF32 hi and
// lo copies of the three flow tensors (T'_V, T'_L, T'_Vhat) with a pair
// stride padded to a multiple of 4 (16-byte TMA strides), zero outside the
// active pairs and columns, and their tensor maps (CUtensorMap storage).
struct TcKr {
  int R = 0;    // r_max: tensors of at most 2R columns
  int PP = 0;   // pair stride of the engine's tensors, 2R (2R + 1) / 2
  int PPp = 0;  // pair stride of the split copies
  float* th[3] = {nullptr, nullptr, nullptr};
  float* tl[3] = {nullptr, nullptr, nullptr};
  alignas(64) unsigned char tm_h[3][128];
  alignas(64) unsigned char tm_l[3][128];
};

// The tensor-core products need the tensor-map encoder of the driver.
bool tc_kr_supported(int R);
cudaError_t tc_kr_init(TcKr* t, int R);
void tc_kr_free(TcKr* t);

// TF32 split of tensor k (0: T'_V, 1: T'_L, 2: T'_Vhat) from Tp (PP x 2R,
// ld PP, packed over the ka active columns: ka = 2r for aug, r otherwise).
cudaError_t tc_kr_split(TcKr* t, int k, const float* Tp, const int32_t* rank, int aug, cudaStream_t st);

// Split counts of the products: kz splits of the pair chunks per 128-row
// tile and 64-column half, about one CTA per SM.
int tc_kr_splits(int N, int R, int aug, int sms, int zmax);

// part[z * N * 2R + i + col(c) * N] (=, or += with accum) scale * (KR(Y, Y) T'_k)[i, c]
// summed over split z of the pair chunks (z < kz), i < N, c < ka, col(c) the
// panel column of active index c (the first r of each half for aug).  Y: the
// N x R (aug = 0) or N x 2R (aug = 1) panel, ld N.  A bounded wait that
// gives up ORs status_timeout into *status.
cudaError_t tc_kr_apply(TcKr* t, int k, int N, int aug, const int32_t* rank, const float* Y, float* part, int kz,
                        double scale, int accum, uint32_t* status, uint32_t status_timeout, cudaStream_t st);

}  // namespace lri
