// tc_pass.h - snapshot passes of the data substeps on the tensor cores
// (tcgen05 + TMA, sm_103a): out = dY X or dY^T X with dY = A1 - A0 formed in
// registers and stored into tensor memory as the A operand, FP32 data split
// into TF32 hi + lo parts (3xTF32 products, FP32 accumulation in tensor
// memory).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace lri {

// Per-stream state of the tensor-core passes: the split copies of the right
// factor, the split-K partial sums and the tensor maps of the split copies
// (CUtensorMap storage, kept opaque here).
struct TcPass {
  int64_t n = 0, m = 0;
  int R = 0, NB = 0, sms = 0;
  float* xh = nullptr;    // max(n, m) x NB: TF32 hi part of the right factor
  float* xl = nullptr;    // max(n, m) x NB: TF32 lo part
  float* part = nullptr;  // split-K partials
  size_t part_elems = 0;
  int ov_splits[2] = {0, 0};  // split-K factor override per mode (0 = automatic)
  int ov_stages = 0;          // pipeline stage override (0 = as many as fit)
  alignas(64) unsigned char tm_xh_m[128];
  alignas(64) unsigned char tm_xl_m[128];
  alignas(64) unsigned char tm_xh_n[128];
  alignas(64) unsigned char tm_xl_n[128];
};

// Shapes the tensor-core passes take: FP32 n x m snapshots with n, m
// multiples of 4 (16-byte TMA strides) and at least 128, panel width R <= 96.
bool tc_pass_supported(int64_t n, int64_t m, int R);

// Allocates the split buffers and partials and encodes their tensor maps.
cudaError_t tc_pass_init(TcPass* t, int64_t n, int64_t m, int R);
void tc_pass_free(TcPass* t);

// Tile overrides of the autotuner: K splits per 128-row output tile for
// dY X (splits_rows) and dY^T X (splits_cols), pipeline stages (2 up to what
// fits); 0 restores the automatic choice.  Grows the partial buffer when
// needed.
cudaError_t tc_pass_set_tiles(TcPass* t, int splits_rows, int splits_cols, int stages);

// out (P x R, ld ldo) = dY X (trans = 0: P = n, X is m x R with ld ldx) or
// dY^T X (trans = 1: P = m, X is n x R), dY = A1 - A0 (A0 may be null: dY = A1) (n x m, column-major,
// 16-byte aligned).  Active columns: ncols when >= 0, else the device rank
// (capped at R); the others are written as zeros.  kd (optional, P x R,
// ld P) receives a copy of out.  A bounded wait that gives up ORs
// status_timeout into *status.
cudaError_t tc_pass_run(TcPass* t, int trans, const float* A1, const float* A0, const float* X, int64_t ldx,
                        const int32_t* rank, int ncols, float* out, int64_t ldo, float* kd, uint32_t* status,
                        uint32_t status_timeout, cudaStream_t st);

// 2-D FP32 tensor map (CUtensorMap storage) of a column-major rows x cols
// matrix with ld = rows (a multiple of 4), box box0 x box1, optionally with
// the 128-byte swizzle; false when the driver's encoder is missing or
// rejects the shape.
bool tc_encode_2d(void* out, const void* ptr, uint64_t rows, uint64_t cols, uint32_t box0, uint32_t box1,
                  bool swizzle);
bool tc_encoder_available();

}  // namespace lri
