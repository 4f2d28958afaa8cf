// tc_pass.cu - the snapshot passes of the data substeps on the 5th-generation
// tensor cores.
//
// The data substeps (src/integrators/data_integrator.jl:13-16, driven by
// dY = A(t+dt) - A(t), src/integrators/unconventional.jl:121-127) need the
// products dY V0 (K step), dY^T U0 (L step) and dY Vhat (S step) of an n x m
// snapshot increment with a tall panel of at most 96 columns.  They read
// the two n x m FP32 snapshots once each and are bound by HBM; on the CUDA
// cores they were bound by FP32 FMA issue instead.
//
// One CTA owns a 128-row tile of the output and a range of K (the
// contraction index) in chunks of 32:
//   warp 4   TMA producer: per chunk, the A(t+dt) and A(t) tiles (128 x 32)
//            and the chunk's 32 rows of the split right factor (hi and lo);
//   warps 0-3 form row i of dY = A(t+dt) - A(t) (exact in FP32 for nearby
//            snapshots) in thread i's registers, split it into TF32 hi + lo
//            parts and store both into tensor memory (tcgen05.st): the A
//            operand never goes back through shared memory, whose bandwidth
//            (TMA writes, operand reads) bounds the pass otherwise;
//   warp 5   allocates tensor memory and issues, per 8-wide K slice,
//            tcgen05.mma (kind::tf32, A from tensor memory, B from shared
//            memory, M = 128, N = active columns rounded up to 16): hi*hi
//            into one FP32 accumulator, hi*lo + lo*hi into a second
//            (correction) one;
//   warps 0-3 also drain the accumulators: the tensor cores' FP32
//            accumulation truncates, so its error grows with the number of
//            MMAs summed into one accumulator (1.4e-5 relative over 2048
//            terms of K).  Every TC_DRAIN chunks (128 terms) the MMAs switch
//            to the other of two accumulator buffers while the four warps
//            add the finished block into FP32 registers (tcgen05.ld, round
//            to nearest) and hand the buffer back;
//   warps 0-3 finally write the CTA's split-K partial; a second kernel sums
//            the partials in a fixed order (deterministic) and writes the
//            panel.
// Rows of dY^T X: the snapshot tile arrives through TMA K-major with the
// 128-byte swizzle (K = rows of the snapshot are contiguous); rows of dY X:
// it arrives row-contiguous and each thread gathers its row down the tile's
// columns.  Two A slots in tensor memory let the split of chunk k + 1 overlap
// the MMAs of chunk k.  3xTF32 drops only the lo*lo term: products accurate
// to about 2^-21 relative, summed in FP32.
//
// Every mbarrier wait is bounded (about two seconds of SM clock); a wait
// that gives up sets a status bit, the CTA stops issuing work, waits (again
// bounded) for its copies and MMAs in flight, frees its tensor memory and
// returns.
#include <cuda.h>  // CUtensorMap and its enums (the encoder comes from the runtime's entry-point query)
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstdint>
#include <cstring>

#include "engine_api.h"
#include "tc_common.cuh"
#include "tc_pass.h"

namespace lri {
namespace {

constexpr int TC_BM = 128;                        // output rows per CTA (UMMA M)
constexpr int TC_BK = 32;                         // K per pipeline stage: one 128-byte swizzle row of FP32
constexpr int TC_THREADS = 192;                   // warps 0-3 transform/epilogue, 4 TMA, 5 MMA
constexpr uint32_t TC_TILE_BYTES = TC_BM * TC_BK * 4;  // 16 KB snapshot tile
constexpr int TC_MAX_STAGES = 4;
constexpr int TC_MAX_NB = 96;                     // panel columns (N <= 96)
constexpr int TC_DRAIN = 4;                       // chunks accumulated in tensor memory between drains
constexpr int TC_DRAIN_LAG = 2;                   // chunks of the next block queued before a drain
constexpr int TC_SMEM_LIMIT = 232448;             // 227 KB opt-in per CTA
constexpr int TC_CTRL_BYTES = 1024;               // barriers, tensor-memory address, abort flag
constexpr long long TC_WAIT_CYCLES = 4000000000LL;  // about 2 s at 2 GHz
constexpr int TC_A_SLOTS = 2;                     // A operand slots in tensor memory (hi: 32, lo: 32 columns each)

struct TcArgs {
  int P, R, NB, nchunks, chunks_per_split, stages, rows_mode, ncols;
  int has_a0;  // 0: the product of the snapshot A1 itself (no A0 tile is loaded)
  const int32_t* rank;
  float* part;
  uint32_t* status;
  uint32_t status_timeout;
};

// bounded wait of this kernel's roles (status bit from the launch)
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, volatile int* abort_flag,
                                          const TcArgs& a, long long limit = TC_WAIT_CYCLES) {
  return mbar_wait_st(bar, parity, abort_flag, a.status, a.status_timeout, limit);
}

__device__ __forceinline__ int active_cols(const TcArgs& a) {
  const int k = (a.ncols >= 0) ? a.ncols : *a.rank;
  return max(0, min(a.R, k));
}

__global__ void __launch_bounds__(TC_THREADS, 1)
    tc_pass_kernel(const __grid_constant__ CUtensorMap tmA1, const __grid_constant__ CUtensorMap tmA0,
                   const __grid_constant__ CUtensorMap tmXh, const __grid_constant__ CUtensorMap tmXl,
                   const TcArgs a) {
  extern __shared__ unsigned char smem_raw[];
  unsigned char* base = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                                         ~static_cast<uintptr_t>(1023));
  const int NS = a.stages;
  const uint32_t xbytes = TC_BK * 4 * a.NB;  // one split-factor tile: NB rows of 128 bytes
  const uint32_t stage_bytes = 2 * TC_TILE_BYTES + 2 * xbytes;
  unsigned char* ctrl = base + NS * stage_bytes;
  const uint32_t bar0 = smem_u32(ctrl);
  auto full = [&](int s) { return bar0 + 8u * s; };                          // TMA bytes landed
  auto tfull = [&](int s) { return bar0 + 8u * (TC_MAX_STAGES + s); };       // operands formed
  auto empty = [&](int s) { return bar0 + 8u * (2 * TC_MAX_STAGES + s); };   // MMAs done with the stage
  auto acc_full = [&](int b) { return bar0 + 8u * (3 * TC_MAX_STAGES + b); };       // a block's MMAs done
  auto acc_empty = [&](int b) { return bar0 + 8u * (3 * TC_MAX_STAGES + 2 + b); };  // a block drained
  const uint32_t done = bar0 + 8u * (3 * TC_MAX_STAGES + 4);                 // every MMA done
  auto aempty = [&](int t) { return bar0 + 8u * (3 * TC_MAX_STAGES + 5 + t); };  // MMAs done with A slot t
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(ctrl + 256);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(ctrl + 260);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int mt = blockIdx.x, sp = blockIdx.y;
  const int kc0 = sp * a.chunks_per_split;
  const int nk = min(a.nchunks, kc0 + a.chunks_per_split) - kc0;
  const int nblocks = (nk + TC_DRAIN - 1) / TC_DRAIN;
  const int ka = active_cols(a);
  const int N = min(a.NB, max(16, (ka + 15) & ~15));
  // accumulator buffer b: hi*hi sums in columns [2 b NB, 2 b NB + N), the
  // hi*lo + lo*hi corrections NB columns further; the A operand of chunk it
  // (dY hi, then lo, 32 columns each) in slot it % 2 from column 4 NB
  const uint32_t a_col = 4u * (uint32_t)a.NB;
  const uint32_t ncols_tmem = (a_col + 64 * TC_A_SLOTS > 256) ? 512u : 256u;

  if (threadIdx.x == 0) {
    for (int s = 0; s < NS; ++s) {
      mbar_init(full(s), 1);
      mbar_init(tfull(s), 128);
      mbar_init(empty(s), 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(acc_full(b), 1);
      mbar_init(acc_empty(b), 128);
    }
    for (int t = 0; t < TC_A_SLOTS; ++t) mbar_init(aempty(t), 1);
    mbar_init(done, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 5) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(ncols_tmem)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 4) {
    // ---------------- TMA producer ----------------
    if (lane == 0) {
      int last_par[TC_MAX_STAGES];
      for (int s = 0; s < TC_MAX_STAGES; ++s) last_par[s] = -1;
      bool ok = true;
      for (int it = 0; it < nk && ok; ++it) {
        const int s = it % NS;
        const uint32_t par = (uint32_t)(it / NS) & 1u;
        if (!(ok = mbar_wait(empty(s), par ^ 1u, abort_flag, a))) break;
        const int kc = kc0 + it;
        const uint32_t st = smem_u32(base + (size_t)s * stage_bytes);
        mbar_expect_tx(full(s), a.has_a0 ? stage_bytes : stage_bytes - TC_TILE_BYTES);
        if (a.rows_mode) {
          tma_load_2d(st, &tmA1, mt * TC_BM, kc * TC_BK, full(s));
          if (a.has_a0) tma_load_2d(st + TC_TILE_BYTES, &tmA0, mt * TC_BM, kc * TC_BK, full(s));
        } else {
          tma_load_2d(st, &tmA1, kc * TC_BK, mt * TC_BM, full(s));
          if (a.has_a0) tma_load_2d(st + TC_TILE_BYTES, &tmA0, kc * TC_BK, mt * TC_BM, full(s));
        }
        tma_load_2d(st + 2 * TC_TILE_BYTES, &tmXh, kc * TC_BK, 0, full(s));
        tma_load_2d(st + 2 * TC_TILE_BYTES + xbytes, &tmXl, kc * TC_BK, 0, full(s));
        last_par[s] = (int)par;
      }
      if (!ok || *abort_flag) {
        // let the copies in flight land before the CTA's shared memory goes away
        for (int s = 0; s < TC_MAX_STAGES; ++s)
          if (last_par[s] >= 0) mbar_wait(full(s), (uint32_t)last_par[s], abort_flag, a, TC_WAIT_CYCLES / 4);
      }
    }
  } else if (warp == 5) {
    // ---------------- MMA issuer ----------------
    if (lane == 0) {
      const uint32_t idesc = idesc_tf32(TC_BM, N);
      for (int it = 0; it < nk; ++it) {
        const int s = it % NS;
        const uint32_t par = (uint32_t)(it / NS) & 1u;
        const int bi = it / TC_DRAIN, b = bi & 1;
        const bool first = (it % TC_DRAIN) == 0;
        // the buffer's previous block (bi - 2) must have been drained
        if (first && bi >= 2 && !mbar_wait(acc_empty(b), (uint32_t)((bi >> 1) - 1) & 1u, abort_flag, a)) break;
        if (!mbar_wait(full(s), par, abort_flag, a) || !mbar_wait(tfull(s), par, abort_flag, a)) break;
        tc_fence_after();
        const uint32_t sxh = smem_u32(base + (size_t)s * stage_bytes) + 2 * TC_TILE_BYTES;
        const uint32_t sxl = sxh + xbytes;
        const uint32_t dmain = tmem + (uint32_t)(2 * b * a.NB), dcorr = dmain + (uint32_t)a.NB;
        const uint32_t tah = tmem + a_col + (uint32_t)(64 * (it % TC_A_SLOTS)), tal = tah + 32u;
#pragma unroll
        for (int kk = 0; kk < TC_BK / 8; ++kk) {
          const uint64_t bh = sw128_desc(sxh + 32u * kk), bl = sw128_desc(sxl + 32u * kk);
          const uint32_t acc = (!first || kk > 0) ? 1u : 0u;
          umma_tf32_ts(dmain, tah + 8u * kk, bh, idesc, acc);
          umma_tf32_ts(dcorr, tah + 8u * kk, bl, idesc, acc);
          umma_tf32_ts(dcorr, tal + 8u * kk, bh, idesc, 1u);
        }
        umma_commit(empty(s));
        umma_commit(aempty(it % TC_A_SLOTS));
        if ((it % TC_DRAIN) == TC_DRAIN - 1 || it == nk - 1) umma_commit(acc_full(b));
      }
      umma_commit(done);  // arrives once every MMA issued above has completed
      if (*abort_flag) mbar_wait(done, 0, abort_flag, a, TC_WAIT_CYCLES / 4);
    }
    __syncwarp();
  } else {
    // -------- form dY, split; drain the accumulators; epilogue (warps 0-3) --------
    const int tid = threadIdx.x;
    const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
    float acc[TC_MAX_NB];
#pragma unroll
    for (int c = 0; c < TC_MAX_NB; ++c) acc[c] = 0.0f;
    bool aborted = false;
    int drained = 0;
    // adds block k's hi*hi and correction sums (FP32, round to nearest) into
    // the registers and hands the buffer back to the MMA issuer
    auto drain = [&](int k) {
      const int b = k & 1;
      const bool ok = mbar_wait(acc_full(b), (uint32_t)(k >> 1) & 1u, abort_flag, a);
      if (bar_any(!ok)) return false;
      tc_fence_after();
      const uint32_t dmain = tmem + lane_base + (uint32_t)(2 * b * a.NB), dcorr = dmain + (uint32_t)a.NB;
#pragma unroll
      for (int c0 = 0; c0 < TC_MAX_NB; c0 += 16) {
        if (c0 < N) {
          float v[16], w[16];
          tmem_ld16(dmain + (uint32_t)c0, v);
          tmem_ld16(dcorr + (uint32_t)c0, w);
#pragma unroll
          for (int q = 0; q < 16; ++q) acc[c0 + q] += v[q] + w[q];
        }
      }
      tc_fence_before();
      mbar_arrive(acc_empty(b));
      return true;
    };
    for (int it = 0; it < nk; ++it) {
      const int s = it % NS;
      const uint32_t par = (uint32_t)(it / NS) & 1u;
      const bool ok = mbar_wait(full(s), par, abort_flag, a);
      if (bar_any(!ok)) {
        aborted = true;
        break;
      }
      const float* a1 = reinterpret_cast<const float*>(base + (size_t)s * stage_bytes);
      const float* a0 = a1 + TC_BM * TC_BK;
      // row tid of dY for the chunk's 32 K values
      float h[TC_BK], l[TC_BK];
      if (a.rows_mode) {
        // tile rows j (32) of 128 contiguous i
#pragma unroll
        for (int j = 0; j < TC_BK; ++j) h[j] = a.has_a0 ? a1[j * TC_BM + tid] - a0[j * TC_BM + tid] : a1[j * TC_BM + tid];
      } else {
        // K-major tile with the 128-byte swizzle: the 16-byte group c of row
        // i sits at group c ^ (i & 7) of the row's 128 bytes
        const int rb = (tid >> 3) * 1024 + (tid & 7) * 128;
        const unsigned char* b1 = reinterpret_cast<const unsigned char*>(a1);
        const unsigned char* b0 = reinterpret_cast<const unsigned char*>(a0);
#pragma unroll
        for (int c = 0; c < TC_BK / 4; ++c) {
          const int off = rb + ((c ^ (tid & 7)) << 4);
          float4 x1 = *reinterpret_cast<const float4*>(b1 + off);
          if (a.has_a0) {
            const float4 x0 = *reinterpret_cast<const float4*>(b0 + off);
            x1.x -= x0.x;
            x1.y -= x0.y;
            x1.z -= x0.z;
            x1.w -= x0.w;
          }
          h[4 * c + 0] = x1.x;
          h[4 * c + 1] = x1.y;
          h[4 * c + 2] = x1.z;
          h[4 * c + 3] = x1.w;
        }
      }
#pragma unroll
      for (int j = 0; j < TC_BK; ++j) split(h[j], h[j], l[j]);
      // A slot it % 2 is free once the MMAs of chunk it - 2 have completed
      if (it >= TC_A_SLOTS) {
        const bool okA = mbar_wait(aempty(it % TC_A_SLOTS), (uint32_t)(it / TC_A_SLOTS - 1) & 1u, abort_flag, a);
        if (bar_any(!okA)) {
          aborted = true;
          break;
        }
        tc_fence_after();
      }
      const uint32_t ta = tmem + lane_base + a_col + (uint32_t)(64 * (it % TC_A_SLOTS));
      tmem_st32(ta, h);
      tmem_st32(ta + 32u, l);
      asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
      tc_fence_before();
      mbar_arrive(tfull(s));
      // the previous block is drained once this block has a few chunks queued
      if ((it % TC_DRAIN) == TC_DRAIN_LAG && it >= TC_DRAIN) {
        if (!drain(drained)) {
          aborted = true;
          break;
        }
        ++drained;
      }
    }
    while (!aborted && drained < nblocks) {
      if (!drain(drained)) aborted = true;
      ++drained;
    }
    if (!aborted) {
      const int row = mt * TC_BM + warp * 32 + lane;
      float* out = a.part + (size_t)sp * a.NB * a.P;
      if (row < a.P) {
#pragma unroll
        for (int c = 0; c < TC_MAX_NB; ++c)
          if (c < N) out[(size_t)c * a.P + row] = acc[c];
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 5) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols_tmem) : "memory");
  }
}

// TF32 hi / lo parts of the active columns of X (rows x R, ld ldx) into
// xh, xl (rows x NB, ld rows); inactive and padding columns become zeros.
__global__ void tc_split_x(int rows, int R, int NB, const int32_t* rank, int ncols, const float* __restrict__ X,
                           int64_t ldx, float* __restrict__ xh, float* __restrict__ xl) {
  const int ka = max(0, min(R, ncols >= 0 ? ncols : *rank));
  const int64_t total = (int64_t)rows * NB;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int row = (int)(e % rows), col = (int)(e / rows);
    const float x = (col < ka) ? X[row + (int64_t)col * ldx] : 0.0f;
    float h, l;
    split(x, h, l);
    xh[e] = h;
    xl[e] = l;
  }
}

// out[:, c] = sum over splits (fixed order) of the partials, c < active;
// zeros for the other columns < R
__global__ void tc_reduce(int P, int R, int NB, int splits, const int32_t* rank, int ncols,
                          const float* __restrict__ part, float* __restrict__ out, int64_t ldo, float* __restrict__ kd) {
  const int ka = max(0, min(R, ncols >= 0 ? ncols : *rank));
  const int64_t total = (int64_t)P * R;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int row = (int)(e % P), col = (int)(e / P);
    float v = 0.0f;
    if (col < ka)
      for (int s = 0; s < splits; ++s) v += part[((int64_t)s * NB + col) * P + row];
    out[row + (int64_t)col * ldo] = v;
    if (kd) kd[e] = v;
  }
}

using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encoder() {
  static std::atomic<void*> fn{nullptr};
  void* f = fn.load(std::memory_order_acquire);
  if (!f) {
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !f)
      return nullptr;
    fn.store(f, std::memory_order_release);
  }
  return reinterpret_cast<EncodeTiledFn>(f);
}

// 2-D FP32 tensor map of a column-major rows x cols matrix (ld = rows)
bool encode_2d(void* out, const void* ptr, uint64_t rows, uint64_t cols, uint32_t box0, uint32_t box1, bool swizzle) {
  EncodeTiledFn enc = encoder();
  if (!enc) return false;
  const cuuint64_t dims[2] = {rows, cols};
  const cuuint64_t strides[1] = {rows * 4};
  const cuuint32_t box[2] = {box0, box1};
  const cuuint32_t es[2] = {1, 1};
  return enc(reinterpret_cast<CUtensorMap*>(out), CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<void*>(ptr), dims,
             strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
             swizzle ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

struct Plan {
  int P, K, tiles, nchunks, cps, splits;
};

Plan plan(int64_t P, int64_t K, int sms, int forced_splits = 0) {
  Plan p{};
  p.P = (int)P;
  p.K = (int)K;
  p.tiles = (int)((P + TC_BM - 1) / TC_BM);
  p.nchunks = (int)((K + TC_BK - 1) / TC_BK);
  int splits = std::max(1, sms / p.tiles);
  splits = std::min(splits, std::max(1, p.nchunks / 4));  // at least 4 chunks (one pipeline fill) per CTA
  if (forced_splits > 0) splits = std::min(forced_splits, p.nchunks);
  p.cps = (p.nchunks + splits - 1) / splits;
  p.splits = (p.nchunks + p.cps - 1) / p.cps;
  return p;
}

int stages_for(int NB) {
  const int stage = 2 * (int)TC_TILE_BYTES + 2 * TC_BK * 4 * NB;
  return std::min(TC_MAX_STAGES, (TC_SMEM_LIMIT - TC_CTRL_BYTES - 1024) / stage);
}

}  // namespace

bool tc_encode_2d(void* out, const void* ptr, uint64_t rows, uint64_t cols, uint32_t box0, uint32_t box1,
                  bool swizzle) {
  return encode_2d(out, ptr, rows, cols, box0, box1, swizzle);
}

bool tc_encoder_available() { return encoder() != nullptr; }

bool tc_pass_supported(int64_t n, int64_t m, int R) {
  return n >= TC_BM && m >= TC_BM && (n % 4) == 0 && (m % 4) == 0 && R >= 1 && R <= TC_MAX_NB &&
         n < (int64_t(1) << 30) && m < (int64_t(1) << 30) && encoder() != nullptr;
}

cudaError_t tc_pass_init(TcPass* t, int64_t n, int64_t m, int R) {
  t->n = n;
  t->m = m;
  t->R = R;
  t->NB = (R + 15) & ~15;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&t->sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return e;
  const int64_t rows = std::max(n, m);
  const Plan pr = plan(n, m, t->sms), pc = plan(m, n, t->sms);
  const size_t part = std::max((size_t)pr.splits * n, (size_t)pc.splits * m) * t->NB;
  e = cudaMalloc((void**)&t->xh, sizeof(float) * rows * t->NB);
  if (e == cudaSuccess) e = cudaMalloc((void**)&t->xl, sizeof(float) * rows * t->NB);
  if (e == cudaSuccess) e = cudaMalloc((void**)&t->part, sizeof(float) * part);
  t->part_elems = part;
  if (e != cudaSuccess) return e;
  const bool ok = encode_2d(t->tm_xh_m, t->xh, m, t->NB, TC_BK, t->NB, true) &&
                  encode_2d(t->tm_xl_m, t->xl, m, t->NB, TC_BK, t->NB, true) &&
                  encode_2d(t->tm_xh_n, t->xh, n, t->NB, TC_BK, t->NB, true) &&
                  encode_2d(t->tm_xl_n, t->xl, n, t->NB, TC_BK, t->NB, true);
  return ok ? cudaSuccess : cudaErrorInvalidValue;
}

cudaError_t tc_pass_set_tiles(TcPass* t, int splits_rows, int splits_cols, int stages) {
  if (splits_rows < 0 || splits_cols < 0 || stages < 0 || (stages > 0 && stages < 2)) return cudaErrorInvalidValue;
  if (stages > stages_for(t->NB)) return cudaErrorInvalidValue;
  const Plan pr = plan(t->n, t->m, t->sms, splits_rows), pc = plan(t->m, t->n, t->sms, splits_cols);
  const size_t need = std::max((size_t)pr.splits * t->n, (size_t)pc.splits * t->m) * t->NB;
  if (need > t->part_elems) {
    float* p = nullptr;
    cudaError_t e = cudaMalloc((void**)&p, sizeof(float) * need);
    if (e != cudaSuccess) return e;
    cudaFree(t->part);  // cudaFree waits for the device: no pass still reads the old buffer
    t->part = p;
    t->part_elems = need;
  }
  t->ov_splits[0] = splits_rows;
  t->ov_splits[1] = splits_cols;
  t->ov_stages = stages;
  return cudaSuccess;
}

void tc_pass_free(TcPass* t) {
  cudaFree(t->xh);
  cudaFree(t->xl);
  cudaFree(t->part);
  t->xh = t->xl = t->part = nullptr;
}

cudaError_t tc_pass_run(TcPass* t, int trans, const float* A1, const float* A0, const float* X, int64_t ldx,
                        const int32_t* rank, int ncols, float* out, int64_t ldo, float* kd, uint32_t* status,
                        uint32_t status_timeout, cudaStream_t st) {
  if ((reinterpret_cast<uintptr_t>(A1) | reinterpret_cast<uintptr_t>(A0)) & 15) return cudaErrorInvalidValue;
  const bool has_a0 = A0 != nullptr;
  if (!has_a0) A0 = A1;  // a valid tensor map; its tile is never loaded
  const int64_t n = t->n, m = t->m;
  const bool rows_mode = (trans == 0);
  const int64_t P = rows_mode ? n : m, K = rows_mode ? m : n;
  alignas(64) unsigned char tm1[128], tm0[128];
  const bool ok = rows_mode ? (encode_2d(tm1, A1, n, m, TC_BM, TC_BK, false) && encode_2d(tm0, A0, n, m, TC_BM, TC_BK, false))
                            : (encode_2d(tm1, A1, n, m, TC_BK, TC_BM, true) && encode_2d(tm0, A0, n, m, TC_BK, TC_BM, true));
  if (!ok) return cudaErrorInvalidValue;
  const Plan pl = plan(P, K, t->sms, t->ov_splits[rows_mode ? 0 : 1]);
  const int NB = t->NB;
  tc_split_x<<<2 * t->sms, 256, 0, st>>>((int)K, t->R, NB, rank, ncols, X, ldx, t->xh, t->xl);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  const int stages = t->ov_stages > 0 ? t->ov_stages : stages_for(NB);
  const size_t smem = (size_t)stages * (2 * TC_TILE_BYTES + 2 * TC_BK * 4 * NB) + TC_CTRL_BYTES + 1024;
  static std::atomic<uint64_t> attr_done{0};  // the largest any panel width needs
  if ((e = set_smem_limit(tc_pass_kernel, TC_SMEM_LIMIT, attr_done)) != cudaSuccess) return e;
  TcArgs a{};
  a.P = (int)P;
  a.R = t->R;
  a.NB = NB;
  a.nchunks = pl.nchunks;
  a.chunks_per_split = pl.cps;
  a.stages = stages;
  a.rows_mode = rows_mode ? 1 : 0;
  a.has_a0 = has_a0 ? 1 : 0;
  a.ncols = ncols;
  a.rank = rank;
  a.part = t->part;
  a.status = status;
  a.status_timeout = status_timeout;
  const CUtensorMap* xh = reinterpret_cast<const CUtensorMap*>(rows_mode ? t->tm_xh_m : t->tm_xh_n);
  const CUtensorMap* xl = reinterpret_cast<const CUtensorMap*>(rows_mode ? t->tm_xl_m : t->tm_xl_n);
  tc_pass_kernel<<<dim3(pl.tiles, pl.splits), TC_THREADS, smem, st>>>(
      *reinterpret_cast<const CUtensorMap*>(tm1), *reinterpret_cast<const CUtensorMap*>(tm0), *xh, *xl, a);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  tc_reduce<<<2 * t->sms, 256, 0, st>>>((int)P, t->R, NB, pl.splits, rank, ncols, t->part, out, ldo, kd);
  return cudaGetLastError();
}

}  // namespace lri
