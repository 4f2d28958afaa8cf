// tc_kr.cu - Khatri-Rao products of the large Burgers engine's flows on the
// 5th-generation tensor cores.
//
// At active widths above 32 each RK stage of the K, L and S substep flows
// needs out = KR(Y, Y) T' (the quadratic Burgers term, see the engine's flow
// kernels): KR(Y, Y)_{i, p(a,b)} = Y_ia Y_ib over the packed pairs a <= b of
// the ka active columns, T' the packed flow tensor (np x ka, np = ka (ka +
// 1) / 2).  At rank 64 that is n P(128) 128 = 4.3 GFMA per S stage, which the
// FP32 pipe runs at about a quarter of its peak; here it is a GEMM with
// M = rows, N = ka, K = np.
//
// One CTA owns a 128-row tile, 64 output columns and a range of the pair
// chunks (32 pairs each):
//   all warps  load the tile's rows of Y (every active column) into shared
//              memory once;
//   warp 8     TMA producer: per chunk, the chunk's 32 rows of the TF32 hi and
//              lo copies of T' (split once per step by tc_kr_split), 64
//              columns, into a 4-stage mbarrier pipeline;
//   warps 0-7  two warpgroups, one per half of the chunk's 32 pairs: thread
//              i of a group forms row i of its 16 A columns, Y_ia Y_ib from
//              a pair table (independent entries: the shared-memory reads
//              overlap), splits them into TF32 hi + lo and stores both into
//              tensor memory (tcgen05.st; four A slots);
//   warp 9     allocates tensor memory and issues per 8-wide K slice
//              tcgen05.mma.kind::tf32 (A from tensor memory, B from shared
//              memory, M = 128, N = 64): hi*hi into one accumulator, hi*lo
//              + lo*hi into a correction accumulator;
//   warps 0-7  drain the accumulators into FP32 registers every 4 chunks,
//              each warpgroup 32 of the 64 columns (two accumulator buffers:
//              the tensor cores' FP32 accumulation truncates, so the number
//              of MMAs summed in one accumulator stays at 12) and finally
//              write the CTA's partial.
// Every mbarrier wait is bounded; a wait that gives up sets a status bit, the
// CTA stops issuing work, waits (bounded) for its copies and MMAs in flight,
// frees its tensor memory and returns.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstdint>

#include "engine_api.h"
#include "tc_common.cuh"
#include "tc_kr.h"
#include "tc_pass.h"

namespace lri {
namespace {

constexpr int KR_BM = 128;            // rows per CTA (UMMA M)
constexpr int KR_BN = 64;             // output columns per CTA (UMMA N)
constexpr int KR_BK = 32;             // pairs per chunk: one 128-byte swizzle row of FP32
constexpr int KR_THREADS = 320;       // warps 0-7 transform/drain/epilogue, 8 TMA, 9 MMA
constexpr int KR_TX = 256;            // transform threads: two warpgroups, one per half of a chunk's pairs
constexpr int KR_STAGES = 4;
constexpr int KR_DRAIN = 4;           // chunks per accumulator block
constexpr int KR_DRAIN_LAG = 2;       // chunks of the next block queued before a drain
constexpr int KR_A_SLOTS = 4;                    // A operand slots: the transform runs up to 3 chunks ahead
constexpr int KR_KMAX = 128;          // active columns (2 r_max, r_max <= 64)
constexpr uint32_t KR_TILE_BYTES = KR_BN * KR_BK * 4;  // one B tile (hi or lo): 8 KB
constexpr int KR_CTRL_BYTES = 1024;
constexpr uint32_t KR_TMEM_COLS = 512;  // 2 x (64 main + 64 correction) + 4 x 64 A columns
constexpr long long KR_WAIT_CYCLES = 4000000000LL;
constexpr int KR_PMAX = KR_KMAX * (KR_KMAX + 1) / 2;  // packed pairs at the widest panel
// shared memory: the stages, the row tile (KR_KMAX x 128 FP32), the pair
// table (a | b << 8 per pair, 16 bits), control
constexpr int KR_TAB_BYTES = ((KR_PMAX * 2 + 1023) / 1024) * 1024;
constexpr int KR_SMEM = KR_STAGES * 2 * KR_TILE_BYTES + KR_KMAX * KR_BM * 4 + KR_TAB_BYTES + KR_CTRL_BYTES + 1024;

struct KrArgs {
  int N, R, aug, kz;
  float scale;
  int accum;
  const int32_t* rank;
  const float* Y;
  float* part;
  uint32_t* status;
  uint32_t status_timeout;
};

__device__ __forceinline__ int kr_col(int c, int r, int R, int aug) { return (aug && c >= r) ? R + (c - r) : c; }

__global__ void __launch_bounds__(KR_THREADS, 1)
    tc_kr_kernel(const __grid_constant__ CUtensorMap tmTh, const __grid_constant__ CUtensorMap tmTl,
                 const KrArgs a) {
  extern __shared__ unsigned char smem_raw[];
  const int r = min(a.R, (int)*a.rank);
  const int ka = a.aug ? 2 * r : r;
  const int np = ka * (ka + 1) / 2;
  const int nchunks = (np + KR_BK - 1) / KR_BK;
  const int mt = blockIdx.x, c0 = blockIdx.y * KR_BN, z = blockIdx.z;
  if (c0 >= ka) return;  // the whole CTA, before any barrier or allocation
  const int i0 = mt * KR_BM;
  const int kc0 = (int)((int64_t)z * nchunks / a.kz), kc1 = (int)((int64_t)(z + 1) * nchunks / a.kz);
  const int nk = kc1 - kc0;
  const int nblocks = (nk + KR_DRAIN - 1) / KR_DRAIN;

  unsigned char* base = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                                         ~static_cast<uintptr_t>(1023));
  unsigned char* stages = base;                                       // KR_STAGES x (hi, lo) B tiles
  float* ys = reinterpret_cast<float*>(base + KR_STAGES * 2 * KR_TILE_BYTES);  // [column][128 rows]
  uint16_t* tab = reinterpret_cast<uint16_t*>(ys + KR_KMAX * KR_BM);           // pair p -> a | b << 8
  unsigned char* ctrl = reinterpret_cast<unsigned char*>(tab) + KR_TAB_BYTES;
  const uint32_t bar0 = smem_u32(ctrl);
  auto full = [&](int s) { return bar0 + 8u * s; };
  auto tfull = [&](int s) { return bar0 + 8u * (KR_STAGES + s); };
  auto empty = [&](int s) { return bar0 + 8u * (2 * KR_STAGES + s); };
  auto acc_full = [&](int b) { return bar0 + 8u * (3 * KR_STAGES + b); };
  auto acc_empty = [&](int b) { return bar0 + 8u * (3 * KR_STAGES + 2 + b); };
  const uint32_t done = bar0 + 8u * (3 * KR_STAGES + 4);
  auto aempty = [&](int t) { return bar0 + 8u * (3 * KR_STAGES + 5 + t); };
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(ctrl + 256);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(ctrl + 260);
  auto wait = [&](uint32_t bar, uint32_t par, long long limit = KR_WAIT_CYCLES) {
    return mbar_wait_st(bar, par, abort_flag, a.status, a.status_timeout, limit);
  };

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  // the tile's rows of Y, every active column (rows beyond N are zero)
  {
    const int rows = min(KR_BM, a.N - i0);
    constexpr int U = 8;  // loads in flight per thread
    const int total = ka * KR_BM;
    for (int e0 = tid; e0 < total; e0 += U * KR_THREADS) {
      float v[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int e = e0 + u * KR_THREADS;
        const int ii = e % KR_BM, c = e / KR_BM;
        v[u] = (e < total && ii < rows) ? a.Y[(int64_t)kr_col(c, r, a.R, a.aug) * a.N + i0 + ii] : 0.0f;
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int e = e0 + u * KR_THREADS;
        if (e < total) ys[e] = v[u];
      }
    }
  }
  // pair table: row a of the triangle starts at a ka - a (a - 1) / 2
  for (int pa = tid; pa < ka; pa += KR_THREADS) {
    const int st0 = pa * ka - pa * (pa - 1) / 2;
    for (int pb = pa; pb < ka; ++pb) tab[st0 + pb - pa] = (uint16_t)(pa | (pb << 8));
  }
  if (tid == 0) {
    for (int s = 0; s < KR_STAGES; ++s) {
      mbar_init(full(s), 1);
      mbar_init(tfull(s), KR_TX);
      mbar_init(empty(s), 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(acc_full(b), 1);
      mbar_init(acc_empty(b), KR_TX);
    }
    for (int t = 0; t < KR_A_SLOTS; ++t) mbar_init(aempty(t), 1);
    mbar_init(done, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 9) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(KR_TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  const uint32_t a_col = 4u * KR_BN;  // A slots after the two accumulator buffers

  if (warp == 8) {
    // ---------------- TMA producer ----------------
    if (lane == 0) {
      int last_par[KR_STAGES];
      for (int s = 0; s < KR_STAGES; ++s) last_par[s] = -1;
      bool ok = true;
      for (int it = 0; it < nk && ok; ++it) {
        const int s = it % KR_STAGES;
        const uint32_t par = (uint32_t)(it / KR_STAGES) & 1u;
        if (!(ok = wait(empty(s), par ^ 1u))) break;
        const int kc = kc0 + it;
        const uint32_t st = smem_u32(stages + (size_t)s * 2 * KR_TILE_BYTES);
        mbar_expect_tx(full(s), 2 * KR_TILE_BYTES);
        tma_load_2d(st, &tmTh, kc * KR_BK, c0, full(s));
        tma_load_2d(st + KR_TILE_BYTES, &tmTl, kc * KR_BK, c0, full(s));
        last_par[s] = (int)par;
      }
      if (!ok || *abort_flag) {
        for (int s = 0; s < KR_STAGES; ++s)
          if (last_par[s] >= 0) wait(full(s), (uint32_t)last_par[s], KR_WAIT_CYCLES / 4);
      }
    }
  } else if (warp == 9) {
    // ---------------- MMA issuer ----------------
    if (lane == 0) {
      const uint32_t idesc = idesc_tf32(KR_BM, KR_BN);
      for (int it = 0; it < nk; ++it) {
        const int s = it % KR_STAGES;
        const uint32_t par = (uint32_t)(it / KR_STAGES) & 1u;
        const int bi = it / KR_DRAIN, b = bi & 1;
        const bool first = (it % KR_DRAIN) == 0;
        if (first && bi >= 2 && !wait(acc_empty(b), (uint32_t)((bi >> 1) - 1) & 1u)) break;
        if (!wait(full(s), par) || !wait(tfull(s), par)) break;
        tc_fence_after();
        const uint32_t sbh = smem_u32(stages + (size_t)s * 2 * KR_TILE_BYTES);
        const uint32_t sbl = sbh + KR_TILE_BYTES;
        const uint32_t dmain = tmem + (uint32_t)(2 * b * KR_BN), dcorr = dmain + (uint32_t)KR_BN;
        const uint32_t tah = tmem + a_col + (uint32_t)(64 * (it % KR_A_SLOTS)), tal = tah + 32u;
#pragma unroll
        for (int kk = 0; kk < KR_BK / 8; ++kk) {
          const uint64_t bh = sw128_desc(sbh + 32u * kk), bl = sw128_desc(sbl + 32u * kk);
          const uint32_t acc = (!first || kk > 0) ? 1u : 0u;
          umma_tf32_ts(dmain, tah + 8u * kk, bh, idesc, acc);
          umma_tf32_ts(dcorr, tah + 8u * kk, bl, idesc, acc);
          umma_tf32_ts(dcorr, tal + 8u * kk, bh, idesc, 1u);
        }
        umma_commit(empty(s));
        umma_commit(aempty(it % KR_A_SLOTS));
        if ((it % KR_DRAIN) == KR_DRAIN - 1 || it == nk - 1) umma_commit(acc_full(b));
      }
      umma_commit(done);
      if (*abort_flag) wait(done, 0, KR_WAIT_CYCLES / 4);
    }
    __syncwarp();
  } else {
    // -------- A operand, drains, epilogue (warps 0-7: group g = half of the pairs and columns) --------
    const int g = tid >> 7, row_t = tid & 127;  // tensor-memory lane = row_t (warp % 4 picks the quarter)
    const uint32_t lane_base = (uint32_t)((warp & 3) * 32) << 16;
    constexpr int HN = KR_BN / 2, HK = KR_BK / 2;
    float acc[HN];
#pragma unroll
    for (int c = 0; c < HN; ++c) acc[c] = 0.0f;
    bool aborted = false;
    int drained = 0;
    auto drain = [&](int k) {
      const int b = k & 1;
      const bool ok = wait(acc_full(b), (uint32_t)(k >> 1) & 1u);
      if (bar_any_n(!ok, KR_TX)) return false;
      tc_fence_after();
      const uint32_t dmain = tmem + lane_base + (uint32_t)(2 * b * KR_BN + HN * g), dcorr = dmain + (uint32_t)KR_BN;
#pragma unroll
      for (int cc = 0; cc < HN; cc += 16) {
        float v[16], w[16];
        tmem_ld16(dmain + (uint32_t)cc, v);
        tmem_ld16(dcorr + (uint32_t)cc, w);
#pragma unroll
        for (int q = 0; q < 16; ++q) acc[cc + q] += v[q] + w[q];
      }
      tc_fence_before();
      mbar_arrive(acc_empty(b));
      return true;
    };
    const float* yrow = ys + row_t;  // column c of this row at yrow[c * KR_BM]
    for (int it = 0; it < nk; ++it) {
      const int p0 = (kc0 + it) * KR_BK + HK * g;  // this group's 16 pairs
      float h[HK], l[HK];
      // the pairs from the table (a broadcast read each): independent
      // entries, so their shared-memory reads overlap
#pragma unroll
      for (int j = 0; j < HK; ++j) {
        const int p = p0 + j;
        float v = 0.0f;
        if (p < np) {
          const uint32_t ab = tab[p];
          v = yrow[(ab & 0xffu) * KR_BM] * yrow[(ab >> 8) * KR_BM];
        }
        split(v, h[j], l[j]);
      }
      if (it >= KR_A_SLOTS) {
        const bool okA = wait(aempty(it % KR_A_SLOTS), (uint32_t)(it / KR_A_SLOTS - 1) & 1u);
        if (bar_any_n(!okA, KR_TX)) {
          aborted = true;
          break;
        }
        tc_fence_after();
      }
      // slot: hi in columns [0, 32), lo in [32, 64); this group's 16 of each
      const uint32_t ta = tmem + lane_base + a_col + (uint32_t)(64 * (it % KR_A_SLOTS) + HK * g);
      tmem_st16(ta, h);
      tmem_st16(ta + 32u, l);
      asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
      tc_fence_before();
      mbar_arrive(tfull(it % KR_STAGES));
      if ((it % KR_DRAIN) == KR_DRAIN_LAG && it >= KR_DRAIN) {
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
      const int row = i0 + row_t;
      if (row < a.N) {
        float* dst = a.part + (int64_t)z * a.N * (2 * a.R);
#pragma unroll
        for (int cc = 0; cc < HN; ++cc) {
          const int c = c0 + HN * g + cc;
          if (c < ka) {
            float* d = dst + row + (int64_t)kr_col(c, r, a.R, a.aug) * a.N;
            *d = a.accum ? fmaf(a.scale, acc[cc], *d) : a.scale * acc[cc];
          }
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 9) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(KR_TMEM_COLS) : "memory");
  }
}

// TF32 hi / lo copies (pair stride PPp) of a packed tensor (PP x 2R, ld PP)
// over its ka active columns; zero beyond the active pairs and columns.
__global__ void tc_kr_split_kernel(int R, int aug, const int32_t* __restrict__ rank, const float* __restrict__ Tp,
                                   int PP, int PPp, float* __restrict__ th, float* __restrict__ tl) {
  const int r = min(R, (int)*rank), ka = aug ? 2 * r : r, np = ka * (ka + 1) / 2;
  const int64_t total = (int64_t)PPp * 2 * R;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int p = (int)(e % PPp), c = (int)(e / PPp);
    const float v = (p < np && c < ka) ? Tp[p + (int64_t)c * PP] : 0.0f;
    float h, l;
    split(v, h, l);
    th[e] = h;
    tl[e] = l;
  }
}

}  // namespace

bool tc_kr_supported(int R) { return R >= 1 && 2 * R <= KR_KMAX && tc_encoder_available(); }

cudaError_t tc_kr_init(TcKr* t, int R) {
  t->R = R;
  t->PP = (2 * R) * (2 * R + 1) / 2;
  t->PPp = (t->PP + 3) & ~3;
  const size_t elems = (size_t)t->PPp * 2 * R;
  cudaError_t e = cudaSuccess;
  for (int k = 0; k < 3 && e == cudaSuccess; ++k) {
    e = cudaMalloc((void**)&t->th[k], sizeof(float) * elems);
    if (e == cudaSuccess) e = cudaMalloc((void**)&t->tl[k], sizeof(float) * elems);
    if (e == cudaSuccess) e = cudaMemset(t->th[k], 0, sizeof(float) * elems);
    if (e == cudaSuccess) e = cudaMemset(t->tl[k], 0, sizeof(float) * elems);
  }
  if (e != cudaSuccess) return e;
  for (int k = 0; k < 3; ++k)
    if (!tc_encode_2d(t->tm_h[k], t->th[k], (uint64_t)t->PPp, (uint64_t)2 * R, KR_BK, KR_BN, true) ||
        !tc_encode_2d(t->tm_l[k], t->tl[k], (uint64_t)t->PPp, (uint64_t)2 * R, KR_BK, KR_BN, true))
      return cudaErrorInvalidValue;
  return cudaSuccess;
}

void tc_kr_free(TcKr* t) {
  for (int k = 0; k < 3; ++k) {
    cudaFree(t->th[k]);
    cudaFree(t->tl[k]);
    t->th[k] = t->tl[k] = nullptr;
  }
}

cudaError_t tc_kr_split(TcKr* t, int k, const float* Tp, const int32_t* rank, int aug, cudaStream_t st) {
  if (k < 0 || k > 2) return cudaErrorInvalidValue;
  tc_kr_split_kernel<<<304, 256, 0, st>>>(t->R, aug, rank, Tp, t->PP, t->PPp, t->th[k], t->tl[k]);
  return cudaGetLastError();
}

int tc_kr_splits(int N, int R, int aug, int sms, int zmax) {
  const int tiles = ((N + KR_BM - 1) / KR_BM) * (((aug ? 2 * R : R) + KR_BN - 1) / KR_BN);
  return std::max(1, std::min(zmax, sms / std::max(1, tiles)));
}

cudaError_t tc_kr_apply(TcKr* t, int k, int N, int aug, const int32_t* rank, const float* Y, float* part, int kz,
                        double scale, int accum, uint32_t* status, uint32_t status_timeout, cudaStream_t st) {
  if (k < 0 || k > 2 || kz < 1 || N < 1) return cudaErrorInvalidValue;
  static std::atomic<uint64_t> attr_done{0};
  cudaError_t e = set_smem_limit(tc_kr_kernel, KR_SMEM, attr_done);
  if (e != cudaSuccess) return e;
  KrArgs a{};
  a.N = N;
  a.R = t->R;
  a.aug = aug;
  a.kz = kz;
  a.scale = (float)scale;
  a.accum = accum;
  a.rank = rank;
  a.Y = Y;
  a.part = part;
  a.status = status;
  a.status_timeout = status_timeout;
  const int kmax = aug ? 2 * t->R : t->R;
  const dim3 grid((N + KR_BM - 1) / KR_BM, (kmax + KR_BN - 1) / KR_BN, kz);
  tc_kr_kernel<<<grid, KR_THREADS, KR_SMEM, st>>>(*reinterpret_cast<const CUtensorMap*>(t->tm_h[k]),
                                                 *reinterpret_cast<const CUtensorMap*>(t->tm_l[k]), a);
  return cudaGetLastError();
}

}  // namespace lri
