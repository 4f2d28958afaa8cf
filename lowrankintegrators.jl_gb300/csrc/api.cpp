// api.cpp - host side of the C ABI declared in include/lri.h.
//
// A batch is the GB300 form of the reference's DLRIntegrator
// (src/primitives.jl:54-63): it owns the per-instance workspace (the
// reference's alg_cache, e.g. src/integrators/unconventional.jl:39-107),
// plans a packed layout for the caller's factors and runs steps as launches
// of the instance-engine kernel, multi-step calls as one CUDA graph.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <numeric>
#include <vector>

#include "../../include/lri.h"
#include "engine_api.h"

using lri::InstDesc;
using lri::Scheme;
using lri::StepArgs;

struct lri_batch {
  lri_batch_desc desc;
  lri_alg_desc alg;
  std::vector<int64_t> n, m, r, rcap;
  std::vector<InstDesc> inst;
  std::vector<int32_t> order;
  int64_t totU = 0, totS = 0, totV = 0, totA = 0, totB = 0, totWork = 0, totSmall = 0, totY = 0;
  size_t esize = 8;
  // device
  InstDesc* d_inst = nullptr;
  int32_t* d_order = nullptr;
  int32_t* d_rank = nullptr;
  int32_t* d_proj_valid = nullptr;
  uint32_t* d_status = nullptr;
  void* d_work = nullptr;
  void* d_small = nullptr;
  void* d_Yprev = nullptr;
  // double-float batches: the engine's own copies of the factors/operators
  void* iU = nullptr;
  void* iS = nullptr;
  void* iV = nullptr;
  void* iA = nullptr;
  void* iB = nullptr;
  void* iYn = nullptr;
  // bound caller buffers
  void* U = nullptr;
  void* S = nullptr;
  void* V = nullptr;
  const void* opA = nullptr;
  const void* opB = nullptr;
  bool bound = false;
  bool data_ready = false;
  int32_t ctas_per_sm = 3;  // register budget of the step kernel (lri_batch_set_occupancy)
  // discrete adjoint (allocated by lri_batch_adjoint_prepare)
  double* d_adj_work = nullptr;
  int64_t* d_adj_off = nullptr;
  int64_t* d_th_off = nullptr;
  // graph cache
  cudaStream_t cap_stream = nullptr;
  cudaGraphExec_t gexec = nullptr;
  int g_steps = 0;
  double g_dt = 0.0;
};

namespace {

lri_status cuda_status(cudaError_t e) { return e == cudaSuccess ? LRI_OK : LRI_ERR_CUDA; }

#define LRI_CUDA(call)                          \
  do {                                          \
    cudaError_t _e = (call);                    \
    if (_e != cudaSuccess) return LRI_ERR_CUDA; \
  } while (0)

bool scheme_ok(const lri_scheme& s) {
  if (s.nstages < 1 || s.nstages > 4 || s.nsub < 1) return false;
  for (int i = 0; i < s.nstages; ++i)
    if (!std::isfinite(s.a[i]) || !std::isfinite(s.b[i]) || !std::isfinite(s.c[i])) return false;
  return true;
}

Scheme to_scheme(const lri_scheme& s) {
  Scheme o{};
  o.nstages = s.nstages;
  o.nsub = s.nsub;
  for (int i = 0; i < 4; ++i) {
    o.a[i] = s.a[i];
    o.b[i] = s.b[i];
    o.c[i] = s.c[i];
  }
  return o;
}

template <typename T>
StepArgs<T> make_args(const lri_batch* b, double t, double dt, const void* Ynext) {
  const bool df = b->desc.dtype == LRI_DF;
  StepArgs<T> g{};
  g.inst = b->d_inst;
  g.order = b->d_order;
  g.rank = b->d_rank;
  g.proj_valid = b->d_proj_valid;
  g.status = b->d_status;
  g.U = static_cast<T*>(df ? b->iU : b->U);
  g.S = static_cast<T*>(df ? b->iS : b->S);
  g.V = static_cast<T*>(df ? b->iV : b->V);
  g.opA = static_cast<const T*>(df ? b->iA : b->opA);
  g.opB = static_cast<const T*>(df ? b->iB : b->opB);
  g.work = static_cast<T*>(b->d_work);
  g.small = static_cast<T*>(b->d_small);
  g.Yprev = static_cast<T*>(b->d_Yprev);
  g.Ynext = static_cast<const T*>(df && Ynext ? b->iYn : Ynext);
  g.t = t;
  g.dt = dt;
  g.alg = b->alg.kind;
  g.ksl_order = b->alg.ksl_order;
  g.op = b->desc.op;
  g.r_min = b->alg.r_min;
  g.two_factor = b->alg.two_factor;
  g.tol = b->alg.tol;
  g.sK = to_scheme(b->alg.K_alg);
  g.sL = to_scheme(b->alg.L_alg);
  g.sS = to_scheme(b->alg.S_alg);
  g.flow = b->desc.flow;
  g.bh = b->desc.burgers_h;
  g.balpha = b->desc.burgers_alpha;
  g.bbeta = b->desc.burgers_beta;
  return g;
}

cudaError_t launch_one(const lri_batch* b, double t, double dt, const void* Ynext, cudaStream_t st) {
  const int count = b->desc.count;
  if (b->desc.dtype == LRI_F32)
    return lri::launch_step<float>(make_args<float>(b, t, dt, Ynext), count, st, b->ctas_per_sm);
  if (b->desc.dtype == LRI_DF) {
    cudaError_t e = cudaSuccess;
    if (Ynext) e = lri::convert_f64_to_df(static_cast<const double*>(Ynext), b->iYn, b->totY, st);
    if (e != cudaSuccess) return e;
    return lri::launch_step<lri::dfloat>(make_args<lri::dfloat>(b, t, dt, Ynext), count, st, b->ctas_per_sm);
  }
  return lri::launch_step<double>(make_args<double>(b, t, dt, Ynext), count, st);
}

// double-float batches: write the engine's factors back to the caller's buffers
cudaError_t writeback(const lri_batch* b, cudaStream_t st) {
  if (b->desc.dtype != LRI_DF) return cudaSuccess;
  cudaError_t e = lri::convert_df_to_f64(b->iU, static_cast<double*>(b->U), b->totU, st);
  if (e == cudaSuccess) e = lri::convert_df_to_f64(b->iS, static_cast<double*>(b->S), b->totS, st);
  if (e == cudaSuccess) e = lri::convert_df_to_f64(b->iV, static_cast<double*>(b->V), b->totV, st);
  return e;
}

void free_graph(lri_batch* b) {
  if (b->gexec) cudaGraphExecDestroy(b->gexec);
  b->gexec = nullptr;
  b->g_steps = 0;
}

}  // namespace

extern "C" {

int lri_abi_version(void) { return LRI_ABI_VERSION; }

const char* lri_status_str(lri_status s) {
  switch (s) {
    case LRI_OK: return "ok";
    case LRI_ERR_ARG: return "invalid argument";
    case LRI_ERR_UNSUPPORTED: return "unsupported configuration";
    case LRI_ERR_BREAKDOWN: return "numerical breakdown (SVD did not converge)";
    case LRI_ERR_NONFINITE: return "non-finite value in the factors";
    case LRI_ERR_RANK_OVERFLOW: return "rank exceeded capacity";
    case LRI_ERR_TIMEOUT: return "bounded device wait timed out";
    case LRI_ERR_CUDA: return "CUDA error or no CUDA device";
    case LRI_ERR_STATE: return "call out of order";
  }
  return "unknown status";
}

int32_t lri_flow_count(void) { return lri::local_flow_count(); }

const char* lri_flow_name(int32_t id) { return lri::local_flow_name(id); }

lri_status lri_device_info(int* device, int* sm_count, int* cc_major, int* cc_minor) {
  int dev = 0;
  LRI_CUDA(cudaGetDevice(&dev));
  cudaDeviceProp p;
  LRI_CUDA(cudaGetDeviceProperties(&p, dev));
  if (device) *device = dev;
  if (sm_count) *sm_count = p.multiProcessorCount;
  if (cc_major) *cc_major = p.major;
  if (cc_minor) *cc_minor = p.minor;
  return LRI_OK;
}

lri_status lri_batch_create(lri_batch** out, const lri_batch_desc* desc, const lri_alg_desc* alg) {
  if (!out || !desc || !alg) return LRI_ERR_ARG;
  *out = nullptr;
  if (desc->count < 1 || !desc->n || !desc->m || !desc->r) return LRI_ERR_ARG;
  if (desc->dtype != LRI_F32 && desc->dtype != LRI_F64 && desc->dtype != LRI_DF) return LRI_ERR_ARG;
  if (desc->op < LRI_OP_ZERO || desc->op > LRI_OP_LOCAL_FLOW) return LRI_ERR_ARG;
  if (desc->op == LRI_OP_LOCAL_FLOW && (desc->flow < 0 || desc->flow >= lri::local_flow_count()))
    return LRI_ERR_ARG;
  if (alg->kind < LRI_ALG_BUG || alg->kind > LRI_ALG_GREEDY) return LRI_ERR_ARG;
  if (alg->kind == LRI_ALG_GREEDY) {
    if (alg->two_factor != 0 && alg->two_factor != 1) return LRI_ERR_ARG;
    // SVD-like greedy fitting needs data; two factors take data or a flow (hybrid)
    if (!alg->two_factor && desc->op != LRI_OP_DATA) return LRI_ERR_UNSUPPORTED;
  }
  if (alg->kind == LRI_ALG_KSL && (alg->ksl_order < 0 || alg->ksl_order > 2)) return LRI_ERR_ARG;
  if (!scheme_ok(alg->K_alg) || !scheme_ok(alg->L_alg) || !scheme_ok(alg->S_alg)) return LRI_ERR_ARG;
  if (alg->kind == LRI_ALG_RA_BUG && (!(alg->tol >= 0.0) || alg->r_min < 1)) return LRI_ERR_ARG;
  if ((desc->op == LRI_OP_BURGERS_PERIODIC || desc->op == LRI_OP_LOCAL_FLOW) &&
      !(desc->burgers_h > 0.0 && std::isfinite(desc->burgers_h) && std::isfinite(desc->burgers_alpha) &&
        std::isfinite(desc->burgers_beta)))
    return LRI_ERR_ARG;
  // Strang needs the data at the half step: with one snapshot per step it is
  // not defined (the reference has no method for it either:
  // update_data! requires integer dt, data_integrator.jl:26).
  if (desc->op == LRI_OP_DATA && alg->kind == LRI_ALG_KSL && alg->ksl_order == LRI_KSL_STRANG)
    return LRI_ERR_UNSUPPORTED;

  lri_batch* b = new lri_batch();
  b->desc = *desc;
  b->alg = *alg;
  b->esize = desc->dtype == LRI_F32 ? 4 : 8;
  const int count = desc->count;
  const bool ra = alg->kind == LRI_ALG_RA_BUG;
  b->n.resize(count);
  b->m.resize(count);
  b->r.resize(count);
  b->rcap.resize(count);
  b->inst.resize(count);
  for (int i = 0; i < count; ++i) {
    const int64_t n = desc->n[i], m = desc->m[i], r = desc->r[i];
    const int64_t rc = desc->r_cap ? desc->r_cap[i] : r;
    const int64_t w = ra ? 2 * rc : rc;
    bool ok = n >= 1 && m >= 1 && r >= 1 && rc >= r && n < (1LL << 30) && m < (1LL << 30);
    ok = ok && w <= 64 && w <= n && w <= m;
    if (desc->op == LRI_OP_DATA || alg->kind == LRI_ALG_GREEDY) ok = ok && (n * m) < (1LL << 40);
    if (!ok) {
      delete b;
      return (w > 64 && n >= w && m >= w && r >= 1 && rc >= r) ? LRI_ERR_UNSUPPORTED : LRI_ERR_ARG;
    }
    b->n[i] = n;
    b->m[i] = m;
    b->r[i] = r;
    b->rcap[i] = rc;
  }
  // packed layout of the caller's buffers and of the workspace
  for (int i = 0; i < count; ++i) {
    const int64_t n = b->n[i], m = b->m[i], rc = b->rcap[i];
    const int64_t w = ra ? 2 * rc : rc;
    InstDesc& d = b->inst[i];
    d.n = (int32_t)n;
    d.m = (int32_t)m;
    d.rcap = (int32_t)rc;
    d.wcap = (int32_t)w;
    d.offU = b->totU;
    b->totU += n * rc;
    d.offS = b->totS;
    b->totS += rc * rc;
    d.offV = b->totV;
    b->totV += m * rc;
    d.offA = b->totA;
    d.offB = b->totB;
    if (desc->op == LRI_OP_SYLVESTER_TRIDIAG) {
      b->totA += 3 * n;
      b->totB += 3 * m;
    } else if (desc->op == LRI_OP_BURGERS_PERIODIC || desc->op == LRI_OP_LOCAL_FLOW) {
      b->totB += m;  // per-column parameter (Burgers: viscosity)
    }
    // side workspaces: PY, PQ (N x W) + PA, PZ0, PZ1 (N x rcap); keep 16-byte alignment
    auto al = [](int64_t x) { return (x + 3) & ~int64_t(3); };
    d.offWK = b->totWork;
    b->totWork += al(n * (2 * w + 3 * rc));
    d.offWL = b->totWork;
    b->totWork += al(m * (2 * w + 3 * rc));
    d.offSmall = b->totSmall;
    b->totSmall += lri::kSmallBlocks * al(w * w);  // blocks padded to 4 elements (see Inst::blk)
    d.offY = b->totY;
    if (desc->op == LRI_OP_DATA || alg->kind == LRI_ALG_GREEDY) b->totY += n * m;
  }
  // longest-processing-time-first launch order: CTAs start in block order
  b->order.resize(count);
  std::iota(b->order.begin(), b->order.end(), 0);
  std::vector<double> cost(count);
  for (int i = 0; i < count; ++i) {
    const double w = (double)b->inst[i].wcap;
    cost[i] = (double)(b->n[i] + b->m[i]) * w * (w + 8.0);
  }
  std::stable_sort(b->order.begin(), b->order.end(), [&](int x, int y) { return cost[x] > cost[y]; });

  cudaError_t e = cudaSuccess;
  auto alloc = [&](void** p, size_t bytes) {
    if (e != cudaSuccess) return;
    e = cudaMalloc(p, bytes < 16 ? 16 : bytes);
  };
  alloc((void**)&b->d_inst, sizeof(InstDesc) * count);
  alloc((void**)&b->d_order, sizeof(int32_t) * count);
  alloc((void**)&b->d_rank, sizeof(int32_t) * count);
  alloc((void**)&b->d_proj_valid, sizeof(int32_t) * count);
  alloc((void**)&b->d_status, sizeof(uint32_t));
  alloc(&b->d_work, b->esize * (size_t)b->totWork);
  alloc(&b->d_small, b->esize * (size_t)b->totSmall);
  if (desc->op == LRI_OP_DATA && alg->kind != LRI_ALG_GREEDY) alloc(&b->d_Yprev, b->esize * (size_t)b->totY);
  if (desc->dtype == LRI_DF) {
    alloc(&b->iU, 8 * (size_t)b->totU);
    alloc(&b->iS, 8 * (size_t)b->totS);
    alloc(&b->iV, 8 * (size_t)b->totV);
    alloc(&b->iA, 8 * (size_t)b->totA);
    alloc(&b->iB, 8 * (size_t)b->totB);
    if (b->totY > 0) alloc(&b->iYn, 8 * (size_t)b->totY);
  }
  if (e == cudaSuccess) e = cudaMemcpy(b->d_inst, b->inst.data(), sizeof(InstDesc) * count, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(b->d_order, b->order.data(), sizeof(int32_t) * count, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(b->d_status, 0, sizeof(uint32_t));
  if (e == cudaSuccess) e = cudaMemset(b->d_proj_valid, 0, sizeof(int32_t) * count);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->cap_stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    lri_batch_destroy(b);
    return LRI_ERR_CUDA;
  }
  std::vector<int32_t> r32(b->r.begin(), b->r.end());
  if (cudaMemcpy(b->d_rank, r32.data(), sizeof(int32_t) * count, cudaMemcpyHostToDevice) != cudaSuccess) {
    lri_batch_destroy(b);
    return LRI_ERR_CUDA;
  }
  *out = b;
  return LRI_OK;
}

lri_status lri_batch_destroy(lri_batch* b) {
  if (!b) return LRI_ERR_ARG;
  free_graph(b);
  if (b->cap_stream) cudaStreamDestroy(b->cap_stream);
  cudaFree(b->d_inst);
  cudaFree(b->d_order);
  cudaFree(b->d_rank);
  cudaFree(b->d_proj_valid);
  cudaFree(b->d_status);
  cudaFree(b->d_work);
  cudaFree(b->d_small);
  cudaFree(b->d_Yprev);
  cudaFree(b->iU);
  cudaFree(b->iS);
  cudaFree(b->iV);
  cudaFree(b->iA);
  cudaFree(b->iB);
  cudaFree(b->iYn);
  cudaFree(b->d_adj_work);
  cudaFree(b->d_adj_off);
  cudaFree(b->d_th_off);
  delete b;
  return LRI_OK;
}

lri_status lri_batch_layout(const lri_batch* b, int64_t* offU, int64_t* offS, int64_t* offV, int64_t* offA,
                            int64_t* offB, int64_t* totals) {
  if (!b) return LRI_ERR_ARG;
  const int count = b->desc.count;
  for (int i = 0; i < count; ++i) {
    if (offU) offU[i] = b->inst[i].offU;
    if (offS) offS[i] = b->inst[i].offS;
    if (offV) offV[i] = b->inst[i].offV;
    if (offA) offA[i] = b->inst[i].offA;
    if (offB) offB[i] = b->inst[i].offB;
  }
  if (totals) {
    totals[0] = b->totU;
    totals[1] = b->totS;
    totals[2] = b->totV;
    totals[3] = b->totA;
    totals[4] = b->totB;
  }
  return LRI_OK;
}

lri_status lri_batch_data_layout(const lri_batch* b, int64_t* offY, int64_t* total) {
  if (!b) return LRI_ERR_ARG;
  if (offY)
    for (int i = 0; i < b->desc.count; ++i) offY[i] = b->inst[i].offY;
  if (total) *total = b->totY;
  return LRI_OK;
}

lri_status lri_batch_bind(lri_batch* b, void* U, void* S, void* V, const void* opA, const void* opB) {
  if (!b || !U || !S || !V) return LRI_ERR_ARG;
  if (b->desc.op == LRI_OP_SYLVESTER_TRIDIAG && (!opA || !opB)) return LRI_ERR_ARG;
  const uintptr_t mask = 15;
  if (((uintptr_t)U | (uintptr_t)S | (uintptr_t)V) & (b->esize - 1)) return LRI_ERR_ARG;
  (void)mask;
  free_graph(b);
  b->U = U;
  b->S = S;
  b->V = V;
  b->opA = opA;
  b->opB = opB;
  const int count = b->desc.count;
  std::vector<int32_t> r32(b->r.begin(), b->r.end());
  LRI_CUDA(cudaMemcpy(b->d_rank, r32.data(), sizeof(int32_t) * count, cudaMemcpyHostToDevice));
  LRI_CUDA(cudaMemset(b->d_proj_valid, 0, sizeof(int32_t) * count));
  if (b->desc.dtype == LRI_DF) {
    // load the engine's double-float copy (synchronous, like the rank upload above)
    LRI_CUDA(lri::convert_f64_to_df(static_cast<const double*>(U), b->iU, b->totU, 0));
    LRI_CUDA(lri::convert_f64_to_df(static_cast<const double*>(S), b->iS, b->totS, 0));
    LRI_CUDA(lri::convert_f64_to_df(static_cast<const double*>(V), b->iV, b->totV, 0));
    if (opA) LRI_CUDA(lri::convert_f64_to_df(static_cast<const double*>(opA), b->iA, b->totA, 0));
    if (opB) LRI_CUDA(lri::convert_f64_to_df(static_cast<const double*>(opB), b->iB, b->totB, 0));
    LRI_CUDA(cudaDeviceSynchronize());
  }
  b->bound = true;
  return LRI_OK;
}

lri_status lri_batch_data_init(lri_batch* b, const void* Y0, void* stream) {
  if (!b || !Y0) return LRI_ERR_ARG;
  if (b->desc.op != LRI_OP_DATA) return LRI_ERR_STATE;
  if (b->alg.kind == LRI_ALG_GREEDY) {  // the greedy steps read y(t + dt) only
    b->data_ready = true;
    return LRI_OK;
  }
  if (b->desc.dtype == LRI_DF) {
    LRI_CUDA(lri::convert_f64_to_df(static_cast<const double*>(Y0), b->d_Yprev, b->totY, (cudaStream_t)stream));
  } else {
    LRI_CUDA(cudaMemcpyAsync(b->d_Yprev, Y0, b->esize * (size_t)b->totY, cudaMemcpyDeviceToDevice,
                             (cudaStream_t)stream));
  }
  b->data_ready = true;
  return LRI_OK;
}

lri_status lri_batch_step(lri_batch* b, double t, double dt, int32_t nsteps, const void* Ynext, void* stream) {
  if (!b || nsteps < 0 || !std::isfinite(dt) || !std::isfinite(t)) return LRI_ERR_ARG;
  if (!b->bound) return LRI_ERR_STATE;
  if (nsteps == 0) return LRI_OK;
  cudaStream_t st = (cudaStream_t)stream;
  const bool greedy = b->alg.kind == LRI_ALG_GREEDY;
  if (b->desc.op == LRI_OP_DATA || greedy) {
    if (!b->data_ready && !greedy) return LRI_ERR_STATE;
    if (!Ynext || nsteps != 1) return LRI_ERR_ARG;
    cudaError_t e = launch_one(b, t, dt, Ynext, st);
    if (e == cudaSuccess) e = writeback(b, st);
    return cuda_status(e);
  }
  if (Ynext) return LRI_ERR_ARG;
  if (nsteps == 1) {
    cudaError_t e = launch_one(b, t, dt, nullptr, st);
    if (e == cudaSuccess) e = writeback(b, st);
    return cuda_status(e);
  }
  const lri_status ps = lri_batch_prepare(b, dt, nsteps);
  if (ps != LRI_OK) return ps;
  return cuda_status(cudaGraphLaunch(b->gexec, st));
}

lri_status lri_batch_prepare(lri_batch* b, double dt, int32_t nsteps) {
  if (!b || nsteps < 2 || !std::isfinite(dt)) return LRI_ERR_ARG;
  if (!b->bound) return LRI_ERR_STATE;
  if (b->desc.op == LRI_OP_DATA || b->alg.kind == LRI_ALG_GREEDY) return LRI_ERR_UNSUPPORTED;
  // The engine's operators are autonomous, so a captured graph depends on
  // (nsteps, dt) only and is reused across calls.
  if (b->gexec && b->g_steps == nsteps && b->g_dt == dt) return LRI_OK;
  free_graph(b);
  cudaGraph_t graph = nullptr;
  LRI_CUDA(cudaStreamBeginCapture(b->cap_stream, cudaStreamCaptureModeThreadLocal));
  cudaError_t e = cudaSuccess;
  for (int k = 0; k < nsteps && e == cudaSuccess; ++k) e = launch_one(b, k * dt, dt, nullptr, b->cap_stream);
  if (e == cudaSuccess) e = writeback(b, b->cap_stream);
  cudaError_t e2 = cudaStreamEndCapture(b->cap_stream, &graph);
  if (e != cudaSuccess || e2 != cudaSuccess) {
    if (graph) cudaGraphDestroy(graph);
    cudaGetLastError();
    return LRI_ERR_CUDA;
  }
  e = cudaGraphInstantiate(&b->gexec, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) {
    b->gexec = nullptr;
    return LRI_ERR_CUDA;
  }
  b->g_steps = nsteps;
  b->g_dt = dt;
  return LRI_OK;
}

lri_status lri_batch_ranks(lri_batch* b, int64_t* r_out, void* stream) {
  if (!b || !r_out) return LRI_ERR_ARG;
  const int count = b->desc.count;
  std::vector<int32_t> r32(count);
  LRI_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
  LRI_CUDA(cudaMemcpy(r32.data(), b->d_rank, sizeof(int32_t) * count, cudaMemcpyDeviceToHost));
  for (int i = 0; i < count; ++i) r_out[i] = r32[i];
  return LRI_OK;
}

lri_status lri_batch_status(lri_batch* b, void* stream) {
  if (!b) return LRI_ERR_ARG;
  LRI_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
  LRI_CUDA(cudaGetLastError());
  uint32_t s = 0;
  LRI_CUDA(cudaMemcpy(&s, b->d_status, sizeof(uint32_t), cudaMemcpyDeviceToHost));
  LRI_CUDA(cudaMemset(b->d_status, 0, sizeof(uint32_t)));
  if (s & lri::ST_BAD_SHAPE) return LRI_ERR_ARG;
  if (s & lri::ST_NONFINITE) return LRI_ERR_NONFINITE;
  if (s & lri::ST_SVD_NOCONV) return LRI_ERR_BREAKDOWN;
  if (s & lri::ST_RANK_OVERFLOW) return LRI_ERR_RANK_OVERFLOW;
  return LRI_OK;
}

lri_status lri_batch_set_occupancy(lri_batch* b, int32_t ctas_per_sm) {
  if (!b || (ctas_per_sm != 2 && ctas_per_sm != 3)) return LRI_ERR_ARG;
  if (b->desc.dtype == LRI_F64 && ctas_per_sm != 3) return LRI_ERR_UNSUPPORTED;
  if (b->ctas_per_sm != ctas_per_sm) free_graph(b);  // the captured graph holds the other kernel
  b->ctas_per_sm = ctas_per_sm;
  return LRI_OK;
}

int32_t lri_batch_launches_per_step(const lri_batch* b) {
  if (!b) return 0;
  // one engine launch; double-float batches add the three write-back
  // conversions (and one snapshot conversion for data problems) per call
  if (b->desc.dtype == LRI_DF) return 4 + (b->totY > 0 ? 1 : 0);
  return 1;
}

}  // extern "C"

// Checks that the batch is one the adjoint covers; returns the stage counts.
static lri_status adjoint_supported(const lri_batch* b, int* nsK, int* nsL) {
  if (b->desc.dtype != LRI_F64 || b->alg.kind != LRI_ALG_BUG || b->desc.op != LRI_OP_SYLVESTER_TRIDIAG)
    return LRI_ERR_UNSUPPORTED;
  for (int i = 0; i < b->desc.count; ++i)
    if (b->r[i] != b->rcap[i]) return LRI_ERR_UNSUPPORTED;  // fixed-rank BUG only
  *nsK = b->alg.K_alg.nstages * b->alg.K_alg.nsub;
  *nsL = b->alg.L_alg.nstages * b->alg.L_alg.nsub;
  const int nsS = b->alg.S_alg.nstages * b->alg.S_alg.nsub;
  const int lim = lri::adjoint_max_stages();
  if (*nsK > lim || *nsL > lim || nsS > lim) return LRI_ERR_UNSUPPORTED;
  return LRI_OK;
}

lri_status lri_batch_adjoint_prepare(lri_batch* b) {
  if (!b) return LRI_ERR_ARG;
  int nsK = 0, nsL = 0;
  const lri_status ok = adjoint_supported(b, &nsK, &nsL);
  if (ok != LRI_OK) return ok;
  if (b->d_adj_work) return LRI_OK;  // the stage counts are fixed at create time
  const int count = b->desc.count;
  std::vector<int64_t> off(count), th(count);
  int64_t tot = 0, toth = 0;
  for (int i = 0; i < count; ++i) {
    off[i] = tot;
    tot += ((int64_t)lri::adjoint_work_elems(b->n[i], b->m[i], b->rcap[i], nsK, nsL) + 3) & ~int64_t(3);
    th[i] = toth;
    toth += b->n[i];
  }
  cudaError_t e = cudaMalloc((void**)&b->d_adj_work, sizeof(double) * (size_t)tot);
  if (e == cudaSuccess) e = cudaMalloc((void**)&b->d_adj_off, sizeof(int64_t) * count);
  if (e == cudaSuccess) e = cudaMalloc((void**)&b->d_th_off, sizeof(int64_t) * count);
  if (e == cudaSuccess)
    e = cudaMemcpy(b->d_adj_off, off.data(), sizeof(int64_t) * count, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(b->d_th_off, th.data(), sizeof(int64_t) * count, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    cudaFree(b->d_adj_work);
    cudaFree(b->d_adj_off);
    cudaFree(b->d_th_off);
    b->d_adj_work = nullptr;
    b->d_adj_off = b->d_th_off = nullptr;
    return LRI_ERR_CUDA;
  }
  return LRI_OK;
}

lri_status lri_batch_adjoint_step(lri_batch* b, double dt, const void* U0, const void* S0, const void* V0, void* Ubar,
                                  void* Sbar, void* Vbar, void* theta_bar, void* stream) {
  if (!b || !U0 || !S0 || !V0 || !Ubar || !Sbar || !Vbar || !theta_bar || !std::isfinite(dt)) return LRI_ERR_ARG;
  if (!b->bound) return LRI_ERR_STATE;
  int nsK = 0, nsL = 0;
  const lri_status ok = adjoint_supported(b, &nsK, &nsL);
  if (ok != LRI_OK) return ok;
  if (!b->d_adj_work) return LRI_ERR_STATE;  // lri_batch_adjoint_prepare allocates the workspace
  const int count = b->desc.count;
  return cuda_status(lri::launch_adjoint_step(
      b->d_inst, b->d_adj_off, b->d_th_off, count, static_cast<const double*>(U0), static_cast<const double*>(S0),
      static_cast<const double*>(V0), static_cast<double*>(Ubar), static_cast<double*>(Sbar),
      static_cast<double*>(Vbar), static_cast<double*>(theta_bar), static_cast<const double*>(b->opA),
      static_cast<const double*>(b->opB), b->d_adj_work, to_scheme(b->alg.K_alg), to_scheme(b->alg.L_alg),
      to_scheme(b->alg.S_alg), dt, (cudaStream_t)stream));
}

// ---------------------------------------------------------------------------
// Solution history: the reference deep-copies the factors into its solution
// after every step (update_sol!, src/primitives.jl:82-90).  Here every
// record is a device-to-device copy into a ring slot on the caller's stream
// and a copy of that slot to host memory on the history's own stream, so the
// steps never wait for PCIe/NVLink-C2C transfers.
// ---------------------------------------------------------------------------
struct lri_history {
  lri_batch* b = nullptr;
  int slots = 0;
  size_t bytesU = 0, bytesS = 0, bytesV = 0, bytesR = 0;
  std::vector<void*> d;               // per slot: U | S | V | ranks (one allocation)
  std::vector<cudaEvent_t> ready;     // the slot's device copy is done
  std::vector<cudaEvent_t> done;      // the slot's host copy is done
  std::vector<int64_t> slot_seq;
  cudaStream_t copy = nullptr;
  int64_t next = 0;
};

extern "C" {

lri_status lri_history_destroy(lri_history* h) {
  if (!h) return LRI_ERR_ARG;
  if (h->copy) cudaStreamSynchronize(h->copy);
  for (void* p : h->d) cudaFree(p);
  for (cudaEvent_t e : h->ready) if (e) cudaEventDestroy(e);
  for (cudaEvent_t e : h->done) if (e) cudaEventDestroy(e);
  if (h->copy) cudaStreamDestroy(h->copy);
  delete h;
  return LRI_OK;
}

lri_status lri_history_create(lri_history** out, lri_batch* b, int32_t slots) {
  if (!out || !b || slots < 1 || slots > 1024) return LRI_ERR_ARG;
  *out = nullptr;
  lri_history* h = new lri_history();
  h->b = b;
  h->slots = slots;
  const size_t es = b->desc.dtype == LRI_F32 ? 4 : 8;  // double-float batches expose FP64 factors
  auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
  h->bytesU = es * (size_t)b->totU;
  h->bytesS = es * (size_t)b->totS;
  h->bytesV = es * (size_t)b->totV;
  h->bytesR = sizeof(int32_t) * (size_t)b->desc.count;
  const size_t per = al(h->bytesU) + al(h->bytesS) + al(h->bytesV) + al(h->bytesR);
  h->d.assign(slots, nullptr);
  h->ready.assign(slots, nullptr);
  h->done.assign(slots, nullptr);
  h->slot_seq.assign(slots, -1);
  cudaError_t e = cudaStreamCreateWithFlags(&h->copy, cudaStreamNonBlocking);
  for (int i = 0; i < slots && e == cudaSuccess; ++i) {
    e = cudaMalloc(&h->d[i], per);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->ready[i], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->done[i], cudaEventDisableTiming);
  }
  if (e != cudaSuccess) {
    lri_history_destroy(h);
    return LRI_ERR_CUDA;
  }
  *out = h;
  return LRI_OK;
}

lri_status lri_history_record(lri_history* h, void* hostU, void* hostS, void* hostV, int32_t* host_ranks, void* stream,
                              int64_t* seq) {
  if (!h || !hostU || !hostS || !hostV) return LRI_ERR_ARG;
  lri_batch* b = h->b;
  if (!b->bound) return LRI_ERR_STATE;
  cudaStream_t st = (cudaStream_t)stream;
  const int slot = (int)(h->next % h->slots);
  auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
  unsigned char* base = static_cast<unsigned char*>(h->d[slot]);
  unsigned char* sU = base;
  unsigned char* sS = sU + al(h->bytesU);
  unsigned char* sV = sS + al(h->bytesS);
  unsigned char* sR = sV + al(h->bytesV);
  // the slot's previous host copy must have finished before it is overwritten
  if (h->slot_seq[slot] >= 0) LRI_CUDA(cudaStreamWaitEvent(st, h->done[slot], 0));
  LRI_CUDA(cudaMemcpyAsync(sU, b->U, h->bytesU, cudaMemcpyDeviceToDevice, st));
  LRI_CUDA(cudaMemcpyAsync(sS, b->S, h->bytesS, cudaMemcpyDeviceToDevice, st));
  LRI_CUDA(cudaMemcpyAsync(sV, b->V, h->bytesV, cudaMemcpyDeviceToDevice, st));
  LRI_CUDA(cudaMemcpyAsync(sR, b->d_rank, h->bytesR, cudaMemcpyDeviceToDevice, st));
  LRI_CUDA(cudaEventRecord(h->ready[slot], st));
  LRI_CUDA(cudaStreamWaitEvent(h->copy, h->ready[slot], 0));
  LRI_CUDA(cudaMemcpyAsync(hostU, sU, h->bytesU, cudaMemcpyDeviceToHost, h->copy));
  LRI_CUDA(cudaMemcpyAsync(hostS, sS, h->bytesS, cudaMemcpyDeviceToHost, h->copy));
  LRI_CUDA(cudaMemcpyAsync(hostV, sV, h->bytesV, cudaMemcpyDeviceToHost, h->copy));
  if (host_ranks) LRI_CUDA(cudaMemcpyAsync(host_ranks, sR, h->bytesR, cudaMemcpyDeviceToHost, h->copy));
  LRI_CUDA(cudaEventRecord(h->done[slot], h->copy));
  h->slot_seq[slot] = h->next;
  if (seq) *seq = h->next;
  ++h->next;
  return LRI_OK;
}

lri_status lri_history_wait(lri_history* h, int64_t seq) {
  if (!h || seq < 0 || seq >= h->next) return LRI_ERR_ARG;
  // a later record of the same slot completes after this one (one copy stream)
  const int slot = (int)(seq % h->slots);
  LRI_CUDA(cudaEventSynchronize(h->done[slot]));
  return LRI_OK;
}

}  // extern "C"
