/*
 * lri.h - C ABI of the GB300 (sm_103a) engine for the per-step hot path of
 * dynamical low-rank approximation (DLRA): the K/L/S substeps of the
 * unconventional "BUG" integrator, its rank-adaptive variant and the
 * projector-splitting (KSL) integrator of LowRankIntegrators.jl.
 *
 * Conventions
 *   - Every matrix is column-major (Julia's layout).  A batch holds `count`
 *     independent problems ("instances") of uneven sizes; instance i owns an
 *     n_i x r_cap_i block of U, an r_cap_i x r_cap_i block of S and an
 *     m_i x r_cap_i block of V inside caller-owned packed device buffers.
 *     `lri_batch_layout` returns the element offsets; only the leading
 *     r_i columns (r_i = current rank) are meaningful.
 *   - Device buffers are passed as raw pointers and stay owned by the caller.
 *     The library allocates its own workspace once, in lri_batch_create; the
 *     step calls allocate nothing.
 *   - A handle is not thread-safe: use one per host thread / stream.
 *   - Errors are returned as lri_status; kernel-side failures (non-finite
 *     values, SVD non-convergence, rank overflow) are accumulated in a device
 *     status word read by lri_batch_status().
 *   - There is no CPU fallback: without a usable CUDA device every entry point
 *     that computes returns LRI_ERR_CUDA.
 *
 * Reference interfaces replaced (paths are within LowRankIntegrators.jl):
 *   MatrixDEProblem / MatrixDataProblem        src/primitives.jl:13-30
 *   init(prob, alg, dt)                         src/integrators/unconventional.jl:109-119,
 *                                               src/integrators/rank_adaptive_unconventional.jl:94-104,
 *                                               src/integrators/projector_splitting.jl:107-115
 *   step!(integrator, alg, dt)                  src/integrators/unconventional.jl:159-164,
 *                                               src/integrators/rank_adaptive_unconventional.jl:171-180,
 *                                               src/integrators/projector_splitting.jl:191-211
 *   set_u!/step! of the substep integrators     src/integrators/unconventional.jl:138-139,146-147,154-155
 *   update_data! + Δy for data problems         src/integrators/data_integrator.jl:22-28,
 *                                               src/integrators/unconventional.jl:121-127
 */
#ifndef LRI_H
#define LRI_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define LRI_API __attribute__((visibility("default")))
#else
#define LRI_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define LRI_ABI_VERSION 1

typedef enum {
  LRI_OK = 0,
  LRI_ERR_ARG = 1,           /* invalid argument (null pointer, bad size, bad enum) */
  LRI_ERR_UNSUPPORTED = 2,   /* combination not provided by the engine */
  LRI_ERR_BREAKDOWN = 3,     /* SVD did not converge */
  LRI_ERR_NONFINITE = 4,     /* NaN/Inf appeared in a factor */
  LRI_ERR_RANK_OVERFLOW = 5, /* rank-adaptive step needed more than r_cap */
  LRI_ERR_TIMEOUT = 6,       /* a bounded device wait gave up */
  LRI_ERR_CUDA = 7,          /* CUDA runtime error or no device */
  LRI_ERR_STATE = 8          /* call out of order (e.g. step before bind) */
} lri_status;

/* Precision of a batch.
 *   LRI_F64  plain FP64: buffers and arithmetic in double.
 *   LRI_F32  fast form: buffers and arithmetic in float.
 *   LRI_DF   double-float: buffers in double at the ABI, arithmetic on the
 *            FP32 units with 48-bit (hi+lo float pair) significands.  The
 *            engine keeps its own double-float copy of the factors: it is
 *            loaded by lri_batch_bind and written back to the caller's
 *            buffers at the end of every lri_batch_step call. */
typedef enum { LRI_F64 = 0, LRI_F32 = 1, LRI_DF = 2 } lri_dtype;

/* Algorithms: UnconventionalAlgorithm (unconventional.jl:13-21),
 * RankAdaptiveUnconventionalAlgorithm (rank_adaptive_unconventional.jl:15-23),
 * ProjectorSplitting (projector_splitting.jl:27-41),
 * GreedyIntegrator (greedy_integrator.jl:17-24; fixed rank):
 *   two_factor = 0, op DATA: SVD-like factors, U = Q of qr(X V),
 *       V = Q of qr(X^T U), S = U^T X V (greedy_integrator.jl:96-104);
 *   two_factor = 1, op DATA: u = U Z^T with Z in the V buffer (S unused):
 *       Z = X^T U, U = polar factor of X Z (:84-94);
 *   two_factor = 1, op ZERO / SYLVESTER / BURGERS: MatrixHybridProblem
 *       (primitives.jl:36-41): Z advanced over [t, t+dt] by the L-substep
 *       flow Z' = F(U Z^T)^T U of the operator (the reference's coefficient
 *       ODE f(Z, U, t) for a flow map F) with the L_alg scheme, then
 *       U = polar factor of X Z (:73-82).
 *   X = y(t+dt) is the snapshot passed to every lri_batch_step call. */
typedef enum { LRI_ALG_BUG = 0, LRI_ALG_RA_BUG = 1, LRI_ALG_KSL = 2, LRI_ALG_GREEDY = 3 } lri_alg_kind;
typedef enum { LRI_KSL_PRIMAL = 0, LRI_KSL_DUAL = 1, LRI_KSL_STRANG = 2 } lri_ksl_order;

/* Flow maps.  The reference accepts any Julia closure F(Y,t) evaluated by
 * LowRankArithmetic; the engine accepts this fixed menu (no closures):
 *   ZERO        F = 0
 *   SYLVESTER   F(X) = A X + X B^T, A (n x n) and B (m x m) tridiagonal,
 *               each stored as three vectors [sub | diag | sup] (sub[0] and
 *               sup[last] unused).  diag(theta) X terms fold into A's diagonal.
 *   BURGERS     F(X) = (Dxx X) diag(nu) + alpha (Dx X).*X + beta Dx(X.*X),
 *               periodic central differences of spacing h along the n rows
 *               (h, alpha, beta in lri_batch_desc, shared by the batch);
 *               nu per column (operator B, m values).  Evaluated tile by
 *               tile on Y = K V^T without forming the n x m matrix.
 *   DATA        MatrixDataProblem: exact substep flows driven by the snapshot
 *               increment Δy = A(t+dt) - A(t) (data_integrator.jl:13-16).
 *   LOCAL_FLOW  a flow map registered in the library when it is built
 *               (csrc/flows.cuh; stands in for the reference's user-supplied
 *               F and K_rhs / L_rhs / S_rhs hooks, unconventional.jl:2-4,
 *               16-21,51-79): F(Y)_ij = f(Y_{i-1,j}, Y_ij, Y_{i+1,j}, c_j;
 *               h, p0, p1), periodic along the rows.  lri_batch_desc.flow
 *               selects it (lri_flow_count / lri_flow_name list them),
 *               burgers_h / _alpha / _beta carry h, p0, p1, operator B the
 *               per-column c (m values).  Evaluated like BURGERS, tile by
 *               tile without forming the n x m matrix.  Flow 0 is the
 *               Burgers flow; flow 1 "reaction_diffusion" is
 *               F = (Dxx Y) diag(c) + p0 Y + p1 Y.^3. */
typedef enum {
  LRI_OP_ZERO = 0,
  LRI_OP_SYLVESTER_TRIDIAG = 1,
  LRI_OP_BURGERS_PERIODIC = 2,
  LRI_OP_DATA = 3,
  LRI_OP_LOCAL_FLOW = 4
} lri_op_kind;

/* Fixed-step explicit Runge-Kutta substep scheme with a sub-diagonal Butcher
 * tableau (Euler, Heun, midpoint, classic RK4), run nsub times per substep
 * interval.  Stands in for the reference's DifferentialEquations solver
 * (default Tsit5, unconventional.jl:18). */
typedef struct {
  int32_t nstages;   /* 1..4 */
  int32_t nsub;      /* >= 1 */
  double a[4];       /* a[s]: weight of k_{s-1} in stage s input; a[0] unused */
  double b[4];
  double c[4];
} lri_scheme;

typedef struct {
  int32_t kind;        /* lri_alg_kind */
  int32_t ksl_order;   /* lri_ksl_order (KSL only) */
  lri_scheme K_alg, L_alg, S_alg;
  double tol;          /* rank-adaptive truncation tolerance (absolute) */
  int32_t r_min;       /* rank-adaptive lower bound (>= 1); no reference counterpart */
  int32_t two_factor;  /* GreedyIntegrator only: 1 = factors U Z^T (TwoFactorRepresentation) */
} lri_alg_desc;

typedef struct {
  int32_t dtype;       /* lri_dtype */
  int32_t op;          /* lri_op_kind */
  int32_t count;       /* number of instances (>= 1) */
  int32_t flow;        /* LRI_OP_LOCAL_FLOW: registered flow id; else 0 */
  const int64_t* n;      /* host [count]: rows of U */
  const int64_t* m;      /* host [count]: rows of V */
  const int64_t* r;      /* host [count]: initial rank */
  const int64_t* r_cap;  /* host [count]: capacity (rank-adaptive r_max), NULL => r */
  double burgers_h, burgers_alpha, burgers_beta;  /* BURGERS: h, alpha, beta; LOCAL_FLOW: h, p0, p1 */
} lri_batch_desc;

typedef struct lri_batch lri_batch;

/* Library / device information. */
LRI_API int lri_abi_version(void);
LRI_API const char* lri_status_str(lri_status s);
LRI_API lri_status lri_device_info(int* device, int* sm_count, int* cc_major, int* cc_minor);
/* The local flow maps compiled into the library (LRI_OP_LOCAL_FLOW): their
 * count and the name of flow id (NULL beyond the count). */
LRI_API int32_t lri_flow_count(void);
LRI_API const char* lri_flow_name(int32_t id);

/* init(prob, alg, dt): validates the shapes, plans the packed layout and
 * allocates the workspace. */
LRI_API lri_status lri_batch_create(lri_batch** out, const lri_batch_desc* desc, const lri_alg_desc* alg);
LRI_API lri_status lri_batch_destroy(lri_batch* b);

/* Element offsets of each instance inside the packed buffers (host arrays of
 * length count, any may be NULL) and the total element counts
 * totals[0..4] = {U, S, V, operator A, operator B}.  Operator A holds 3*n_i
 * elements per instance (SYLVESTER) or nothing; operator B holds 3*m_i
 * (SYLVESTER) or m_i (BURGERS: nu) elements. */
LRI_API lri_status lri_batch_layout(const lri_batch* b, int64_t* offU, int64_t* offS, int64_t* offV,
                            int64_t* offA, int64_t* offB, int64_t* totals);

/* Binds the caller's device buffers (dtype of the batch).  U, S, V hold Y0 on
 * entry and are updated in place by every step, like the reference's
 * integrator.u (unconventional.jl:151-156).  opA/opB may be NULL for ZERO and
 * DATA.  Binding resets the cached projections and ranks to the host r. */
LRI_API lri_status lri_batch_bind(lri_batch* b, void* U, void* S, void* V, const void* opA, const void* opB);

/* DATA problems: device buffer with every instance's first snapshot A(t0)
 * (packed like lri_batch_layout's "data" region: n_i x m_i column-major,
 * offsets returned by lri_batch_data_layout).  Copied into the library's
 * previous-snapshot buffer (unconventional.jl:91-93). */
LRI_API lri_status lri_batch_data_layout(const lri_batch* b, int64_t* offY, int64_t* total);
LRI_API lri_status lri_batch_data_init(lri_batch* b, const void* Y0, void* stream);

/* step!(integrator, alg, dt), nsteps times, starting at time t.  For DATA
 * problems and GreedyIntegrator batches nsteps must be 1 and Ynext points at
 * A(t+dt) for every instance (same packing as lri_batch_data_init; the
 * greedy steps need no lri_batch_data_init); for other batches Ynext is NULL.
 * Runs asynchronously on `stream` (cudaStream_t, NULL = legacy default);
 * multi-step calls run as one captured CUDA graph. */
LRI_API lri_status lri_batch_step(lri_batch* b, double t, double dt, int32_t nsteps, const void* Ynext,
                          void* stream);

/* Builds (without running) the CUDA graph that lri_batch_step uses for a
 * call with this (dt, nsteps), so the first such call does not pay for the
 * capture.  No counterpart in the reference. */
LRI_API lri_status lri_batch_prepare(lri_batch* b, double dt, int32_t nsteps);

/* Register budget of the batch's step kernel, the autotuner's knob for the
 * instance engine: 3 CTAs per SM (at most 80 registers per thread; the
 * default) or 2 (at most 128 registers: fewer spills, less latency hiding).
 * FP64 batches take 3 only.  No counterpart in the reference. */
LRI_API lri_status lri_batch_set_occupancy(lri_batch* b, int32_t ctas_per_sm);

/* Current ranks (host array of length count; synchronises the stream). */
LRI_API lri_status lri_batch_ranks(lri_batch* b, int64_t* r_out, void* stream);

/* Device status word accumulated by the kernels since the last call
 * (synchronises `stream`, then clears the word). */
LRI_API lri_status lri_batch_status(lri_batch* b, void* stream);

/* Allocation-free BUG step (no counterpart in the reference).  For callers
 * that cannot call cudaMalloc - their device memory is owned by another
 * allocator, or their time loop must not trigger the device-wide
 * synchronisation of cudaMalloc/cudaFree - this advances ONE instance of
 * F(X) = A X + X B^T (tridiagonal A, B as in LRI_OP_SYLVESTER_TRIDIAG) by
 * nsteps BUG steps with the step kernel of lri_batch_step, using a fixed
 * 4 MiB scratch array compiled into the library (held by every GPU that loads
 * it until the process exits) instead of allocated workspace.
 *   dtype   LRI_F64 or LRI_F32 (LRI_DF: LRI_ERR_UNSUPPORTED)
 *   U (n x r), S (r x r), V (m x r)  caller's device buffers, column-major,
 *           updated in place; A (3n), B (3m) device coefficient vectors
 *   Sizes whose workspace exceeds the scratch, elem_size * (5r(n+m) + 23r^2)
 *   + 256 bytes > 4 MiB (each term padded to 4 elements; for example
 *   n + m > 3120 at r = 32 in FP64), are rejected with LRI_ERR_ARG.
 * The first call on a device looks up the scratch array's device address
 * (cudaGetSymbolAddress) with that device current; make that first call
 * before any stream capture.  All calls share the one array and leave their
 * contents in it (the call clears what must start at zero), so calls whose
 * work overlaps on the GPU (other streams, other host threads) race.
 * The one scheme drives the K, L and S substeps, and the time of step k of
 * a call is k * dt (each call starts at t = 0; the Sylvester flow is
 * autonomous, so only the step count matters).  LRI_F32 is accurate to the
 * FP32 level only while kappa(S0) <= 2^21; for worse-conditioned cores use
 * LRI_F64 (the batch API's mixed form switches to double-float there).
 * status_out (host pointer, optional): when given, the call waits for its
 * steps and stores the device status mapped as lri_batch_status does
 * (LRI_OK, LRI_ERR_NONFINITE, LRI_ERR_BREAKDOWN, LRI_ERR_RANK_OVERFLOW, or
 * LRI_ERR_ARG for a shape the kernel rejected); nsteps == 0 stores LRI_OK. */
LRI_API lri_status lri_bug_step_noalloc(int32_t dtype, int64_t n, int64_t m, int64_t r, void* U, void* S, void* V,
                                        const void* A, const void* B, double dt, int32_t nsteps,
                                        const lri_scheme* scheme, void* stream, int32_t* status_out);

/* Discrete adjoint of one BUG step (no counterpart in the reference, which
 * has no differentiation; gradients of a loss of Y(T) by a reverse sweep).  For an
 * LRI_F64, LRI_ALG_BUG, LRI_OP_SYLVESTER_TRIDIAG batch at fixed rank
 * (r = r_cap) whose operator A carries a diagonal shift theta
 * (F = (A0 + diag theta) X + X B^T, A as bound):
 *   U0, S0, V0      the step's input factors (device, packed like the bound
 *                   U, S, V; e.g. saved before the step during a replay)
 *   Ubar, Sbar, Vbar in: adjoints of the step's outputs; out: adjoints of
 *                   its inputs (same packing)
 *   theta_bar       device, sum_i n_i doubles (instance i at sum_{j<i} n_j):
 *                   accumulates d loss / d theta
 * Each instance recomputes its step in stage form (RK stage inputs, both
 * QRs, basis changes, projections, S stages) and sweeps back through it;
 * the thin-QR adjoint is (Q_bar + Q copyltu(-Q_bar^T Q)) R^{-T}.  While
 * twice the instance count fits the device's SMs, each instance runs on a
 * 2-CTA thread-block cluster (the K side on one SM, the L side on another);
 * larger batches take one CTA per instance.  The
 * workspace comes from lri_batch_adjoint_prepare (LRI_ERR_STATE without it);
 * the step allocates nothing.  Schemes with nstages * nsub > 16 and other
 * batch kinds return LRI_ERR_UNSUPPORTED. */
LRI_API lri_status lri_batch_adjoint_prepare(lri_batch* b);
LRI_API lri_status lri_batch_adjoint_step(lri_batch* b, double dt, const void* U0, const void* S0, const void* V0,
                                          void* Ubar, void* Sbar, void* Vbar, void* theta_bar, void* stream);

/* ---- One large data stream on the whole GPU -------------------------------
 * Rank-adaptive BUG for a MatrixDataProblem whose n x m snapshots are too
 * large for the one-CTA-per-instance batch (the reference's
 * rankadaptive_unconventional_step! with the data substeps,
 * rank_adaptive_unconventional.jl:182-233, data_integrator.jl:13-16; the
 * snapshot stream of primitives.jl:23-30).  Every kernel spreads over the
 * whole GPU: three streaming passes over the snapshot pair per step (dY V,
 * dY^T U, dY Vhat, with dY = A(t+dt) - A(t) formed in the loader), Gram
 * reductions in FP64, single-CTA FP64 kernels for the r x r and 2r x 2r
 * work.  Uhat = [U0 | orthonormal basis of (I - U0 U0^T) dY V0] spans the
 * same space as the reference's orth([K1 | U0]).
 *   dtype   LRI_F32 or LRI_F64 (snapshots and factors)
 *   r0      initial rank, r_max <= 96 the buffers' width, tol the absolute
 *           truncation tolerance, r_min >= 1 the lower bound
 * The caller's U (n x r_max), S (r_max x r_max), V (m x r_max) hold Y0 with
 * zeros beyond rank r0 and are updated in place; the rank stays on the
 * device (lri_stream_rank reads it).  No counterpart handle in the reference
 * (its DLRIntegrator, primitives.jl:54-63). */
typedef struct lri_stream lri_stream;
LRI_API lri_status lri_stream_create(lri_stream** out, int32_t dtype, int64_t n, int64_t m, int64_t r0,
                                     int64_t r_max, double tol, int32_t r_min);
LRI_API lri_status lri_stream_destroy(lri_stream* s);
LRI_API lri_status lri_stream_bind(lri_stream* s, void* U, void* S, void* V);
/* One step from snapshot A_prev = A(t) to A_next = A(t+dt) (device, n x m,
 * column-major, dtype of the stream). */
LRI_API lri_status lri_stream_step(lri_stream* s, const void* A_prev, const void* A_next, void* stream);
/* GreedyIntegrator step on the stream's bound SVD-like factors
 * (greedy_integrator.jl:96-104): with X = A_next = y(t+dt) (n x m, the
 * stream's dtype), U = orthonormal basis of X V, V = orthonormal basis of
 * X^T U, S = U^T X V with the new bases; the rank stays.  Three passes over
 * the single snapshot (tensor cores for FP32 streams as above). */
LRI_API lri_status lri_stream_greedy_step(lri_stream* s, const void* A_next, void* stream);
LRI_API lri_status lri_stream_rank(lri_stream* s, int64_t* r_out, void* stream);
LRI_API lri_status lri_stream_status(lri_stream* s, void* stream);

/* The snapshot passes of an FP32 stream run on the tensor cores (tcgen05,
 * operands staged by TMA; dY split into TF32 hi + lo parts, 3xTF32 products
 * with FP32 accumulation) when n and m are multiples of 4 and at least 128;
 * otherwise, and for FP64 streams, on the CUDA cores.  set_tensor_cores(0)
 * selects the CUDA-core passes (LRI_ERR_UNSUPPORTED when asking for tensor
 * cores the stream cannot use).  No counterpart in the reference. */
LRI_API lri_status lri_stream_set_tensor_cores(lri_stream* s, int32_t enable);
LRI_API lri_status lri_stream_uses_tensor_cores(const lri_stream* s, int32_t* out);
/* Tile choices of the tensor-core passes (the autotuner's knobs): K splits
 * per 128-row output tile of dY X (splits_rows) and of dY^T X (splits_cols),
 * and pipeline stages (2 .. what fits in shared memory); 0 keeps the
 * automatic choice (splits filling the SMs, as many stages as fit).  No
 * counterpart in the reference. */
LRI_API lri_status lri_stream_set_pass_tiles(lri_stream* s, int32_t splits_rows, int32_t splits_cols, int32_t stages);

/* One product of the data substeps (the increments left^T dY right of
 * src/integrators/data_integrator.jl:13-16, dY = A(t+dt) - A(t) as in
 * src/integrators/unconventional.jl:121-127) with the stream's passes:
 *   trans = 0: out (n x ncols) = dY X,   X m x ncols (ld ldx)
 *   trans = 1: out (m x ncols) = dY^T X, X n x ncols
 * A_prev = A(t), A_next = A(t+dt) (n x m, column-major, the stream's
 * dtype), 1 <= ncols <= r_max; out has leading dimension ldo (the CUDA-core
 * passes need ldo = rows of out).  Uses the stream's workspace, so it must
 * not overlap a step of the same stream. */
LRI_API lri_status lri_stream_data_product(lri_stream* s, int32_t trans, const void* A_prev, const void* A_next,
                                           const void* X, int64_t ldx, int64_t ncols, void* out, int64_t ldo,
                                           void* stream);

/* One large Burgers instance (the Burgers-UQ workload: n grid points x m
 * samples too large for the batch) on the same engine: rank-adaptive BUG
 * (rank_adaptive_unconventional.jl:194-233) for LRI_OP_BURGERS_PERIODIC with
 * the given substep scheme.  The flow evaluations F(K V^T) V, F(U L^T)^T U,
 * Uhat^T F(Uhat S Vhat^T) Vhat never form the n x m matrix: the diffusion
 * term is (Dxx K)(V^T diag(nu) V), the quadratic terms are Khatri-Rao
 * products with the symmetric tensor sum_j v_j (x) v_j (x) v_j built once per
 * step (likewise for the L and S substeps).  r_max <= 64.  bind: the
 * caller's U, S, V (as lri_stream_bind) and nu (m viscosities, device).
 * lri_burgers_step with nsteps > 1 runs the first step, captures one step
 * as a CUDA graph and replays it (kept while dt and the binding stay).
 * Destroy with lri_stream_destroy; rank and status as for the stream. */
LRI_API lri_status lri_burgers_create(lri_stream** out, int32_t dtype, int64_t n, int64_t m, int64_t r0,
                                      int64_t r_max, double tol, int32_t r_min, double h, double alpha,
                                      double beta, const lri_scheme* scheme);
LRI_API lri_status lri_burgers_bind(lri_stream* s, void* U, void* S, void* V, const void* nu);
LRI_API lri_status lri_burgers_step(lri_stream* s, double dt, int32_t nsteps, void* stream);

/* Solution history (update_sol!, src/primitives.jl:82-90, which deep-copies
 * the factors after every step).  A history owns `slots` device copies of
 * the batch's factors and ranks and a copy stream of its own.
 * lri_history_record queues, on `stream` after the work already queued
 * there, a device-to-device copy of the bound U, S, V and the ranks into the
 * next slot, then (on the history's stream) the copy of that slot into the
 * caller's host buffers: U, S, V packed like the bound buffers in the
 * batch's dtype (FP64 for double-float batches), ranks as int32 per
 * instance (optional).  The host buffers should be page-locked for the copy
 * to overlap the next steps, and must stay valid until lri_history_wait
 * returns for the record.  When a slot comes round again, `stream` first
 * waits for its previous host copy.  *seq receives the record's number
 * (0, 1, ...).  lri_history_wait blocks the calling thread until record seq
 * is on the host.  No counterpart in the reference's API. */
typedef struct lri_history lri_history;
LRI_API lri_status lri_history_create(lri_history** out, lri_batch* b, int32_t slots);
LRI_API lri_status lri_history_destroy(lri_history* h);
LRI_API lri_status lri_history_record(lri_history* h, void* hostU, void* hostS, void* hostV, int32_t* host_ranks,
                                      void* stream, int64_t* seq);
LRI_API lri_status lri_history_wait(lri_history* h, int64_t seq);

/* Number of kernel launches a single-step lri_batch_step call makes. */
LRI_API int32_t lri_batch_launches_per_step(const lri_batch* b);

#ifdef __cplusplus
}
#endif

#endif /* LRI_H */
