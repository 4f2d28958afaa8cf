"""Benchmark: batched BUG steps/sec on the 4096-instance Lyapunov ensemble,
followed (N = 1) by the other workloads in the same JSON line.

Headline workload (one "step" = one BUG step of every instance, one kernel
launch per precision class):
  4096 independent F_i(X) = A_i X + X B_i^T, n_i, m_i ~ U{64..1024},
  r_i ~ U{4..32}, tridiagonal A_i, B_i, X0_i with spectrum 2^-k (seed 4),
  dt = 1e-2, RK4 substeps (nsub = 1), mixed form (FP32 for well-conditioned
  cores, double-float for the others); the plain FP64 form runs the same
  steps for the speed ratio and the accuracy check.

``workloads`` (N = 1, unless --no-legs): the 256 x 256 Laplacian flow (FP64,
1000 steps), the 8192 x 4096 data-compression stream (rank-adaptive, FP32),
the 4096 x 16384 Burgers-UQ instance (rank 16..64) and the 2048 x 2048
discrete-adjoint sweep with its finite-difference check, each with its own
timing, clocks, accuracy and CPU sample.  --laplace / --stream / --burgers /
--adjoint print one of them alone.

Prints one JSON line (rank 0).  ``--impl reference`` times the CPU
restatement of the reference integrator on the host cores instead.
"""
from __future__ import annotations

import argparse
import json
import math
import multiprocessing as mp
import os
import statistics
import subprocess
import tempfile
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "lowrankintegrators.jl_gb300"))

METRIC = "BUG steps/sec @ <=1e-5 rel. Frobenius err vs FP64 (batched Lyapunov ensemble, 4096 instances)"
UNIT = "batched steps/s"
DT = 1e-2
NSUB = 1


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), float(p["bf16_tflops"]), "measured"
    except Exception:
        return 6800.0, 1900.0, "fallback"


# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per instance and
# step of each class's step kernel, from an ncu capture of the 1024-instance
# slice of this ensemble (655 FP32-class and 369 double-float-class
# instances: 0.2596 GB and 1.7816 GB per steady launch of step_kernel<T, 3>);
# scaled by the instance counts.
TRAFFIC_PER_INSTANCE = {"fp32": 0.2596e9 / 655, "df": 1.7816e9 / 369}


def algorithmic(shapes, nsub=NSUB, esize=4):
    """Per batched step: compulsory DRAM bytes (factors and operators read,
    factors written) and algorithmic flops of the implemented BUG step."""
    n, m, r = (np.asarray(x, np.float64) for x in shapes)
    nm = n + m
    bytes_ = np.sum((2 * nm * r + 2 * r * r + 3 * nm) * esize)
    flops = np.sum((12 + 16 * nsub) * nm * r * r + (36 * nsub + 5) * nm * r + (4 + 32 * nsub) * r ** 3)
    return float(bytes_), float(flops)


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during a region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index=0):
        self.dev = device_index
        self.proc = None
        self.path = os.path.join(tempfile.gettempdir(), f"lri_clocks_{os.getpid()}.csv")

    def __enter__(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.dev}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                p = [x.strip() for x in line.split(",")]
                if len(p) < 9:
                    continue
                try:
                    sm.append(float(p[1]))
                    smax.append(float(p[2]))
                except ValueError:
                    continue
                for nm, v in zip(names, p[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------------
# CPU baseline: the oracle (FP64 restatement of the reference integrator),
# one process per host core over a bounded sample of instances.
# ---------------------------------------------------------------------------

def _pool_init():
    os.environ["OPENBLAS_NUM_THREADS"] = "1"
    os.environ["OMP_NUM_THREADS"] = "1"


def _cpu_worker(args):
    idx, steps, warmup, count = args
    os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")
    import workloads
    from oracle import lri_oracle as O
    integs = []
    for i in idx:
        e = workloads.lyapunov_ensemble(count=count, first=i, limit=1)[0]
        p = O.MatrixDEProblem(O.SylvesterTridiagOp(e.A, e.B), O.SVDLikeRepresentation(e.U, e.S, e.V),
                              (0.0, DT * (steps + warmup)))
        integs.append(O.init(p, O.UnconventionalAlgorithm(O.RK4(NSUB)), DT))
    for _ in range(warmup):
        for integ in integs:
            O.step(integ, integ.alg, DT)
    t0 = time.perf_counter()
    for _ in range(steps):
        for integ in integs:
            O.step(integ, integ.alg, DT)
    return time.perf_counter() - t0


def _oracle_finals(args):
    """The oracle's factors (dense) after `steps` steps of each instance."""
    idx, steps, count = args
    import workloads
    from oracle import lri_oracle as O
    out = []
    for i in idx:
        e = workloads.lyapunov_ensemble(count=count, first=i, limit=1)[0]
        p = O.MatrixDEProblem(O.SylvesterTridiagOp(e.A, e.B), O.SVDLikeRepresentation(e.U, e.S, e.V),
                              (0.0, DT * steps))
        integ = O.init(p, O.UnconventionalAlgorithm(O.RK4(NSUB)), DT)
        for _ in range(steps):
            O.step(integ, integ.alg, DT)
        out.append((i, integ.u.full()))
    return out


def cpu_baseline(count, sample_every, steps, warmup=0, cores=None):
    """The oracle on every `sample_every`-th instance of the ensemble, one
    process per host core: `warmup` untimed steps, then `steps` timed steps
    of every sampled instance.  Returns (batched steps/s extrapolated to
    `count` instances, cores, description of the sample, timed steps)."""
    cores = cores or os.cpu_count() or 1
    sample = list(range(0, count, sample_every))
    chunks = [sample[k::cores] for k in range(cores)]
    chunks = [c for c in chunks if c]
    ctx = mp.get_context("spawn")
    t0 = time.perf_counter()
    with ctx.Pool(len(chunks), initializer=_pool_init) as pool:
        busy = pool.map(_cpu_worker, [(c, steps, warmup, count) for c in chunks])
    wall = time.perf_counter() - t0
    # instance-steps per second of the whole pool, scaled to the full ensemble
    inst_steps = len(sample) * steps
    per_inst_step = sum(busy) / inst_steps            # core-seconds per instance-step
    batched_per_s = len(chunks) / (per_inst_step * count)
    desc = (f"{len(sample)} of {count} instances (every {sample_every}th), {warmup} untimed + {steps} timed "
            f"steps of each, {len(chunks)} processes, {wall:.1f} s wall; the ensemble's step time is the "
            f"sample's core-seconds per instance-step x {count} / {len(chunks)} cores")
    return batched_per_s, len(chunks), desc


# ---------------------------------------------------------------------------


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if ws > 1:
        import torch
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
        pg = dist
    return ws, rank, local, pg


def rank_barrier(dist):
    if dist is not None:
        dist.barrier()


def rank_max(x: float, dist) -> float:
    """Maximum of x over the ranks (the slowest rank's time)."""
    if dist is None:
        return x
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def weak_value(ws: int, steps: int, seconds: float) -> float:
    """Whole-job batched steps/s: every rank advances its own ensemble by
    ``steps`` steps; the job takes the slowest rank's time."""
    return ws * steps / seconds


def run_reference(args, ws, rank):
    """The reference arm: the oracle (the NumPy FP64 restatement of the
    reference integrator; Julia is not available) on the host cores, W
    untimed and K timed steps of every 64th ensemble member, extrapolated to
    the 4096-instance ensemble."""
    if rank != 0:
        return
    val, cores, desc = cpu_baseline(args.count, args.cpu_sample_every, args.steps, args.warmup)
    line = {"impl": "reference", "metric": METRIC, "value": val, "unit": UNIT, "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 / val, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "lyapunov_ensemble_4096", "instances": args.count, "dt": DT,
                       "scheme": f"RK4(nsub={NSUB})", "algorithm": "BUG",
                       "instances_timed": len(range(0, args.count, args.cpu_sample_every)),
                       "steps_timed": args.steps},
            "cpu_baseline": {"value": val, "unit": UNIT, "cores": cores, "kind": "port", "sample": desc},
            "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def leg_stream(steps, warmup):
    """The data-compression workload on one GPU: n = 8192, m = 4096 FP32
    snapshots of the rotating-mode stream (500 on [0, 1], generated on the
    device), rank-adaptive BUG with tol 1e-6 and r <= 96 from the rank-64
    noise-free part of A(0), on the large-stream engine.  W warm-up steps, then
    K timed steps (snapshots resident in HBM); accuracy of 3 steps against the
    FP64 oracle on the same snapshots; the oracle's step timed on the host."""
    import torch
    import __graft_entry__ as ge
    import workloads
    from oracle import lri_oracle as O
    lri = ge.load_package()
    n, m, nsnap, R, tol = 8192, 4096, 500, 96, 1e-6
    K, W = min(steps, nsnap - 1 - warmup), warmup
    snap = workloads.data_stream_device(n, m, nsnap)
    A = [snap(j) for j in range(W + K + 1)]
    torch.cuda.synchronize()
    Us, ss, Vs = snap.signal0  # Y0: the rank-64 noise-free part of A(0)
    Y0 = lri.SVDLikeRepresentation(Us, np.diag(ss), Vs)
    eng = lri.DataStreamEngine(n, m, 64, R, tol, 1, "fp32")
    eng.bind(Y0)
    for j in range(W):
        eng.step(A[j], A[j + 1])
    eng.check_status()
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    sampler = ClockSampler(torch.cuda.current_device())
    sampler.__enter__()
    e0.record(stream)
    for j in range(W, W + K):
        eng.step(A[j], A[j + 1])
    e1.record(stream)
    torch.cuda.synchronize()
    sampler.__exit__()
    ms = e0.elapsed_time(e1) / K
    eng.check_status()
    rank_end = eng.rank()
    tc_used = eng.uses_tensor_cores()
    eng_tiles = eng.tuning or {"shape": None, "note": "automatic: K splits filling the SMs, as many stages as fit"}

    # the dominant kernel: one snapshot pass (dY X, dY^T X with 96 columns)
    # timed alone, on the tensor cores and on the CUDA cores
    def time_pass(trans, tc, reps=20):
        eng.set_tensor_cores(tc)
        X = torch.randn((n if trans else m) * R, dtype=torch.float32, device=A[0].device)
        out = eng.data_product(A[0], A[1], X, trans=trans)
        f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        f0.record(stream)
        for j in range(reps):  # alternate snapshot pairs: 268 MB per pass, more than L2
            eng.data_product(A[j % 4], A[j % 4 + 1], X, trans=trans, out=out)
        f1.record(stream)
        torch.cuda.synchronize()
        return f0.elapsed_time(f1) / reps
    pass_ms = {}
    if tc_used:
        pass_ms["tensor_cores"] = {"dY_X_ms": time_pass(False, True), "dYt_X_ms": time_pass(True, True)}
    pass_ms["cuda_cores"] = {"dY_X_ms": time_pass(False, False), "dYt_X_ms": time_pass(True, False)}
    # the same steps with the CUDA-core passes, for comparison (same warm-up)
    eng.set_tensor_cores(False)
    eng.bind(Y0)
    for j in range(W):
        eng.step(A[j], A[j + 1])
    torch.cuda.synchronize()
    e0.record(stream)
    for j in range(W, W + K):
        eng.step(A[j], A[j + 1])
    e1.record(stream)
    torch.cuda.synchronize()
    ms_cuda_core = e0.elapsed_time(e1) / K
    eng.set_tensor_cores(tc_used)
    eng.check_status()
    # e2e: every snapshot from pinned host memory (the first two inside the
    # timed region), the rank read back after every step; the snapshot two
    # steps ahead is copied on a second stream while the current step runs
    # (a ring of three device buffers)
    nE = max(1, min(K, 8))
    hostA = [A[j].cpu().pin_memory() for j in range(nE + 1)]
    dA = [torch.empty_like(A[0]) for _ in range(3)]
    copy_stream = torch.cuda.Stream()
    eng.bind(Y0)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    dA[0].copy_(hostA[0], non_blocking=True)
    dA[1].copy_(hostA[1], non_blocking=True)
    landed = [None, None, None]
    for j in range(nE):
        if j + 2 <= nE:  # the slot of snapshot j + 2 was last read by step j - 1
            copy_stream.wait_stream(stream)
            with torch.cuda.stream(copy_stream):
                dA[(j + 2) % 3].copy_(hostA[j + 2], non_blocking=True)
                landed[(j + 2) % 3] = torch.cuda.Event()
                landed[(j + 2) % 3].record(copy_stream)
        if landed[(j + 1) % 3] is not None:
            stream.wait_event(landed[(j + 1) % 3])
        eng.step(dA[j % 3], dA[(j + 1) % 3])
        eng.rank()
    e2e_s = (time.perf_counter() - t0) / nE
    Yg = eng.download()  # after nE steps
    eng.close()
    # accuracy vs the FP64 oracle (the same nE steps from the same Y0), and the oracle's step time
    snaps64 = [a.double().cpu().numpy().T.copy() for a in hostA]
    Y0o = O.SVDLikeRepresentation(Y0.U, Y0.S, Y0.V)
    t0 = time.perf_counter()
    so = O.solve(O.MatrixDataProblem(snaps64, Y0o), O.RankAdaptiveUnconventionalAlgorithm(tol, rmax=R),
                 save_everystep=False)
    cpu_step = (time.perf_counter() - t0) / nE
    Yo = so.Y[-1]
    # relative Frobenius error without forming n x m: ||Y_g - Y_o||^2 from the factors
    def gram_fro(a, b):
        return np.trace((a.U.T @ b.U) @ b.S @ (b.V.T @ a.V) @ a.S.T)
    d2 = gram_fro(Yg, Yg) - 2 * gram_fro(Yg, Yo) + gram_fro(Yo, Yo)
    err = float(np.sqrt(max(d2, 0.0) / gram_fro(Yo, Yo)))
    hbm, bf16, src = peaks()
    alg_bytes = 2 * 2 * n * m * 4
    pass_bytes = 2 * n * m * 4  # one pass reads both snapshots once
    kern = pass_ms.get("tensor_cores", pass_ms["cuda_cores"])
    t_pass = 0.5 * (kern["dY_X_ms"] + kern["dYt_X_ms"]) * 1e-3
    achieved = pass_bytes / t_pass / 1e9
    for v in pass_ms.values():
        v["GB_per_s"] = pass_bytes / (0.5 * (v["dY_X_ms"] + v["dYt_X_ms"]) * 1e-3) / 1e9
    flops_pass = 2.0 * n * m * R
    line = {"metric": "rank-adaptive BUG steps/s (8192x4096 FP32 data stream, r <= 96)", "value": 1e3 / ms,
            "unit": "steps/s", "n_gpus": 1, "steps": K, "warmup": W, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (device-generated stream)",
            "config": {"workload": "data_stream_8192x4096", "snapshots": nsnap, "tol": tol, "r_max": R, "r0": 64,
                       "rank_after": rank_end, "l2": "inputs larger than L2 (134 MB per snapshot)"},
            "accuracy": {"steps": nE, "rel_fro_vs_fp64_oracle": err, "rank_gpu": Yg.S.shape[0],
                         "rank_oracle": Yo.S.shape[0]},
            "passes": pass_ms,
            "pass_tiles": eng_tiles,
            "ms_per_step_cuda_core_passes": ms_cuda_core,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                         "traffic": None, "peak_source": src,
                         "kernel": "tc_pass_kernel (tcgen05 + TMA, 3xTF32)" if tc_used else "pass_rows/pass_cols",
                         "algorithmic_bytes_per_launch": pass_bytes,
                         "tensor_tflops": flops_pass * 3 / t_pass / 1e12,
                         "note": "one snapshot pass (both snapshots read once, 96 columns), mean of dY X and dY^T X, "
                                 "CUDA events around the whole call (TF32 split of the panel, the pass, the "
                                 "split-K sum); a step makes three passes (dY V0, dY^T U0, dY Q_V), "
                                 "step-level bytes %.0f MB / %.3f ms = %.0f GB/s"
                                 % (alg_bytes / 1e6, ms, alg_bytes / (ms * 1e-3) / 1e9)},
            "gpu_launches": None,
            "clocks": sampler.summary(),
            "cpu_baseline": {"value": 1.0 / cpu_step, "unit": "steps/s", "cores": os.cpu_count(), "kind": "port",
                             "sample": f"{nE} oracle steps at full size (NumPy FP64, threaded BLAS)"},
            "e2e": {"value": 1.0 / e2e_s, "unit": "steps/s", "h2d_bytes_per_step": (nE + 1) * n * m * 4 / nE,
                    "d2h_bytes_per_step": 8, "steps": nE}}
    return line


FP32_FFMA_TFLOPS = 74.6  # FP32 FMA-loop probe on a GB300 (152 SMs at 2070 MHz)


def leg_burgers(steps, warmup):
    """The Burgers-UQ workload on one GPU: u_t + (u^2/2)_x = nu u_xx,
    periodic, n = 4096 grid points, m = 16384 samples (nu_j ~ U[0.005, 0.02],
    u0_j = sin 2 pi x + a_j sin(4 pi x + phi_j)), rank-adaptive BUG with
    rmin = 16, rmax = 64, tol = 1e-4, dt = 1e-4, FP32 panels, on the large
    Burgers engine from the exact rank-3 initial data (padded to 16).  The
    diffusion term is stiff (4 nu / h^2 = 1.34e6, dt * lambda = 134), so the
    substeps are RK4 with 64 substeps (dt * lambda / 64 = 2.1, inside RK4's
    stability interval of 2.78; the reference's adaptive Tsit5 takes steps of
    that size too).  W warm-up steps, then K timed steps; the same at a fixed
    rank 64 (rmin = rmax) for the upper end of the rank range; accuracy of 3
    steps against the FP64 engine at full size (whose oracle parity the tests
    check at smaller sizes); the oracle's step timed on a bounded sample."""
    import torch
    import __graft_entry__ as ge
    import workloads
    from oracle import lri_oracle as O
    lri = ge.load_package()
    n, m, r0, R, tol, dt, nsub = 4096, 16384, 16, 64, 1e-4, 1e-4, 64
    K, W = steps, warmup
    h, nu, U0, s0, V0 = workloads.burgers_uq_factors(n, m, r0)
    Y0 = lri.SVDLikeRepresentation(U0, np.diag(s0), V0)
    op = lri.BurgersOperator(h, nu, alpha=0.0, beta=-0.5)
    stream = torch.cuda.current_stream()

    def timed(rmin, k, w, precision="fp32", sample=False):
        eng = lri.BurgersLargeEngine(op, n, m, r0 if rmin < R else R, R, tol, lri.RK4(nsub), rmin, precision)
        if rmin < R:
            eng.bind(Y0)
        else:  # rank 64 from the start: Y0 padded with zero directions
            _, _, U64, s64, V64 = workloads.burgers_uq_factors(n, m, R)
            eng.bind(lri.SVDLikeRepresentation(U64, np.diag(s64), V64))
        eng.advance(dt, w)
        eng.check_status()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        sampler = ClockSampler(torch.cuda.current_device()) if sample else None
        if sampler:
            sampler.__enter__()
        e0.record(stream)
        eng.advance(dt, k)
        e1.record(stream)
        torch.cuda.synchronize()
        if sampler:
            sampler.__exit__()
        eng.check_status()
        rank = eng.rank()
        y = eng.download()
        eng.close()
        return e0.elapsed_time(e1) / k, rank, (sampler.summary() if sampler else None), y

    ms, rank_end, clocks, _ = timed(16, K, W, sample=True)
    ms64, _, _, _ = timed(R, 3, 1)
    # accuracy: 3 steps in FP32 against the same 3 steps in FP64 (full size)
    _, _, _, y32 = timed(16, 1, 2)
    ms_f64, _, _, y64 = timed(16, 1, 2, precision="fp64")

    def gram_fro(a, b):
        return np.trace((a.U.T @ b.U) @ b.S @ (b.V.T @ a.V) @ a.S.T)
    d2 = gram_fro(y32, y32) - 2 * gram_fro(y32, y64) + gram_fro(y64, y64)
    err = float(np.sqrt(max(d2, 0.0) / gram_fro(y64, y64)))
    # e2e through the public solve: factors from host memory, every step's
    # factors back to the host (save_everystep), K steps
    kE = max(1, K)
    prob = lri.MatrixDEProblem(op, Y0, (0.0, kE * dt))
    alg = lri.RankAdaptiveUnconventionalAlgorithm(tol, rmax=R, K_alg=lri.RK4(nsub), rmin=16)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    sol_e2e = lri.solve_burgers_large(prob, alg, dt, save_everystep=True)
    e2e_s = (time.perf_counter() - t0) / kE
    d2h_e2e = 4 * (R * n + R * R + R * m)  # each step's U, S, V buffers (FP32, r_max wide)
    del sol_e2e
    # CPU: the oracle's first step on the first m_s = 2048 samples with 1 and
    # 2 RK4 substeps; the step's cost is linear in m and in the substeps, so
    # t(m, 64) = (m / m_s) (t1 + 63 (t2 - t1))
    ms_cols = 2048
    Ys = O.SVDLikeRepresentation(U0, np.diag(s0), V0[:ms_cols])
    Ys.V = np.linalg.qr(V0[:ms_cols])[0]
    tcpu = []
    for ns in (1, 2):
        po = O.MatrixDEProblem(O.BurgersOp(n, h, nu[:ms_cols], alpha=0.0, beta=-0.5), Ys.copy(), (0.0, dt))
        t0 = time.perf_counter()
        O.solve(po, O.RankAdaptiveUnconventionalAlgorithm(tol, rmax=R, K_alg=O.RK4(ns), rmin=16), dt,
                save_everystep=False)
        tcpu.append(time.perf_counter() - t0)
    cpu_step = (m / ms_cols) * (tcpu[0] + (nsub - 1) * max(tcpu[1] - tcpu[0], 0.0))

    # flops of the structured flow at active rank r (w = 2r, pairs P(k) =
    # k (k + 1) / 2), per RK stage: K substep (Dxx K) N_nu and KR(K, K) T'_V
    # (n r^2 + n P(r) r multiply-adds), L substep the same over m rows, S
    # substep A = Uhat S and Uhat^T M (2 n w^2), A_xx S N_nu (2 w^3) and
    # KR(A, A) T'_Vhat (n P(w) w); once per step the tensors T'_V, T'_L
    # (m P(r) r, n P(r) r) and T'_Vhat (m P(w) w)
    def step_flops(r):
        P = lambda k: k * (k + 1) // 2
        w = 2 * r
        stage = (n * r * r + n * P(r) * r) + (m * r * r + m * P(r) * r) + (2 * n * w * w + 2 * w ** 3 + n * P(w) * w)
        once = m * P(r) * r + n * P(r) * r + m * P(w) * w
        return 2.0 * (nsub * 4 * stage + once)
    achieved = step_flops(rank_end) / (ms * 1e-3) / 1e12
    line = {"metric": "rank-adaptive BUG steps/s (Burgers UQ, n=4096, m=16384, r 16..64)", "value": 1e3 / ms,
            "unit": "steps/s", "n_gpus": 1, "steps": K, "warmup": W, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded Burgers-UQ samples)",
            "config": {"workload": "burgers_uq_4096x16384", "dt": dt, "tol": tol, "r_min": 16, "r_max": R,
                       "rank_after": rank_end, "scheme": f"RK4, {nsub} substeps",
                       "ms_per_step_at_rank_64": ms64, "ms_per_step_fp64_engine": ms_f64,
                       "l2": "no n x m matrix exists; factors (4096 + 16384) x 128 FP32 stay in L2"},
            "accuracy": {"steps": 3, "rel_fro_fp32_vs_fp64_engine": err, "rank_fp32": y32.S.shape[0],
                         "rank_fp64": y64.S.shape[0]},
            "roofline": {"bound": "fp32", "achieved": achieved, "peak": FP32_FFMA_TFLOPS, "unit": "TFLOP/s",
                         "frac": achieved / FP32_FFMA_TFLOPS, "traffic": None,
                         "peak_source": "measured FP32 FMA probe (not tensor cores: the flow tiles run on the "
                                        "FP32 pipe)",
                         "algorithmic_flops_per_step": step_flops(rank_end)},
            "gpu_launches": None,
            "clocks": clocks,
            "cpu_baseline": {"value": 1.0 / cpu_step, "unit": "steps/s", "cores": os.cpu_count(), "kind": "port",
                             "sample": f"oracle step on {ms_cols} of {m} samples with 1 and 2 RK4 substeps "
                                       f"({tcpu[0]:.1f} s, {tcpu[1]:.1f} s), scaled linearly to {m} samples "
                                       f"and {nsub} substeps"},
            "e2e": {"value": 1.0 / e2e_s, "unit": "steps/s",
                    "h2d_bytes_per_step": ((n + m) * r0 + r0 * r0 + m) * 4 / kE,
                    "d2h_bytes_per_step": d2h_e2e, "steps": kE}}
    return line


def leg_adjoint():
    """The adjoint workload on one GPU: one loss + gradient sweep (forward
    with checkpoints every 20 steps, segment replays, 200 adjoint-step
    launches), timed after a warm-up sweep over the first 20 steps (same
    kernels and graph shapes), then the gradient against FP64 central
    differences on 32 random directions (64 perturbed forward solves in one
    batch)."""
    import torch
    import __graft_entry__ as ge
    import workloads
    lri = ge.load_package()
    A0, theta, U, S, V, (P, d, Q) = workloads.adjoint_2048()
    dt, T = 1e-4, 0.02
    alg = lri.UnconventionalAlgorithm(lri.RK4(1))
    target = lri.SVDLikeRepresentation(P, np.diag(d), Q)
    prob = lri.MatrixDEProblem(lri.SylvesterTridiagOperator(A0, A0, theta), lri.SVDLikeRepresentation(U, S, V),
                               (0.0, T))
    warm = lri.MatrixDEProblem(prob.f, prob.u0, (0.0, 20 * dt))
    lri.bug_gradient(warm, alg, dt, target, checkpoint_every=20)  # warm-up (builds, graph capture)
    torch.cuda.synchronize()
    sampler = ClockSampler(torch.cuda.current_device())
    sampler.__enter__()
    t0 = time.perf_counter()
    loss, thb, gr = lri.bug_gradient(prob, alg, dt, target, checkpoint_every=20)
    torch.cuda.synchronize()
    sweep = time.perf_counter() - t0
    sampler.__exit__()
    t0 = time.perf_counter()
    lri.solve(prob, alg, dt, precision="fp64", save_everystep=False)
    torch.cuda.synchronize()
    fwd = time.perf_counter() - t0
    g = np.random.default_rng(11)
    h = 1e-6
    dirs = [tuple(g.standard_normal(x.shape) for x in (theta, U, S, V)) for _ in range(32)]
    probs = []
    for (dth, dU, dS, dV) in dirs:
        for sgn in (1.0, -1.0):
            e = sgn * h
            probs.append(lri.MatrixDEProblem(lri.SylvesterTridiagOperator(A0, A0, theta + e * dth),
                                             lri.SVDLikeRepresentation(U + e * dU, S + e * dS, V + e * dV), (0.0, T)))
    t0 = time.perf_counter()
    finals = lri.solve_ensemble(probs, alg, dt, precision="fp64")
    fd_time = time.perf_counter() - t0
    losses = [lri.terminal_loss(Y, target)[0] for Y in finals]
    rel = []
    for i, (dth, dU, dS, dV) in enumerate(dirs):
        fd = (losses[2 * i] - losses[2 * i + 1]) / (2 * h)
        an = np.sum(thb * dth) + np.sum(gr.U * dU) + np.sum(gr.S * dS) + np.sum(gr.V * dV)
        rel.append(abs(fd - an) / abs(an))
    nsteps = lri.n_steps((0.0, T), dt)
    line = {"metric": "BUG loss + gradient sweep (checkpointed discrete adjoint)", "value": sweep, "unit": "s",
            "higher_is_better": False, "n_gpus": 1, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "adjoint_2048", "n": 2048, "m": 2048, "r": 32, "steps": nsteps, "dt": dt,
                       "scheme": "RK4(nsub=1)", "checkpoint_every": 20, "loss": "||Y(T) - X_t||_F^2, X_t rank 40"},
            "forward_only_s": fwd, "sweep_over_forward": sweep / fwd,
            "gpu_launches": {"forward": nsteps, "replay": nsteps, "adjoint": nsteps},
            "fd_check": {"directions": len(dirs), "h": h, "worst_rel": float(max(rel)),
                         "median_rel": float(np.median(rel)), "batched_forward_solves_s": fd_time,
                         "tolerance": 1e-4, "passed": bool(max(rel) <= 1e-4)},
            "clocks": sampler.summary(),
            "loss": loss}
    return line


def leg_laplace(warmup):
    """The stiff 256 x 256 workload: plain BUG in FP64 on F(X) = A X + X A^T,
    A = Laplacian/h^2 - 0.1 I (h = 1/257), Y0 rank 8, dt = 1e-4, RK4 with 20
    substeps, 1000 steps on [0, 0.1] as one CUDA graph on the device-resident
    factors; accuracy of the first 100 steps against the oracle, whose time
    for those steps is the CPU baseline; end to end through solve() from host
    arrays with the final factors read back."""
    import torch
    import __graft_entry__ as ge
    import workloads
    from oracle import lri_oracle as O
    lri = ge.load_package()
    inst, dt, tspan, nsub = workloads.sylvester_256()
    nsteps = lri.n_steps(tspan, dt)
    alg = lri.UnconventionalAlgorithm(lri.RK4(nsub))
    Y0 = lri.SVDLikeRepresentation(inst.U, inst.S, inst.V)
    op = lri.SylvesterTridiagOperator(inst.A, inst.B)
    OPK = lri._native.LRI_OP_SYLVESTER_TRIDIAG
    stream = torch.cuda.current_stream()

    def batch(prec):
        b = lri.Batch([256], [256], [8], alg, OPK, prec)
        b.upload([Y0], [op])
        return b

    res = {}
    clocks = None
    for prec in ("fp64", "df"):
        b = batch(prec)
        for k in range(warmup):
            b.step(k * dt, dt, 1)
        b.check_status()
        b.upload([Y0], [op])
        b.prepare(dt, nsteps)
        torch.cuda.synchronize()
        sampler = ClockSampler(torch.cuda.current_device()) if prec == "fp64" else None
        if sampler:
            sampler.__enter__()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        b.step(0.0, dt, nsteps)
        e1.record(stream)
        torch.cuda.synchronize()
        if sampler:
            sampler.__exit__()
            clocks = sampler.summary()
        b.check_status()
        res[prec] = e0.elapsed_time(e1) / nsteps
        b.close()
    # accuracy over the first 100 steps, against the oracle and the oracle's
    # own response to a 1e-16 relative perturbation of the core every step
    k_acc = 100
    b = batch("fp64")
    b.step(0.0, dt, k_acc)
    b.check_status()
    yg = b.download()[0]
    b.close()
    Yo = O.SVDLikeRepresentation(inst.U, inst.S, inst.V)
    mk = lambda: O.init(O.MatrixDEProblem(O.SylvesterTridiagOp(inst.A, inst.B), Yo, tspan),
                        O.UnconventionalAlgorithm(O.RK4(nsub)), dt)
    io, ip = mk(), mk()
    g = np.random.default_rng(0)
    t0 = time.perf_counter()
    for _ in range(k_acc):
        O.step(io, io.alg, dt)
    cpu_s = (time.perf_counter() - t0) / k_acc
    for _ in range(k_acc):
        O.step(ip, ip.alg, dt)
        ip.u.S = ip.u.S * (1 + 1e-16 * g.standard_normal(ip.u.S.shape))
    err = O.rel_fro_err(yg.full(), io.u.full())
    sens = O.rel_fro_err(ip.u.full(), io.u.full())
    # e2e: the public solve() from host arrays (H2D of Y0 and operators, one
    # graph of all steps, D2H of the final factors)
    prob = lri.MatrixDEProblem(op, Y0, tspan)
    lri.solve(prob, alg, dt, save_everystep=False)  # warm-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    lri.solve(prob, alg, dt, save_everystep=False)
    e2e_s = time.perf_counter() - t0
    ms = res["fp64"]
    # per rhs evaluation 5nr (stencil) + 2nr^2 (K P^T); 3 substep flows x 4
    # stages x nsub per step, plus QR and basis change ~14 (n + m) r^2
    flops = 4 * nsub * 3 * (5 * 256 * 8 + 2 * 256 * 8 * 8) + 14 * 512 * 64
    return {"metric": "BUG steps/s (256x256 Laplacian flow, r = 8, RK4 x 20 substeps, FP64)",
            "value": 1e3 / ms, "unit": "steps/s", "n_gpus": 1, "steps": nsteps, "warmup": warmup,
            "ms_per_step": ms, "higher_is_better": True, "dtype": "f64", "data": "synthetic (seed 1)",
            "config": {"workload": "sylvester_256", "n": 256, "m": 256, "r": 8, "dt": dt, "scheme": "RK4(nsub=20)",
                       "one_launch_per_step": True, "graph_steps": nsteps},
            "double_float": {"ms_per_step": res["df"], "steps_per_s": 1e3 / res["df"]},
            "accuracy": {"steps": k_acc, "rel_fro_vs_fp64_oracle": err, "oracle_self_sensitivity": sens,
                         "bound": max(1e-11, 100.0 * sens),
                         "passed": bool(err <= max(1e-11, 100.0 * sens))},
            "roofline": {"bound": "latency", "note": "one instance of 66 KB state on a 2-CTA cluster (FP64: the K "
                                                     "and L steps on two SMs, the S step on the first; the "
                                                     "double-float form on one CTA); flops per step %.3g, "
                                                     "%.3f TFLOP/s" % (flops, flops / (ms * 1e-3) / 1e12)},
            "gpu_launches": nsteps,
            "clocks": clocks,
            "cpu_baseline": {"value": 1.0 / cpu_s, "unit": "steps/s", "cores": 1, "kind": "port",
                             "sample": f"{k_acc} oracle steps (NumPy FP64)"},
            "e2e": {"value": nsteps / e2e_s, "unit": "steps/s",
                    "h2d_bytes_per_step": (2 * 256 * 8 + 64 + 6 * 256) * 8 / nsteps,
                    "d2h_bytes_per_step": (2 * 256 * 8 + 64) * 8 / nsteps}}


def run_leg(name, args):
    """One of the other workloads; its own dict (or the error it raised)."""
    import torch
    try:
        if name == "stream":
            out = leg_stream(min(args.steps, 20), args.warmup)
        elif name == "burgers":
            out = leg_burgers(min(args.steps, 20), args.warmup)
        elif name == "adjoint":
            out = leg_adjoint()
        else:
            out = leg_laplace(args.warmup)
    except Exception as exc:  # a failing leg must not hide the others
        out = {"error": f"{type(exc).__name__}: {exc}"}
    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--count", type=int, default=4096)
    ap.add_argument("--fp64-steps", type=int, default=None, help="plain FP64 steps timed (default: all)")
    ap.add_argument("--cpu-sample-every", type=int, default=64)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--oracle-sample", type=int, default=64, help="ensemble instances checked against the oracle")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--adjoint", action="store_true",
                    help="instead of the ensemble: the adjoint workload (loss + gradient, FD check)")
    ap.add_argument("--burgers", action="store_true",
                    help="instead of the ensemble: the Burgers-UQ workload (n=4096, m=16384, rank 16..64)")
    ap.add_argument("--stream", action="store_true",
                    help="instead of the ensemble: the 8192 x 4096 data-compression stream (rank-adaptive)")
    ap.add_argument("--laplace", action="store_true",
                    help="instead of the ensemble: the 256 x 256 Laplacian flow (FP64, 1000 steps)")
    ap.add_argument("--no-legs", action="store_true",
                    help="N = 1: skip the other workloads that follow the ensemble in the same JSON line")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    ws, rank, local, dist = dist_setup()
    if args.impl == "reference":
        run_reference(args, ws, rank)
        return
    legs = {"adjoint": args.adjoint, "stream": args.stream, "burgers": args.burgers, "laplace": args.laplace}
    only = [k for k, v in legs.items() if v]
    if only:
        if rank == 0:
            for k in only:
                print(json.dumps(run_leg(k, args)), flush=True)
        return

    # CPU baseline first: its spawn pool starts before any GPU work
    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = cpu_baseline(args.count, args.cpu_sample_every, 2, 1)

    import torch
    import __graft_entry__ as ge
    import workloads
    lri = ge.load_package()
    torch.cuda.set_device(local)
    dev_index = torch.cuda.current_device()

    seed = 4 + rank  # weak scaling: every rank advances its own ensemble
    insts = workloads.lyapunov_ensemble(count=args.count, seed=seed)
    shapes = ([e.U.shape[0] for e in insts], [e.V.shape[0] for e in insts], [e.S.shape[0] for e in insts])
    factors = [lri.SVDLikeRepresentation(e.U, e.S, e.V) for e in insts]
    ops = [lri.SylvesterTridiagOperator(e.A, e.B) for e in insts]
    alg = lri.UnconventionalAlgorithm(lri.RK4(NSUB))
    K, W = args.steps, args.warmup
    OPK = lri._native.LRI_OP_SYLVESTER_TRIDIAG

    def barrier():
        rank_barrier(dist)

    def max_over_ranks(x):
        return rank_max(x, dist)

    stream = torch.cuda.current_stream()

    def timed_run(make, k_timed, k_total, sample_clocks=False):
        """W warm-up steps, k_timed timed steps (CUDA events on the current
        stream, barrier + synchronize on both sides), then the rest untimed so
        every form ends at step W + k_total.  Returns (ms, factors, launches,
        clocks)."""
        obj = make()
        t = 0.0
        for _ in range(W):
            obj.step(t, DT, 1)
            t += DT
        obj.check_status()
        obj.prepare(DT, k_timed)  # graph capture outside the timed region
        torch.cuda.synchronize()
        barrier()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        sampler = ClockSampler(dev_index) if sample_clocks else None
        if sampler:
            sampler.__enter__()
        e0.record(stream)
        obj.step(t, DT, k_timed)  # one CUDA graph of k_timed steps per batch
        t += k_timed * DT
        e1.record(stream)
        torch.cuda.synchronize()
        if sampler:
            sampler.__exit__()
        barrier()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        for _ in range(k_total - k_timed):
            obj.step(t, DT, 1)
            t += DT
        obj.check_status()
        launches = obj.launches(k_timed)
        ys = obj.download()
        obj.close()
        return ms, ys, launches, (sampler.summary() if sampler else None)

    class Single:
        """one homogeneous batch behind the same interface as MixedEnsemble"""

        def __init__(self, prec):
            self.b = lri.Batch(*shapes, alg, OPK, prec)
            self.b.upload(factors, ops)

        def step(self, t, dt, k):
            self.b.step(t, dt, k)

        def check_status(self):
            self.b.check_status()

        def launches_per_step(self):
            return int(self.b.lib.lri_batch_launches_per_step(self.b.handle))

        def prepare(self, dt, k):
            self.b.prepare(dt, k)

        def launches(self, k):
            return self.b.launches(k)

        def download(self):
            return self.b.download()

        def close(self):
            self.b.close()

    # headline: the mixed form (FP32 batch for well-conditioned cores,
    # double-float batch for the rest, two streams)
    ms, ymix, launches, clocks = timed_run(lambda: lri.MixedEnsemble(factors, ops, alg, OPK), K, K, True)
    ms_max = max_over_ranks(ms)
    value = weak_value(ws, K, ms_max * 1e-3)
    kap = np.array([lri.core_condition(Y.S) for Y in factors])
    n_fp32 = int((kap <= lri.MIXED_KAPPA_MAX).sum())
    # the autotuned register budget of each precision class (tuning.json)
    ensemble_tiles = {}
    for prec, sel in (("fp32", np.flatnonzero(kap <= lri.MIXED_KAPPA_MAX)),
                      ("df", np.flatnonzero(kap > lri.MIXED_KAPPA_MAX))):
        c, bucket = lri._tuning.ensemble_occupancy(prec, [shapes[0][i] for i in sel], [shapes[1][i] for i in sel],
                                                   [shapes[2][i] for i in sel])
        ensemble_tiles[prec] = {"ctas_per_sm": c, "tuned_bucket": bucket,
                                "micro_tile": "4x4 per thread, rows per tile 4*256/ceil(c/4) (c = panel columns)"}
    # pure FP32 form and plain FP64 form, same steps
    ms32, y32, _, _ = timed_run(lambda: Single("fp32"), K, K)
    k64 = K if args.fp64_steps is None else min(K, args.fp64_steps)
    ms64, y64, _, _ = timed_run(lambda: Single("fp64"), k64, K)
    fp64_ms = ms64 / k64

    def rel_errs(ys):
        return np.array([np.linalg.norm(a.full() - c.full()) / np.linalg.norm(c.full()) for a, c in zip(ys, y64)])

    err_mix = rel_errs(ymix)
    err_32 = rel_errs(y32)
    # aggregate over the ensemble: ||[Y_i] - [Y_i^64]||_F / ||[Y_i^64]||_F
    num = sum(np.linalg.norm(a.full() - c.full()) ** 2 for a, c in zip(ymix, y64))
    den = sum(np.linalg.norm(c.full()) ** 2 for c in y64)
    err_mix_agg = float(math.sqrt(num / den))

    # ---------------- accuracy vs the CPU oracle on a sample -----------------
    oracle_err = None
    if rank == 0:
        # every 64th instance (64 of 4096), the oracle's full trajectory of
        # W + K steps, one spawned process per host core
        sample = list(range(0, args.count, max(1, args.count // args.oracle_sample)))[:args.oracle_sample]
        cores = os.cpu_count() or 1
        chunks = [c for c in (sample[k::cores] for k in range(cores)) if c]
        t0 = time.perf_counter()
        with mp.get_context("spawn").Pool(len(chunks), initializer=_pool_init) as pool:
            finals = pool.map(_oracle_finals, [(c, W + K, args.count) for c in chunks])
        wall = time.perf_counter() - t0
        ref = {i: Y for part in finals for i, Y in part}
        from oracle import lri_oracle as O
        em = [O.rel_fro_err(ymix[i].full(), ref[i]) for i in sample]
        e64 = [O.rel_fro_err(y64[i].full(), ref[i]) for i in sample]
        oracle_err = {"instances": len(sample), "every": max(1, args.count // args.oracle_sample),
                      "mixed_max": float(max(em)), "mixed_median": float(np.median(em)),
                      "mixed_above_1e-5": int(sum(e > 1e-5 for e in em)), "fp64_max": float(max(e64)),
                      "oracle_wall_s": wall}

    # ---------------- e2e through the public API with host buffers -----------------
    e2e = None
    if not args.no_e2e:
        ens = lri.MixedEnsemble(factors, ops, alg, OPK)
        pinned = []
        for prec, sel, b, st in ens.parts:
            hU, hS, hV = b.pack_factors([factors[i] for i in sel])
            hA = np.zeros(int(b.opA.numel()), b.np_dtype)
            hB = np.zeros(int(b.opB.numel()), b.np_dtype)
            for j, i in enumerate(sel):
                a_, b_ = ops[i].packed()
                hA[b.offA[j]:b.offA[j] + len(a_)] = a_
                hB[b.offB[j]:b.offB[j] + len(b_)] = b_
            src = [torch.from_numpy(x).pin_memory() for x in (hU, hS, hV, hA, hB)]
            # every step's factors go to the host through the library's
            # solution history: a device ring slot per record, copied to
            # page-locked host buffers on the history's own stream, so the
            # transfers overlap the following steps (three host buffer sets
            # per class, each reused once its previous record has landed)
            hist = lri.History(b, slots=4)
            hosts = [hist.host_buffers() for _ in range(3)]
            pinned.append((b, st, src, (hist, hosts)))
        h2d = sum(int(x.numel()) * x.element_size() for _, _, src, _ in pinned for x in src)
        d2h = sum(int(x.numel()) * x.element_size() for _, _, _, (_, hosts) in pinned for x in hosts[0])

        def one_solve():
            for b, st, src, _ in pinned:
                st.wait_stream(torch.cuda.current_stream())
                with torch.cuda.stream(st):
                    for dst, x in zip((b.U, b.S, b.V, b.opA, b.opB), src):
                        dst.copy_(x, non_blocking=True)
                    st.synchronize()
                    b.bind()
            tt = 0.0
            seqs = [[None] * 3 for _ in pinned]
            for k in range(K):
                for j, (b, st, src, (hist, hosts)) in enumerate(pinned):
                    with torch.cuda.stream(st):
                        b.step(tt, DT, 1)
                        slot = k % 3
                        if seqs[j][slot] is not None:
                            hist.wait(seqs[j][slot])  # that buffer's record is on the host
                        seqs[j][slot] = hist.record(host=hosts[slot])
                tt += DT
            for j, (_, _, _, (hist, _)) in enumerate(pinned):
                for q in seqs[j]:
                    if q is not None:
                        hist.wait(q)  # every step's factors are on the host
                hist.pending = []
            return tt

        one_solve()  # warm-up solve
        torch.cuda.synchronize()
        barrier()
        t0 = time.perf_counter()
        one_solve()
        torch.cuda.synchronize()
        barrier()
        el = max_over_ranks(time.perf_counter() - t0)
        ens.check_status()
        for _, _, _, (hist, _) in pinned:
            hist.close()
        ens.close()
        e2e = {"value": ws * K / el, "unit": UNIT, "h2d_bytes_per_step": h2d / K, "d2h_bytes_per_step": d2h,
               "note": "one solve of K steps through the public API: H2D of Y0 and operators from pinned "
                       "memory, every step's U, S, V and ranks read back to pinned host buffers through the "
                       "solution history (device ring, copies on the history's stream overlapping the next "
                       "steps), all of them landed before the clock stops"}

    if rank != 0:
        return
    hbm, bf16, src = peaks()
    alg_bytes, alg_flops = algorithmic(shapes)
    t_launch = ms / K * 1e-3
    # FP32 FMA peak: SMs x 128 lanes x 2 flops x the SM clock sampled during
    # the timed region (nominal maximum when no sample was taken)
    sms = torch.cuda.get_device_properties(dev_index).multi_processor_count
    clk = (clocks or {}).get("sm_mhz") or 2070.0
    fp32_peak = sms * 128 * 2 * clk * 1e6 / 1e12
    fp32_src = "%d SMs x 128 FP32 lanes x 2 x %.0f MHz (%s)" % (
        sms, clk, "sampled SM clock" if (clocks or {}).get("sm_mhz") else "nominal maximum clock")
    achieved = alg_bytes / t_launch / 1e9
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": K, "warmup": W,
        "ms_per_step": ms_max / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+df32", "data": "synthetic",
        "config": {"workload": "lyapunov_ensemble_4096", "instances": args.count,
                   "n_m_range": [64, 1024], "r_range": [4, 32], "dt": DT, "scheme": f"RK4(nsub={NSUB})",
                   "algorithm": "BUG (UnconventionalAlgorithm)",
                   "precision": "mixed: FP32 for kappa(S0) <= %.0e (%d instances), double-float for the other %d"
                                % (lri.MIXED_KAPPA_MAX, n_fp32, args.count - n_fp32),
                   "instance_steps_per_s": value * args.count,
                   "tiles": ensemble_tiles,
                   "l2": "inputs larger than L2: factors %.0f MB + operators + workspace > 129 MB"
                         % (alg_bytes / 2e6)},
        "accuracy": {"mixed_vs_fp64_gpu_rel_fro_max": float(err_mix.max()),
                     "mixed_vs_fp64_gpu_rel_fro_median": float(np.median(err_mix)),
                     "mixed_vs_fp64_gpu_rel_fro_aggregate": err_mix_agg,
                     "fp32_only_vs_fp64_gpu_rel_fro_max": float(err_32.max()),
                     "fp32_only_instances_above_1e-5": int((err_32 > 1e-5).sum()),
                     "vs_oracle_sample": oracle_err, "steps_compared": W + K},
        "fp32_only": {"ms_per_step": ms32 / K, "steps_per_s": 1e3 * K / ms32},
        "plain_fp64": {"ms_per_step": fp64_ms, "steps_per_s": 1e3 / fp64_ms, "timed_steps": k64,
                       "speedup_mixed_over_fp64": (value / ws) / (1e3 / fp64_ms)},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "traffic": TRAFFIC_PER_INSTANCE["fp32"] * n_fp32
                                + TRAFFIC_PER_INSTANCE["df"] * (args.count - n_fp32),
                     "traffic_source": "ncu dram bytes per instance-step of each class (1024-instance capture of "
                                       "step_kernel<T, 3>), scaled by the instance counts",
                     "peak_source": src,
                     "algorithmic_bytes_per_launch": alg_bytes,
                     "note": "compulsory bytes per batched step (factors and operators read, factors "
                             "written) / mixed step time; the step kernels are FP32-issue bound on the CUDA "
                             "cores, see compute"},
        "compute": {"flops_per_step": alg_flops, "achieved_tflops": alg_flops / t_launch / 1e12,
                    "fp32_fma_peak_tflops": fp32_peak, "fp32_peak_source": fp32_src,
                    "frac_fp32_pipe": alg_flops / t_launch / 1e12 / fp32_peak,
                    "frac_bf16_tensor_peak": alg_flops / t_launch / 1e12 / bf16,
                    "note": "algorithmic flops of the implemented BUG step (FP32 and double-float "
                            "multiply-adds counted once; a double-float one costs 12-15 FP32 instructions)"},
        "gpu_launches": launches,
        "clocks": clocks,
    }
    if cpu is not None:
        line["cpu_baseline"] = {"value": cpu[0], "unit": UNIT, "cores": cpu[1], "kind": "port", "sample": cpu[2]}
    if e2e is not None:
        line["e2e"] = e2e
    if ws == 1 and not args.no_legs:
        # the other workloads, each timed on its own with its own clocks,
        # accuracy, roofline and CPU sample
        line["workloads"] = {"laplace_256": run_leg("laplace", args),
                             "data_stream_8192x4096": run_leg("stream", args),
                             "burgers_uq_4096x16384": run_leg("burgers", args),
                             "adjoint_2048": run_leg("adjoint", args)}
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
