"""Autotuner of the engine's tile choices, run on the GPU it tunes for.

    python lowrankintegrators.jl_gb300/autotune.py [--out PATH] [--count N] [--steps K]

Writes ``tuning.json`` beside this file (see ``_tuning.py`` for how the
library reads it):

* the instance engine: for each precision class of the 4096-instance
  Lyapunov ensemble (FP32 for kappa(S0) <= 2^21, double-float above, as the
  mixed form splits it) and each rank bucket holding at least 32 instances,
  the BUG step of that sub-population timed with the step kernel's two
  register budgets (3 CTAs per SM with at most 80 registers per thread, or
  2 with at most 128); K steps in one CUDA graph after 3 warm-up steps, CUDA
  events on the launching stream;
* the tensor-core snapshot passes: for each stream shape, dY X and dY^T X
  (both snapshots resident, alternating pairs so every pass reads HBM)
  timed over the K splits per 128-row tile and the pipeline stages; the
  stage count shared by both passes minimises their summed best times.
"""
from __future__ import annotations

import argparse
import datetime
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)


def time_batch(lri, torch, shapes, factors, ops, alg, prec, ctas, steps, dt):
    b = lri.Batch(*shapes, alg, lri._native.LRI_OP_SYLVESTER_TRIDIAG, prec)
    try:
        b.upload(factors, ops)
        b.set_occupancy(ctas)
        for k in range(3):
            b.step(k * dt, dt, 1)
        b.prepare(dt, steps)
        stream = torch.cuda.current_stream()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        b.step(3 * dt, dt, steps)
        e1.record(stream)
        torch.cuda.synchronize()
        b.check_status()
        return e0.elapsed_time(e1) / steps
    finally:
        b.close()


def tune_ensemble(lri, torch, count, steps):
    import workloads
    from _tuning import rank_bucket
    insts = workloads.lyapunov_ensemble(count=count, seed=4)
    kap = np.array([lri.core_condition(e.S) for e in insts])
    alg = lri.UnconventionalAlgorithm(lri.RK4(1))
    table, meas = {}, {}
    for prec, sel in (("fp32", np.flatnonzero(kap <= lri.MIXED_KAPPA_MAX)),
                      ("df", np.flatnonzero(kap > lri.MIXED_KAPPA_MAX))):
        buckets = {}
        for i in sel:
            buckets.setdefault(rank_bucket(insts[i].S.shape[0]), []).append(i)
        for bucket, idx in sorted(buckets.items()):
            if len(idx) < 32:
                continue
            es = [insts[i] for i in idx]
            shapes = ([e.U.shape[0] for e in es], [e.V.shape[0] for e in es], [e.S.shape[0] for e in es])
            factors = [lri.SVDLikeRepresentation(e.U, e.S, e.V) for e in es]
            ops = [lri.SylvesterTridiagOperator(e.A, e.B) for e in es]
            ms = {c: time_batch(lri, torch, shapes, factors, ops, alg, prec, c, steps, 1e-2) for c in (3, 2)}
            best = min(ms, key=ms.get)
            table.setdefault(prec, {})[bucket] = {"ctas_per_sm": best}
            meas.setdefault(prec, {})[bucket] = {"instances": len(idx), "ms_per_step": {str(c): v for c, v in ms.items()}}
            print(f"ensemble {prec} {bucket}: {len(idx)} instances, ms/step {ms} -> {best} CTAs/SM", flush=True)
    return table, meas


def tune_stream(lri, torch, n, m, R, reps=20):
    eng = lri.DataStreamEngine(n, m, R, R, 1e-6, 1, "fp32")
    try:
        if not eng.uses_tensor_cores():
            return None, None
        g = torch.Generator(device="cuda").manual_seed(1)
        snaps = [torch.randn(n * m, device="cuda", generator=g) for _ in range(3)]
        stream = torch.cuda.current_stream()
        res = {}
        for trans, cands in ((False, (1, 2, 3, 4)), (True, (2, 3, 4, 5, 6))):
            X = torch.randn((n if trans else m) * R, device="cuda", generator=g)
            out = eng.data_product(snaps[0], snaps[1], X, trans=trans)
            for stages in (2, 3, 4):
                for sp in cands:
                    try:
                        eng.set_pass_tiles(sp if not trans else 0, sp if trans else 0, stages)
                    except lri.LriError:
                        continue
                    eng.data_product(snaps[0], snaps[1], X, trans=trans, out=out)
                    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                    torch.cuda.synchronize()
                    e0.record(stream)
                    for j in range(reps):
                        eng.data_product(snaps[j % 2], snaps[j % 2 + 1], X, trans=trans, out=out)
                    e1.record(stream)
                    torch.cuda.synchronize()
                    res[(trans, stages, sp)] = e0.elapsed_time(e1) / reps
        eng.check_status()
    finally:
        eng.close()
    best = None
    for stages in (2, 3, 4):
        rows = {sp: v for (tr, st, sp), v in res.items() if not tr and st == stages}
        cols = {sp: v for (tr, st, sp), v in res.items() if tr and st == stages}
        if not rows or not cols:
            continue
        sr, sc = min(rows, key=rows.get), min(cols, key=cols.get)
        tot = rows[sr] + cols[sc]
        if best is None or tot < best[0]:
            best = (tot, stages, sr, sc, rows[sr], cols[sc])
    _, stages, sr, sc, tr_ms, tc_ms = best
    entry = {"splits_rows": sr, "splits_cols": sc, "stages": stages}
    meas = {f"{'dYt_X' if tr else 'dY_X'} stages={st} splits={sp}": v for (tr, st, sp), v in sorted(res.items())}
    print(f"stream {n}x{m}x{R}: {entry}, dY X {tr_ms:.4f} ms, dY^T X {tc_ms:.4f} ms", flush=True)
    return entry, meas


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=os.path.join(HERE, "tuning.json"))
    ap.add_argument("--count", type=int, default=4096)
    ap.add_argument("--steps", type=int, default=20)
    args = ap.parse_args()
    import torch
    import __graft_entry__ as ge
    lri = ge.load_package()
    props = torch.cuda.get_device_properties(torch.cuda.current_device())
    ens, ens_meas = tune_ensemble(lri, torch, args.count, args.steps)
    stream, stream_meas = {}, {}
    for (n, m, R) in ((8192, 4096, 96), (1024, 512, 48)):
        e, meas = tune_stream(lri, torch, n, m, R)
        if e is not None:
            stream[f"{n}x{m}x{R}"] = e
            stream_meas[f"{n}x{m}x{R}"] = meas
    out = {"device": props.name, "sm_count": props.multi_processor_count,
           "when": datetime.datetime.now(datetime.timezone.utc).isoformat(timespec="seconds"),
           "ensemble": ens, "stream": stream,
           "measurements": {"ensemble_ms_per_step": ens_meas, "stream_ms_per_pass": stream_meas}}
    with open(args.out, "w") as f:
        json.dump(out, f, indent=1)
    print(f"wrote {args.out}")


if __name__ == "__main__":
    main()
