"""Parity cases for the data-compression and Burgers-UQ configurations at
sizes the instance engine holds (panels of at most 64 columns, so r <= 32
for the rank-adaptive step), against the FP64 oracle.

* Data stream (the compression workload's generator: 64 rotating modes with
  oscillating amplitudes e^{-k/8}(1 + 0.3 sin 2 pi f t) plus 1e-4 noise),
  512 x 256, 12 snapshots, rank-adaptive BUG with tol 1e-6, r <= 32 from
  r0 = 16; the rank trajectory must match the oracle's exactly.
* Burgers UQ (conservative form, per-sample viscosity), 256 grid points x 128
  samples, rank-adaptive with r in [16, 32], dt = 1e-4.
"""
import os
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                                "lowrankintegrators.jl_gb300"))
import workloads  # noqa: E402


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("df", 1e-9)])
def test_data_stream_rank_adaptive(lri, oracle, precision, tol):
    snaps = workloads.data_stream(512, 256, 12)
    X0o = oracle.truncated_svd(snaps[0], r=16)
    X0 = lri.SVDLikeRepresentation(X0o.U, X0o.S, X0o.V)
    sg = lri.solve(lri.MatrixDataProblem(snaps, X0), lri.RankAdaptiveUnconventionalAlgorithm(1e-6, rmax=32),
                   precision=precision)
    so = oracle.solve(oracle.MatrixDataProblem(snaps, X0o), oracle.RankAdaptiveUnconventionalAlgorithm(1e-6, rmax=32))
    assert [y.S.shape[0] for y in sg.Y] == [y.S.shape[0] for y in so.Y]
    for k, (yg, yo) in enumerate(zip(sg.Y, so.Y)):
        err = oracle.rel_fro_err(yg.full(), yo.full())
        assert err <= tol, f"snapshot {k}: {err:.3e}"


def test_data_stream_bug_fp32(lri, oracle):
    """The FP32 engine on the same stream (fixed rank 16, BUG)."""
    snaps = workloads.data_stream(512, 256, 12)
    X0o = oracle.truncated_svd(snaps[0], r=16)
    X0 = lri.SVDLikeRepresentation(X0o.U, X0o.S, X0o.V)
    yg = lri.solve(lri.MatrixDataProblem(snaps, X0), lri.UnconventionalAlgorithm(), precision="fp32",
                   save_everystep=False).Y[-1]
    yo = oracle.solve(oracle.MatrixDataProblem(snaps, X0o), oracle.UnconventionalAlgorithm(),
                      save_everystep=False).Y[-1]
    assert oracle.rel_fro_err(yg.full(), yo.full()) <= 1e-5


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("df", 1e-9)])
def test_burgers_uq_rank_adaptive(lri, oracle, precision, tol):
    n, m = 256, 128
    h, nu, X0d = workloads.burgers_uq(n, m)
    Y0 = oracle.truncated_svd(X0d, r=16)
    dt, T = 1e-4, 2e-3
    ag = lri.RankAdaptiveUnconventionalAlgorithm(1e-6, rmax=32, K_alg=lri.RK4(1), rmin=16)
    ao = oracle.RankAdaptiveUnconventionalAlgorithm(1e-6, rmax=32, K_alg=oracle.RK4(1), rmin=16)
    pg = lri.MatrixDEProblem(lri.BurgersOperator(h, nu, alpha=0.0, beta=-0.5),
                             lri.SVDLikeRepresentation(Y0.U, Y0.S, Y0.V), (0.0, T))
    po = oracle.MatrixDEProblem(oracle.BurgersOp(n, h, nu, alpha=0.0, beta=-0.5), Y0, (0.0, T))
    sg = lri.solve(pg, ag, dt, precision=precision)
    so = oracle.solve(po, ao, dt)
    assert [y.S.shape[0] for y in sg.Y] == [y.S.shape[0] for y in so.Y]
    for k, (yg, yo) in enumerate(zip(sg.Y, so.Y)):
        err = oracle.rel_fro_err(yg.full(), yo.full())
        assert err <= tol, f"step {k}: {err:.3e}"
