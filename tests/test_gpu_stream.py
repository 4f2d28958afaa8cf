"""The large-stream engine (lri_stream_*: multi-CTA passes over the snapshot
pair, rank-adaptive BUG) against the FP64 oracle on the data-compression
generator, with panels wider than the one-CTA batch holds (r_max = 48, so
2 r_max = 96 columns).  Rank trajectories must match exactly; FP64 to 1e-10,
FP32 to 1e-5 relative Frobenius error every step."""
import os
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                                "lowrankintegrators.jl_gb300"))
import workloads  # noqa: E402


@pytest.fixture(scope="module")
def stream_case(oracle):
    snaps = workloads.data_stream(1024, 512, 10)
    X0 = oracle.truncated_svd(snaps[0], r=16)
    so = oracle.solve(oracle.MatrixDataProblem(snaps, X0), oracle.RankAdaptiveUnconventionalAlgorithm(1e-6, rmax=48))
    return snaps, X0, so


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("fp32", 1e-5)])
def test_stream_engine_matches_oracle(lri, oracle, stream_case, precision, tol):
    snaps, X0, so = stream_case
    prob = lri.MatrixDataProblem(snaps, lri.SVDLikeRepresentation(X0.U, X0.S, X0.V))
    sg = lri.solve_stream(prob, lri.RankAdaptiveUnconventionalAlgorithm(1e-6, rmax=48), precision=precision)
    assert [y.S.shape[0] for y in sg.Y] == [y.S.shape[0] for y in so.Y]
    for k, (yg, yo) in enumerate(zip(sg.Y, so.Y)):
        err = oracle.rel_fro_err(yg.full(), yo.full())
        assert err <= tol, f"snapshot {k}: {err:.3e}"
    Yf = sg.Y[-1]
    assert np.linalg.norm(Yf.U.T @ Yf.U - np.eye(Yf.U.shape[1])) <= (1e-12 if precision == "fp64" else 1e-5)


def test_stream_engine_agrees_with_batch_engine(lri, oracle):
    """Below the batch's 64-column limit both engines run the same step."""
    snaps = workloads.data_stream(384, 256, 6, seed=7)
    X0 = oracle.truncated_svd(snaps[0], r=8)
    Y0 = lri.SVDLikeRepresentation(X0.U, X0.S, X0.V)
    alg = lri.RankAdaptiveUnconventionalAlgorithm(1e-6, rmax=24)
    a = lri.solve_stream(lri.MatrixDataProblem(snaps, Y0), alg, precision="fp64", save_everystep=False).Y[-1]
    b = lri.solve(lri.MatrixDataProblem(snaps, Y0), alg, precision="fp64", save_everystep=False).Y[-1]
    assert a.S.shape == b.S.shape
    assert oracle.rel_fro_err(a.full(), b.full()) <= 1e-10


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-9), ("fp32", 1e-5)])
def test_stream_engine_wide_core(lri, oracle, precision, tol):
    """Rank 90 of r_max 96: the 2r x 2r core (180) no longer fits the core
    kernel's shared memory, so its SVD runs on the global-memory scratch.
    A noise-free stream of exact rank 90 (the integrator reproduces it; the
    truncation has a clear gap: sigma_90 = 1.2e-5 against tol = 5e-6)."""
    snaps = workloads.data_stream(1024, 512, 6, seed=11, K=90, noise=0.0)
    X0 = oracle.truncated_svd(snaps[0], r=90)
    alg_o = oracle.RankAdaptiveUnconventionalAlgorithm(5e-6, rmax=96)
    so = oracle.solve(oracle.MatrixDataProblem(snaps, X0), alg_o)
    prob = lri.MatrixDataProblem(snaps, lri.SVDLikeRepresentation(X0.U, X0.S, X0.V))
    sg = lri.solve_stream(prob, lri.RankAdaptiveUnconventionalAlgorithm(5e-6, rmax=96), precision=precision)
    assert [y.S.shape[0] for y in sg.Y] == [y.S.shape[0] for y in so.Y] == [90] * 6
    for k, (yg, yo) in enumerate(zip(sg.Y, so.Y)):
        err = oracle.rel_fro_err(yg.full(), yo.full())
        assert err <= tol, f"snapshot {k}: {err:.3e}"
    Yf = sg.Y[-1]
    assert np.abs(Yf.U.T @ Yf.U - np.eye(90)).max() <= (1e-12 if precision == "fp64" else 1e-5)


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("fp32", 1e-5)])
def test_stream_engine_low_rank(lri, oracle, precision, tol):
    """From rank 1 on a noise-free rank-3 stream (the oracle's ranks: 1, 2,
    4, 8, 8, 8 with r_max 8): the core has 2 to 16 columns, so most of the
    core SVD's column blocks (16 over the cluster) are empty or hold one
    column."""
    snaps = workloads.data_stream(384, 256, 6, seed=3, K=3, noise=0.0)
    X0 = oracle.truncated_svd(snaps[0], r=1)
    so = oracle.solve(oracle.MatrixDataProblem(snaps, X0), oracle.RankAdaptiveUnconventionalAlgorithm(1e-6, rmax=8))
    prob = lri.MatrixDataProblem(snaps, lri.SVDLikeRepresentation(X0.U, X0.S, X0.V))
    sg = lri.solve_stream(prob, lri.RankAdaptiveUnconventionalAlgorithm(1e-6, rmax=8), precision=precision)
    ranks = [y.S.shape[0] for y in sg.Y]
    assert ranks == [y.S.shape[0] for y in so.Y]
    assert max(ranks) > 1
    for k, (yg, yo) in enumerate(zip(sg.Y, so.Y)):
        err = oracle.rel_fro_err(yg.full(), yo.full())
        assert err <= tol, f"snapshot {k}: {err:.3e}"
