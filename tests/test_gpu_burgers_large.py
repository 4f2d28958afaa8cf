"""The large Burgers engine (lri_burgers_*: grid-wide tile-fused flow
evaluations, rank-adaptive BUG) against the FP64 oracle on the Burgers-UQ
problem (conservative form, per-sample viscosity), with panels wider than
the batch holds (r_max = 48, so 96-column augmented bases).

The workload's own initial data has exact rank 3, padded to r_min = 16: then
[K1 | U0] is numerically rank deficient and the reference's Householder QR
completes the augmented basis with arbitrary directions, which no other basis
construction reproduces.  Those directions carry singular values at the
rounding level only, so the dense solutions still agree to that level; the
factors are compared through Y = U S V^T, and initial data with full
numerical rank (1e-3 noise added) is checked step by step with ranks."""
import os
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                                "lowrankintegrators.jl_gb300"))
import workloads  # noqa: E402


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("fp32", 1e-5)])
def test_burgers_large_matches_oracle(lri, oracle, precision, tol):
    n, m = 256, 320
    h, nu, X0d = workloads.burgers_uq(n, m)
    X0d = X0d + 1e-3 * np.random.default_rng(1).standard_normal(X0d.shape)
    Y0 = oracle.truncated_svd(X0d, r=16)
    dt, T = 1e-4, 1e-3
    pg = lri.MatrixDEProblem(lri.BurgersOperator(h, nu, alpha=0.0, beta=-0.5),
                             lri.SVDLikeRepresentation(Y0.U, Y0.S, Y0.V), (0.0, T))
    po = oracle.MatrixDEProblem(oracle.BurgersOp(n, h, nu, alpha=0.0, beta=-0.5), Y0, (0.0, T))
    ag = lri.RankAdaptiveUnconventionalAlgorithm(1e-6, rmax=48, K_alg=lri.RK4(1), rmin=16)
    ao = oracle.RankAdaptiveUnconventionalAlgorithm(1e-6, rmax=48, K_alg=oracle.RK4(1), rmin=16)
    sg = lri.solve_burgers_large(pg, ag, dt, precision=precision, save_everystep=True)
    so = oracle.solve(po, ao, dt)
    assert [y.S.shape[0] for y in sg.Y] == [y.S.shape[0] for y in so.Y]
    for k, (yg, yo) in enumerate(zip(sg.Y, so.Y)):
        err = oracle.rel_fro_err(yg.full(), yo.full())
        assert err <= tol, f"step {k}: {err:.3e}"


def test_burgers_large_agrees_with_batch_engine(lri, oracle):
    n, m = 192, 160
    h, nu, X0d = workloads.burgers_uq(n, m, seed=9)
    X0d = X0d + 1e-3 * np.random.default_rng(2).standard_normal(X0d.shape)
    Y0 = oracle.truncated_svd(X0d, r=8)
    prob = lri.MatrixDEProblem(lri.BurgersOperator(h, nu, alpha=0.0, beta=-0.5),
                               lri.SVDLikeRepresentation(Y0.U, Y0.S, Y0.V), (0.0, 1e-3))
    alg = lri.RankAdaptiveUnconventionalAlgorithm(1e-7, rmax=24, K_alg=lri.RK4(2), rmin=8)
    a = lri.solve_burgers_large(prob, alg, 1e-4, precision="fp64").Y[-1]
    b = lri.solve(prob, alg, 1e-4, precision="fp64", save_everystep=False).Y[-1]
    assert a.S.shape == b.S.shape
    assert oracle.rel_fro_err(a.full(), b.full()) <= 1e-10


def test_burgers_large_padded_workload_is_finite(lri, oracle):
    n, m = 256, 320
    h, nu, X0d = workloads.burgers_uq(n, m)
    Y0 = oracle.truncated_svd(X0d, r=16)
    prob = lri.MatrixDEProblem(lri.BurgersOperator(h, nu, alpha=0.0, beta=-0.5),
                               lri.SVDLikeRepresentation(Y0.U, Y0.S, Y0.V), (0.0, 2e-3))
    alg = lri.RankAdaptiveUnconventionalAlgorithm(1e-6, rmax=48, K_alg=lri.RK4(1), rmin=16)
    for precision in ("fp32", "fp64"):
        y = lri.solve_burgers_large(prob, alg, 1e-4, precision=precision).Y[-1]
        Y = y.full()
        assert np.all(np.isfinite(Y)) and y.S.shape[0] >= 16
        assert np.linalg.norm(Y) <= 1.01 * np.linalg.norm(X0d)


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-9), ("fp32", 1e-5)])
def test_burgers_large_padded_exact_rank_matches_oracle(lri, oracle, precision, tol):
    """The bench's initial data: exact rank 3 in factor form, completed to
    rank 16 with orthonormal directions at singular value 0."""
    n, m = 256, 320
    h, nu, U0, s0, V0 = workloads.burgers_uq_factors(n, m, 16)
    dt, T = 1e-4, 1e-3
    Y0 = oracle.SVDLikeRepresentation(U0, np.diag(s0), V0)
    pg = lri.MatrixDEProblem(lri.BurgersOperator(h, nu, alpha=0.0, beta=-0.5),
                             lri.SVDLikeRepresentation(U0, np.diag(s0), V0), (0.0, T))
    po = oracle.MatrixDEProblem(oracle.BurgersOp(n, h, nu, alpha=0.0, beta=-0.5), Y0, (0.0, T))
    ag = lri.RankAdaptiveUnconventionalAlgorithm(1e-4, rmax=48, K_alg=lri.RK4(1), rmin=16)
    ao = oracle.RankAdaptiveUnconventionalAlgorithm(1e-4, rmax=48, K_alg=oracle.RK4(1), rmin=16)
    sg = lri.solve_burgers_large(pg, ag, dt, precision=precision, save_everystep=True)
    so = oracle.solve(po, ao, dt)
    for k, (yg, yo) in enumerate(zip(sg.Y, so.Y)):
        err = oracle.rel_fro_err(yg.full(), yo.full())
        assert err <= tol, f"step {k}: {err:.3e} (ranks {yg.S.shape[0]} / {yo.S.shape[0]})"
        U = np.asarray(yg.U, np.float64)
        assert np.abs(U.T @ U - np.eye(U.shape[1])).max() <= (1e-12 if precision == "fp64" else 1e-5)
