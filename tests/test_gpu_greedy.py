"""GreedyIntegrator and MatrixHybridProblem on the GPU (the instance
engine's greedy_step, src/integrators/greedy_integrator.jl:73-104) against
the oracle, every step, through the C ABI:

* SVD-like factors on a data stream (U = Q of qr(X V), V = Q of qr(X^T U),
  S = U^T X V), compared through Y = U S V^T (QR sign conventions differ);
* two factors u = U Z^T on the same stream (Z = X^T U, U = polar(X Z)):
  the polar factor is unique, so U and Z are compared directly;
* the hybrid problem of test/data_informed_approximation.jl (Burgers flow
  nu Dxx u - (Dx u) .* u on a periodic grid, coefficients Z' = F(U Z^T)^T U,
  U refitted to the snapshots), on a smaller grid.
Tolerances: FP64 1e-11 (1e-10 for the nonlinear hybrid), double-float
1e-10, FP32 1e-5 relative."""
import os
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                                "lowrankintegrators.jl_gb300"))
import workloads  # noqa: E402

TOL = {"fp64": 1e-11, "df": 1e-10, "fp32": 1e-5}


@pytest.fixture(scope="module")
def stream():
    return workloads.data_stream(256, 192, 8, seed=4)


@pytest.mark.parametrize("precision", ["fp64", "df", "fp32"])
def test_greedy_svd_like_matches_oracle(lri, oracle, stream, precision):
    Y0 = oracle.truncated_svd(stream[0], r=8)
    so = oracle.solve(oracle.MatrixDataProblem(stream, Y0), oracle.GreedyIntegrator())
    sg = lri.solve(lri.MatrixDataProblem(stream, lri.SVDLikeRepresentation(Y0.U, Y0.S, Y0.V)),
                   lri.GreedyIntegrator(), precision=precision)
    assert len(sg.Y) == len(so.Y)
    for k, (yg, yo) in enumerate(zip(sg.Y, so.Y)):
        err = oracle.rel_fro_err(yg.full(), yo.full())
        assert err <= TOL[precision], f"snapshot {k}: {err:.3e}"
    U = sg.Y[-1].U
    assert np.abs(U.T @ U - np.eye(8)).max() <= (1e-5 if precision == "fp32" else 1e-12)


@pytest.mark.parametrize("precision", ["fp64", "df", "fp32"])
def test_greedy_two_factor_matches_oracle(lri, oracle, stream, precision):
    Y0 = oracle.truncated_svd(stream[0], r=6)
    U0, Z0 = Y0.U, stream[0].T @ Y0.U
    so = oracle.solve(oracle.MatrixDataProblem(stream, oracle.TwoFactorRepresentation(U0, Z0)),
                      oracle.GreedyIntegrator())
    sg = lri.solve(lri.MatrixDataProblem(stream, lri.TwoFactorRepresentation(U0, Z0)), lri.GreedyIntegrator(),
                   precision=precision)
    for k, (yg, yo) in enumerate(zip(sg.Y, so.Y)):
        assert isinstance(yg, lri.TwoFactorRepresentation)
        eu = np.linalg.norm(yg.U - yo.U) / np.linalg.norm(yo.U)
        ez = np.linalg.norm(yg.Z - yo.Z) / np.linalg.norm(yo.Z)
        assert max(eu, ez) <= TOL[precision], f"snapshot {k}: U {eu:.3e}, Z {ez:.3e}"


def _burgers_data(n, m, dt, nsteps, seed=0):
    """Snapshots of nu u_xx - u u_x on [0, pi) (periodic), m samples of a
    seeded initial condition with two random modes, by FP64 RK4 with 4
    substeps per snapshot interval (the reference test solves the same ODEs
    with DifferentialEquations, test/data_informed_approximation.jl:43-67)."""
    g = np.random.default_rng(seed)
    L, nu = np.pi, 0.005
    h = L / n
    x = h / 2 + h * np.arange(n)
    xi = g.uniform(-1, 1, (2, m))
    U = (0.5 * (np.exp(np.cos(x)) - 1.5) * np.sin(x + 2 * np.pi * 0.37))[:, None] \
        + 0.5 * xi[0][None, :] * np.sin(2 * np.pi * x)[:, None] + 0.5 * xi[1][None, :] * np.sin(3 * np.pi * x)[:, None]

    def F(Y):
        Yp, Ym = np.roll(Y, -1, axis=0), np.roll(Y, 1, axis=0)
        return nu * (Yp - 2 * Y + Ym) / h ** 2 - ((Yp - Ym) / (2 * h)) * Y

    snaps = [U.copy()]
    hh = dt / 4
    for _ in range(nsteps):
        for _ in range(4):
            k1 = F(U)
            k2 = F(U + 0.5 * hh * k1)
            k3 = F(U + 0.5 * hh * k2)
            k4 = F(U + hh * k3)
            U = U + hh / 6 * (k1 + 2 * k2 + 2 * k3 + k4)
        snaps.append(U.copy())
    return h, nu, snaps


@pytest.mark.parametrize("precision", ["fp64", "df"])
def test_hybrid_burgers_matches_oracle(lri, oracle, precision):
    n, m, r, dt, nsteps = 128, 16, 5, 1e-3, 20
    h, nu, snaps = _burgers_data(n, m, dt, nsteps)
    X0 = oracle.truncated_svd(np.hstack([snaps[0], snaps[1]]), r=r)
    U0, Z0 = X0.U, snaps[0].T @ X0.U
    y = lambda t: snaps[int(round(t / dt))]
    T = dt * nsteps
    op_o = oracle.BurgersOp(n, h, nu, alpha=-1.0, beta=0.0)
    po = oracle.MatrixHybridProblem(y, lambda Z, U, t: op_o.L_rhs(Z, U, t),
                                    oracle.TwoFactorRepresentation(U0, Z0), (0.0, T))
    so = oracle.solve(po, oracle.GreedyIntegrator(oracle.RK4(1)), dt)
    pg = lri.MatrixHybridProblem(y, lri.BurgersOperator(h, nu, alpha=-1.0, beta=0.0),
                                 lri.TwoFactorRepresentation(U0, Z0), (0.0, T))
    sg = lri.solve(pg, lri.GreedyIntegrator(lri.RK4(1)), dt, precision=precision)
    assert len(sg.Y) == len(so.Y) == nsteps + 1
    tol = 1e-10
    for k, (yg, yo) in enumerate(zip(sg.Y, so.Y)):
        eu = np.linalg.norm(yg.U - yo.U) / np.linalg.norm(yo.U)
        ez = np.linalg.norm(yg.Z - yo.Z) / np.linalg.norm(yo.Z)
        assert max(eu, ez) <= tol, f"step {k}: U {eu:.3e}, Z {ez:.3e}"
    # the reference test's own bar: relative error of the data-informed solution
    Yf = sg.Y[-1].full()
    assert np.linalg.norm(snaps[-1] - Yf) / np.linalg.norm(snaps[-1]) <= 0.1


def test_greedy_rejects_svd_like_without_data(lri):
    Y0 = lri.SVDLikeRepresentation(np.eye(8, 2), np.eye(2), np.eye(6, 2))
    prob = lri.MatrixDEProblem(lri.ZeroOperator(), Y0, (0.0, 1.0))
    with pytest.raises(lri.LriError):
        lri.solve(prob, lri.GreedyIntegrator(), 0.5)


@pytest.mark.parametrize("precision,tc,tol", [("fp64", False, 1e-10), ("fp32", True, 1e-5), ("fp32", False, 1e-5)])
def test_greedy_on_stream_engine_matches_oracle(lri, oracle, precision, tc, tol):
    """The large-stream engine's greedy step (single-snapshot passes on the
    tensor or CUDA cores, orthonormal bases by pivoted Cholesky + Newton-Schulz
    or CholeskyQR) against the oracle's Householder-based greedy step,
    through Y = U S V^T."""
    snaps = workloads.data_stream(1024, 512, 6, seed=12)
    Y0 = oracle.truncated_svd(snaps[0], r=12)
    so = oracle.solve(oracle.MatrixDataProblem(snaps, Y0), oracle.GreedyIntegrator())
    eng = lri.DataStreamEngine(1024, 512, 12, 12, 0.0, 1, precision)
    try:
        if precision == "fp32":
            eng.set_tensor_cores(tc)
        eng.bind(lri.SVDLikeRepresentation(Y0.U, Y0.S, Y0.V))
        for k in range(1, len(snaps)):
            eng.greedy_step(eng.to_device(snaps[k]))
            eng.check_status()
            yg = eng.download()
            err = oracle.rel_fro_err(yg.full(), so.Y[k].full())
            assert err <= tol, f"snapshot {k}: {err:.3e}"
    finally:
        eng.close()
