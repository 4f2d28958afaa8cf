"""GPU parity of the Burgers flow map (tile-fused, F never materialised)
against the FP64 oracle, which evaluates F on the dense n x m matrix.

Algorithms: BUG, KSL primal / dual / Strang, rank-adaptive BUG.  The
reference's own smoke test (test/data_agnostic_approximation.jl: n = 1000
grid points, 20^2 samples, rank 5, dt = 1e-2, nu = 0.005) runs here on
[0, 0.1] with RK4(10) substeps, the fixed-step stand-in for the reference's
adaptive Tsit5 (the Laplacian's stiffness needs ten substeps for RK4).
Tolerances: FP64 1e-10 and double-float 1e-9 relative Frobenius error
(different summation order in a nonlinear flow); FP32 1e-4.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = {"fp64": 1e-10, "df": 1e-9, "fp32": 1e-4}


def burgers_instance(n, mgrid, r, oracle):
    dx = math.pi / n
    x = np.arange(dx / 2, math.pi, dx)[:n]
    xi = np.linspace(-1, 1, mgrid)
    cols = []
    for x2 in xi:
        for x1 in xi:
            ub = 0.5 * (np.exp(np.cos(x)) - 1.5) * np.sin(x + 2 * math.pi * 0.37)
            cols.append(ub + 0.5 * x1 * np.sin(2 * math.pi * x) + 0.5 * x2 * np.sin(3 * math.pi * x))
    rho0 = np.array(cols).T
    return dx, oracle.truncated_svd(rho0, r=r)


def algs(lri, O, kind, nsub):
    if kind == "bug":
        return lri.UnconventionalAlgorithm(lri.RK4(nsub)), O.UnconventionalAlgorithm(O.RK4(nsub))
    if kind == "ra":
        return (lri.RankAdaptiveUnconventionalAlgorithm(1e-4, rmax=10, K_alg=lri.RK4(nsub)),
                O.RankAdaptiveUnconventionalAlgorithm(1e-4, rmax=10, K_alg=O.RK4(nsub)))
    order = {"primal": "PrimalLieTrotter", "dual": "DualLieTrotter", "strang": "Strang"}[kind]
    return (lri.ProjectorSplitting(getattr(lri, order)(), lri.RK4(nsub)),
            O.ProjectorSplitting(getattr(O, order)(), O.RK4(nsub)))


@pytest.mark.parametrize("precision", ["fp64", "df", "fp32"])
@pytest.mark.parametrize("kind", ["bug", "primal", "dual", "strang", "ra"])
def test_burgers_small_every_step(lri, oracle, kind, precision):
    n, mgrid, r = 128, 6, 4
    dx, Y0 = burgers_instance(n, mgrid, r, oracle)
    ag, ao = algs(lri, oracle, kind, 2)
    pg = lri.MatrixDEProblem(lri.BurgersOperator(dx, 0.005, alpha=-1.0, beta=0.0),
                             lri.SVDLikeRepresentation(Y0.U, Y0.S, Y0.V), (0.0, 0.1))
    po = oracle.MatrixDEProblem(oracle.BurgersOp(n, dx, 0.005, alpha=-1.0, beta=0.0), Y0, (0.0, 0.1))
    sg = lri.solve(pg, ag, 1e-2, precision=precision)
    so = oracle.solve(po, ao, 1e-2)
    assert len(sg.Y) == len(so.Y)
    for k, (yg, yo) in enumerate(zip(sg.Y, so.Y)):
        if kind == "ra" and precision != "fp32":
            assert yg.S.shape == yo.S.shape, f"step {k}: rank {yg.S.shape[0]} vs {yo.S.shape[0]}"
        err = oracle.rel_fro_err(yg.full(), yo.full())
        assert err <= TOL[precision], f"step {k}: {err:.3e}"


def test_burgers_conservative_form_per_column_viscosity(lri, oracle):
    """The Burgers-UQ form: alpha = 0, beta = -1/2, one viscosity per sample."""
    n, mgrid, r = 96, 5, 5
    dx, Y0 = burgers_instance(n, mgrid, r, oracle)
    nu = np.random.default_rng(3).uniform(0.005, 0.02, mgrid * mgrid)
    pg = lri.MatrixDEProblem(lri.BurgersOperator(dx, nu, alpha=0.0, beta=-0.5),
                             lri.SVDLikeRepresentation(Y0.U, Y0.S, Y0.V), (0.0, 0.05))
    po = oracle.MatrixDEProblem(oracle.BurgersOp(n, dx, nu, alpha=0.0, beta=-0.5), Y0, (0.0, 0.05))
    yg = lri.solve(pg, lri.UnconventionalAlgorithm(lri.RK4(2)), 1e-2, save_everystep=False).Y[-1]
    yo = oracle.solve(po, oracle.UnconventionalAlgorithm(oracle.RK4(2)), 1e-2, save_everystep=False).Y[-1]
    assert oracle.rel_fro_err(yg.full(), yo.full()) <= TOL["fp64"]


@pytest.mark.parametrize("kind", ["bug", "primal", "dual", "strang", "ra"])
def test_reference_burgers_smoke_gpu(lri, oracle, kind):
    n, mgrid, r = 1000, 20, 5
    dx, Y0 = burgers_instance(n, mgrid, r, oracle)
    ag, ao = algs(lri, oracle, kind, 10)
    pg = lri.MatrixDEProblem(lri.BurgersOperator(dx, 0.005), lri.SVDLikeRepresentation(Y0.U, Y0.S, Y0.V),
                             (0.0, 0.1))
    po = oracle.MatrixDEProblem(oracle.BurgersOp(n, dx, 0.005), Y0, (0.0, 0.1))
    yg = lri.solve(pg, ag, 1e-2, save_everystep=False).Y[-1]
    yo = oracle.solve(po, ao, 1e-2, save_everystep=False).Y[-1]
    assert np.all(np.isfinite(yg.full()))
    assert oracle.rel_fro_err(yg.full(), yo.full()) <= TOL["fp64"]
