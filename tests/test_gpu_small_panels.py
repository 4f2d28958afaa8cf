"""GPU parity of the instance engine's register-resident paths for short
panels (at most 256 rows and 8 columns: the K and L substeps with one row per
thread) and small cores (p*q <= 256: the S substep with one entry per
thread), against the FP64 oracle.

* Non-orthonormal initial factors in FP64: the literal rhs F(K V^T) V =
  T K (V^T V) + K P^T with V^T V far from I takes the full Gram product (the
  FP32 correction for V^T V = I + E applies only when E is at rounding
  level); every later step has orthonormal bases.  Tolerance 1e-11 (the FP64
  tolerance of the engine tests: same discrete scheme, different summation
  order).
* Panel heights and widths on both sides of the path's limits (256 / 257
  rows, 8 / 9 columns), FP64 (1e-11) and double-float (1e-10).
"""
import os
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "lowrankintegrators.jl_gb300"))
import workloads  # noqa: E402

TOL = {"fp64": 1e-11, "df": 1e-10}


def instance(seed, n, m, r, skew=0.0):
    g = np.random.default_rng(seed)
    A = (g.uniform(0.5, 1.0, n), -2.0 - g.uniform(0, 1, n), g.uniform(0.5, 1.0, n))
    B = (g.uniform(0.5, 1.0, m), -2.0 - g.uniform(0, 1, m), g.uniform(0.5, 1.0, m))
    U = workloads.random_orthonormal(g, n, r)
    V = workloads.random_orthonormal(g, m, r)
    if skew:
        # columns of norm ~1 +- skew, no longer orthogonal: X^T X - I ~ skew
        U = U + skew * g.standard_normal(U.shape) / np.sqrt(n)
        V = V + skew * g.standard_normal(V.shape) / np.sqrt(m)
    S = np.diag(np.linspace(1.0, 0.2, r))
    return A, B, U, S, V


def algs(lri, O, kind):
    if kind == "bug":
        return lri.UnconventionalAlgorithm(lri.RK4(3)), O.UnconventionalAlgorithm(O.RK4(3))
    # KSL primal: its backward S substep runs on (U1, V0), so the small-core
    # path sees a non-orthonormal V0 as well
    return (lri.ProjectorSplitting(lri.PrimalLieTrotter(), lri.RK4(3)),
            O.ProjectorSplitting(O.PrimalLieTrotter(), O.RK4(3)))


def compare(lri, O, A, B, U, S, V, kind, precision, dt=0.02, T=0.1):
    ag, ao = algs(lri, O, kind)
    pg = lri.MatrixDEProblem(lri.SylvesterTridiagOperator(A, B), lri.SVDLikeRepresentation(U, S, V), (0.0, T))
    po = O.MatrixDEProblem(O.SylvesterTridiagOp(A, B), O.SVDLikeRepresentation(U, S, V), (0.0, T))
    sg = lri.solve(pg, ag, dt, precision=precision)
    so = O.solve(po, ao, dt)
    assert len(sg.Y) == len(so.Y)
    for k, (yg, yo) in enumerate(zip(sg.Y, so.Y)):
        assert yg.rank == yo.rank, f"step {k}: rank {yg.rank} != {yo.rank}"
        err = O.rel_fro_err(yg.full(), yo.full())
        assert err <= TOL[precision], f"step {k}: {err:.3e}"


@pytest.mark.parametrize("kind", ["bug", "primal"])
@pytest.mark.parametrize("shape", [(48, 40, 3), (60, 52, 7), (256, 200, 8)])
def test_non_orthonormal_initial_factors_fp64(lri, oracle, kind, shape):
    n, m, r = shape
    A, B, U, S, V = instance(11, n, m, r, skew=0.3)
    assert np.abs(V.T @ V - np.eye(r)).max() > 1e-3  # the full Gram product is taken
    compare(lri, oracle, A, B, U, S, V, kind, "fp64")


@pytest.mark.parametrize("precision", ["fp64", "df"])
@pytest.mark.parametrize("shape", [(256, 257, 8), (257, 256, 8), (256, 256, 9), (120, 255, 4), (33, 256, 5)])
def test_panel_limits(lri, oracle, precision, shape):
    n, m, r = shape
    A, B, U, S, V = instance(5, n, m, r)
    compare(lri, oracle, A, B, U, S, V, "bug", precision)
