"""Edge shapes of the batch engine against the FP64 oracle: rank 1, a
full-rank square instance (r = n = m), the widest panels the one-CTA engine
takes (BUG at r = 64, rank-adaptive at r_max = 32, i.e. 64 columns), and a
batch mixing all of them with a tiny and a tall-skinny instance."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = {"fp64": 1e-10, "df": 1e-9, "fp32": 1e-4}


def inst(seed, n, m, r):
    g = np.random.default_rng(seed)
    A = (g.uniform(0.5, 1.0, n), -2.0 - g.uniform(0, 1, n), g.uniform(0.5, 1.0, n))
    B = (g.uniform(0.5, 1.0, m), -2.0 - g.uniform(0, 1, m), g.uniform(0.5, 1.0, m))
    U, _ = np.linalg.qr(g.standard_normal((n, r)))
    V, _ = np.linalg.qr(g.standard_normal((m, r)))
    S = np.diag(np.linspace(1.0, 0.5, r))
    return A, B, U, S, V


def both(lri, O, shape, alg_g, alg_o, precision, dt=0.02, T=0.1, seed=3):
    A, B, U, S, V = inst(seed, *shape)
    pg = lri.MatrixDEProblem(lri.SylvesterTridiagOperator(A, B), lri.SVDLikeRepresentation(U, S, V), (0.0, T))
    po = O.MatrixDEProblem(O.SylvesterTridiagOp(A, B), O.SVDLikeRepresentation(U, S, V), (0.0, T))
    yg = lri.solve(pg, alg_g, dt, precision=precision, save_everystep=False).Y[-1]
    yo = O.solve(po, alg_o, dt, save_everystep=False).Y[-1]
    return yg, yo


@pytest.mark.parametrize("precision", ["fp64", "df", "fp32"])
@pytest.mark.parametrize("shape", [(40, 30, 1), (8, 8, 8), (200, 180, 64), (1, 1, 1)])
def test_bug_edge_shapes(lri, oracle, shape, precision):
    yg, yo = both(lri, oracle, shape, lri.UnconventionalAlgorithm(lri.RK4(1)),
                  oracle.UnconventionalAlgorithm(oracle.RK4(1)), precision)
    assert oracle.rel_fro_err(yg.full(), yo.full()) <= TOL[precision]


@pytest.mark.parametrize("precision", ["fp64", "df"])
def test_rank_adaptive_widest_panel(lri, oracle, precision):
    yg, yo = both(lri, oracle, (160, 150, 20), lri.RankAdaptiveUnconventionalAlgorithm(1e-5, rmax=32),
                  oracle.RankAdaptiveUnconventionalAlgorithm(1e-5, rmax=32), precision)
    assert yg.S.shape == yo.S.shape
    assert oracle.rel_fro_err(yg.full(), yo.full()) <= TOL[precision]


def test_mixed_edge_batch(lri, oracle):
    shapes = [(40, 30, 1), (8, 8, 8), (200, 180, 64), (1, 1, 1), (1000, 64, 3), (65, 64, 64)]
    insts = [inst(50 + i, *s) for i, s in enumerate(shapes)]
    probs = [lri.MatrixDEProblem(lri.SylvesterTridiagOperator(A, B), lri.SVDLikeRepresentation(U, S, V), (0.0, 0.1))
             for (A, B, U, S, V) in insts]
    out = lri.solve_ensemble(probs, lri.UnconventionalAlgorithm(lri.RK4(1)), 0.02, precision="fp64")
    for i, (A, B, U, S, V) in enumerate(insts):
        po = oracle.MatrixDEProblem(oracle.SylvesterTridiagOp(A, B), oracle.SVDLikeRepresentation(U, S, V),
                                    (0.0, 0.1))
        yo = oracle.solve(po, oracle.UnconventionalAlgorithm(oracle.RK4(1)), 0.02, save_everystep=False).Y[-1]
        assert oracle.rel_fro_err(out[i].full(), yo.full()) <= 1e-10, shapes[i]
