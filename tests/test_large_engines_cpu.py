"""Host-side checks of the large engines' entry points (solve_stream,
solve_burgers_large): problems the engines do not take are rejected before
any device work, so these run without a GPU."""
import numpy as np
import pytest


def _y0(lri, n, m, r):
    g = np.random.default_rng(0)
    U = np.linalg.qr(g.standard_normal((n, r)))[0]
    V = np.linalg.qr(g.standard_normal((m, r)))[0]
    return lri.SVDLikeRepresentation(U, np.diag(2.0 ** -np.arange(r)), V)


def test_stream_engine_takes_snapshot_lists_only(lri):
    y0 = _y0(lri, 64, 48, 4)
    prob = lri.MatrixDataProblem(lambda t: np.zeros((64, 48)), y0, (0.0, 1.0))
    with pytest.raises(ValueError):
        lri.solve_stream(prob, lri.RankAdaptiveUnconventionalAlgorithm(1e-6, rmax=8))


def test_burgers_engine_takes_burgers_problems_only(lri):
    y0 = _y0(lri, 64, 48, 4)
    sub = np.full(64, 1.0)
    dia = np.full(64, -2.0)
    prob = lri.MatrixDEProblem(lri.SylvesterTridiagOperator((sub, dia, sub), (sub[:48], dia[:48], sub[:48])),
                               y0, (0.0, 1e-3))
    with pytest.raises(lri.LriError):
        lri.solve_burgers_large(prob, lri.RankAdaptiveUnconventionalAlgorithm(1e-6, rmax=8), 1e-4)


def test_data_problem_with_function_needs_tspan(lri):
    y0 = _y0(lri, 16, 12, 2)
    with pytest.raises(ValueError):
        lri.MatrixDataProblem(lambda t: np.zeros((16, 12)), y0)
    prob = lri.MatrixDataProblem([np.zeros((16, 12))] * 3, y0)
    assert prob.tspan == (1, 3)
