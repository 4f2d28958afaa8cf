"""Registered local flow maps (LRI_OP_LOCAL_FLOW, csrc/flows.cuh: the
engine's build-time stand-in for the reference's user-supplied F and
K_rhs / L_rhs / S_rhs hooks, src/integrators/unconventional.jl:2-4,51-79)
against the oracle's dense flow maps, every step: the reaction-diffusion
flow (Allen-Cahn form) for BUG, rank-adaptive BUG and KSL in every
precision, flow 0 against the dedicated Burgers operator (the same
functor: identical bits), and a hybrid greedy problem driven by a local
flow.  Tolerances: FP64 1e-11, double-float 1e-10, FP32 1e-5."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = {"fp64": 1e-11, "df": 1e-10, "fp32": 1e-5}


def _initial(n, m, r, seed):
    g = np.random.default_rng(seed)
    x = (np.arange(n) + 0.5) / n
    cols = [0.6 * np.sin(2 * np.pi * x + g.uniform(0, 2 * np.pi)) + 0.2 * g.standard_normal() * np.cos(4 * np.pi * x)
            for _ in range(m)]
    X = np.stack(cols, axis=1)
    X = X + 1e-3 * g.standard_normal(X.shape)
    U, s, Vt = np.linalg.svd(X, full_matrices=False)
    return 1.0 / n, g.uniform(0.002, 0.01, m), U[:, :r], np.diag(s[:r]), Vt[:r].T


def test_registry_lists_the_flows(lri):
    assert lri.registered_flows()[:2] == ["burgers", "reaction_diffusion"]


@pytest.mark.parametrize("precision", ["fp64", "df", "fp32"])
@pytest.mark.parametrize("kind", ["bug", "ra", "ksl"])
def test_reaction_diffusion_matches_oracle(lri, oracle, precision, kind):
    n, m, r = 96, 40, 6
    h, c, U, S, V = _initial(n, m, r, seed=21)
    dt, T = 1e-3, 8e-3
    if kind == "bug":
        ag, ao = lri.UnconventionalAlgorithm(lri.RK4(2)), oracle.UnconventionalAlgorithm(oracle.RK4(2))
    elif kind == "ra":
        ag = lri.RankAdaptiveUnconventionalAlgorithm(1e-5 if precision != "fp32" else 1e-3, rmax=12,
                                                     K_alg=lri.RK4(2))
        ao = oracle.RankAdaptiveUnconventionalAlgorithm(ag.tol, rmax=12, K_alg=oracle.RK4(2))
    else:
        ag, ao = lri.ProjectorSplitting(lri.PrimalLieTrotter(), lri.RK4(2)), \
            oracle.ProjectorSplitting(oracle.PrimalLieTrotter(), oracle.RK4(2))
    pg = lri.MatrixDEProblem(lri.ReactionDiffusionOperator(h, c, 1.0, -1.0), lri.SVDLikeRepresentation(U, S, V),
                             (0.0, T))
    po = oracle.MatrixDEProblem(oracle.ReactionDiffusionOp(n, h, c, 1.0, -1.0), oracle.SVDLikeRepresentation(U, S, V),
                                (0.0, T))
    sg = lri.solve(pg, ag, dt, precision=precision)
    so = oracle.solve(po, ao, dt)
    assert [y.S.shape[0] for y in sg.Y] == [y.S.shape[0] for y in so.Y]
    for k, (yg, yo) in enumerate(zip(sg.Y, so.Y)):
        err = oracle.rel_fro_err(yg.full(), yo.full())
        assert err <= TOL[precision], f"step {k}: {err:.3e}"


def test_flow_zero_is_the_burgers_operator(lri):
    n, m, r = 64, 24, 5
    h, nu, U, S, V = _initial(n, m, r, seed=3)
    Y0 = lri.SVDLikeRepresentation(U, S, V)
    alg = lri.UnconventionalAlgorithm(lri.RK4(2))
    a = lri.solve(lri.MatrixDEProblem(lri.BurgersOperator(h, nu, -1.0, 0.0), Y0, (0.0, 5e-3)), alg, 1e-3,
                  save_everystep=False).Y[-1]
    b = lri.solve(lri.MatrixDEProblem(lri.LocalFlowOperator("burgers", h, nu, -1.0, 0.0), Y0, (0.0, 5e-3)), alg,
                  1e-3, save_everystep=False).Y[-1]
    assert np.array_equal(a.full(), b.full())


def test_hybrid_with_local_flow_matches_oracle(lri, oracle):
    n, m, r = 96, 30, 4
    h, c, U, S, V = _initial(n, m, r, seed=8)
    g = np.random.default_rng(9)
    snaps = [(U @ S @ V.T) * (1.0 - 0.1 * k) + 1e-3 * g.standard_normal((n, m)) for k in range(7)]
    dt = 1e-3
    y = lambda t: snaps[int(round(t / dt))]
    Z0 = snaps[0].T @ U
    op_o = oracle.ReactionDiffusionOp(n, h, c, 1.0, -1.0)
    so = oracle.solve(oracle.MatrixHybridProblem(y, lambda Z, Uc, t: op_o.L_rhs(Z, Uc, t),
                                                 oracle.TwoFactorRepresentation(U, Z0), (0.0, 6 * dt)),
                      oracle.GreedyIntegrator(oracle.RK4(2)), dt)
    sg = lri.solve(lri.MatrixHybridProblem(y, lri.ReactionDiffusionOperator(h, c, 1.0, -1.0),
                                           lri.TwoFactorRepresentation(U, Z0), (0.0, 6 * dt)),
                   lri.GreedyIntegrator(lri.RK4(2)), dt, precision="fp64")
    for k, (yg, yo) in enumerate(zip(sg.Y, so.Y)):
        e = max(np.linalg.norm(yg.U - yo.U) / np.linalg.norm(yo.U), np.linalg.norm(yg.Z - yo.Z) / np.linalg.norm(yo.Z))
        assert e <= 1e-10, f"step {k}: {e:.3e}"
