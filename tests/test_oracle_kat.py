"""Pins of the FP64 oracle that do not depend on the oracle itself.

* closed-form known answers (F = 0; invariant eigen-subspaces of a linear F,
  where BUG/KSL with RK4 substeps reproduce an analytic RK4 polynomial);
* the exactness property of the integrators on rank-r data streams
  (Ceruti-Lubich 2021, Lubich-Oseledets 2014);
* the reference's own assertion (test/data_driven_approximation.jl:22-31):
  continuous stream and discrete snapshots agree;
* the reference's Burgers smoke test (test/data_agnostic_approximation.jl),
  re-expressed as "runs, stays finite and bounded";
* the truncation rule and the time loop of src/primitives.jl:68-80.
"""
import math

import numpy as np
import pytest

from oracle import lri_oracle as O


def rk4_poly(z, nsub):
    """Stability polynomial of classic RK4 composed nsub times (step z/nsub)."""
    w = z / nsub
    return (1 + w + w ** 2 / 2 + w ** 3 / 6 + w ** 4 / 24) ** nsub


def sym_tridiag_eig(n, a, b):
    """Eigenpairs of the symmetric tridiagonal Toeplitz matrix tridiag(b, a, b)."""
    k = np.arange(1, n + 1)
    lam = a + 2 * b * np.cos(k * np.pi / (n + 1))
    Q = np.sqrt(2.0 / (n + 1)) * np.sin(np.outer(np.arange(1, n + 1), k) * np.pi / (n + 1))
    return lam, Q


def invariant_problem(n=24, m=20, r=3, a=-2.0, b=0.7, c=-1.5, d=0.4):
    lamA, QA = sym_tridiag_eig(n, a, b)
    lamB, QB = sym_tridiag_eig(m, c, d)
    ia = [1, 4, 7][:r]
    ib = [0, 2, 5][:r]
    U = QA[:, ia]
    V = QB[:, ib]
    S = np.diag([1.0, 0.3, 0.05][:r])
    A = (np.full(n, b), np.full(n, a), np.full(n, b))
    B = (np.full(m, d), np.full(m, c), np.full(m, d))
    return A, B, U, S, V, lamA[ia], lamB[ib]


@pytest.mark.parametrize("alg", [
    O.UnconventionalAlgorithm(O.RK4(3)),
    O.ProjectorSplitting(O.PrimalLieTrotter(), O.RK4(3)),
    O.ProjectorSplitting(O.DualLieTrotter(), O.RK4(3)),
])
def test_invariant_subspace_closed_form(alg):
    """A U0 = U0 diag(la), B V0 = V0 diag(lb): with RK4 substeps every step
    multiplies S_ij by R4(dt (la_i + lb_j)) (BUG: K, then S on the new basis;
    the closed form follows from the substep flows being diagonal)."""
    A, B, U, S, V, la, lb = invariant_problem()
    dt, nsteps, nsub = 0.05, 8, 3
    prob = O.MatrixDEProblem(O.SylvesterTridiagOp(A, B), O.SVDLikeRepresentation(U, S, V), (0.0, dt * nsteps))
    Y = O.solve(prob, alg, dt).Y[-1].full()
    if isinstance(alg, O.UnconventionalAlgorithm):
        # K/L steps keep the bases (up to column signs); the Galerkin S-step
        # from M S N^T multiplies S_ij by R(dt (la_i + lb_j)) once per step.
        fac = rk4_poly(dt * (la[:, None] + lb[None, :]), nsub)
    else:
        # KSL: K forward (R), S backward (R(-z)), L forward (R) per step.
        z = dt * (la[:, None] + lb[None, :])
        fac = rk4_poly(z, nsub) * rk4_poly(-z, nsub) * rk4_poly(z, nsub)
    Sd = np.diag(S)[:, None] * np.eye(len(la))
    Yref = U @ (Sd * fac ** nsteps) @ V.T
    assert O.rel_fro_err(Y, Yref) < 1e-13


def test_zero_flow_is_constant():
    rng = np.random.default_rng(3)
    U, _ = np.linalg.qr(rng.standard_normal((30, 4)))
    V, _ = np.linalg.qr(rng.standard_normal((25, 4)))
    S = rng.standard_normal((4, 4))
    Y0 = O.SVDLikeRepresentation(U, S, V)
    for alg in [O.UnconventionalAlgorithm(), O.ProjectorSplitting(O.Strang()),
                O.RankAdaptiveUnconventionalAlgorithm(1e-10, rmax=8)]:
        sol = O.solve(O.MatrixDEProblem(O.ZeroOp(), Y0, (0.0, 0.1)), alg, 0.01)
        assert O.rel_fro_err(sol.Y[-1], Y0) < 1e-14


def rank_r_stream(seed=5, n=40, m=30, r=3, decay3=None):
    """A(t) = Q_n(t) U0 diag(s(t)) V0^T Q_m(t)^T with rotations Q(t) = expm(0.3 t W),
    so the singular values of A(t) are s(t) exactly."""
    rng = np.random.default_rng(seed)
    from scipy.linalg import expm

    Wn = rng.standard_normal((n, n))
    Wn = Wn - Wn.T
    Wm = rng.standard_normal((m, m))
    Wm = Wm - Wm.T
    U0, _ = np.linalg.qr(rng.standard_normal((n, r)))
    V0, _ = np.linalg.qr(rng.standard_normal((m, r)))
    s0 = np.array([1.0, 0.5, 0.2])[:r]

    def sv(t):
        s = s0 * np.exp(-t * np.arange(1, r + 1))
        if decay3 is not None:
            s[-1] = 0.2 * np.exp(-decay3 * t)
        return s

    def Y(t):
        return expm(0.3 * t * Wn) @ U0 @ np.diag(sv(t)) @ V0.T @ expm(0.3 * t * Wm).T

    Y.sv = sv
    return Y


@pytest.mark.parametrize("alg", [
    O.UnconventionalAlgorithm(),
    O.ProjectorSplitting(O.PrimalLieTrotter()),
    O.ProjectorSplitting(O.DualLieTrotter()),
    O.RankAdaptiveUnconventionalAlgorithm(1e-10, rmax=6),
])
def test_exactness_on_rank_r_data(alg):
    """Data A(t) of exact rank r, Y0 = A(t0): the integrators reproduce A(t)
    (exactness property of projector splitting and of BUG)."""
    Y = rank_r_stream()
    Y0 = O.truncated_svd(Y(0.0), r=3)
    sol = O.solve(O.MatrixDataProblem(Y, Y0, (0.0, 0.5)), alg, 0.05)
    assert O.rel_fro_err(sol.Y[-1], Y(sol.t[-1])) < 1e-10


def test_rank_adaptive_follows_numerical_rank():
    """Rank-3 data whose third singular value decays as 0.2 exp(-100 t): the
    integrator is exact on it, so its core singular values are those of A(t)
    and the truncation (tol = 1e-8) must give the analytic rank trajectory."""
    Y = rank_r_stream(decay3=100.0)
    Y0 = O.truncated_svd(Y(0.0), r=3)
    tol = 1e-8
    sol = O.solve(O.MatrixDataProblem(Y, Y0, (0.0, 0.3)), O.RankAdaptiveUnconventionalAlgorithm(tol, rmax=6), 0.025)
    ranks = [y.rank for y in sol.Y]
    expected = [3] + [O.truncate_to_tolerance(np.concatenate([Y.sv(t), np.zeros(3)]), tol) for t in sol.t[1:]]
    assert ranks == expected
    assert 2 in ranks and ranks[-1] == 2
    assert O.rel_fro_err(sol.Y[-1], Y(sol.t[-1])) < 1e-8


def test_reference_continuous_vs_discrete():
    """test/data_driven_approximation.jl:22-31 with a seeded stream: a
    function stream with dt = 0.01 and the 101 snapshots give the same final
    factors, elementwise isapprox with rtol = sqrt(eps) (Julia's default)."""
    import sys, os
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(__file__)), "lowrankintegrators.jl_gb300"))
    import workloads

    Y = workloads.data_rotation(seed=0, N=100)
    X0 = O.truncated_svd(Y(0.0), tol=1e-4)
    data = [Y(t) for t in np.arange(0, 101) * 0.01]
    rtol = math.sqrt(np.finfo(float).eps)
    for alg in [O.UnconventionalAlgorithm(), O.ProjectorSplitting(O.PrimalLieTrotter()),
                O.ProjectorSplitting(O.DualLieTrotter()), O.RankAdaptiveUnconventionalAlgorithm(1e-8, rmax=20)]:
        sol = O.solve(O.MatrixDataProblem(Y, X0, (0.0, 1.0)), alg, 1e-2)
        dsol = O.solve(O.MatrixDataProblem(data, X0), alg)
        a, b = sol.Y[-1].full(), dsol.Y[-1].full()
        assert np.all(np.abs(a - b) <= rtol * np.maximum(np.abs(a), np.abs(b))), type(alg).__name__


def test_reference_burgers_smoke():
    """test/data_agnostic_approximation.jl: Burgers n=1000, m=20^2, r=5,
    dt=1e-2 on [0,1] for BUG, KSL (three orders) and RA(1e-4, rmax=10).
    Here on a shortened span [0, 0.1] with RK4(10) substeps."""
    n, m = 1000, 20
    dx = math.pi / n
    x = np.arange(dx / 2, math.pi, dx)[:n]
    xi = np.linspace(-1, 1, m)
    cols = []
    for x2 in xi:
        for x1 in xi:
            ub = 0.5 * (np.exp(np.cos(x)) - 1.5) * np.sin(x + 2 * math.pi * 0.37)
            cols.append(ub + 0.5 * x1 * np.sin(2 * math.pi * x) + 0.5 * x2 * np.sin(3 * math.pi * x))
    rho0 = np.array(cols).T
    Y0 = O.truncated_svd(rho0, r=5)
    op = O.BurgersOp(n, dx, 0.005, alpha=-1.0, beta=0.0)
    nrm0 = np.linalg.norm(Y0.full())
    for alg in [O.UnconventionalAlgorithm(O.RK4(10)), O.ProjectorSplitting(O.PrimalLieTrotter(), O.RK4(10)),
                O.ProjectorSplitting(O.DualLieTrotter(), O.RK4(10)), O.ProjectorSplitting(O.Strang(), O.RK4(10)),
                O.RankAdaptiveUnconventionalAlgorithm(1e-4, rmax=10, K_alg=O.RK4(10))]:
        sol = O.solve(O.MatrixDEProblem(op, Y0, (0.0, 0.1)), alg, 1e-2, save_everystep=False)
        Yf = sol.Y[-1].full()
        assert np.all(np.isfinite(Yf))
        assert np.linalg.norm(Yf) < 2 * nrm0


def test_dense_and_factored_rhs_agree():
    rng = np.random.default_rng(11)
    n, m, r = 30, 26, 4
    A = (rng.uniform(0.5, 1, n), -2 - rng.uniform(0, 1, n), rng.uniform(0.5, 1, n))
    B = (rng.uniform(0.5, 1, m), -2 - rng.uniform(0, 1, m), rng.uniform(0.5, 1, m))
    U, _ = np.linalg.qr(rng.standard_normal((n, r)))
    V, _ = np.linalg.qr(rng.standard_normal((m, r)))
    Y0 = O.SVDLikeRepresentation(U, np.diag([1, .5, .25, .1]), V)
    for alg in [O.UnconventionalAlgorithm(O.RK4(2)), O.ProjectorSplitting(O.Strang(), O.RK4(2)),
                O.RankAdaptiveUnconventionalAlgorithm(1e-6, rmax=8, K_alg=O.RK4(2))]:
        a = O.solve(O.MatrixDEProblem(O.SylvesterTridiagOp(A, B, True), Y0, (0, .1)), alg, .01).Y[-1]
        b = O.solve(O.MatrixDEProblem(O.SylvesterTridiagOp(A, B, False), Y0, (0, .1)), alg, .01).Y[-1]
        assert O.rel_fro_err(a, b) < 1e-13


def test_bug_first_order_convergence():
    """Linear F whose exact solution stays rank r (A, B symmetric, Y0 built
    from eigenvectors plus a rotation): the BUG error against expm decreases
    at least linearly in dt."""
    from scipy.linalg import expm
    n = m = 24
    a, b = -2.0, 0.8
    A = (np.full(n, b), np.full(n, a), np.full(n, b))
    Ad = O.tri_dense(*A)
    rng = np.random.default_rng(2)
    U, _ = np.linalg.qr(rng.standard_normal((n, 3)))
    V, _ = np.linalg.qr(rng.standard_normal((m, 3)))
    Y0 = O.SVDLikeRepresentation(U, np.diag([1.0, 0.4, 0.1]), V)
    T = 0.2
    Xex = expm(T * Ad) @ Y0.full() @ expm(T * Ad).T
    errs = []
    for dt in [0.04, 0.02, 0.01]:
        y = O.solve(O.MatrixDEProblem(O.SylvesterTridiagOp(A, A), Y0, (0, T)), O.UnconventionalAlgorithm(O.RK4(2)),
                    dt).Y[-1]
        errs.append(O.rel_fro_err(y, Xex))
    assert errs[2] < errs[1] < errs[0]
    assert errs[0] / errs[2] > 3.0


def test_truncate_to_tolerance():
    s = np.array([1.0, 0.1, 0.01, 0.001])
    assert O.truncate_to_tolerance(s, 0.0) == 4   # nothing may be dropped
    assert O.truncate_to_tolerance(s, 0.0011) == 3  # tail 0.001 < tol
    assert O.truncate_to_tolerance(s, 0.001) == 4  # strict inequality keeps it
    assert O.truncate_to_tolerance(s, 0.02) == 2
    assert O.truncate_to_tolerance(s, 10.0) == 1   # at least one kept


def test_time_loop_step_count():
    """src/primitives.jl:70-74: t accumulates, loop while (tf-t)/T > 1e-8."""
    assert O.n_steps((0.0, 0.1), 1e-4) == 1000
    assert O.n_steps((0.0, 1.0), 1e-2) == 100
    assert O.n_steps((0.0, 2.0), 1e-2) == 200
    assert O.n_steps((1, 101), 1) == 100
    assert O.n_steps((0.0, 0.5), 0.3) == 2  # no clipping to tf
