"""The oracle's restatement of GreedyIntegrator and MatrixHybridProblem
(src/integrators/greedy_integrator.jl:73-104, src/primitives.jl:32-41)
against closed-form properties, on the CPU:

* SVD-like greedy fitting reproduces data of exact rank <= r at every step
  (X V and X^T U span the data's ranges, so U S V^T = X);
* the two-factor update U <- polar(X X^T U) for a constant snapshot is a
  power iteration: U converges to the dominant left singular subspace;
* a hybrid problem with F = 0 keeps Z and sets U = polar(X Z);
* every U stays orthonormal, and the polar factor agrees with the
  Newton iteration's limit.
"""
import numpy as np

from oracle import lri_oracle as O


def _low_rank_stream(n, m, r, nsnap, seed=0):
    g = np.random.default_rng(seed)
    U, _ = np.linalg.qr(g.standard_normal((n, r)))
    V, _ = np.linalg.qr(g.standard_normal((m, r)))
    W = g.standard_normal((r, r))
    W = W - W.T
    snaps = []
    for k in range(nsnap):
        t = 0.1 * k
        R = np.linalg.qr(np.eye(r) + t * W)[0]
        s = 2.0 ** -np.arange(r) * (1 + 0.2 * np.sin(t + np.arange(r)))
        snaps.append((U @ R) @ np.diag(s) @ (V @ R).T)
    return snaps


def test_greedy_svd_like_reproduces_exact_rank_data():
    snaps = _low_rank_stream(40, 30, 4, 6)
    Y0 = O.truncated_svd(snaps[0], r=4)
    sol = O.solve(O.MatrixDataProblem(snaps, Y0), O.GreedyIntegrator())
    for k, (Y, X) in enumerate(zip(sol.Y, snaps)):
        assert np.linalg.norm(Y.full() - X) <= 1e-12 * np.linalg.norm(X), f"snapshot {k}"
        assert np.abs(Y.U.T @ Y.U - np.eye(4)).max() <= 1e-13


def test_greedy_two_factor_power_iteration():
    g = np.random.default_rng(3)
    n, m, r = 50, 40, 3
    # singular values 3, 2.5, 2 | 0.5 ... 0.1: a gap of 4 in the power iteration's ratio per step
    Ux, _ = np.linalg.qr(g.standard_normal((n, m)))
    s = np.concatenate([[3.0, 2.5, 2.0], np.linspace(0.5, 0.1, m - 3)])
    X = Ux @ np.diag(s) @ np.linalg.qr(g.standard_normal((m, m)))[0].T
    U0, _ = np.linalg.qr(g.standard_normal((n, r)))
    u0 = O.TwoFactorRepresentation(U0, X.T @ U0)
    sol = O.solve(O.MatrixDataProblem(lambda t: X, u0, (0.0, 60.0)), O.GreedyIntegrator(), 1.0,
                  save_everystep=False)
    U = sol.Y[-1].U
    P = np.linalg.svd(X)[0][:, :r]
    assert np.linalg.norm(U @ U.T - P @ P.T) <= 1e-8
    assert np.abs(U.T @ U - np.eye(r)).max() <= 1e-13


def test_hybrid_with_zero_flow_keeps_z():
    g = np.random.default_rng(5)
    n, m, r = 30, 20, 3
    snaps = [g.standard_normal((n, m)) for _ in range(4)]
    U0, _ = np.linalg.qr(g.standard_normal((n, r)))
    Z0 = g.standard_normal((m, r))
    prob = O.MatrixHybridProblem(lambda t: snaps[int(round(t))], lambda Z, U, t: np.zeros_like(Z),
                                 O.TwoFactorRepresentation(U0, Z0), (0.0, 3.0))
    sol = O.solve(prob, O.GreedyIntegrator(), 1.0)
    for k in range(1, 4):
        Y = sol.Y[k]
        assert np.array_equal(Y.Z, Z0)
        A = snaps[k] @ Z0
        # polar factor: U = A (A^T A)^{-1/2}
        w, Q = np.linalg.eigh(A.T @ A)
        Up = A @ (Q @ np.diag(w ** -0.5) @ Q.T)
        assert np.linalg.norm(Y.U - Up) <= 1e-12


def test_hybrid_coefficients_follow_the_flow():
    """With X = U0 Z^T data of the coefficient flow itself, the polar step
    keeps U = U0 and Z follows the L-substep flow of the operator."""
    n, m, r = 24, 10, 2
    g = np.random.default_rng(7)
    U0, _ = np.linalg.qr(g.standard_normal((n, r)))
    Z0 = g.standard_normal((m, r))
    lam = -0.5
    f = lambda Z, U, t: lam * Z
    expZ = lambda t: np.exp(lam * t) * Z0
    prob = O.MatrixHybridProblem(lambda t: U0 @ expZ(t).T, f, O.TwoFactorRepresentation(U0, Z0), (0.0, 0.5))
    sol = O.solve(prob, O.GreedyIntegrator(O.RK4(4)), 0.1)
    Y = sol.Y[-1]
    assert np.linalg.norm(Y.U @ Y.U.T - U0 @ U0.T) <= 1e-12
    assert np.linalg.norm(Y.Z - expZ(0.5)) <= 1e-7 * np.linalg.norm(Z0)
