"""The CPU discrete adjoint of the BUG step (the oracle of the GPU adjoint):
its forward step reproduces the oracle's bug_step, and its gradient matches
FP64 central finite differences on random directions."""
import numpy as np
import pytest

from oracle import lri_adjoint as AD
from oracle import lri_oracle as O


def problem(seed=5, n=24, m=20, r=4, rt=6):
    g = np.random.default_rng(seed)
    A0 = (np.ones(n), -2.0 * np.ones(n), np.ones(n))
    B = (g.uniform(0.5, 1, m), -2.0 - g.uniform(0, 1, m), g.uniform(0.5, 1, m))
    theta = g.normal(0.0, 0.1, n)
    U, _ = np.linalg.qr(g.standard_normal((n, r)))
    V, _ = np.linalg.qr(g.standard_normal((m, r)))
    S = np.diag(2.0 ** (-np.arange(1, r + 1) / 4.0)) + 0.05 * g.standard_normal((r, r))
    P, _ = np.linalg.qr(g.standard_normal((n, rt)))
    Q, _ = np.linalg.qr(g.standard_normal((m, rt)))
    d = 2.0 ** (-np.arange(1, rt + 1) / 4.0)
    return A0, B, theta, U, S, V, (P, d, Q)


def test_forward_matches_oracle_bug_step():
    A0, B, theta, U, S, V, _ = problem()
    A = (A0[0], A0[1] + theta, A0[2])
    sch = O.RK4(2)
    U1, S1, V1, _ = AD.bug_step_forward(U, S, V, A, B, sch, 0.05)
    prob = O.MatrixDEProblem(O.SylvesterTridiagOp(A, B), O.SVDLikeRepresentation(U, S, V), (0.0, 0.05))
    Y = O.solve(prob, O.UnconventionalAlgorithm(sch), 0.05).Y[-1]
    assert np.linalg.norm(U1 @ S1 @ V1.T - Y.full()) <= 1e-13 * np.linalg.norm(Y.full())


def test_qr_backward_matches_differences():
    g = np.random.default_rng(1)
    Kx = g.standard_normal((15, 4))
    W = g.standard_normal((15, 4))
    f = lambda K: float(np.sum(W * np.linalg.qr(K, mode="reduced")[0]))
    Q, R = np.linalg.qr(Kx, mode="reduced")
    G = AD.qr_backward(Q, R, W)
    D = g.standard_normal(Kx.shape)
    h = 1e-6
    fd = (f(Kx + h * D) - f(Kx - h * D)) / (2 * h)
    assert abs(fd - np.sum(G * D)) <= 1e-7 * max(1.0, abs(fd))


@pytest.mark.parametrize("scheme", [("RK4", 1), ("Heun", 2)])
def test_gradient_matches_central_differences(scheme):
    A0, B, theta, U, S, V, target = problem()
    sch = getattr(O, scheme[0])(scheme[1])
    dt, nsteps = 0.05, 7
    loss, thb, Ub, Sb, Vb = AD.loss_and_grad(U, S, V, A0, theta, B, sch, dt, nsteps, target, checkpoint_every=3)
    assert np.isclose(loss, AD.loss_only(U, S, V, A0, theta, B, sch, dt, nsteps, target), rtol=1e-13)
    g = np.random.default_rng(7)
    h = 1e-6
    for _ in range(6):
        dth, dU, dS, dV = (g.standard_normal(x.shape) for x in (theta, U, S, V))
        f = lambda e: AD.loss_only(U + e * dU, S + e * dS, V + e * dV, A0, theta + e * dth, B, sch, dt, nsteps,
                                   target)
        fd = (f(h) - f(-h)) / (2 * h)
        an = np.sum(thb * dth) + np.sum(Ub * dU) + np.sum(Sb * dS) + np.sum(Vb * dV)
        assert abs(fd - an) <= 1e-6 * abs(an), (fd, an)
