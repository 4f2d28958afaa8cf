"""GPU discrete adjoint of the BUG step (lri_batch_adjoint_step through
lri.bug_gradient) against the CPU adjoint of the same discrete step
(oracle/lri_adjoint.py) and against FP64 central finite differences.

The full-size case is the adjoint workload: F(X; theta) = A X + X A^T +
diag(theta) X with A = tridiag(1, -2, 1) (unscaled), n = m = 2048, r = 32,
theta ~ N(0, 0.1), 200 steps at dt = 1e-4 (RK4 substeps), loss
||Y(T) - X_t||_F^2 with a seeded rank-40 target of spectrum 2^{-k/4};
checkpoints every 20 steps; 32 random directions, h = 1e-6, the directional
derivatives must agree to 1e-4 relative.  The finite differences run as one
batch of 64 perturbed problems.
"""
import os
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                                "lowrankintegrators.jl_gb300"))
import workloads  # noqa: E402


def small_problem(seed=5, n=40, m=36, r=4, rt=6):
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


@pytest.mark.parametrize("scheme", [("RK4", 1), ("RK4", 2), ("Heun", 3)])
def test_adjoint_matches_cpu_adjoint(lri, oracle, scheme):
    from oracle import lri_adjoint as AD
    A0, B, theta, U, S, V, (P, d, Q) = small_problem()
    dt, T = 0.05, 0.35
    sg = getattr(lri, scheme[0])(scheme[1])
    so = getattr(oracle, scheme[0])(scheme[1])
    nsteps = lri.n_steps((0.0, T), dt)
    loss_c, thb_c, Ub_c, Sb_c, Vb_c = AD.loss_and_grad(U, S, V, A0, theta, B, so, dt, nsteps, (P, d, Q),
                                                       checkpoint_every=3)
    prob = lri.MatrixDEProblem(lri.SylvesterTridiagOperator(A0, B, theta), lri.SVDLikeRepresentation(U, S, V),
                               (0.0, T))
    target = lri.SVDLikeRepresentation(P, np.diag(d), Q)
    loss, thb, gr = lri.bug_gradient(prob, lri.UnconventionalAlgorithm(sg), dt, target, checkpoint_every=3)
    rel = lambda a, b: np.linalg.norm(a - b) / np.linalg.norm(b)
    assert abs(loss - loss_c) <= 1e-11 * abs(loss_c)
    assert rel(thb, thb_c) <= 1e-9
    assert rel(gr.U, Ub_c) <= 1e-9
    assert rel(gr.S, Sb_c) <= 1e-9
    assert rel(gr.V, Vb_c) <= 1e-9


def test_adjoint_workload_against_central_differences(lri):
    A0, theta, U, S, V, (P, d, Q) = workloads.adjoint_2048()
    n, r = U.shape
    dt, T = 1e-4, 0.02
    alg = lri.UnconventionalAlgorithm(lri.RK4(1))
    target = lri.SVDLikeRepresentation(P, np.diag(d), Q)
    prob = lri.MatrixDEProblem(lri.SylvesterTridiagOperator(A0, A0, theta), lri.SVDLikeRepresentation(U, S, V),
                               (0.0, T))
    loss, thb, gr = lri.bug_gradient(prob, alg, dt, target, checkpoint_every=20)
    g = np.random.default_rng(11)
    h = 1e-6
    dirs = [tuple(g.standard_normal(x.shape) for x in (theta, U, S, V)) for _ in range(32)]
    probs = []
    for (dth, dU, dS, dV) in dirs:
        for sgn in (1.0, -1.0):
            e = sgn * h
            probs.append(lri.MatrixDEProblem(lri.SylvesterTridiagOperator(A0, A0, theta + e * dth),
                                             lri.SVDLikeRepresentation(U + e * dU, S + e * dS, V + e * dV), (0.0, T)))
    finals = lri.solve_ensemble(probs, alg, dt, precision="fp64")
    losses = [lri.terminal_loss(Y, target)[0] for Y in finals]
    worst = 0.0
    for i, (dth, dU, dS, dV) in enumerate(dirs):
        fd = (losses[2 * i] - losses[2 * i + 1]) / (2 * h)
        an = np.sum(thb * dth) + np.sum(gr.U * dU) + np.sum(gr.S * dS) + np.sum(gr.V * dV)
        worst = max(worst, abs(fd - an) / abs(an))
    assert worst <= 1e-4, f"worst relative disagreement {worst:.3e}"
