"""FP64 CPU discrete adjoint of the BUG step (the oracle for the GPU adjoint).

TEST INFRASTRUCTURE ONLY, like ``lri_oracle``: only ``tests/`` and the
benchmark's CPU leg may import it; the product never calls it.

The reference (LowRankIntegrators.jl) has no differentiation; this module is
the "plain CPU gradient of the same discrete step" that the GPU adjoint is
checked against, next to central finite differences.  The forward step is the
oracle's ``bug_step`` (src/integrators/unconventional.jl:121-157) for the
Sylvester flow F(X) = A X + X B^T with A = A0 + diag(theta), written out with
its intermediates kept (``tape``); ``tests/test_adjoint_cpu.py`` checks that it
reproduces ``lri_oracle.bug_step`` and that the reverse sweep matches central
differences.

Forward (one step, fixed-step RK with sub-diagonal tableau, nsub substeps):
  K-step  K' = A K G_V + K P_V^T,  G_V = V0^T V0, P_V = V0^T B V0,  K0 = U0 S0
  U1 = Q(K1) (Householder, thin),   M = U1^T U0
  L-step  L' = B L G_U + L P_U^T,  G_U = U0^T U0, P_U = U0^T A U0,  L0 = V0 S0^T
  V1 = Q(L1),                      N = V1^T V0
  S-step  S' = Pu S Gv + Gu S Pv^T  on (U1, V1), from S~0 = M S0 N^T
Reverse: the adjoint of each map in the opposite order.  For A = QR (thin,
R invertible) with only Q used downstream:
  A_bar = (Q_bar + Q copyltu(-Q_bar^T Q)) R^{-T},
  copyltu(X) = tril(X) + tril(X, -1)^T.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import List, Tuple

import numpy as np

from .lri_oracle import SubstepScheme, tri_apply


def tri_transpose(sub, dia, sup):
    """Coefficients of T^T for T = tridiag(sub, dia, sup) (sub[0], sup[-1] unused)."""
    n = len(dia)
    subT = np.zeros(n)
    supT = np.zeros(n)
    subT[1:] = sup[:-1]
    supT[:-1] = sub[1:]
    return subT, np.asarray(dia, dtype=np.float64), supT


def _rk_forward(L, y0, scheme: SubstepScheme, dt):
    """Stage form of the scheme on y' = L(y); returns y1 and the stage inputs
    of every substep (list of lists)."""
    h = dt / scheme.nsub
    y = y0
    stages = []
    for _ in range(scheme.nsub):
        zs = []
        acc = None
        kprev = None
        for s in range(len(scheme.b)):
            z = y if s == 0 else y + (h * scheme.a[s]) * kprev
            zs.append(z)
            k = L(z)
            acc = scheme.b[s] * k if acc is None else acc + scheme.b[s] * k
            kprev = k
        stages.append(zs)
        y = y + h * acc
    return y, stages


def _rk_reverse(LT, coef_grad, stages, ybar1, scheme: SubstepScheme, dt):
    """Adjoint of ``_rk_forward`` for a linear L: returns y0_bar; calls
    coef_grad(kbar, z) for every stage (the operator-coefficient gradients)."""
    h = dt / scheme.nsub
    ns = len(scheme.b)
    ybar = ybar1
    for zs in reversed(stages):
        yb_next = ybar            # adjoint of the substep's output
        ybar = yb_next.copy()     # identity term y1 = y + ...
        kbar_next_in = None       # adjoint of stage s+1's input, to propagate into k_s
        for s in reversed(range(ns)):
            kbar = (h * scheme.b[s]) * yb_next
            if kbar_next_in is not None:
                kbar = kbar + (h * scheme.a[s + 1]) * kbar_next_in
            coef_grad(kbar, zs[s])
            zbar = LT(kbar)
            ybar = ybar + zbar
            kbar_next_in = zbar
    return ybar


def qr_backward(Q, R, Qbar):
    """Adjoint of the thin QR A = QR when only Q is used downstream."""
    Mx = -(Qbar.T @ Q)
    C = Qbar + Q @ (np.tril(Mx) + np.tril(Mx, -1).T)
    # A_bar = C R^{-T}
    return np.linalg.solve(R, C.T).T


@dataclass
class StepTape:
    U0: np.ndarray
    S0: np.ndarray
    V0: np.ndarray
    U1: np.ndarray
    V1: np.ndarray
    RK: np.ndarray
    RL: np.ndarray
    M: np.ndarray
    N: np.ndarray
    GV: np.ndarray
    PV: np.ndarray
    GU: np.ndarray
    PU: np.ndarray
    Kst: list
    Lst: list
    Sst: list
    Pu1: np.ndarray
    Gu1: np.ndarray
    Pv1: np.ndarray
    Gv1: np.ndarray


def bug_step_forward(U0, S0, V0, A, B, scheme: SubstepScheme, dt, sS: SubstepScheme = None, sL: SubstepScheme = None):
    """One BUG step (unconventional.jl:133-157) for F = A X + X B^T; A and B
    are (sub, diag, sup) triples (theta already on A's diagonal)."""
    sK = scheme
    sL = sL or scheme
    sS = sS or scheme
    GV = V0.T @ V0
    PV = V0.T @ tri_apply(*B, V0)
    K1, Kst = _rk_forward(lambda K: tri_apply(*A, K) @ GV + K @ PV.T, U0 @ S0, sK, dt)
    U1, RK = np.linalg.qr(K1, mode="reduced")
    M = U1.T @ U0
    GU = U0.T @ U0
    PU = U0.T @ tri_apply(*A, U0)
    L1, Lst = _rk_forward(lambda L: tri_apply(*B, L) @ GU + L @ PU.T, V0 @ S0.T, sL, dt)
    V1, RL = np.linalg.qr(L1, mode="reduced")
    N = V1.T @ V0
    Pu1 = U1.T @ tri_apply(*A, U1)
    Gu1 = U1.T @ U1
    Pv1 = V1.T @ tri_apply(*B, V1)
    Gv1 = V1.T @ V1
    S1, Sst = _rk_forward(lambda S: Pu1 @ S @ Gv1 + Gu1 @ S @ Pv1.T, M @ S0 @ N.T, sS, dt)
    tape = StepTape(U0, S0, V0, U1, V1, RK, RL, M, N, GV, PV, GU, PU, Kst, Lst, Sst, Pu1, Gu1, Pv1, Gv1)
    return U1, S1, V1, tape


def bug_step_vjp(tape: StepTape, A, B, scheme: SubstepScheme, dt, Ub1, Sb1, Vb1,
                 sS: SubstepScheme = None, sL: SubstepScheme = None):
    """Reverse sweep of one step: (U1_bar, S1_bar, V1_bar) -> (U0_bar,
    S0_bar, V0_bar, theta_bar) with theta the diagonal shift of A."""
    sK = scheme
    sL = sL or scheme
    sS = sS or scheme
    t = tape
    AT = tri_transpose(*A)
    BT = tri_transpose(*B)
    n = t.U0.shape[0]
    thb = np.zeros(n)
    # S-step: S' = Pu S Gv + Gu S Pv^T
    cg = {"Pu": 0.0, "Gv": 0.0, "Gu": 0.0, "Pv": 0.0}

    def s_coef(kb, z):
        cg["Pu"] = cg["Pu"] + kb @ t.Gv1.T @ z.T
        cg["Gv"] = cg["Gv"] + (t.Pu1 @ z).T @ kb
        cg["Gu"] = cg["Gu"] + kb @ t.Pv1 @ z.T
        cg["Pv"] = cg["Pv"] + kb.T @ t.Gu1 @ z

    St0b = _rk_reverse(lambda X: t.Pu1.T @ X @ t.Gv1.T + t.Gu1.T @ X @ t.Pv1, s_coef, t.Sst, Sb1, sS, dt)
    # S~0 = M S0 N^T
    Mb = St0b @ t.N @ t.S0.T
    Nb = St0b.T @ t.M @ t.S0
    S0b = t.M.T @ St0b @ t.N
    # coefficients of the S-step from U1, V1
    U1b = Ub1 + t.U0 @ Mb.T + t.U1 @ (cg["Gu"] + cg["Gu"].T) + tri_apply(*A, t.U1) @ cg["Pu"].T \
        + tri_apply(*AT, t.U1) @ cg["Pu"]
    thb += np.sum((t.U1 @ cg["Pu"].T) * t.U1, axis=1)
    V1b = Vb1 + t.V0 @ Nb.T + t.V1 @ (cg["Gv"] + cg["Gv"].T) + tri_apply(*B, t.V1) @ cg["Pv"].T \
        + tri_apply(*BT, t.V1) @ cg["Pv"]
    U0b = t.U1 @ Mb
    V0b = t.V1 @ Nb
    # K-step
    K1b = qr_backward(t.U1, t.RK, U1b)
    kg = {"G": 0.0, "P": 0.0}

    def k_coef(kb, z):
        kg["G"] = kg["G"] + tri_apply(*A, z).T @ kb
        kg["P"] = kg["P"] + kb.T @ z
        thb[:] += np.sum(kb * (z @ t.GV), axis=1)

    K0b = _rk_reverse(lambda X: tri_apply(*AT, X) @ t.GV.T + X @ t.PV, k_coef, t.Kst, K1b, sK, dt)
    U0b += K0b @ t.S0.T
    S0b += t.U0.T @ K0b
    V0b += t.V0 @ (kg["G"] + kg["G"].T) + tri_apply(*B, t.V0) @ kg["P"].T + tri_apply(*BT, t.V0) @ kg["P"]
    # L-step
    L1b = qr_backward(t.V1, t.RL, V1b)
    lg = {"G": 0.0, "P": 0.0}

    def l_coef(kb, z):
        lg["G"] = lg["G"] + tri_apply(*B, z).T @ kb
        lg["P"] = lg["P"] + kb.T @ z

    L0b = _rk_reverse(lambda X: tri_apply(*BT, X) @ t.GU.T + X @ t.PU, l_coef, t.Lst, L1b, sL, dt)
    V0b += L0b @ t.S0
    S0b += L0b.T @ t.V0
    U0b += t.U0 @ (lg["G"] + lg["G"].T) + tri_apply(*A, t.U0) @ lg["P"].T + tri_apply(*AT, t.U0) @ lg["P"]
    thb += np.sum((t.U0 @ lg["P"].T) * t.U0, axis=1)
    return U0b, S0b, V0b, thb


def terminal_loss(U, S, V, target):
    """L = ||U S V^T - X_t||_F^2 with X_t = P diag(d) Q^T, and its gradient
    with respect to the factors (the n x m matrices are never formed)."""
    P, d, Q = target
    W = (P * d)                       # X_t = W Q^T
    VtV = V.T @ V
    UtU = U.T @ U
    QtV = Q.T @ V
    PtU = W.T @ U                     # (P d)^T U
    loss = (np.trace(S.T @ UtU @ S @ VtV) - 2.0 * np.trace(S.T @ PtU.T @ QtV)
            + np.sum((W.T @ W) * (Q.T @ Q)))
    # Ybar = 2 (U S V^T - W Q^T)
    Ub = 2.0 * (U @ S @ VtV @ S.T - W @ QtV @ S.T)
    Sb = 2.0 * (UtU @ S @ VtV - PtU.T @ QtV)
    Vb = 2.0 * (V @ S.T @ UtU @ S - Q @ PtU @ S)
    return float(loss), Ub, Sb, Vb


def loss_and_grad(U0, S0, V0, A0, theta, B, scheme: SubstepScheme, dt, nsteps, target, checkpoint_every=20):
    """Loss after nsteps BUG steps and its gradient with respect to theta and
    the initial factors, by checkpointed recomputation (checkpoints every
    ``checkpoint_every`` steps, each segment replayed once)."""
    A = (A0[0], A0[1] + theta, A0[2])
    ckpts: List[Tuple[np.ndarray, np.ndarray, np.ndarray]] = []
    U, S, V = U0, S0, V0
    for k in range(nsteps):
        if k % checkpoint_every == 0:
            ckpts.append((U, S, V))
        U, S, V, _ = bug_step_forward(U, S, V, A, B, scheme, dt)
    loss, Ub, Sb, Vb = terminal_loss(U, S, V, target)
    thb = np.zeros_like(theta)
    for c in reversed(range(len(ckpts))):
        k0 = c * checkpoint_every
        k1 = min(nsteps, k0 + checkpoint_every)
        U, S, V = ckpts[c]
        tapes = []
        for _ in range(k0, k1):
            U, S, V, tp = bug_step_forward(U, S, V, A, B, scheme, dt)
            tapes.append(tp)
        for tp in reversed(tapes):
            Ub, Sb, Vb, tb = bug_step_vjp(tp, A, B, scheme, dt, Ub, Sb, Vb)
            thb += tb
    return loss, thb, Ub, Sb, Vb


def loss_only(U0, S0, V0, A0, theta, B, scheme: SubstepScheme, dt, nsteps, target):
    A = (A0[0], A0[1] + theta, A0[2])
    U, S, V = U0, S0, V0
    for _ in range(nsteps):
        U, S, V, _ = bug_step_forward(U, S, V, A, B, scheme, dt)
    return terminal_loss(U, S, V, target)[0]
