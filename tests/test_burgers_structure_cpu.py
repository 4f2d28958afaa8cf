"""The algebra the large Burgers engine (lri_burgers_*) evaluates its substep
flows with, checked on the CPU against the oracle's dense flow map
(oracle.BurgersOp, F(Y) = (Dxx Y) diag(nu) + alpha (Dx Y).*Y + beta Dx(Y.*Y)).

The engine never forms Y = K V^T: the diffusion term is (Dxx K)(V^T diag(nu) V)
and the quadratic terms are Khatri-Rao products with symmetric 3-tensors built
once per step, stored over packed pairs a <= b with the off-diagonal pairs
counted twice, T'[p(a,b), c] = c_ab T[a,b,c], KR(P,Q)_{i,p(a,b)} =
(P_ia Q_ib + P_ib Q_ia) / 2 (kr_gram_part / kr_reduce / kr_apply_part).  The
kernels compute sum_p KR(X,X)_ip T'_pc as sum_a X_ia sum_{b >= a} X_ib T'_(a,b)c
over contiguous pair rows; both forms are restated here in NumPy.  The pair
decoding is the kernels' (pair_ab).
"""
import math

import numpy as np
import pytest

from oracle import lri_oracle as O


def pairs(ka):
    return [(a, b) for a in range(ka) for b in range(a, ka)]


def kr(P, Q):
    return np.stack([0.5 * (P[:, a] * Q[:, b] + P[:, b] * Q[:, a]) for a, b in pairs(P.shape[1])], axis=1)


def packed_tensor(P, Q, Y, coef=1.0):
    c = np.array([1.0 if a == b else 2.0 for a, b in pairs(P.shape[1])])
    return coef * c[:, None] * (kr(P, Q).T @ Y)


def kr_apply_rows(X, Tp):
    """sum_a diag(X[:, a]) X[:, a:] T'_a: the loop order of kr_apply_part."""
    ka = X.shape[1]
    out = np.zeros((X.shape[0], Tp.shape[1]))
    start = 0
    for a in range(ka):
        rows = Tp[start:start + ka - a]
        out += X[:, [a]] * (X[:, a:] @ rows)
        start += ka - a
    return out


def stencils(n, h):
    def dxx(X):
        return (np.roll(X, 1, 0) - 2 * X + np.roll(X, -1, 0)) / h ** 2

    def dx(X):
        return (np.roll(X, -1, 0) - np.roll(X, 1, 0)) / (2 * h)

    return dxx, dx


@pytest.mark.parametrize("alpha,beta", [(0.0, -0.5), (-1.0, 0.0), (-0.7, 0.4)])
def test_structured_substep_flows_match_dense(alpha, beta):
    g = np.random.default_rng(7)
    n, m, k = 48, 36, 5
    h = 1.0 / n
    nu = g.uniform(0.005, 0.02, m)
    op = O.BurgersOp(n, h, nu, alpha=alpha, beta=beta)
    dxx, dx = stencils(n, h)
    U = np.linalg.qr(g.standard_normal((n, k)))[0]
    V = np.linalg.qr(g.standard_normal((m, k)))[0]
    K = g.standard_normal((n, k))
    L = g.standard_normal((m, k))
    # K substep: F(K V^T) V
    Tv = packed_tensor(V, V, V)
    Nnu = V.T @ (nu[:, None] * V)
    Kd = dxx(K) @ Nnu + alpha * kr(dx(K), K) @ Tv + beta * dx(kr(K, K) @ Tv)
    ref = op(K @ V.T, 0.0) @ V
    assert np.abs(Kd - ref).max() <= 1e-12 * np.abs(ref).max()
    # the kernels' loop order for the symmetric product, and the 1/2 (X,Y)+(Y,X) split
    assert np.allclose(kr_apply_rows(K, Tv), kr(K, K) @ Tv, rtol=0, atol=1e-12 * np.abs(Tv).max() * k * k)
    # L substep: F(U L^T)^T U = diag(nu) L (U^T Dxx U) + KR(L, L) T'_L
    Tl = packed_tensor(dx(U), U, U, alpha) + packed_tensor(U, U, dx(U), -beta)
    Ld = nu[:, None] * (L @ (U.T @ dxx(U))) + kr(L, L) @ Tl
    ref = op(U @ L.T, 0.0).T @ U
    assert np.abs(Ld - ref).max() <= 1e-12 * np.abs(ref).max()
    # S substep on augmented bases: Uh^T F(Uh S Vh^T) Vh
    Uh = np.linalg.qr(g.standard_normal((n, 2 * k)))[0]
    Vh = np.linalg.qr(g.standard_normal((m, 2 * k)))[0]
    S = g.standard_normal((2 * k, 2 * k))
    Th = packed_tensor(Vh, Vh, Vh)
    A = Uh @ S
    Sd = (Uh.T @ dxx(Uh)) @ S @ (Vh.T @ (nu[:, None] * Vh)) \
        + Uh.T @ (alpha * kr(dx(A), A) @ Th + beta * dx(kr(A, A) @ Th))
    ref = Uh.T @ op(Uh @ S @ Vh.T, 0.0) @ Vh
    assert np.abs(Sd - ref).max() <= 1e-12 * np.abs(ref).max()


def pair_ab(p, ka):
    """The kernels' decoding of a packed pair index (row-wise, a <= b)."""
    q = 2.0 * ka + 1.0
    x = int((q - math.sqrt(q * q - 8.0 * p)) * 0.5)
    x = max(0, min(x, ka - 1))
    while x > 0 and x * ka - x * (x - 1) // 2 > p:
        x -= 1
    while x + 1 < ka and (x + 1) * ka - (x + 1) * x // 2 <= p:
        x += 1
    return x, x + (p - (x * ka - x * (x - 1) // 2))


@pytest.mark.parametrize("ka", [1, 2, 3, 17, 64, 128, 192])
def test_pair_decoding_is_row_wise_packing(ka):
    assert [pair_ab(p, ka) for p in range(ka * (ka + 1) // 2)] == pairs(ka)
