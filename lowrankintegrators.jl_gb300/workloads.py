"""Seeded synthetic inputs of the benchmark workloads (host NumPy).

sylvester_256      plain BUG on F(X) = A X + X A^T, A = Laplacian/h^2 - 0.1 I,
                   n = m = 256, h = 1/257, Dirichlet; X0 = sum_{k<=20} 2^-k u_k v_k^T
                   (seed 1); Y0 = rank-8 truncated SVD; dt = 1e-4 on [0, 0.1];
                   RK4 substeps with nsub = 20 (|dt*lambda| ~ 53 needs ~19).
lyapunov_ensemble  4096 independent F_i(X) = A_i X + X B_i^T; n_i, m_i ~ U{64..1024},
                   r_i ~ U{4..32}; A_i, B_i tridiagonal, diagonal -2-U[0,1],
                   off-diagonals U[0.5,1]; X0_i = sum_{k<=r_i} 2^-k u_k v_k^T with
                   seeded orthonormal u, v (seed 4); dt = 1e-2, 200 steps, RK4 nsub = 1.
data_rotation      the reference test's stream Y(t) = exp(t W1) e^t D exp(t W2),
                   N = 100, W skew, D = diag(2^-j) (seeded; the reference's is not).
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import List, Tuple

import numpy as np


def laplacian_tridiag(n: int, h: float, shift: float = 0.0):
    sub = np.full(n, 1.0 / (h * h))
    dia = np.full(n, -2.0 / (h * h) - shift)
    sup = np.full(n, 1.0 / (h * h))
    return sub, dia, sup


def random_orthonormal(rng, n: int, k: int) -> np.ndarray:
    Q, R = np.linalg.qr(rng.standard_normal((n, k)))
    return Q * np.sign(np.diag(R))[None, :]


@dataclass
class SylvesterInstance:
    A: Tuple[np.ndarray, np.ndarray, np.ndarray]
    B: Tuple[np.ndarray, np.ndarray, np.ndarray]
    U: np.ndarray
    S: np.ndarray
    V: np.ndarray


def sylvester_256(seed: int = 1, n: int = 256, r: int = 8, nterms: int = 20):
    """Returns (instance, dt, tspan, nsub)."""
    rng = np.random.default_rng(seed)
    h = 1.0 / (n + 1)
    A = laplacian_tridiag(n, h, 0.1)
    u = random_orthonormal(rng, n, nterms)
    v = random_orthonormal(rng, n, nterms)
    s = 2.0 ** -np.arange(1, nterms + 1)
    X0 = (u * s[None, :]) @ v.T
    Uf, sf, Vtf = np.linalg.svd(X0)
    inst = SylvesterInstance(A, A, Uf[:, :r].copy(), np.diag(sf[:r]), Vtf[:r].T.copy())
    return inst, 1e-4, (0.0, 0.1), 20


def lyapunov_ensemble(count: int = 4096, seed: int = 4, nmin: int = 64, nmax: int = 1024, rmin: int = 4,
                      rmax: int = 32, first: int = 0, limit: int = None) -> List[SylvesterInstance]:
    """Instances [first, first+limit) of the seeded ensemble (sizes and data
    of instance i do not depend on which slice is requested)."""
    rng = np.random.default_rng(seed)
    n = rng.integers(nmin, nmax + 1, count)
    m = rng.integers(nmin, nmax + 1, count)
    r = rng.integers(rmin, rmax + 1, count)
    seeds = rng.integers(0, 2 ** 63 - 1, count)
    last = count if limit is None else min(count, first + limit)
    out = []
    for i in range(first, last):
        g = np.random.default_rng(int(seeds[i]))
        ni, mi, ri = int(n[i]), int(m[i]), int(r[i])
        A = (g.uniform(0.5, 1.0, ni), -2.0 - g.uniform(0.0, 1.0, ni), g.uniform(0.5, 1.0, ni))
        B = (g.uniform(0.5, 1.0, mi), -2.0 - g.uniform(0.0, 1.0, mi), g.uniform(0.5, 1.0, mi))
        U = random_orthonormal(g, ni, ri)
        V = random_orthonormal(g, mi, ri)
        S = np.diag(2.0 ** -np.arange(1, ri + 1))
        out.append(SylvesterInstance(A, B, U, S, V))
    return out


def lyapunov_ensemble_shapes(count: int = 4096, seed: int = 4, nmin: int = 64, nmax: int = 1024, rmin: int = 4,
                             rmax: int = 32):
    rng = np.random.default_rng(seed)
    n = rng.integers(nmin, nmax + 1, count)
    m = rng.integers(nmin, nmax + 1, count)
    r = rng.integers(rmin, rmax + 1, count)
    return n, m, r


def skew(rng, N: int) -> np.ndarray:
    W = rng.standard_normal((N, N))
    return np.triu(W, 1) - np.triu(W, 1).T


def data_rotation(seed: int = 0, N: int = 100):
    """Returns the stream t -> Y(t) of the reference data test."""
    from scipy.linalg import expm

    rng = np.random.default_rng(seed)
    W1, W2 = skew(rng, N), skew(rng, N)
    D = np.diag(2.0 ** -np.arange(1, N + 1))

    def Y(t):
        return expm(t * W1) @ (np.exp(t) * D) @ expm(t * W2)

    return Y


def adjoint_2048(seed: int = 5, n: int = 2048, r: int = 32, rt: int = 40):
    """The adjoint workload: F(X; theta) = A X + X A^T + diag(theta) X with A
    the unscaled 1D Laplacian tridiag(1, -2, 1), n = m = 2048, theta with
    variance 0.1, Y0 rank 32 (seeded orthonormal factors, spectrum
    2^{-k/4}), target X_t seeded rank 40 with spectrum 2^{-k/4}.  Returns
    (A0, theta, U, S, V, (P, d, Q)) with X_t = P diag(d) Q^T."""
    g = np.random.default_rng(seed)
    A0 = (np.ones(n), -2.0 * np.ones(n), np.ones(n))
    theta = g.normal(0.0, np.sqrt(0.1), n)
    U, _ = np.linalg.qr(g.standard_normal((n, r)))
    V, _ = np.linalg.qr(g.standard_normal((n, r)))
    S = np.diag(2.0 ** (-np.arange(1, r + 1) / 4.0))
    P, _ = np.linalg.qr(g.standard_normal((n, rt)))
    Q, _ = np.linalg.qr(g.standard_normal((n, rt)))
    d = 2.0 ** (-np.arange(1, rt + 1) / 4.0)
    return A0, theta, U, S, V, (P, d, Q)


def data_stream(n: int, m: int, nsnap: int, seed: int = 2, K: int = 64, sub: int = 128, noise: float = 1e-4):
    """Snapshots A(t_j), t_j = j / (nsnap - 1), of the compressed data stream
    A(t) = sum_{k<=K} sigma_k(t) u_k(t) v_k(t)^T + noise * N(0, 1):
    sigma_k(t) = e^{-k/8} (1 + 0.3 sin(2 pi f_k t)), f_k ~ U[0.5, 2];
    u_k(t) = Q_u exp(t Omega_u) [I_K; 0] with Q_u an n x sub seeded orthonormal
    basis and Omega_u a sub x sub skew matrix with N(0, 0.1) entries (the
    same for v); the noise is one fixed realisation.  The full-size stream
    is n = 8192, m = 4096, 500 snapshots."""
    from scipy.linalg import expm

    g = np.random.default_rng(seed)
    f = g.uniform(0.5, 2.0, K)
    Qu = random_orthonormal(g, n, sub)
    Qv = random_orthonormal(g, m, sub)
    Wu = g.normal(0.0, np.sqrt(0.1), (sub, sub))
    Wv = g.normal(0.0, np.sqrt(0.1), (sub, sub))
    Ou, Ov = np.triu(Wu, 1) - np.triu(Wu, 1).T, np.triu(Wv, 1) - np.triu(Wv, 1).T
    E = noise * g.standard_normal((n, m))
    k = np.arange(1, K + 1)
    out = []
    for j in range(nsnap):
        t = j / max(1, nsnap - 1)
        sig = np.exp(-k / 8.0) * (1.0 + 0.3 * np.sin(2 * np.pi * f * t))
        Ut = Qu @ expm(t * Ou)[:, :K]
        Vt = Qv @ expm(t * Ov)[:, :K]
        out.append((Ut * sig) @ Vt.T + E)
    return out


def burgers_uq(n: int, m: int, seed: int = 3):
    """The Burgers-UQ problem u_t + (u^2/2)_x = nu u_xx on the periodic grid
    x_i = i/n (h = 1/n), one column per sample: nu_j ~ U[0.005, 0.02],
    u0_j = sin(2 pi x) + a_j sin(4 pi x + phi_j), a_j ~ U[0, 0.5],
    phi_j ~ U[0, 2 pi].  Returns (h, nu, X0) with X0 the n x m initial data
    (exact rank 3).  The full-size problem is n = 4096, m = 16384."""
    g = np.random.default_rng(seed)
    x = np.arange(n) / n
    nu = g.uniform(0.005, 0.02, m)
    a = g.uniform(0.0, 0.5, m)
    phi = g.uniform(0.0, 2 * np.pi, m)
    X0 = np.sin(2 * np.pi * x)[:, None] + a[None, :] * np.sin(4 * np.pi * x[:, None] + phi[None, :])
    return 1.0 / n, nu, X0


def burgers_uq_factors(n: int, m: int, r: int, seed: int = 3):
    """The initial data of ``burgers_uq`` (same seed, same samples) as an
    SVD-like rank-r factorisation without forming X0: X0 = B C^T with
    B = [sin 2 pi x, sin 4 pi x, cos 4 pi x] and C = [1, a cos phi, a sin phi]
    (exact rank 3), thin QR of both and the SVD of the 3 x 3 core; the
    columns 4..r of U and V complete them with seeded orthonormal directions
    at singular value 0.  Returns (h, nu, U, s, V)."""
    g = np.random.default_rng(seed)
    x = np.arange(n) / n
    nu = g.uniform(0.005, 0.02, m)
    a = g.uniform(0.0, 0.5, m)
    phi = g.uniform(0.0, 2 * np.pi, m)
    B = np.stack([np.sin(2 * np.pi * x), np.sin(4 * np.pi * x), np.cos(4 * np.pi * x)], axis=1)
    C = np.stack([np.ones(m), a * np.cos(phi), a * np.sin(phi)], axis=1)
    Qb, Rb = np.linalg.qr(B)
    Qc, Rc = np.linalg.qr(C)
    P, s3, Qt = np.linalg.svd(Rb @ Rc.T)
    g2 = np.random.default_rng(seed + 1000)

    def complete(Q):
        Z = g2.standard_normal((Q.shape[0], r - 3))
        for _ in range(2):
            Z -= Q @ (Q.T @ Z)
        return np.hstack([Q, np.linalg.qr(Z)[0]])

    U = complete(Qb @ P)
    V = complete(Qc @ Qt.T)
    s = np.concatenate([s3, np.zeros(r - 3)])
    return 1.0 / n, nu, U, s, V


def data_stream_device(n: int, m: int, nsnap: int, seed: int = 2, K: int = 64, sub: int = 128,
                       noise: float = 1e-4, dtype=None, device="cuda"):
    """The data-compression stream of ``data_stream`` generated on the device
    (mode bases and amplitudes from the seeded host generator, the fixed
    noise realisation from the device generator).  Returns snap(j) -> a
    device tensor with the n x m snapshot A(t_j), t_j = j / (nsnap - 1),
    stored column-major (shape (m, n) row-major)."""
    import torch
    from scipy.linalg import expm

    dtype = dtype or torch.float32
    g = np.random.default_rng(seed)
    f = g.uniform(0.5, 2.0, K)
    Qu = random_orthonormal(g, n, sub)
    Qv = random_orthonormal(g, m, sub)
    Wu = g.normal(0.0, np.sqrt(0.1), (sub, sub))
    Wv = g.normal(0.0, np.sqrt(0.1), (sub, sub))
    Ou, Ov = np.triu(Wu, 1) - np.triu(Wu, 1).T, np.triu(Wv, 1) - np.triu(Wv, 1).T
    gen = torch.Generator(device=device)
    gen.manual_seed(seed)
    E = noise * torch.randn((m, n), generator=gen, device=device, dtype=dtype)
    k = np.arange(1, K + 1)

    def snap(j: int):
        t = j / max(1, nsnap - 1)
        sig = np.exp(-k / 8.0) * (1.0 + 0.3 * np.sin(2 * np.pi * f * t))
        Ut = torch.from_numpy(Qu @ expm(t * Ou)[:, :K] * sig).to(device, dtype)
        Vt = torch.from_numpy(Qv @ expm(t * Ov)[:, :K]).to(device, dtype)
        return torch.addmm(E, Vt, Ut.T)  # (m, n) row-major = n x m column-major

    # the noise-free rank-K part of A(0): orthonormal factors and amplitudes
    snap.signal0 = (Qu[:, :K].copy(), np.exp(-k / 8.0), Qv[:, :K].copy())
    return snap
