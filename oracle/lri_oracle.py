"""FP64 CPU oracle: a NumPy restatement of LowRankIntegrators.jl's per-step hot path.

TEST INFRASTRUCTURE ONLY.  This module checks the engine; only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg may import it;
the product (the CUDA library and its host wrapper) never calls it.

Parity status: **parity unpinned** against the Julia reference itself.  The
reference ships no golden vectors, Julia is not available to run it, and two
pieces of its hot path live in third-party packages that are not in the
reference tree:

* ``DifferentialEquations`` v7 (version not pinned; ``Project.toml:7,14``)
  integrates every substep with adaptive ``Tsit5`` by default
  (``src/integrators/unconventional.jl:18``).  This oracle, like the GPU
  library, uses a *fixed-step* explicit Runge-Kutta substep scheme
  (``RK4``/``Euler``/``Heun``/``Midpoint``, ``nsub`` steps per substep) so
  that both sides run the same discrete scheme.
* ``LowRankArithmetic`` >= 0.1.2 (``Project.toml:9,15``) evaluates the user's
  ``F`` on factored operands and provides ``truncate_to_tolerance``.  Here
  ``F(K V^T) V`` is evaluated either densely (for small sizes; the literal
  meaning of ``F(TwoFactorRepresentation(K,V),t)*V``) or through the
  operator's exact factored form, and the truncation rule is restated from
  its published criterion (tail of squared singular values below ``tol^2``).

What *is* pinned: the reference's only assertion on the hot path
(``test/data_driven_approximation.jl:22-31``: continuous data stream and
discrete snapshots give the same answer), the exactness and invariance
properties of the published integrators (known-answer tests in ``tests/``),
and LAPACK's Householder QR / SVD, which NumPy shares with Julia.

Every function cites the reference line it follows.  Paths are relative to
the reference project root.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Callable, List, Optional, Sequence, Tuple, Union

import numpy as np

__all__ = [
    "SVDLikeRepresentation", "TwoFactorRepresentation",
    "MatrixDEProblem", "MatrixDataProblem", "MatrixHybridProblem", "GreedyIntegrator",
    "DLRSolution", "DLRIntegrator",
    "UnconventionalAlgorithm", "RankAdaptiveUnconventionalAlgorithm",
    "ProjectorSplitting", "PrimalLieTrotter", "DualLieTrotter", "Strang",
    "SubstepScheme", "Euler", "Heun", "Midpoint", "RK4",
    "SylvesterTridiagOp", "BurgersOp", "ReactionDiffusionOp", "DenseOp", "ZeroOp",
    "solve", "init", "step", "truncate_to_tolerance", "truncated_svd",
    "rel_fro_err", "to_dense",
]


# --------------------------------------------------------------------------
# Low-rank containers (LowRankArithmetic.jl, not vendored; used at
# src/integrators/unconventional.jl:53,63,73 and
# src/integrators/rank_adaptive_unconventional.jl:80,231)
# --------------------------------------------------------------------------

@dataclass
class SVDLikeRepresentation:
    """Y = U S V^T with U (n x r), S (r x r), V (m x r)."""
    U: np.ndarray
    S: np.ndarray
    V: np.ndarray

    @property
    def rank(self) -> int:
        return self.S.shape[0]

    @property
    def shape(self) -> Tuple[int, int]:
        return (self.U.shape[0], self.V.shape[0])

    def full(self) -> np.ndarray:
        return self.U @ self.S @ self.V.T

    def copy(self) -> "SVDLikeRepresentation":
        return SVDLikeRepresentation(self.U.copy(), self.S.copy(), self.V.copy())


@dataclass
class TwoFactorRepresentation:
    """Y = U Z^T."""
    U: np.ndarray
    Z: np.ndarray

    def full(self) -> np.ndarray:
        return self.U @ self.Z.T

    def copy(self) -> "TwoFactorRepresentation":
        return TwoFactorRepresentation(self.U.copy(), self.Z.copy())


def to_dense(Y) -> np.ndarray:
    return Y.full() if hasattr(Y, "full") else np.asarray(Y)


def truncated_svd(A: np.ndarray, r: Optional[int] = None, tol: Optional[float] = None
                  ) -> SVDLikeRepresentation:
    """Rank-r (or tolerance-) truncated SVD (LowRankArithmetic ``truncated_svd``,
    called at test/data_agnostic_approximation.jl:45 and
    test/data_driven_approximation.jl:18)."""
    U, s, Vt = np.linalg.svd(A, full_matrices=False)
    if r is None:
        r = truncate_to_tolerance(s, tol)
    return SVDLikeRepresentation(U[:, :r].copy(), np.diag(s[:r]), Vt[:r, :].T.copy())


def truncate_to_tolerance(s: Sequence[float], tol: float) -> int:
    """Rank selection used at src/integrators/rank_adaptive_unconventional.jl:223.

    Keeps the smallest leading count r1 >= 1 such that the discarded tail
    satisfies sum_{j>r1} s_j^2 < tol^2 (absolute tolerance), i.e. the
    Ceruti-Kusch-Lubich criterion.  Restated: accumulate s_j^2 from the
    smallest singular value upwards until the sum reaches tol^2; the value
    that crossed the threshold is the last one kept.
    """
    s = np.asarray(s, dtype=np.float64)
    acc = 0.0
    r = len(s)
    tol2 = tol * tol
    while acc < tol2 and r > 0:
        acc += s[r - 1] ** 2
        r -= 1
    # with tol == 0 the loop never runs; keep every value rather than len+1
    return min(r + 1, len(s))


# --------------------------------------------------------------------------
# Problems / solution / integrator (src/primitives.jl)
# --------------------------------------------------------------------------

@dataclass
class MatrixDEProblem:
    """dX/dt = F(X,t), X(t0) ~= u0 (src/primitives.jl:13-17)."""
    f: "Operator"
    u0: SVDLikeRepresentation
    tspan: Tuple[float, float]


class MatrixDataProblem:
    """Track the low-rank decomposition of a data stream A(t)
    (src/primitives.jl:23-30).  ``y`` is a callable t -> A(t) or a list of
    snapshots; for a list, tspan defaults to (1, len(y)) and dt to 1."""

    def __init__(self, y, u0: SVDLikeRepresentation, tspan=None):
        self.y = y
        self.u0 = u0
        if tspan is None:
            if callable(y):
                raise ValueError("tspan is required for a data stream given as a function")
            tspan = (1, len(y))
        self.tspan = tspan


class MatrixHybridProblem:
    """Data-informed basis: y(t) ~= U(t) Z(t)^T with dZ/dt = f(Z, U, t)
    (src/primitives.jl:32-41).  ``y`` is a callable t -> snapshot, ``u0`` a
    TwoFactorRepresentation."""

    def __init__(self, y, f, u0: "TwoFactorRepresentation", tspan):
        self.y = y
        self.f = f
        self.u0 = u0
        self.tspan = tspan


@dataclass
class DLRSolution:
    """History of the factors and times (src/primitives.jl:46-49)."""
    Y: List[Optional[SVDLikeRepresentation]]
    t: List[float]


@dataclass
class DLRIntegrator:
    """src/primitives.jl:54-63."""
    u: SVDLikeRepresentation
    t: float
    dt: float
    sol: DLRSolution
    alg: object
    cache: object
    prob: object
    iter: int = 0


def init_sol(dt, t0, tf, u0) -> DLRSolution:
    """Preallocated history (src/primitives.jl:92-104)."""
    if isinstance(dt, (int, np.integer)) and isinstance(t0, (int, np.integer)):
        steps = list(range(t0, tf + 1, dt))
        return DLRSolution([None] * len(steps), [float(s) for s in steps])
    n = int(math.floor((tf - t0) / dt)) + 1
    return DLRSolution([None] * n, list(np.linspace(t0, tf, n)))


def update_sol(integ: DLRIntegrator) -> None:
    """Deep copy of the factors after every step (src/primitives.jl:82-90)."""
    if integ.iter <= len(integ.sol.Y) - 1:
        integ.sol.Y[integ.iter] = integ.u.copy()
        integ.sol.t[integ.iter] = integ.t
    else:
        integ.sol.Y.append(integ.u.copy())
        integ.sol.t.append(integ.t)


def solve(prob, alg, dt=None, save_everystep: bool = True) -> DLRSolution:
    """Time loop of src/primitives.jl:68-80: ``while (tf-t)/T > 1e-8``,
    ``t += dt`` by accumulation, history saved after every step.
    ``save_everystep=False`` keeps only the first and last entries (used for
    large runs; the loop is unchanged)."""
    if dt is None:
        if not isinstance(prob, MatrixDataProblem) or callable(prob.y):
            raise ValueError("If the data is not provided as array, integration stepsize needs to be specified")
        dt = 1
    integ = init(prob, alg, dt)
    T = prob.tspan[1] - prob.tspan[0]
    while (prob.tspan[1] - integ.t) / T > 1e-8:
        step(integ, alg, dt)
        if save_everystep:
            update_sol(integ)
    if not save_everystep:
        integ.sol.Y = [integ.sol.Y[0], integ.u.copy()]
        integ.sol.t = [integ.sol.t[0], integ.t]
    return integ.sol


def n_steps(tspan, dt) -> int:
    """Number of iterations the time loop of src/primitives.jl:70-74 makes."""
    t0, tf = tspan
    T = tf - t0
    t = t0
    k = 0
    while (tf - t) / T > 1e-8:
        t += dt
        k += 1
    return k


# --------------------------------------------------------------------------
# Flow-map operators.  The reference accepts an arbitrary Julia closure F;
# the GPU library accepts a fixed menu, restated here with the same maths.
# Each operator provides the dense F(X,t) and the three projected rhs
#   K_rhs(K,V,t) = F(K V^T, t) V            (unconventional.jl:52-54)
#   L_rhs(L,U,t) = F(U L^T, t)^T U          (unconventional.jl:62-64)
#   S_rhs(S,U,V,t) = U^T F(U S V^T, t) V    (unconventional.jl:72-74)
# --------------------------------------------------------------------------

def tri_apply(sub: np.ndarray, diag: np.ndarray, sup: np.ndarray, X: np.ndarray) -> np.ndarray:
    """(T X) for tridiagonal T with T[i,i-1]=sub[i], T[i,i]=diag[i],
    T[i,i+1]=sup[i] (sub[0] and sup[n-1] are ignored)."""
    Y = diag[:, None] * X
    Y[1:] += sub[1:, None] * X[:-1]
    Y[:-1] += sup[:-1, None] * X[1:]
    return Y


def tri_dense(sub, diag, sup) -> np.ndarray:
    n = len(diag)
    T = np.diag(diag).astype(np.float64)
    T += np.diag(sub[1:], -1) + np.diag(sup[:-1], 1)
    return T


class Operator:
    dense_ok = True

    def __call__(self, X: np.ndarray, t: float) -> np.ndarray:
        raise NotImplementedError

    # Dense evaluation of the projected right-hand sides: the literal meaning
    # of F applied to the factored state and multiplied by the fixed factor.
    def K_rhs(self, K, V, t):
        return self(K @ V.T, t) @ V

    def L_rhs(self, L, U, t):
        return self(U @ L.T, t).T @ U

    def S_rhs(self, S, U, V, t):
        return U.T @ self(U @ S @ V.T, t) @ V

    # rhs closures for one substep (the fixed factor does not change during a
    # substep); operators with a factored form precompute their projections.
    def K_rhs_fn(self, V):
        return lambda K, t: self.K_rhs(K, V, t)

    def L_rhs_fn(self, U):
        return lambda L, t: self.L_rhs(L, U, t)

    def S_rhs_fn(self, U, V):
        return lambda S, t: self.S_rhs(S, U, V, t)


class ZeroOp(Operator):
    """F == 0."""

    def __call__(self, X, t):
        return np.zeros_like(X)

    def K_rhs(self, K, V, t):
        return np.zeros_like(K)

    def L_rhs(self, L, U, t):
        return np.zeros_like(L)

    def S_rhs(self, S, U, V, t):
        return np.zeros_like(S)


class DenseOp(Operator):
    """Arbitrary dense F(X, t) (small sizes only)."""

    def __init__(self, f: Callable[[np.ndarray, float], np.ndarray]):
        self.f = f

    def __call__(self, X, t):
        return self.f(X, t)


class SylvesterTridiagOp(Operator):
    """F(X) = A X + X B^T with tridiagonal A (n x n) and B (m x m).

    Each of A and B is given as three length-n (length-m) vectors
    (sub, diag, sup).  A ``diag(theta) X`` term is folded into A's diagonal.
    The factored rhs are exact algebraic rewrites of the dense ones:
      F(K V^T) V   = A K (V^T V) + K (V^T B V)^T
      F(U L^T)^T U = B L (U^T U) + L (U^T A U)^T
      U^T F(U S V^T) V = (U^T A U) S (V^T V) + (U^T U) S (V^T B V)^T
    """

    def __init__(self, A: Tuple[np.ndarray, np.ndarray, np.ndarray],
                 B: Tuple[np.ndarray, np.ndarray, np.ndarray], factored: bool = True):
        self.A = tuple(np.asarray(a, dtype=np.float64) for a in A)
        self.B = tuple(np.asarray(b, dtype=np.float64) for b in B)
        self.factored = factored

    def Ad(self):
        return tri_dense(*self.A)

    def Bd(self):
        return tri_dense(*self.B)

    def __call__(self, X, t):
        return tri_apply(*self.A, X) + tri_apply(*self.B, X.T).T

    def K_rhs(self, K, V, t):
        if not self.factored:
            return super().K_rhs(K, V, t)
        G = V.T @ V
        P = V.T @ tri_apply(*self.B, V)
        return tri_apply(*self.A, K) @ G + K @ P.T

    def L_rhs(self, L, U, t):
        if not self.factored:
            return super().L_rhs(L, U, t)
        G = U.T @ U
        P = U.T @ tri_apply(*self.A, U)
        return tri_apply(*self.B, L) @ G + L @ P.T

    def S_rhs(self, S, U, V, t):
        if not self.factored:
            return super().S_rhs(S, U, V, t)
        PU = U.T @ tri_apply(*self.A, U)
        PV = V.T @ tri_apply(*self.B, V)
        return PU @ S @ (V.T @ V) + (U.T @ U) @ S @ PV.T

    def K_rhs_fn(self, V):
        if not self.factored:
            return super().K_rhs_fn(V)
        G = V.T @ V
        PT = (V.T @ tri_apply(*self.B, V)).T
        A = self.A
        return lambda K, t: tri_apply(*A, K) @ G + K @ PT

    def L_rhs_fn(self, U):
        if not self.factored:
            return super().L_rhs_fn(U)
        G = U.T @ U
        PT = (U.T @ tri_apply(*self.A, U)).T
        B = self.B
        return lambda L, t: tri_apply(*B, L) @ G + L @ PT

    def S_rhs_fn(self, U, V):
        if not self.factored:
            return super().S_rhs_fn(U, V)
        PU = U.T @ tri_apply(*self.A, U)
        PVT = (V.T @ tri_apply(*self.B, V)).T
        GU = U.T @ U
        GV = V.T @ V
        return lambda S, t: PU @ S @ GV + GU @ S @ PVT


class BurgersOp(Operator):
    """Periodic central-difference Burgers flow map, column j = sample j:

        F(X) = (Dxx X) diag(nu) + alpha * (Dx X) .* X + beta * Dx (X .* X)

    with Dxx = tridiag(1,-2,1)/h^2 and Dx = tridiag(-1,0,1)/(2h), both
    periodic.  The reference test (test/data_agnostic_approximation.jl:16-33)
    is nu = 0.005 for every column, alpha = -1, beta = 0; the Burgers-UQ
    workload is per-column nu, alpha = 0, beta = -1/2 (conservative form).
    """

    def __init__(self, n: int, h: float, nu, alpha: float = -1.0, beta: float = 0.0):
        self.n = n
        self.h = float(h)
        self.nu = np.asarray(nu, dtype=np.float64)
        self.alpha = float(alpha)
        self.beta = float(beta)

    def _dxx(self, X):
        return (np.roll(X, 1, axis=0) - 2.0 * X + np.roll(X, -1, axis=0)) / (self.h * self.h)

    def _dx(self, X):
        return (np.roll(X, -1, axis=0) - np.roll(X, 1, axis=0)) / (2.0 * self.h)

    def __call__(self, X, t):
        nu = self.nu if self.nu.ndim else np.full(X.shape[1], float(self.nu))
        out = self._dxx(X) * nu[None, :]
        if self.alpha != 0.0:
            out += self.alpha * self._dx(X) * X
        if self.beta != 0.0:
            out += self.beta * self._dx(X * X)
        return out


class ReactionDiffusionOp(BurgersOp):
    """Periodic reaction-diffusion flow map, column j = sample j:

        F(X) = (Dxx X) diag(c) + p0 X + p1 X.^3

    (Allen-Cahn for c = eps^2, p0 = 1, p1 = -1).  The dense restatement of
    the library's registered local flow "reaction_diffusion": a flow map the
    reference would take as a user closure F (unconventional.jl:51-79)."""

    def __init__(self, n: int, h: float, c, p0: float = 0.0, p1: float = 0.0):
        super().__init__(n, h, c, 0.0, 0.0)
        self.p0 = float(p0)
        self.p1 = float(p1)

    def __call__(self, X, t):
        c = self.nu if self.nu.ndim else np.full(X.shape[1], float(self.nu))
        return self._dxx(X) * c[None, :] + self.p0 * X + self.p1 * X ** 3


# --------------------------------------------------------------------------
# Fixed-step substep schemes (stand-in for DifferentialEquations' Tsit5;
# the reference calls set_u! + step!(integ, dt, true), e.g.
# src/integrators/unconventional.jl:138-139)
# --------------------------------------------------------------------------

@dataclass(frozen=True)
class SubstepScheme:
    """Explicit Runge-Kutta scheme with a sub-diagonal Butcher tableau,
    applied ``nsub`` times with step dt/nsub over each substep interval."""
    name: str
    a: Tuple[float, ...]     # a[s] = coefficient of k_{s-1} in stage s input (a[0] unused)
    b: Tuple[float, ...]
    c: Tuple[float, ...]
    nsub: int = 1

    def with_nsub(self, nsub: int) -> "SubstepScheme":
        return SubstepScheme(self.name, self.a, self.b, self.c, int(nsub))

    def integrate(self, rhs: Callable[[np.ndarray, float], np.ndarray], y0: np.ndarray,
                  t0: float, dt: float) -> np.ndarray:
        h = dt / self.nsub
        y = y0
        t = t0
        for _ in range(self.nsub):
            acc = None
            kprev = None
            for s in range(len(self.b)):
                z = y if s == 0 else y + (h * self.a[s]) * kprev
                k = rhs(z, t + self.c[s] * h)
                acc = self.b[s] * k if acc is None else acc + self.b[s] * k
                kprev = k
            y = y + h * acc
            t = t + h
        return y


def Euler(nsub: int = 1) -> SubstepScheme:
    return SubstepScheme("Euler", (0.0,), (1.0,), (0.0,), nsub)


def Heun(nsub: int = 1) -> SubstepScheme:
    return SubstepScheme("Heun", (0.0, 1.0), (0.5, 0.5), (0.0, 1.0), nsub)


def Midpoint(nsub: int = 1) -> SubstepScheme:
    return SubstepScheme("Midpoint", (0.0, 0.5), (0.0, 1.0), (0.0, 0.5), nsub)


def RK4(nsub: int = 1) -> SubstepScheme:
    return SubstepScheme("RK4", (0.0, 0.5, 0.5, 1.0), (1 / 6, 1 / 3, 1 / 3, 1 / 6),
                         (0.0, 0.5, 0.5, 1.0), nsub)


# --------------------------------------------------------------------------
# Algorithms (src/integrators/*.jl)
# --------------------------------------------------------------------------

@dataclass
class UnconventionalAlgorithm:
    """BUG integrator parameters (src/integrators/unconventional.jl:13-21)."""
    K_alg: SubstepScheme = field(default_factory=RK4)
    L_alg: Optional[SubstepScheme] = None
    S_alg: Optional[SubstepScheme] = None

    def __post_init__(self):
        self.L_alg = self.L_alg or self.K_alg
        self.S_alg = self.S_alg or self.K_alg


@dataclass
class RankAdaptiveUnconventionalAlgorithm:
    """Rank-adaptive BUG (src/integrators/rank_adaptive_unconventional.jl:15-23).
    ``rmin`` has no counterpart in the reference (it defaults to 1)."""
    tol: float
    rmax: int = 2 ** 62
    K_alg: SubstepScheme = field(default_factory=RK4)
    L_alg: Optional[SubstepScheme] = None
    S_alg: Optional[SubstepScheme] = None
    rmin: int = 1

    def __post_init__(self):
        self.L_alg = self.L_alg or self.K_alg
        self.S_alg = self.S_alg or self.K_alg


class PrimalLieTrotter:
    pass


class DualLieTrotter:
    pass


class Strang:
    pass


@dataclass
class ProjectorSplitting:
    """KSL projector-splitting integrator (src/integrators/projector_splitting.jl:1-41)."""
    order: object = field(default_factory=PrimalLieTrotter)
    K_alg: SubstepScheme = field(default_factory=RK4)
    L_alg: Optional[SubstepScheme] = None
    S_alg: Optional[SubstepScheme] = None

    def __post_init__(self):
        self.L_alg = self.L_alg or self.K_alg
        self.S_alg = self.S_alg or self.K_alg


@dataclass
class GreedyIntegrator:
    """Greedy basis fitting (src/integrators/greedy_integrator.jl:17-24);
    Z_alg integrates the coefficient ODE of a MatrixHybridProblem."""
    Z_alg: SubstepScheme = field(default_factory=RK4)


# --------------------------------------------------------------------------
# Data-stream bookkeeping (src/integrators/data_integrator.jl)
# --------------------------------------------------------------------------

class _DataCache:
    def __init__(self, prob: MatrixDataProblem, t0):
        y = prob.y
        # unconventional.jl:91-93
        self.y = y
        self.yprev = np.array(y[0], dtype=np.float64) if not callable(y) else np.array(y(t0), dtype=np.float64)
        self.ycurr = self.yprev.copy()
        self.dy = np.zeros_like(self.yprev)

    def advance(self, t, dt):
        """update_data! + ``Δy .= ycurr - yprev; yprev .= ycurr``
        (unconventional.jl:121-127, data_integrator.jl:22-28).  Snapshot
        lists are 1-indexed in the reference: y[t+dt]."""
        if callable(self.y):
            self.ycurr = np.array(self.y(t + dt), dtype=np.float64)
        else:
            idx = int(round(t + dt))
            if abs((t + dt) - idx) > 1e-12:
                raise TypeError("discrete snapshot data needs an integer time step")
            self.ycurr = np.array(self.y[idx - 1], dtype=np.float64)
        self.dy = self.ycurr - self.yprev
        self.yprev = self.ycurr.copy()


def _qr(A: np.ndarray) -> Tuple[np.ndarray, np.ndarray]:
    """Householder QR with the thin Q formed (``qr!`` + ``Matrix(Q)``,
    LAPACK geqrt/orgqr; unconventional.jl:141-142)."""
    Q, R = np.linalg.qr(A, mode="reduced")
    return Q, R


class _Substeps:
    """The three substep flows of one problem: DiffEq-style integration of
    the projected rhs for MatrixDEProblem, exact data increments for
    MatrixDataProblem (data_integrator.jl:13-16: ``u .+= sign*left'*Δy*right``)."""

    def __init__(self, prob, alg):
        self.prob = prob
        self.alg = alg
        self.is_data = isinstance(prob, MatrixDataProblem)

    def K(self, K0, V, t, dt):
        if self.is_data:
            return K0 + self.data.dy @ V
        return self.alg.K_alg.integrate(self.prob.f.K_rhs_fn(V), K0, t, dt)

    def L(self, L0, U, t, dt):
        if self.is_data:
            return L0 + self.data.dy.T @ U
        return self.alg.L_alg.integrate(self.prob.f.L_rhs_fn(U), L0, t, dt)

    def S(self, S0, U, V, t, dt, sign=1.0):
        if self.is_data:
            return S0 + sign * (U.T @ self.data.dy @ V)
        rhs = self.prob.f.S_rhs_fn(U, V)
        if sign == 1.0:
            return self.alg.S_alg.integrate(rhs, S0, t, dt)
        return self.alg.S_alg.integrate(lambda S, tt: sign * rhs(S, tt), S0, t, dt)


def init(prob, alg, dt) -> DLRIntegrator:
    """init(prob, alg, dt) (unconventional.jl:109-119,
    rank_adaptive_unconventional.jl:94-104, projector_splitting.jl:107-115)."""
    t0, tf = prob.tspan
    if not tf > t0:
        raise AssertionError("Integration in reverse time direction is not supported")
    u = prob.u0.copy()
    sol = init_sol(dt, t0, tf, prob.u0)
    if isinstance(alg, GreedyIntegrator):
        cache = _GreedyCache(prob)
    else:
        cache = _Substeps(prob, alg)
        if cache.is_data:
            cache.data = _DataCache(prob, t0)
    sol.Y[0] = prob.u0.copy()
    return DLRIntegrator(u, t0, dt, sol, alg, cache, prob, 0)


class _GreedyCache:
    """GreedyIntegrator_Cache (src/integrators/greedy_integrator.jl:1-52):
    the data source and, for a hybrid problem, the coefficient integrator's
    right-hand side f(Z, U, t) (its parameter is the integrator's U,
    aliased, :41-47)."""

    def __init__(self, prob):
        self.prob = prob
        self.hybrid = isinstance(prob, MatrixHybridProblem)

    def snapshot(self, t, dt):
        """update_data!(X, y, t, dt): X = y(t + dt) (data_integrator.jl:22-28;
        snapshot lists are 1-indexed)."""
        y = self.prob.y
        if callable(y):
            return np.array(y(t + dt), dtype=np.float64)
        idx = int(round(t + dt))
        if abs((t + dt) - idx) > 1e-12:
            raise TypeError("discrete snapshot data needs an integer time step")
        return np.array(y[idx - 1], dtype=np.float64)


def _polar(A: np.ndarray) -> np.ndarray:
    """Q P^T from svd(A) = Q Sigma P^T (greedy_integrator.jl:80-81,92-93)."""
    Q, _, Pt = np.linalg.svd(A, full_matrices=False)
    return Q @ Pt


def greedy_step(u, cache: _GreedyCache, alg: GreedyIntegrator, t, dt) -> None:
    """greedy_step! (src/integrators/greedy_integrator.jl:73-104)."""
    if cache.hybrid:
        # :73-82: advance Z over [t, t+dt] with U fixed, then U = polar(X Z)
        U = u.U
        f = cache.prob.f
        u.Z = alg.Z_alg.integrate(lambda Z, tt: f(Z, U, tt), u.Z, t, dt)
        X = cache.snapshot(t, dt)
        u.U = _polar(X @ u.Z)
    elif isinstance(u, TwoFactorRepresentation):
        # :84-94
        X = cache.snapshot(t, dt)
        u.Z = X.T @ u.U
        u.U = _polar(X @ u.Z)
    else:
        # :96-104
        X = cache.snapshot(t, dt)
        XV = X @ u.V
        XU = X.T @ u.U
        u.U, _ = _qr(XV)
        u.V, _ = _qr(XU)
        u.S = u.U.T @ (X @ u.V)


def _advance_data(cache, t, dt):
    if cache.is_data:
        cache.data.advance(t, dt)


def bug_step(u: SVDLikeRepresentation, cache: _Substeps, t, dt) -> None:
    """unconventional_step! (src/integrators/unconventional.jl:121-157)."""
    _advance_data(cache, t, dt)
    U0, S0, V0 = u.U, u.S, u.V
    # K step (:136-142)
    US = U0 @ S0
    US = cache.K(US, V0, t, dt)
    QK, _ = _qr(US)
    M = QK.T @ U0
    # L step (:144-150); the L rhs still sees the old U (u.U is replaced at :152)
    VS = V0 @ S0.T
    VS = cache.L(VS, U0, t, dt)
    QL, _ = _qr(VS)
    N = QL.T @ V0
    u.V = QL          # :151
    u.U = QK          # :152
    # S step on the new bases (:154-156)
    u.S = cache.S(M @ S0 @ N.T, u.U, u.V, t, dt)


def ra_bug_step(u: SVDLikeRepresentation, cache: _Substeps, t, dt, alg) -> bool:
    """rankadaptive_unconventional_step! (src/integrators/rank_adaptive_unconventional.jl:182-233).
    Returns True when the rank changed (the reference then rebuilds its cache,
    :171-180; with no cache to rebuild, only the factors' shapes change)."""
    _advance_data(cache, t, dt)
    U0, S0, V0 = u.U, u.S, u.V
    r = S0.shape[0]
    # K step (:197-206): Uhat = orth([K1 | U0])
    US = cache.K(U0 @ S0, V0, t, dt)
    Uhat, _ = _qr(np.hstack([US, U0]))
    M = Uhat.T @ U0
    # L step (:208-217)
    VS = cache.L(V0 @ S0.T, U0, t, dt)
    Vhat, _ = _qr(np.hstack([VS, V0]))
    N = Vhat.T @ V0
    # S step on the augmented bases (:219-220)
    S1 = cache.S(M @ S0 @ N.T, Uhat, Vhat, t, dt)
    # truncation (:222-231)
    P, sig, Qt = np.linalg.svd(S1)
    r_new = min(alg.rmax, truncate_to_tolerance(sig, alg.tol))
    r_new = max(r_new, alg.rmin)
    r_new = min(r_new, len(sig))
    u.U = Uhat @ P[:, :r_new]
    u.S = np.diag(sig[:r_new])
    u.V = Vhat @ Qt.T[:, :r_new]
    return r_new != r


def primal_lt_step(u: SVDLikeRepresentation, cache: _Substeps, t, dt) -> None:
    """primal_LT_step! (src/integrators/projector_splitting.jl:117-152):
    K -> QR -> backward S -> L -> QR, S = R^T."""
    _advance_data(cache, t, dt)
    # K step (:133-138)
    US = cache.K(u.U @ u.S, u.V, t, dt)
    Q, R = _qr(US)
    u.U = Q
    # S step, backward (rhs negated at :64; data sign -1 at :99) (:141-142)
    S = cache.S(R, u.U, u.V, t, dt, sign=-1.0)
    # L step (:145-151)
    VS = cache.L(u.V @ S.T, u.U, t, dt)
    Q, R = _qr(VS)
    u.V = Q
    u.S = R.T


def dual_lt_step(u: SVDLikeRepresentation, cache: _Substeps, t, dt) -> None:
    """dual_LT_step! (src/integrators/projector_splitting.jl:154-189):
    L -> QR -> backward S -> K -> QR, S = R."""
    _advance_data(cache, t, dt)
    VS = cache.L(u.V @ u.S.T, u.U, t, dt)
    Q, R = _qr(VS)
    u.V = Q
    S = cache.S(R.T.copy(), u.U, u.V, t, dt, sign=-1.0)
    US = cache.K(u.U @ S, u.V, t, dt)
    Q, R = _qr(US)
    u.U = Q
    u.S = R


def step(integ: DLRIntegrator, alg, dt) -> None:
    """step!(integrator, alg, dt) for every algorithm
    (unconventional.jl:159-164, rank_adaptive_unconventional.jl:171-180,
    projector_splitting.jl:191-211)."""
    u, t, cache = integ.u, integ.t, integ.cache
    if isinstance(alg, GreedyIntegrator):
        greedy_step(u, cache, alg, t, dt)
    elif isinstance(alg, UnconventionalAlgorithm):
        bug_step(u, cache, t, dt)
    elif isinstance(alg, RankAdaptiveUnconventionalAlgorithm):
        ra_bug_step(u, cache, t, dt, alg)
    elif isinstance(alg, ProjectorSplitting):
        if isinstance(alg.order, PrimalLieTrotter):
            primal_lt_step(u, cache, t, dt)
        elif isinstance(alg.order, DualLieTrotter):
            dual_lt_step(u, cache, t, dt)
        elif isinstance(alg.order, Strang):
            primal_lt_step(u, cache, t, dt / 2)
            dual_lt_step(u, cache, t + dt / 2, dt / 2)
        else:
            raise TypeError("unknown projector-splitting order")
    else:
        raise TypeError("unknown algorithm")
    integ.t += dt
    integ.iter += 1


# --------------------------------------------------------------------------
# Measures
# --------------------------------------------------------------------------

def rel_fro_err(Y, Yref) -> float:
    """||Y - Yref||_F / ||Yref||_F on the dense matrices."""
    A = to_dense(Y)
    B = to_dense(Yref)
    return float(np.linalg.norm(A - B) / np.linalg.norm(B))
