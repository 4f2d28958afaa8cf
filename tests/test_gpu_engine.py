"""GPU parity of the instance engine against the FP64 oracle.

Tolerances (relative Frobenius error of Y = U S V^T):
  plain FP64 form:   1e-11 (same discrete scheme, different summation order);
  double-float form: 1e-10 (48-bit significands);
  FP32 / mixed form: 1e-5  (the metric's accuracy bar).
Factors are compared gauge-invariantly through Y and the singular values.

Fixed-rank BUG amplifies perturbations of the factors by roughly
kappa(S) * dt per step, so a trajectory whose core becomes very
ill-conditioned is reproducible only to that level even between two FP64
implementations; tests on such trajectories calibrate their tolerance to the
oracle's own response to a 1e-16 relative perturbation.
"""
import os
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "lowrankintegrators.jl_gb300"))
import workloads  # noqa: E402

TOL = {"fp64": 1e-11, "df": 1e-10, "fp32": 1e-5, "mixed": 1e-5}


def sylv_instance(seed, n, m, r, graded=True):
    g = np.random.default_rng(seed)
    A = (g.uniform(0.5, 1.0, n), -2.0 - g.uniform(0, 1, n), g.uniform(0.5, 1.0, n))
    B = (g.uniform(0.5, 1.0, m), -2.0 - g.uniform(0, 1, m), g.uniform(0.5, 1.0, m))
    U = workloads.random_orthonormal(g, n, r)
    V = workloads.random_orthonormal(g, m, r)
    s = 2.0 ** -np.arange(1, r + 1) if graded else np.linspace(1.0, 0.3, r)
    return A, B, U, np.diag(s), V


def pair_algs(lri, O, kind, scheme=("RK4", 2), ra_tol=1e-7):
    gs = getattr(lri, scheme[0])(scheme[1])
    os_ = getattr(O, scheme[0])(scheme[1])
    if kind == "bug":
        return lri.UnconventionalAlgorithm(gs), O.UnconventionalAlgorithm(os_)
    if kind == "ra":
        return (lri.RankAdaptiveUnconventionalAlgorithm(ra_tol, rmax=10, K_alg=gs),
                O.RankAdaptiveUnconventionalAlgorithm(ra_tol, rmax=10, K_alg=os_))
    order = {"primal": "PrimalLieTrotter", "dual": "DualLieTrotter", "strang": "Strang"}[kind]
    return (lri.ProjectorSplitting(getattr(lri, order)(), gs), O.ProjectorSplitting(getattr(O, order)(), os_))


def run_both(lri, O, kind, precision, n=48, m=40, r=5, dt=0.02, T=0.3, scheme=("RK4", 2), seed=1, graded=True):
    A, B, U, S, V = sylv_instance(seed, n, m, r, graded)
    # rank decisions are compared exactly, so the FP32 run truncates well above its rounding level
    ag, ao = pair_algs(lri, O, kind, scheme, ra_tol=1e-3 if precision == "fp32" else 1e-7)
    pg = lri.MatrixDEProblem(lri.SylvesterTridiagOperator(A, B), lri.SVDLikeRepresentation(U, S, V), (0.0, T))
    po = O.MatrixDEProblem(O.SylvesterTridiagOp(A, B), O.SVDLikeRepresentation(U, S, V), (0.0, T))
    sg = lri.solve(pg, ag, dt, precision=precision)
    so = O.solve(po, ao, dt)
    return sg, so


@pytest.mark.parametrize("precision", ["fp64", "df", "fp32"])
@pytest.mark.parametrize("kind", ["bug", "primal", "dual", "strang", "ra"])
def test_sylvester_small_every_step(lri, oracle, kind, precision):
    sg, so = run_both(lri, oracle, kind, precision)
    assert len(sg.Y) == len(so.Y)
    for k, (yg, yo) in enumerate(zip(sg.Y, so.Y)):
        assert yg.rank == yo.rank, f"step {k}: rank {yg.rank} != {yo.rank}"
        err = oracle.rel_fro_err(yg.full(), yo.full())
        assert err <= TOL[precision], f"step {k}: {err:.3e}"
    # orthonormal bases
    yg = sg.Y[-1]
    tol_o = 2e-6 if precision == "fp32" else 1e-12
    assert np.abs(yg.U.T @ yg.U - np.eye(yg.rank)).max() < tol_o
    assert np.abs(yg.V.T @ yg.V - np.eye(yg.rank)).max() < tol_o


@pytest.mark.parametrize("scheme", [("Euler", 3), ("Heun", 2), ("Midpoint", 1)])
def test_substep_schemes(lri, oracle, scheme):
    sg, so = run_both(lri, oracle, "bug", "fp64", scheme=scheme, T=0.1)
    assert oracle.rel_fro_err(sg.Y[-1].full(), so.Y[-1].full()) <= TOL["fp64"]


def test_zero_operator_keeps_y(lri, oracle):
    A, B, U, S, V = sylv_instance(3, 30, 34, 4)
    Y0 = lri.SVDLikeRepresentation(U, S, V)
    for alg in [lri.UnconventionalAlgorithm(), lri.ProjectorSplitting(lri.Strang()),
                lri.RankAdaptiveUnconventionalAlgorithm(1e-12, rmax=8)]:
        sol = lri.solve(lri.MatrixDEProblem(lri.ZeroOperator(), Y0, (0.0, 0.05)), alg, 0.01)
        assert oracle.rel_fro_err(sol.Y[-1].full(), Y0.full()) < 1e-13


def test_invariant_subspace_closed_form_gpu(lri):
    """The analytic BUG answer (see test_oracle_kat) on the GPU, FP64."""
    from test_oracle_kat import invariant_problem, rk4_poly
    A, B, U, S, V, la, lb = invariant_problem()
    dt, nsteps, nsub = 0.05, 8, 3
    prob = lri.MatrixDEProblem(lri.SylvesterTridiagOperator(A, B), lri.SVDLikeRepresentation(U, S, V),
                               (0.0, dt * nsteps))
    Y = lri.solve(prob, lri.UnconventionalAlgorithm(lri.RK4(nsub)), dt).Y[-1].full()
    fac = rk4_poly(dt * (la[:, None] + lb[None, :]), nsub)
    Yref = U @ (np.diag(np.diag(S)) * fac ** nsteps) @ V.T
    assert np.linalg.norm(Y - Yref) / np.linalg.norm(Yref) < 1e-13


@pytest.mark.parametrize("precision", ["fp64", "df", "mixed"])
def test_batched_uneven_instances(lri, oracle, precision):
    """Eleven instances of uneven n, m, r in one batch (one CTA each); the
    r = 32 member has a core condition number of 2^31."""
    shapes = [(64, 70, 4), (128, 90, 8), (200, 256, 12), (96, 96, 16), (300, 180, 5), (72, 64, 32),
              (257, 129, 7), (64, 1024, 9), (1024, 64, 3), (150, 150, 20), (99, 101, 6)]
    insts = [sylv_instance(100 + i, *s) for i, s in enumerate(shapes)]
    dt, T = 1e-2, 0.1
    probs = [lri.MatrixDEProblem(lri.SylvesterTridiagOperator(A, B), lri.SVDLikeRepresentation(U, S, V), (0.0, T))
             for (A, B, U, S, V) in insts]
    out = lri.solve_ensemble(probs, lri.UnconventionalAlgorithm(lri.RK4(1)), dt, precision=precision)
    for i, (A, B, U, S, V) in enumerate(insts):
        po = oracle.MatrixDEProblem(oracle.SylvesterTridiagOp(A, B), oracle.SVDLikeRepresentation(U, S, V), (0.0, T))
        yo = oracle.solve(po, oracle.UnconventionalAlgorithm(oracle.RK4(1)), dt, save_everystep=False).Y[-1]
        err = oracle.rel_fro_err(out[i].full(), yo.full())
        assert err <= TOL[precision], f"instance {i} {shapes[i]}: {err:.3e}"


@pytest.mark.parametrize("precision", ["fp64", "df", "fp32"])
def test_prepared_graph_matches_single_steps(lri, precision):
    """lri_batch_prepare builds the graph of a multi-step call ahead of time;
    running it must give what the same steps give as single-step calls."""
    shapes = [(64, 70, 4), (128, 90, 8), (96, 96, 16)]
    insts = [sylv_instance(300 + i, *s, graded=False) for i, s in enumerate(shapes)]
    alg = lri.UnconventionalAlgorithm(lri.RK4(1))
    nat = lri._native
    ys = []
    for graph in (False, True):
        b = lri.Batch([s[0] for s in shapes], [s[1] for s in shapes], [s[2] for s in shapes], alg,
                      nat.LRI_OP_SYLVESTER_TRIDIAG, precision)
        b.upload([lri.SVDLikeRepresentation(U, S, V) for (A, B, U, S, V) in insts],
                 [lri.SylvesterTridiagOperator(A, B) for (A, B, U, S, V) in insts])
        if graph:
            b.prepare(1e-2, 9)
            b.step(0.0, 1e-2, 9)
        else:
            for k in range(9):
                b.step(k * 1e-2, 1e-2, 1)
        b.check_status()
        ys.append([f.full() for f in b.download()])
        b.close()
    for y1, y2 in zip(*ys):
        assert np.linalg.norm(y1 - y2) <= 1e-13 * np.linalg.norm(y1)


@pytest.mark.parametrize("precision", ["fp64", "df", "mixed", "fp32"])
def test_lyapunov_ensemble_slice(lri, oracle, precision):
    """32 instances of the 4096-member Lyapunov ensemble, full 200 steps.
    The pure FP32 form is checked on the well-conditioned members only (the
    ones the mixed form gives to FP32)."""
    insts = workloads.lyapunov_ensemble(first=0, limit=32)
    if precision == "fp32":
        insts = [e for e in insts if lri.core_condition(e.S) <= lri.MIXED_KAPPA_MAX]
        assert len(insts) >= 8
    dt, T = 1e-2, 2.0
    probs = [lri.MatrixDEProblem(lri.SylvesterTridiagOperator(e.A, e.B), lri.SVDLikeRepresentation(e.U, e.S, e.V),
                                 (0.0, T)) for e in insts]
    out = lri.solve_ensemble(probs, lri.UnconventionalAlgorithm(lri.RK4(1)), dt, precision=precision)
    errs = []
    for i, e in enumerate(insts):
        po = oracle.MatrixDEProblem(oracle.SylvesterTridiagOp(e.A, e.B), oracle.SVDLikeRepresentation(e.U, e.S, e.V),
                                    (0.0, T))
        yo = oracle.solve(po, oracle.UnconventionalAlgorithm(oracle.RK4(1)), dt, save_everystep=False).Y[-1]
        errs.append(oracle.rel_fro_err(out[i].full(), yo.full()))
    # members with kappa(S0) up to 2^31 amplify double-float rounding (~1e-14)
    # by ~1e4 over 200 steps; the FP64 form tracks the oracle to 1e-11
    tol = 1e-8 if precision == "df" else TOL[precision]
    assert max(errs) <= tol, f"max err {max(errs):.3e}"


@pytest.mark.parametrize("precision", ["fp64", "df"])
def test_sylvester_256_every_100_steps(lri, oracle, precision):
    """The stiff 256 x 256, r = 8 workload (RK4 nsub = 20, 1000 steps).  As
    the stiff modes decay the core's condition number passes 1e10, so the
    tolerance is calibrated against the oracle's own sensitivity: a second
    oracle run whose core gets a 1e-16 relative perturbation every step."""
    inst, dt, tspan, nsub = workloads.sylvester_256()
    Yo = oracle.SVDLikeRepresentation(inst.U, inst.S, inst.V)
    mk = lambda: oracle.init(oracle.MatrixDEProblem(oracle.SylvesterTridiagOp(inst.A, inst.B), Yo, tspan),
                             oracle.UnconventionalAlgorithm(oracle.RK4(nsub)), dt)
    integ_o, integ_p = mk(), mk()
    rng = np.random.default_rng(0)
    b = lri.Batch([256], [256], [8], lri.UnconventionalAlgorithm(lri.RK4(nsub)),
                  lri._native.LRI_OP_SYLVESTER_TRIDIAG, precision)
    b.upload([lri.SVDLikeRepresentation(inst.U, inst.S, inst.V)],
             [lri.SylvesterTridiagOperator(inst.A, inst.B)])
    t = 0.0
    for chunk in range(10):
        b.step(t, dt, 100)
        for _ in range(100):
            oracle.step(integ_o, integ_o.alg, dt)
            oracle.step(integ_p, integ_p.alg, dt)
            integ_p.u.S = integ_p.u.S * (1 + 1e-16 * rng.standard_normal(integ_p.u.S.shape))
            t += dt
        yg = b.download()[0]
        err = oracle.rel_fro_err(yg.full(), integ_o.u.full())
        sens = oracle.rel_fro_err(integ_p.u.full(), integ_o.u.full())
        tol = max(TOL[precision], 100.0 * sens * (100.0 if precision == "df" else 1.0))
        assert err <= tol, f"after {100 * (chunk + 1)} steps: {err:.3e} (oracle sensitivity {sens:.3e})"
    b.check_status()


def test_data_reference_continuous_vs_discrete_gpu(lri, oracle):
    """test/data_driven_approximation.jl:22-31 on the GPU (FP64): function
    stream vs 101 snapshots agree elementwise (rtol sqrt(eps)), and both
    agree with the oracle."""
    import math
    Y = workloads.data_rotation(seed=0, N=100)
    X0o = oracle.truncated_svd(Y(0.0), tol=1e-4)
    X0 = lri.SVDLikeRepresentation(X0o.U, X0o.S, X0o.V)
    data = [Y(t) for t in np.arange(0, 101) * 0.01]
    rtol = math.sqrt(np.finfo(float).eps)
    for ag, ao in [(lri.UnconventionalAlgorithm(), oracle.UnconventionalAlgorithm()),
                   (lri.ProjectorSplitting(lri.PrimalLieTrotter()), oracle.ProjectorSplitting(oracle.PrimalLieTrotter())),
                   (lri.ProjectorSplitting(lri.DualLieTrotter()), oracle.ProjectorSplitting(oracle.DualLieTrotter())),
                   (lri.RankAdaptiveUnconventionalAlgorithm(1e-8, rmax=20),
                    oracle.RankAdaptiveUnconventionalAlgorithm(1e-8, rmax=20))]:
        sol = lri.solve(lri.MatrixDataProblem(Y, X0, (0.0, 1.0)), ag, 1e-2, save_everystep=False)
        dsol = lri.solve(lri.MatrixDataProblem(data, X0), ag, save_everystep=False)
        a, b = sol.Y[-1].full(), dsol.Y[-1].full()
        assert np.all(np.abs(a - b) <= rtol * np.maximum(np.abs(a), np.abs(b)) + 1e-15 * np.abs(a).max()), \
            type(ag).__name__
        yo = oracle.solve(oracle.MatrixDataProblem(data, X0o), ao, save_everystep=False).Y[-1]
        assert oracle.rel_fro_err(b, yo.full()) <= 1e-10, type(ag).__name__


def test_rank_adaptive_trajectory_gpu(lri, oracle):
    """Analytic rank trajectory of test_oracle_kat on the GPU (FP64)."""
    from test_oracle_kat import rank_r_stream
    Y = rank_r_stream(decay3=100.0)
    Y0o = oracle.truncated_svd(Y(0.0), r=3)
    Y0 = lri.SVDLikeRepresentation(Y0o.U, Y0o.S, Y0o.V)
    tol = 1e-8
    sol = lri.solve(lri.MatrixDataProblem(Y, Y0, (0.0, 0.3)), lri.RankAdaptiveUnconventionalAlgorithm(tol, rmax=6),
                    0.025)
    ranks = [y.rank for y in sol.Y]
    expected = [3] + [oracle.truncate_to_tolerance(np.concatenate([Y.sv(t), np.zeros(3)]), tol) for t in sol.t[1:]]
    assert ranks == expected


def test_nonfinite_factor_is_reported(lri):
    """Host-side fault injection: a NaN in S is reported as LRI_ERR_NONFINITE."""
    A, B, U, S, V = sylv_instance(9, 40, 40, 4)
    S = S.copy()
    S[1, 1] = np.nan
    b = lri.Batch([40], [40], [4], lri.UnconventionalAlgorithm(), lri._native.LRI_OP_SYLVESTER_TRIDIAG, "fp64")
    b.upload([lri.SVDLikeRepresentation(U, S, V)], [lri.SylvesterTridiagOperator(A, B)])
    b.step(0.0, 0.01, 1)
    with pytest.raises(lri.LriError) as ei:
        b.check_status()
    assert ei.value.code == 4
    b.check_status()  # the status word was cleared


def test_step_before_bind_is_rejected(lri):
    b = lri.Batch([40], [40], [4], lri.UnconventionalAlgorithm(), lri._native.LRI_OP_SYLVESTER_TRIDIAG, "fp64")
    import ctypes as C
    code = b.lib.lri_batch_step(b.handle, 0.0, 0.01, 1, None, None)
    assert code == 8  # LRI_ERR_STATE
