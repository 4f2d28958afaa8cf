"""The solution history (lri_history_*: a device ring of factor copies, each
copied to page-locked host memory on the history's own stream; the
reference's update_sol!, src/primitives.jl:82-90) against synchronous
downloads after every step: the records must hold exactly the factors the
steps produced, also when the ring (2 slots) wraps many times, for
rank-adaptive batches whose rank changes, and in solve(save_everystep=True)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _sylvester(seed, n, m, r):
    g = np.random.default_rng(seed)
    A = (g.uniform(0.5, 1, n), -2 - g.uniform(0, 1, n), g.uniform(0.5, 1, n))
    B = (g.uniform(0.5, 1, m), -2 - g.uniform(0, 1, m), g.uniform(0.5, 1, m))
    U, _ = np.linalg.qr(g.standard_normal((n, r)))
    V, _ = np.linalg.qr(g.standard_normal((m, r)))
    S = np.diag(2.0 ** -np.arange(1, r + 1))
    return A, B, U, S, V


@pytest.mark.parametrize("precision,slots", [("fp64", 2), ("fp32", 3), ("df", 8)])
def test_history_records_every_step(lri, precision, slots):
    shapes = [(64, 70, 4), (128, 90, 8), (96, 96, 6)]
    insts = [_sylvester(10 + i, *s) for i, s in enumerate(shapes)]
    alg = lri.UnconventionalAlgorithm(lri.RK4(1))
    kind = lri._native.LRI_OP_SYLVESTER_TRIDIAG
    factors = [lri.SVDLikeRepresentation(U, S, V) for (A, B, U, S, V) in insts]
    ops = [lri.SylvesterTridiagOperator(A, B) for (A, B, U, S, V) in insts]
    mk = lambda: lri.Batch([s[0] for s in shapes], [s[1] for s in shapes], [s[2] for s in shapes], alg, kind,
                           precision)
    ref = mk()
    ref.upload(factors, ops)
    expected = []
    for k in range(9):
        ref.step(k * 1e-2, 1e-2, 1)
        expected.append([y.full() for y in ref.download()])
    ref.close()
    b = mk()
    b.upload(factors, ops)
    h = lri.History(b, slots=slots)
    for k in range(9):
        b.step(k * 1e-2, 1e-2, 1)
        h.record()
    recs = h.collect()
    h.close()
    b.check_status()
    b.close()
    assert len(recs) == 9
    for k, (rec, exp) in enumerate(zip(recs, expected)):
        for i, (y, e) in enumerate(zip(rec, exp)):
            assert np.array_equal(y.full(), e), f"step {k}, instance {i}"


def test_history_tracks_rank_changes(lri, oracle):
    """Rank-adaptive steps on a data stream: every record carries the rank of
    its step."""
    import os
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                                    "lowrankintegrators.jl_gb300"))
    import workloads
    snaps = workloads.data_stream(200, 160, 7, seed=9)
    X0 = oracle.truncated_svd(snaps[0], r=3)
    prob = lri.MatrixDataProblem(snaps, lri.SVDLikeRepresentation(X0.U, X0.S, X0.V))
    alg = lri.RankAdaptiveUnconventionalAlgorithm(1e-3, rmax=20)
    sol = lri.solve(prob, alg, precision="fp64", save_everystep=True)
    integ = lri.init(prob, alg, 1, precision="fp64")
    ranks = []
    for k in range(1, len(snaps)):
        lri.step(integ, alg, 1)
        ranks.append(integ.u.S.shape[0])
        assert np.array_equal(sol.Y[k].full(), integ.u.full()), f"snapshot {k}"
    integ.batch.close()
    assert [y.S.shape[0] for y in sol.Y[1:]] == ranks
    assert len(set(ranks)) > 1, "the rank should change along this stream"


def test_history_reused_host_buffers(lri):
    """Three caller-owned host buffer sets cycled over nine records (each
    reused once wait() returned for its previous record): every record, read
    right after its wait, holds exactly the factors of its step."""
    shapes = [(64, 70, 4), (96, 96, 6)]
    insts = [_sylvester(30 + i, *s) for i, s in enumerate(shapes)]
    alg = lri.UnconventionalAlgorithm(lri.RK4(1))
    kind = lri._native.LRI_OP_SYLVESTER_TRIDIAG
    factors = [lri.SVDLikeRepresentation(U, S, V) for (A, B, U, S, V) in insts]
    ops = [lri.SylvesterTridiagOperator(A, B) for (A, B, U, S, V) in insts]
    mk = lambda: lri.Batch([s[0] for s in shapes], [s[1] for s in shapes], [s[2] for s in shapes], alg, kind, "fp32")
    ref = mk()
    ref.upload(factors, ops)
    expected = []
    for k in range(9):
        ref.step(k * 1e-2, 1e-2, 1)
        expected.append([y.full() for y in ref.download()])
    ref.close()
    b = mk()
    b.upload(factors, ops)
    h = lri.History(b, slots=2)
    bufs = [h.host_buffers() for _ in range(3)]
    seq = [None] * 3
    got = [None] * 9
    owner = [None] * 3

    def harvest(slot):
        hU, hS, hV, hR = bufs[slot]
        k = owner[slot]
        got[k] = [y.full() for y in b.unpack(hU.numpy()[:b.U.numel()], hS.numpy()[:b.S.numel()],
                                             hV.numpy()[:b.V.numel()], hR.numpy()[:b.count])]

    for k in range(9):
        b.step(k * 1e-2, 1e-2, 1)
        slot = k % 3
        if seq[slot] is not None:
            h.wait(seq[slot])
            harvest(slot)
        seq[slot] = h.record(host=bufs[slot])
        owner[slot] = k
    for slot in range(3):
        h.wait(seq[slot])
        harvest(slot)
    h.close()
    b.check_status()
    b.close()
    for k in range(9):
        for i, (y, e) in enumerate(zip(got[k], expected[k])):
            assert np.array_equal(y, e), f"step {k}, instance {i}"
