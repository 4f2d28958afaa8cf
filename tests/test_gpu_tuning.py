"""The autotuner's knobs change how the work is scheduled, not what is
computed: the step kernel sized for 2 CTAs per SM gives the results of the
default 3-CTA kernel (FP32 and double-float ensembles), and every tile
choice of the tensor-core passes gives the same product within the
products' tolerance (2e-6); invalid choices are rejected."""
import os
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                                "lowrankintegrators.jl_gb300"))
import workloads  # noqa: E402


@pytest.mark.parametrize("precision", ["fp32", "df"])
def test_occupancy_variants_agree(lri, precision):
    insts = workloads.lyapunov_ensemble(first=0, limit=24)
    shapes = ([e.U.shape[0] for e in insts], [e.V.shape[0] for e in insts], [e.S.shape[0] for e in insts])
    alg = lri.UnconventionalAlgorithm(lri.RK4(1))
    outs = []
    for ctas in (3, 2):
        b = lri.Batch(*shapes, alg, lri._native.LRI_OP_SYLVESTER_TRIDIAG, precision)
        b.upload([lri.SVDLikeRepresentation(e.U, e.S, e.V) for e in insts],
                 [lri.SylvesterTridiagOperator(e.A, e.B) for e in insts])
        b.set_occupancy(ctas)
        b.step(0.0, 1e-2, 12)
        b.check_status()
        outs.append([y.full() for y in b.download()])
        b.close()
    for i, (a, c) in enumerate(zip(*outs)):
        assert np.linalg.norm(a - c) <= 1e-12 * np.linalg.norm(c), f"instance {i}"


def test_occupancy_rejects_invalid(lri):
    b = lri.Batch([40], [36], [4], lri.UnconventionalAlgorithm(), lri._native.LRI_OP_ZERO, "fp64")
    with pytest.raises(lri.LriError):
        b.set_occupancy(2)  # FP64 batches have the default kernel only
    with pytest.raises(lri.LriError):
        b.set_occupancy(5)
    b.close()


def test_pass_tiles_agree(lri):
    torch = lri._torch()
    n, m, R = 1024, 512, 48
    eng = lri.DataStreamEngine(n, m, R, R, 1e-6, 1, "fp32")
    try:
        g = torch.Generator(device="cuda").manual_seed(3)
        A0, A1 = (torch.randn(n * m, device="cuda", generator=g) for _ in range(2))
        for trans in (False, True):
            X = torch.randn((n if trans else m) * R, device="cuda", generator=g)
            eng.set_pass_tiles(0, 0, 0)
            ref = eng.data_product(A0, A1, X, trans=trans).cpu().numpy().astype(np.float64)
            for sp in (1, 2, 3, 5):
                for stages in (2, 3, 4):
                    eng.set_pass_tiles(sp, sp, stages)
                    o = eng.data_product(A0, A1, X, trans=trans).cpu().numpy().astype(np.float64)
                    assert np.linalg.norm(o - ref) <= 2e-6 * np.linalg.norm(ref), (trans, sp, stages)
        with pytest.raises(lri.LriError):
            eng.set_pass_tiles(1, 1, 1)   # one stage cannot overlap copies and MMAs
        with pytest.raises(lri.LriError):
            eng.set_pass_tiles(1, 1, 9)   # more stages than shared memory holds
        eng.check_status()
    finally:
        eng.close()
