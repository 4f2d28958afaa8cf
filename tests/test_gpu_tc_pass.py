"""The snapshot passes of the data substeps on the tensor cores (tc_pass.cu:
tcgen05 + TMA, dY split into TF32 hi + lo parts, 3xTF32 products with FP32
accumulation) through lri_stream_data_product: dY X and dY^T X against the
FP64 product of the same FP32 snapshots and panel, against the CUDA-core
passes, at sizes with partial 128-row tiles and at the full 8192 x 4096
data-compression size; then the stream engine on either pass kind against
the oracle.  Tolerance: 2e-6 relative Frobenius error for one product (FP32
rounding of the output and of the summation order), 1e-5 for the steps."""
import os
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                                "lowrankintegrators.jl_gb300"))
import workloads  # noqa: E402

PRODUCT_TOL = 2e-6


def _dev(torch, x):
    return torch.from_numpy(np.asarray(x, np.float32).ravel(order="F")).cuda()


def _check_product(lri, n, m, R, ncols, seed, snaps=None):
    torch = lri._torch()
    eng = lri.DataStreamEngine(n, m, 1, R, 1e-6, 1, "fp32")
    try:
        assert eng.uses_tensor_cores()
        if snaps is None:
            snaps = workloads.data_stream(n, m, 2, seed=seed)
        A0, A1 = (np.asarray(a, np.float32) for a in snaps[:2])
        dA0, dA1 = eng.to_device(A0), eng.to_device(A1)
        dY = A1.astype(np.float64) - A0.astype(np.float64)
        g = np.random.default_rng(seed)
        for trans in (False, True):
            rows_x, rows_o = (n, m) if trans else (m, n)
            X = np.linalg.qr(g.standard_normal((rows_x, ncols)))[0].astype(np.float32)
            ref = (dY.T if trans else dY) @ X.astype(np.float64)
            outs = []
            for tc in (True, False):
                eng.set_tensor_cores(tc)
                out = eng.data_product(dA0, dA1, _dev(torch, X), trans=trans)
                torch.cuda.synchronize()
                o = out.cpu().numpy().astype(np.float64).reshape((R, rows_o)).T
                assert np.all(o[:, ncols:] == 0.0), "inactive columns must be zero"
                o = o[:, :ncols]
                err = np.linalg.norm(o - ref) / np.linalg.norm(ref)
                assert err <= PRODUCT_TOL, f"{'tensor' if tc else 'CUDA'} cores, trans={trans}: {err:.3e}"
                outs.append(o)
            diff = np.linalg.norm(outs[0] - outs[1]) / np.linalg.norm(ref)
            assert diff <= PRODUCT_TOL, f"tensor vs CUDA cores, trans={trans}: {diff:.3e}"
        eng.check_status()
    finally:
        eng.close()


@pytest.mark.parametrize("n,m,R,ncols", [(1024, 512, 48, 48), (1024, 512, 48, 17), (256, 384, 64, 1),
                                         (1000, 516, 96, 96), (516, 1000, 40, 33)])
def test_data_product_matches_fp64(lri, n, m, R, ncols):
    _check_product(lri, n, m, R, ncols, seed=3)


def test_data_product_full_size(lri):
    """8192 x 4096 snapshots of the data-compression stream, 96 columns."""
    _check_product(lri, 8192, 4096, 96, 96, seed=2)


def test_tensor_cores_unavailable_for_fp64_and_small(lri):
    e64 = lri.DataStreamEngine(1024, 512, 4, 48, 1e-6, 1, "fp64")
    try:
        assert not e64.uses_tensor_cores()
        with pytest.raises(lri.LriError):
            e64.set_tensor_cores(True)
    finally:
        e64.close()
    small = lri.DataStreamEngine(96, 200, 4, 24, 1e-6, 1, "fp32")  # n < 128: CUDA-core passes
    try:
        assert not small.uses_tensor_cores()
    finally:
        small.close()


@pytest.mark.parametrize("tc", [True, False])
def test_stream_engine_both_pass_kinds_match_oracle(lri, oracle, tc):
    snaps = workloads.data_stream(1024, 512, 8, seed=5)
    X0 = oracle.truncated_svd(snaps[0], r=16)
    so = oracle.solve(oracle.MatrixDataProblem(snaps, X0), oracle.RankAdaptiveUnconventionalAlgorithm(1e-6, rmax=48))
    eng = lri.DataStreamEngine(1024, 512, 16, 48, 1e-6, 1, "fp32")
    try:
        eng.set_tensor_cores(tc)
        eng.bind(lri.SVDLikeRepresentation(X0.U, X0.S, X0.V))
        prev = eng.to_device(snaps[0])
        for k in range(1, len(snaps)):
            nxt = eng.to_device(snaps[k])
            eng.step(prev, nxt)
            prev = nxt
            eng.check_status()
            yg, yo = eng.download(), so.Y[k]
            assert yg.S.shape == yo.S.shape, f"step {k}: rank {yg.S.shape[0]} vs {yo.S.shape[0]}"
            err = oracle.rel_fro_err(yg.full(), yo.full())
            assert err <= 1e-5, f"step {k}: {err:.3e}"
    finally:
        eng.close()
