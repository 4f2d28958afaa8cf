"""The allocation-free entry point lri_bug_step_noalloc.

It serves callers that cannot call cudaMalloc (device memory owned by another
allocator, or a time loop that must not trigger cudaMalloc's device-wide
synchronisation): it runs the batch API's step kernel on a fixed 4 MiB
scratch array inside the library.  Here two calls in a row must reproduce
what the existing entry point (lri_batch_create / lri_batch_step) computes
for the same total number of steps, within the tolerances of the other GPU
tests.  Collected last so a run that stops at the first failure has run
everything else first.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = {"fp64": 1e-11, "fp32": 1e-5}


def problem(seed=21, n=120, m=100, r=6):
    g = np.random.default_rng(seed)
    A = (g.uniform(0.5, 1.0, n), -2.0 - g.uniform(0, 1, n), g.uniform(0.5, 1.0, n))
    B = (g.uniform(0.5, 1.0, m), -2.0 - g.uniform(0, 1, m), g.uniform(0.5, 1.0, m))
    U, _ = np.linalg.qr(g.standard_normal((n, r)))
    V, _ = np.linalg.qr(g.standard_normal((m, r)))
    S = np.diag(np.linspace(1.0, 0.2, r))
    return A, B, U, S, V


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_noalloc_matches_batch_entry_point(lri, precision):
    import torch

    native = lri._native
    lib = native.load()
    A, B, U, S, V = problem()
    n, m, r = U.shape[0], V.shape[0], S.shape[0]
    dt, k1, k2 = 1e-2, 7, 5
    alg = lri.UnconventionalAlgorithm(lri.RK4(2))

    # existing entry point (allocating batch), k1 + k2 steps
    b = lri.Batch([n], [m], [r], alg, native.LRI_OP_SYLVESTER_TRIDIAG, precision)
    b.upload([lri.SVDLikeRepresentation(U, S, V)], [lri.SylvesterTridiagOperator(A, B)])
    b.step(0.0, dt, k1 + k2)
    b.check_status()
    ref = b.download()[0].full()
    b.close()

    # allocation-free entry point: two calls in a row on caller-owned buffers
    dt_t = torch.float64 if precision == "fp64" else torch.float32
    dev = torch.device("cuda")
    col = lambda X: torch.from_numpy(np.asarray(X, dtype=np.float64).ravel(order="F")).to(dev, dt_t)
    dU, dS, dV = col(U), col(S), col(V)
    dA, dB = col(np.concatenate(A)), col(np.concatenate(B))
    sch = alg.K_alg.to_c()
    dtype = native.LRI_F64 if precision == "fp64" else native.LRI_F32
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    ptr = lambda x: C.c_void_p(x.data_ptr())
    st = C.c_int32(-1)
    for k in (k1, k2):
        code = lib.lri_bug_step_noalloc(dtype, n, m, r, ptr(dU), ptr(dS), ptr(dV), ptr(dA), ptr(dB), dt, k,
                                        C.byref(sch), stream, C.byref(st))
        assert code == 0, native.STATUS_NAMES.get(code, code)
        assert st.value == 0
    torch.cuda.synchronize()
    Ug = dU.double().cpu().numpy().reshape((r, n)).T
    Sg = dS.double().cpu().numpy().reshape((r, r)).T
    Vg = dV.double().cpu().numpy().reshape((r, m)).T
    Y = Ug @ Sg @ Vg.T
    err = np.linalg.norm(Y - ref) / np.linalg.norm(ref)
    assert err <= TOL[precision], f"{err:.3e}"


def test_noalloc_rejects_sizes_beyond_its_scratch(lri):
    native = lri._native
    lib = native.load()
    sch = lri.RK4(1).to_c()
    one = C.c_void_p(16)  # never dereferenced: the size check comes first
    code = lib.lri_bug_step_noalloc(native.LRI_F64, 4000, 4000, 32, one, one, one, one, one, 1e-2, 1,
                                    C.byref(sch), None, None)
    assert code == 1  # LRI_ERR_ARG
