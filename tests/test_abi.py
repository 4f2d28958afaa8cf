"""C ABI checks that need no GPU: the library builds, loads, exports every
symbol include/lri.h declares, and rejects bad arguments on the host before
touching the device."""
import ctypes as C
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "lri.h")).read()
    return sorted(set(re.findall(r"LRI_API\s+[\w\s\*]+?\b(lri_\w+)\s*\(", src)))


def test_header_and_binding_agree(lri):
    from importlib import import_module
    native = import_module(lri.__name__ + "._native")
    assert declared_symbols() == sorted(native.EXPORTED)


def test_library_exports_every_declared_symbol(lri):
    native = __import__(lri.__name__ + "._native", fromlist=["_native"])
    lib = native.load()
    for name in declared_symbols():
        assert hasattr(lib, name), name
    assert lib.lri_abi_version() == 1
    assert lib.lri_status_str(0) == b"ok"
    assert b"CUDA" in lib.lri_status_str(7)


def _desc(native, n, m, r, rcap=None, op=None, dtype=None):
    d = native.lri_batch_desc()
    d.dtype = native.LRI_F64 if dtype is None else dtype
    d.op = native.LRI_OP_SYLVESTER_TRIDIAG if op is None else op
    d.count = len(n)
    keep = [np.asarray(x, np.int64) for x in (n, m, r)]
    P = C.POINTER(C.c_int64)
    d.n, d.m, d.r = (x.ctypes.data_as(P) for x in keep)
    if rcap is not None:
        keep.append(np.asarray(rcap, np.int64))
        d.r_cap = keep[-1].ctypes.data_as(P)
    return d, keep


def _alg(lri, alg):
    return lri._alg_desc(alg)


@pytest.mark.parametrize("case", [
    dict(n=[10], m=[10], r=[0]),            # rank 0
    dict(n=[10], m=[10], r=[11]),           # rank above rows
    dict(n=[10], m=[3], r=[4]),             # rank above columns
    dict(n=[200], m=[200], r=[4], rcap=[3]),  # capacity below rank
])
def test_create_rejects_bad_shapes(lri, case):
    native = __import__(lri.__name__ + "._native", fromlist=["_native"])
    lib = native.load()
    d, keep = _desc(native, case["n"], case["m"], case["r"], case.get("rcap"))
    a = _alg(lri, lri.UnconventionalAlgorithm())
    h = C.c_void_p()
    assert lib.lri_batch_create(C.byref(h), C.byref(d), C.byref(a)) == 1  # LRI_ERR_ARG


def test_create_rejects_bad_scheme_and_unsupported(lri):
    native = __import__(lri.__name__ + "._native", fromlist=["_native"])
    lib = native.load()
    h = C.c_void_p()
    d, keep = _desc(native, [40], [40], [4])
    a = _alg(lri, lri.UnconventionalAlgorithm())
    a.K_alg.nstages = 5
    assert lib.lri_batch_create(C.byref(h), C.byref(d), C.byref(a)) == 1
    a = _alg(lri, lri.UnconventionalAlgorithm())
    a.S_alg.nsub = 0
    assert lib.lri_batch_create(C.byref(h), C.byref(d), C.byref(a)) == 1
    # panels wider than the engine's 64 columns
    d, keep = _desc(native, [400], [400], [65])
    assert lib.lri_batch_create(C.byref(h), C.byref(d), C.byref(_alg(lri, lri.UnconventionalAlgorithm()))) == 2
    # rank-adaptive needs 2*r_cap <= min(n, m)
    d, keep = _desc(native, [20], [40], [4], rcap=[12])
    a = _alg(lri, lri.RankAdaptiveUnconventionalAlgorithm(1e-6, rmax=12))
    assert lib.lri_batch_create(C.byref(h), C.byref(d), C.byref(a)) == 1
    # Strang on snapshot data has no half-step snapshot
    d, keep = _desc(native, [40], [40], [4], op=native.LRI_OP_DATA)
    a = _alg(lri, lri.ProjectorSplitting(lri.Strang()))
    assert lib.lri_batch_create(C.byref(h), C.byref(d), C.byref(a)) == 2
    # null arguments
    assert lib.lri_batch_create(None, C.byref(d), C.byref(a)) == 1
    assert lib.lri_batch_step(None, 0.0, 0.1, 1, None, None) == 1
    assert lib.lri_batch_prepare(None, 0.1, 5) == 1
    # the large-stream engine: r_max above 96, double-float, too few rows
    hs = C.c_void_p()
    assert lib.lri_stream_create(C.byref(hs), native.LRI_F32, 8192, 4096, 16, 97, 1e-6, 1) == 1
    assert lib.lri_stream_create(C.byref(hs), native.LRI_DF, 8192, 4096, 16, 96, 1e-6, 1) == 2
    assert lib.lri_stream_create(C.byref(hs), native.LRI_F32, 100, 4096, 16, 64, 1e-6, 1) == 1
    assert lib.lri_stream_step(None, None, None, None) == 1
    # the large Burgers engine: r_max above 64, bad grid spacing, non-finite
    # coefficients, bad schemes, null handles (all rejected before any device work)
    sch = lri.RK4(64).to_c()
    bad = lri.RK4(1).to_c()
    bad.nstages = 5
    assert lib.lri_burgers_create(C.byref(hs), native.LRI_F32, 4096, 16384, 16, 65, 1e-4, 16,
                                  1.0 / 4096, 0.0, -0.5, C.byref(sch)) == 1
    assert lib.lri_burgers_create(C.byref(hs), native.LRI_F32, 4096, 16384, 16, 64, 1e-4, 16,
                                  0.0, 0.0, -0.5, C.byref(sch)) == 1
    assert lib.lri_burgers_create(C.byref(hs), native.LRI_F32, 4096, 16384, 16, 64, 1e-4, 16,
                                  1.0 / 4096, float("nan"), -0.5, C.byref(sch)) == 1
    assert lib.lri_burgers_create(C.byref(hs), native.LRI_F32, 4096, 16384, 16, 64, 1e-4, 16,
                                  1.0 / 4096, 0.0, -0.5, C.byref(bad)) == 1
    assert lib.lri_burgers_create(C.byref(hs), native.LRI_F32, 4096, 16384, 16, 64, 1e-4, 16,
                                  1.0 / 4096, 0.0, -0.5, None) == 1
    assert lib.lri_burgers_bind(None, None, None, None, None) == 1
    assert lib.lri_burgers_step(None, 1e-4, 1, None) == 1
    assert lib.lri_batch_destroy(None) == 1


def test_unsupported_flow_map_raises(lri):
    prob = lri.MatrixDEProblem(lambda X, t: X, lri.SVDLikeRepresentation(np.eye(4, 2), np.eye(2), np.eye(4, 2)),
                               (0.0, 1.0))
    with pytest.raises(lri.LriError):
        lri._op_kind(prob)


def test_step_count_matches_reference_loop(lri, oracle):
    for tspan, dt in [((0.0, 0.1), 1e-4), ((0.0, 1.0), 1e-2), ((0.0, 0.5), 0.3), ((1, 101), 1)]:
        assert lri.n_steps(tspan, dt) == oracle.n_steps(tspan, dt)
