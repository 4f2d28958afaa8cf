"""ctypes binding of the C ABI in include/lri.h (liblri_gb300.so).

This is the same binding a Julia ``ccall`` shim makes: plain pointers, sizes
and small structs.  Loading fails loudly when the library or a CUDA device
is missing; there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional

from . import _build

LRI_OK = 0
STATUS_NAMES = {
    0: "LRI_OK", 1: "LRI_ERR_ARG", 2: "LRI_ERR_UNSUPPORTED", 3: "LRI_ERR_BREAKDOWN",
    4: "LRI_ERR_NONFINITE", 5: "LRI_ERR_RANK_OVERFLOW", 6: "LRI_ERR_TIMEOUT", 7: "LRI_ERR_CUDA",
    8: "LRI_ERR_STATE",
}

LRI_F64, LRI_F32, LRI_DF = 0, 1, 2
LRI_ALG_BUG, LRI_ALG_RA_BUG, LRI_ALG_KSL, LRI_ALG_GREEDY = 0, 1, 2, 3
LRI_KSL_PRIMAL, LRI_KSL_DUAL, LRI_KSL_STRANG = 0, 1, 2
LRI_OP_ZERO, LRI_OP_SYLVESTER_TRIDIAG, LRI_OP_BURGERS_PERIODIC, LRI_OP_DATA, LRI_OP_LOCAL_FLOW = 0, 1, 2, 3, 4

# Every symbol include/lri.h declares (checked by the CPU test suite).
EXPORTED = [
    "lri_abi_version", "lri_status_str", "lri_device_info", "lri_flow_count", "lri_flow_name", "lri_batch_create", "lri_batch_destroy",
    "lri_batch_layout", "lri_batch_bind", "lri_batch_data_layout", "lri_batch_data_init", "lri_batch_step",
    "lri_batch_ranks", "lri_batch_status", "lri_batch_launches_per_step", "lri_bug_step_noalloc",
    "lri_batch_prepare", "lri_batch_adjoint_prepare", "lri_batch_adjoint_step",
    "lri_stream_create", "lri_stream_destroy", "lri_stream_bind", "lri_stream_step", "lri_stream_rank",
    "lri_stream_status", "lri_stream_set_tensor_cores", "lri_stream_uses_tensor_cores", "lri_stream_data_product",
    "lri_stream_set_pass_tiles", "lri_batch_set_occupancy", "lri_stream_greedy_step",
    "lri_burgers_create", "lri_burgers_bind", "lri_burgers_step",
    "lri_history_create", "lri_history_destroy", "lri_history_record", "lri_history_wait",
]


class LriError(RuntimeError):
    def __init__(self, code: int, where: str):
        self.code = code
        super().__init__(f"{where}: {STATUS_NAMES.get(code, code)}")


class lri_scheme(C.Structure):
    _fields_ = [("nstages", C.c_int32), ("nsub", C.c_int32), ("a", C.c_double * 4),
                ("b", C.c_double * 4), ("c", C.c_double * 4)]


class lri_alg_desc(C.Structure):
    _fields_ = [("kind", C.c_int32), ("ksl_order", C.c_int32), ("K_alg", lri_scheme),
                ("L_alg", lri_scheme), ("S_alg", lri_scheme), ("tol", C.c_double),
                ("r_min", C.c_int32), ("two_factor", C.c_int32)]


class lri_batch_desc(C.Structure):
    _fields_ = [("dtype", C.c_int32), ("op", C.c_int32), ("count", C.c_int32), ("flow", C.c_int32),
                ("n", C.POINTER(C.c_int64)), ("m", C.POINTER(C.c_int64)), ("r", C.POINTER(C.c_int64)),
                ("r_cap", C.POINTER(C.c_int64)), ("burgers_h", C.c_double), ("burgers_alpha", C.c_double),
                ("burgers_beta", C.c_double)]


_lib: Optional[C.CDLL] = None


def _declare(lib: C.CDLL) -> None:
    P = C.c_void_p
    I64P = C.POINTER(C.c_int64)
    lib.lri_abi_version.restype = C.c_int
    lib.lri_status_str.restype = C.c_char_p
    lib.lri_status_str.argtypes = [C.c_int]
    lib.lri_flow_count.restype = C.c_int32
    lib.lri_flow_name.restype = C.c_char_p
    lib.lri_flow_name.argtypes = [C.c_int32]
    lib.lri_device_info.restype = C.c_int
    lib.lri_device_info.argtypes = [C.POINTER(C.c_int)] * 4
    lib.lri_batch_create.restype = C.c_int
    lib.lri_batch_create.argtypes = [C.POINTER(P), C.POINTER(lri_batch_desc), C.POINTER(lri_alg_desc)]
    lib.lri_batch_destroy.restype = C.c_int
    lib.lri_batch_destroy.argtypes = [P]
    lib.lri_batch_layout.restype = C.c_int
    lib.lri_batch_layout.argtypes = [P, I64P, I64P, I64P, I64P, I64P, I64P]
    lib.lri_batch_bind.restype = C.c_int
    lib.lri_batch_bind.argtypes = [P, P, P, P, P, P]
    lib.lri_batch_data_layout.restype = C.c_int
    lib.lri_batch_data_layout.argtypes = [P, I64P, I64P]
    lib.lri_batch_data_init.restype = C.c_int
    lib.lri_batch_data_init.argtypes = [P, P, P]
    lib.lri_batch_step.restype = C.c_int
    lib.lri_batch_step.argtypes = [P, C.c_double, C.c_double, C.c_int32, P, P]
    lib.lri_batch_ranks.restype = C.c_int
    lib.lri_batch_ranks.argtypes = [P, I64P, P]
    lib.lri_batch_status.restype = C.c_int
    lib.lri_batch_status.argtypes = [P, P]
    lib.lri_batch_launches_per_step.restype = C.c_int32
    lib.lri_batch_launches_per_step.argtypes = [P]
    lib.lri_stream_create.restype = C.c_int
    lib.lri_stream_create.argtypes = [C.POINTER(P), C.c_int32, C.c_int64, C.c_int64, C.c_int64, C.c_int64,
                                      C.c_double, C.c_int32]
    lib.lri_stream_destroy.restype = C.c_int
    lib.lri_stream_destroy.argtypes = [P]
    lib.lri_stream_bind.restype = C.c_int
    lib.lri_stream_bind.argtypes = [P, P, P, P]
    lib.lri_stream_step.restype = C.c_int
    lib.lri_stream_step.argtypes = [P, P, P, P]
    lib.lri_stream_rank.restype = C.c_int
    lib.lri_stream_rank.argtypes = [P, C.POINTER(C.c_int64), P]
    lib.lri_stream_status.restype = C.c_int
    lib.lri_stream_status.argtypes = [P, P]
    lib.lri_stream_set_tensor_cores.restype = C.c_int
    lib.lri_stream_set_tensor_cores.argtypes = [P, C.c_int32]
    lib.lri_stream_greedy_step.restype = C.c_int
    lib.lri_stream_greedy_step.argtypes = [P, P, P]
    lib.lri_stream_set_pass_tiles.restype = C.c_int
    lib.lri_stream_set_pass_tiles.argtypes = [P, C.c_int32, C.c_int32, C.c_int32]
    lib.lri_batch_set_occupancy.restype = C.c_int
    lib.lri_batch_set_occupancy.argtypes = [P, C.c_int32]
    lib.lri_stream_uses_tensor_cores.restype = C.c_int
    lib.lri_stream_uses_tensor_cores.argtypes = [P, C.POINTER(C.c_int32)]
    lib.lri_stream_data_product.restype = C.c_int
    lib.lri_stream_data_product.argtypes = [P, C.c_int32, P, P, P, C.c_int64, C.c_int64, P, C.c_int64, P]
    lib.lri_history_create.restype = C.c_int
    lib.lri_history_create.argtypes = [C.POINTER(P), P, C.c_int32]
    lib.lri_history_destroy.restype = C.c_int
    lib.lri_history_destroy.argtypes = [P]
    lib.lri_history_record.restype = C.c_int
    lib.lri_history_record.argtypes = [P, P, P, P, C.POINTER(C.c_int32), P, C.POINTER(C.c_int64)]
    lib.lri_history_wait.restype = C.c_int
    lib.lri_history_wait.argtypes = [P, C.c_int64]
    lib.lri_burgers_create.restype = C.c_int
    lib.lri_burgers_create.argtypes = [C.POINTER(P), C.c_int32, C.c_int64, C.c_int64, C.c_int64, C.c_int64,
                                       C.c_double, C.c_int32, C.c_double, C.c_double, C.c_double, P]
    lib.lri_burgers_bind.restype = C.c_int
    lib.lri_burgers_bind.argtypes = [P, P, P, P, P]
    lib.lri_burgers_step.restype = C.c_int
    lib.lri_burgers_step.argtypes = [P, C.c_double, C.c_int32, P]
    lib.lri_batch_adjoint_prepare.restype = C.c_int
    lib.lri_batch_adjoint_prepare.argtypes = [P]
    lib.lri_batch_adjoint_step.restype = C.c_int
    lib.lri_batch_adjoint_step.argtypes = [P, C.c_double, P, P, P, P, P, P, P, P]
    lib.lri_batch_prepare.restype = C.c_int
    lib.lri_batch_prepare.argtypes = [P, C.c_double, C.c_int32]
    lib.lri_bug_step_noalloc.restype = C.c_int
    lib.lri_bug_step_noalloc.argtypes = [C.c_int32, C.c_int64, C.c_int64, C.c_int64, P, P, P, P, P, C.c_double,
                                         C.c_int32, C.POINTER(lri_scheme), P, C.POINTER(C.c_int32)]


def library_path() -> str:
    return _build.LIB_PATH


def load(build_if_missing: bool = True) -> C.CDLL:
    """Loads liblri_gb300.so (building it when missing or stale)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB_PATH
    if build_if_missing and _build.is_stale():
        _build.build()
    if not os.path.exists(path):
        raise RuntimeError(f"liblri_gb300.so is missing ({path}); run the build first")
    lib = C.CDLL(path)
    _declare(lib)
    _lib = lib
    return lib


def check(code: int, where: str) -> None:
    if code != LRI_OK:
        raise LriError(code, where)
