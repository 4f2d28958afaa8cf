"""Builds the in-tree CUDA library ``_build/liblri_gb300.so`` for sm_103a.

Twelve translation units (FP32, FP64 and double-float engines, the FP32 and
double-float engines sized for two CTAs per SM, host C ABI,
the allocation-free entry point, the discrete adjoint, the large-stream
engine, its tensor-core snapshot passes, its cluster core SVD, the large
Burgers engine's tensor-core Khatri-Rao products) compile in parallel with nvcc and
link into one shared library.  The library is rebuilt
when a source or the public header is newer than it.
"""
from __future__ import annotations

import concurrent.futures
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "liblri_gb300.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "lri.h")

SOURCES = ["engine_f32.cu", "engine_f64.cu", "engine_df.cu", "engine_f32_occ2.cu", "engine_df_occ2.cu", "api.cpp",
           "noalloc.cu", "adjoint.cu", "stream.cu", "tc_pass.cu", "core_svd.cu", "tc_kr.cu"]
ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden"]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build liblri_gb300.so")
    return cand


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(HEADER)
    files.append(os.path.abspath(__file__))
    return files


def is_stale() -> bool:
    if not os.path.exists(LIB_PATH):
        return True
    t = os.path.getmtime(LIB_PATH)
    return any(os.path.getmtime(f) > t for f in _deps())


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile (if needed) and return the path of the shared library."""
    if not force and not is_stale():
        return LIB_PATH
    nvcc = _nvcc()
    os.makedirs(BUILD_DIR, exist_ok=True)

    def compile_one(src: str) -> str:
        obj = os.path.join(BUILD_DIR, os.path.splitext(src)[0] + ".o")
        cmd = [nvcc, *ARCH_FLAGS, *COMMON_FLAGS, "-I", os.path.dirname(HEADER), "-c",
               os.path.join(CSRC, src), "-o", obj]
        if src.endswith(".cu"):
            cmd[1:1] = ["-Xptxas", "-v"] if verbose else []
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{res.stderr}")
        if verbose and res.stderr:
            print(res.stderr)
        return obj

    with concurrent.futures.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB_PATH + ".tmp"
    cmd = [nvcc, *ARCH_FLAGS, "-shared", "-o", tmp, *objs, "-cudart", "shared"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stderr}")
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build(force=True, verbose=True))
