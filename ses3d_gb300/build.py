"""Builds the native library ``libses3d_gpu.so`` (sm_103a) in-tree.

The CUDA translation units are compiled with nvcc for ``sm_103a`` only; the host
set-up code is compiled with ``-ffp-contract=off`` so that its FP32 arithmetic
rounds exactly as the reference's gfortran build (index/location work is
bit-exact). Objects are rebuilt only when a source is newer than the library.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libses3d_gpu.so")
DRIVER = os.path.join(HERE, "ses3d_gpu_main")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
              "-I" + os.path.join(ROOT, "include")]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-Wall",
             "-I" + os.path.join(ROOT, "include")]

CU_SOURCES = ["kernels.cu", "adjoint.cu", "capi.cu"]
CXX_SOURCES = ["setup.cpp"]
DRIVER_SOURCES = ["driver.cpp", "formats.cpp"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libses3d_gpu.so")


def _cuda_home(nvcc: str) -> str:
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))


def _newer(src_paths, target) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(p) > t for p in src_paths)


def _run(cmd, verbose):
    if verbose:
        print(" ".join(cmd), flush=True)
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("command failed: %s\n%s\n%s" % (" ".join(cmd), res.stdout, res.stderr))
    return res


def build(verbose: bool = False, force: bool = False) -> str:
    """Compiles and links libses3d_gpu.so (and the reference-style driver). Returns the library path."""
    nvcc = _nvcc()
    os.makedirs(OUT_DIR, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".hpp", ".cuh", ".h"))]
    headers.append(os.path.join(ROOT, "include", "ses3d_gpu.h"))
    jobs = []
    objs = []
    for f in CU_SOURCES:
        src = os.path.join(CSRC, f)
        obj = os.path.join(OUT_DIR, f + ".o")
        objs.append(obj)
        if force or _newer([src] + headers, obj):
            jobs.append([nvcc] + ARCH + NVCC_FLAGS + ["-c", src, "-o", obj])
    for f in CXX_SOURCES:
        src = os.path.join(CSRC, f)
        obj = os.path.join(OUT_DIR, f + ".o")
        objs.append(obj)
        if force or _newer([src] + headers, obj):
            jobs.append(["g++"] + CXX_FLAGS + ["-c", src, "-o", obj])
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        list(ex.map(lambda c: _run(c, verbose), jobs))
    if force or jobs or not os.path.exists(LIB):
        cuda_lib = os.path.join(_cuda_home(nvcc), "lib64")
        _run([nvcc] + ARCH + ["-shared", "-cudart", "static", "-o", LIB] + objs + ["-L" + cuda_lib], verbose)
    drv_src = [os.path.join(CSRC, f) for f in DRIVER_SOURCES if os.path.exists(os.path.join(CSRC, f))]
    if len(drv_src) == len(DRIVER_SOURCES) and (force or _newer(drv_src + headers + [LIB], DRIVER)):
        _run(["g++"] + CXX_FLAGS + ["-o", DRIVER] + drv_src +
             ["-L" + HERE, "-lses3d_gpu", "-Wl,-rpath,$ORIGIN"], verbose)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
