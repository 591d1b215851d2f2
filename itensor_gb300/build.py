"""Builds the in-tree shared library itensor_gb300/libitg.so for sm_103a.

CUDA sources are compiled by nvcc with one -gencode (compute_103a -> sm_103a),
host C++ by g++, all translation units in parallel; the result is linked
against the CUDA runtime. Rebuilds only what changed (mtime check).

    python -m itensor_gb300.build      (or itensor_gb300.build.build())
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libitg.so")
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = ["contract.cu", "ozaki.cu", "ops.cu", "eigh.cu", "eigh_tri.cu", "svd.cu", "peaks.cu", "noalloc.cu"]
CPP_SOURCES = ["tridiag_ql.cpp", "tensor.cpp", "algo_core.cpp", "heff_program.cpp", "svd_split.cpp", "models.cpp", "dmrg.cpp", "fiber.cpp", "pool.cpp", "mps_io.cpp", "capi.cpp"]
HEADERS = ["common.h", "tensor.h", "engine.h", "ops.h", "algo.h", "fiber.h", "pool.h", "eigh_tri.h", "tridiag_ql.h",
           "mps_io.h", "ozaki_tc.cuh"]


def _newest(paths):
    return max(os.path.getmtime(p) for p in paths if os.path.exists(p))


def _compile(src):
    path = os.path.join(CSRC, src)
    obj = os.path.join(BUILD, src + ".o")
    deps = [path] + [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(HERE, "..", "include", "itg.h")]
    if os.path.exists(obj) and os.path.getmtime(obj) >= _newest(deps):
        return obj
    if src.endswith(".cu"):
        cmd = [NVCC] + ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-c", path, "-o", obj]
    else:
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-I" + os.path.join(CUDA_HOME, "include"), "-c", path, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return obj


def build(verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    srcs = CU_SOURCES + CPP_SOURCES
    with ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        objs = list(ex.map(_compile, srcs))
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= _newest(objs):
        return LIB
    cmd = [NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
