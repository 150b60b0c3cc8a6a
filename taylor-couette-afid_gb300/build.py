"""Build libtcgb300.so (the C ABI of include/tc_capi.h) in-tree for sm_103a.

Each translation unit is compiled in parallel, then linked with the static
CUDA runtime, so the library depends only on the driver at run time.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libtcgb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]
SOURCES = ["tc_capi.cu", "tc_kernels.cu", "tc_host.cpp", "tc_noalloc.cu", "tc_batch.cu", "tc_selftest.cu", "tc_h5.cpp", "tc_stats.cu", "tc_persist.cu"]


def _nvcc() -> str:
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps.append(os.path.join(HERE, "..", "include", "tc_capi.h"))
    deps.append(__file__)
    return any(os.path.getmtime(p) > t for p in deps if os.path.exists(p))


def build(force: bool = False, verbose: bool = False, extra: list[str] | None = None) -> str:
    if not force and not _stale():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    extra = list(extra or [])

    def compile_one(src: str) -> str:
        obj = os.path.join(BUILD, src + ".o")
        path = os.path.join(CSRC, src)
        if src.endswith(".cu"):
            cmd = [nvcc, *ARCH, *NVCC_FLAGS, *extra, "-c", path, "-o", obj]
        else:
            cmd = ["g++", "-O3", "-std=c++17", "-fPIC", "-Wall", "-ffp-contract=off", "-c", path, "-o", obj,
                   "-I", os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if verbose or r.returncode != 0:
            sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
        if r.returncode != 0:
            raise RuntimeError(f"compiling {src} failed")
        return obj

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB + ".tmp"
    cmd = [nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-cudart", "static"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
        raise RuntimeError("linking libtcgb300.so failed")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
