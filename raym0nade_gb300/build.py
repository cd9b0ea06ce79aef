"""Build librmn.so in-tree: nvcc for the CUDA kernels (sm_103a only), g++ for
the host C++, linked into raym0nade_gb300/_build/librmn.so.

Every translation unit is compiled without floating-point contraction
(nvcc -fmad=false, g++ -ffp-contract=off) so that the traversal reproduces the
reference's float results bit for bit on both the x86-64 build host and the
aarch64 GPU host. Objects are rebuilt only when a source or header is newer.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "librmn.so")
ROOT = os.path.dirname(HERE)
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-fmad=false", "-Xcompiler", "-fPIC", "-Xcompiler",
              "-ffp-contract=off", "-I" + CSRC, "-I" + os.path.join(ROOT, "include")]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-pthread", "-I" + CSRC,
             "-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(CUDA_HOME, "include")]


def _headers():
    return glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        [os.path.join(ROOT, "include", "rmn.h")]


def _stale(obj, src, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(p) > t for p in [src] + deps)


def _compile(src, verbose_ptxas=False):
    base = os.path.splitext(os.path.basename(src))[0]
    obj = os.path.join(OUT, base + (".cu.o" if src.endswith(".cu") else ".o"))
    if not _stale(obj, src, _headers()):
        return obj, None
    if src.endswith(".cu"):
        cmd = [NVCC] + ARCH + NVCC_FLAGS + (["-Xptxas", "-v"] if verbose_ptxas else []) + ["-c", src, "-o", obj]
    else:
        cmd = ["g++"] + CXX_FLAGS + ["-c", src, "-o", obj]
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{p.stdout}\n{p.stderr}")
    return obj, p.stderr if verbose_ptxas else None


def build(verbose_ptxas: bool = False, jobs: int | None = None) -> str:
    os.makedirs(OUT, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))
    with cf.ThreadPoolExecutor(jobs or min(8, len(srcs))) as ex:
        results = list(ex.map(lambda s: _compile(s, verbose_ptxas), srcs))
    objs = [o for o, _ in results]
    if verbose_ptxas:
        for _, log in results:
            if log:
                sys.stderr.write(log)
    if not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        cmd = [NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-cudart", "shared", "-Xlinker",
                                                                 "-rpath=" + os.path.join(CUDA_HOME, "lib64")]
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{p.stdout}\n{p.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose_ptxas="-v" in sys.argv))
