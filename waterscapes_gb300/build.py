"""Build libmpetgpu.so in-tree with nvcc for sm_103a (GB300).

Each translation unit is compiled in parallel, then linked into
``waterscapes_gb300/libmpetgpu.so``.  No cmake, no torch extension
machinery: the library is a plain C-ABI shared object loaded by ctypes.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libmpetgpu.so")
SOURCES = ["setup.cu", "assemble.cu", "elem_tc.cu", "facets.cu", "solve.cu", "api.cu", "noalloc.cu",
           "amg_device.cu", "amg_setup.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    p = shutil.which("nvcc")
    if p is None and os.path.exists("/usr/local/cuda/bin/nvcc"):
        p = "/usr/local/cuda/bin/nvcc"
    if p is None:
        raise RuntimeError("nvcc not found")
    return p


def _compile(src, extra=()):
    out = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    path = os.path.join(CSRC, src)
    deps = [path, os.path.join(CSRC, "mpet_internal.cuh"),
            os.path.join(HERE, "..", "include", "mpet_gpu.h")]
    if os.path.exists(out) and all(os.path.getmtime(out) >= os.path.getmtime(d) for d in deps):
        return out
    cmd = [nvcc(), "-std=c++17", "-O3", "-lineinfo", *ARCH, "-Xcompiler", "-fPIC,-fopenmp",
           "-c", path, "-o", out, *extra]
    if src.endswith(".cpp"):
        # no fused multiply-add contraction on the host (aarch64 compilers contract by
        # default): the host AMG set-up rounds like the device one
        cmd = [nvcc(), "-std=c++17", "-O3", "-x", "c++", "-Xcompiler", "-fPIC,-fopenmp,-ffp-contract=off",
               "-c", path, "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr))
    return out


def build(verbose=False, ptxas_info=False):
    os.makedirs(BUILD, exist_ok=True)
    extra = ["-Xptxas", "-v"] if ptxas_info else []
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), SOURCES))
    newest = max(os.path.getmtime(o) for o in objs)
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= newest:
        return LIB
    tmp = LIB + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-Xcompiler", "-fopenmp", "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    os.replace(tmp, LIB)
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True, ptxas_info="-v" in sys.argv)
