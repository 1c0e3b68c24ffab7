"""Compile libnmaggpu.so in-tree for sm_103a (nvcc, no CMake).

Each .cu file is compiled to an object in parallel; the setup kernels
(mesh_kernels.cu, bem_kernels.cu) use --fmad=false so their arithmetic follows
the written operation order exactly.  The CUDA runtime is linked statically.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(ROOT, "csrc")
BUILD = os.path.join(ROOT, "_build")
LIB = os.path.join(PKG, "libnmaggpu.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-fno-strict-aliasing",
          "--expt-relaxed-constexpr"]
NO_FMA = {"mesh_kernels.cu", "bem_kernels.cu", "adjoint.cu"}
SOURCES = ["mesh_kernels.cu", "bem_kernels.cu", "rhs_kernels.cu", "nmg_ts.cu", "nmg_api.cu", "nmg_static.cu",
           "adjoint.cu", "batch.cu", "bem_tc.cu", "nmg_sites.cu"]


def nvcc():
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libnmaggpu.so")
    return p


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(os.path.join(ROOT, "..", "include", "nmag_gpu.h"))
    files.append(os.path.abspath(__file__))
    return files


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(f) <= t for f in _deps() if os.path.exists(f))


def _compile(src, extra=()):
    obj = os.path.join(BUILD, src.replace(".cu", ".o"))
    flags = list(COMMON) + (["--fmad=false"] if src in NO_FMA else []) + list(extra)
    cmd = [nvcc()] + ARCH + flags + ["-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr[-6000:]))
    return obj, r.stderr


def build(force=False, verbose=False, extra=()):
    """Build libnmaggpu.so next to this file; returns its path."""
    if not force and up_to_date():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(lambda s: _compile(s, extra), SOURCES))
    objs = [o for o, _ in results]
    if verbose:
        for _, log in results:
            if log.strip():
                print(log)
    tmp = LIB + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart_static", "-lrt", "-lpthread", "-ldl"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stderr[-4000:]))
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose=True,
                extra=["-Xptxas", "-v"] if "--ptxas" in sys.argv else ()))
