"""Build libhssgpu.so in-tree with nvcc for sm_103a (GB300).

Each translation unit is compiled in parallel, then linked into
``hssc_directsolver_gb300/libhssgpu.so``.  Host code is compiled with
``-ffp-contract=off`` so that the host-side geometry rounds identically on
x86-64 and aarch64.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "libhssgpu.so")
BUILD = os.path.join(HERE, "_build")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["dense.cu", "skinny_tc.cu", "kgen.cu", "hss2d.cu", "hss1d.cu", "hss1d_algebra.cu", "capi.cu", "noalloc.cu", "mlp.cu", "hss2d_lowrank.cu", "krylov.cu", "hss2d_tree.cpp", "drweights.cpp"]


def nvcc() -> str:
    for c in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _flags():
    return ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
            "--expt-relaxed-constexpr", "-diag-suppress", "177"]


def _compile(src: str) -> str:
    obj = os.path.join(BUILD, src + ".o")
    path = os.path.join(CSRC, src)
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(
            os.path.getmtime(os.path.join(CSRC, f)) for f in os.listdir(CSRC)) and \
            os.path.getmtime(obj) >= os.path.getmtime(os.path.join(HERE, "..", "include", "hssgpu.h")):
        return obj
    cmd = [nvcc(), *ARCH, *_flags(), "-c", path, "-o", obj]
    if src.endswith(".cpp"):
        cmd = [nvcc(), *_flags(), "-x", "c++", "-c", path, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=min(len(SOURCES), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(_compile, SOURCES))
    cmd = [nvcc(), *ARCH, "-shared", "-o", OUT + ".tmp", *objs, "-lcudart", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(OUT + ".tmp", OUT)
    if verbose:
        print(f"built {OUT}")
    return OUT


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
