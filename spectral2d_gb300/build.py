"""Build the sm_103a shared library ``libspectral2d_gb300.so`` in-tree.

Each translation unit is compiled by nvcc in parallel, then linked with
``nvcc -shared``.  Only one ``-gencode`` (``compute_103a`` / ``sm_103a``) is
emitted.  The result is loaded by :mod:`spectral2d_gb300._lib` through ctypes.

Usage: ``python -m spectral2d_gb300.build [--verbose]``.
"""

from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libspectral2d_gb300.so")
DRIVER = os.path.join(PKG, "spectral2d_run")

SOURCES = ["s2d_kernels.cu", "s2d_capi.cu", "s2d_ic.cpp", "s2d_ic_dev.cu", "s2d_noalloc.cu", "s2d_batch.cu",
           "s2d_closure.cu", "s2d_io.cu", "s2d_slab.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
          "-Xcompiler", "-fvisibility=hidden", "-I", os.path.join(ROOT, "include"),
          "-I", CSRC]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd, verbose):
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if p.returncode != 0:
        raise RuntimeError(f"command failed ({p.returncode}): {' '.join(cmd)}\n{p.stdout}")
    if verbose and p.stdout:
        print(p.stdout, file=sys.stderr)
    return p.stdout


def build(verbose: bool = False, ptxas_info: bool = False) -> str:
    """Compile every source and link the library; returns its path."""
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    extra = ["-Xptxas", "-v"] if ptxas_info else []
    jobs = []
    for src in SOURCES:
        path = os.path.join(CSRC, src)
        obj = os.path.join(BUILD, src + ".o")
        cmd = [nvcc, *ARCH, *COMMON, *extra, "-c", path, "-o", obj]
        if src.endswith(".cpp"):
            cmd = [nvcc, *COMMON, "-x", "c++", "-c", path, "-o", obj]
        jobs.append((cmd, obj))
    with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        outs = list(ex.map(lambda j: _run(j[0], verbose or ptxas_info), jobs))
    if ptxas_info:
        for o in outs:
            print(o, file=sys.stderr)
    tmp = LIB + ".tmp"
    _run([nvcc, *ARCH, "-shared", "-o", tmp, *[o for _, o in jobs]], verbose)
    os.replace(tmp, LIB)
    # the main program (src/Spectral2D.F90) linked against the library
    tmp = DRIVER + ".tmp"
    _run(["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"),
          os.path.join(CSRC, "s2d_driver.cpp"), "-o", tmp, "-L", PKG, "-lspectral2d_gb300",
          "-Wl,-rpath,$ORIGIN"], verbose)
    os.replace(tmp, DRIVER)
    return LIB


if __name__ == "__main__":
    print(build(verbose="--verbose" in sys.argv, ptxas_info="--ptxas" in sys.argv))
