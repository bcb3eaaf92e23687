"""Build recipe of the engine library ``libfwigpu.so`` (sm_103a only).

    python fwi2dacoustic-mpi-lbfgs_gb300/build.py [--force]

Compiles ``csrc/fwi_engine.cu`` (which includes ``csrc/fwi_kernels.cuh``) with
nvcc for ``-gencode arch=compute_103a,code=sm_103a`` into
``libfwigpu.so`` next to this file.  The CUDA runtime is linked statically so
the library only needs the driver at run time.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
LIB = os.path.join(PKG, "libfwigpu.so")
SOURCES = [os.path.join(PKG, "csrc", "fwi_engine.cu")]
DEPS = SOURCES + [os.path.join(PKG, "csrc", "fwi_kernels.cuh"), os.path.join(ROOT, "include", "fwi_gb300.h")]
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.isfile(cand):
            return cand
    raise RuntimeError("nvcc not found: the engine needs the CUDA toolkit to build")


def stale() -> bool:
    if not os.path.isfile(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(d) > t for d in DEPS)


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and not stale():
        return LIB
    tmp = LIB + ".tmp"
    cmd = [nvcc(), ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-shared",
           "-I", os.path.join(ROOT, "include"), "-o", tmp] + SOURCES
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed:\n" + r.stdout + r.stderr)
    if verbose:
        sys.stderr.write(r.stderr)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
