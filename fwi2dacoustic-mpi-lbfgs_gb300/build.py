"""Build recipe of the engine library ``libfwigpu.so`` (sm_103a only).

    python fwi2dacoustic-mpi-lbfgs_gb300/build.py [--force]

Compiles, in parallel, ``csrc/fwi_engine.cu`` (which includes
``csrc/fwi_kernels.cuh`` and ``csrc/fwi_kernels8.cuh``) and
``csrc/fwi_aux.cu`` (``csrc/fwi_aux.cuh``) and ``csrc/fwi_lbfgs.cu`` with
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
SOURCES = [os.path.join(PKG, "csrc", n) for n in ("fwi_engine.cu", "fwi_aux.cu", "fwi_lbfgs.cu")]
DEPS = SOURCES + [os.path.join(PKG, "csrc", n) for n in ("fwi_kernels.cuh", "fwi_kernels8.cuh", "fwi_aux.cuh",
                                                       "fwi_aux_kernels.cuh", "cpu_emu.h")] + \
    [os.path.join(ROOT, "include", "fwi_gb300.h")]
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


def build(force: bool = False, verbose: bool = False, defines=(), out: str | None = None) -> str:
    """Compiles the three translation units in parallel, then links them.

    defines (e.g. ("FWI_TIMELINE",)) and out build a diagnostics variant into
    its own library and object directory; the product library is LIB."""
    lib = out or LIB
    if not force and not defines and not stale():
        return LIB
    tmp = lib + ".tmp"
    flags = [ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", os.path.join(ROOT, "include")]
    flags += ["-D" + d for d in defines]
    # FWI_NVCC_EXTRA adds diagnostics flags, e.g. -DFWI_SELF_CHECK
    flags = os.environ.get("FWI_NVCC_EXTRA", "").split() + flags
    if verbose:
        flags.append("-Xptxas=-v")
    objdir = os.path.join(PKG, "_build", *(["variant_" + "_".join(d.lower() for d in defines)] if defines else []))
    os.makedirs(objdir, exist_ok=True)
    objs = [os.path.join(objdir, os.path.basename(src)[:-3] + ".o") for src in SOURCES]
    procs = [subprocess.Popen([nvcc()] + flags + ["-c", src, "-o", obj], stdout=subprocess.PIPE,
                              stderr=subprocess.PIPE, text=True) for src, obj in zip(SOURCES, objs)]
    errors = ""
    for p in procs:
        so, se = p.communicate()
        if verbose:
            sys.stderr.write(se)
        if p.returncode != 0:
            errors += so + se
    if errors:
        raise RuntimeError("nvcc failed:\n" + errors)
    r = subprocess.run([nvcc(), ARCH, "-shared", "-o", tmp] + objs, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc link failed:\n" + r.stdout + r.stderr)
    os.replace(tmp, lib)
    return lib


EMU_LIB = os.path.join(PKG, "libfwiemu.so")


def build_emu(force: bool = False, sanitize: bool = True) -> str:
    """CPU emulation build of the same sources (csrc/cpu_emu.h) for memory-
    safety checks without a GPU: every kernel runs on host threads, every
    device buffer is an exact-size heap block, AddressSanitizer on."""
    if not force and os.path.isfile(EMU_LIB) and all(os.path.getmtime(d) <= os.path.getmtime(EMU_LIB)
                                                     for d in DEPS + [os.path.join(PKG, "csrc", "cpu_emu.h")]):
        return EMU_LIB
    cxx = os.environ.get("CXX", "g++")
    cmd = [cxx, "-x", "c++", "-std=c++20", "-O1", "-g", "-fPIC", "-shared", "-DFWI_CPU_EMU",
           "-Wno-unknown-pragmas", "-I", os.path.join(ROOT, "include"), "-o", EMU_LIB + ".tmp"] + SOURCES + ["-lpthread"]
    if sanitize:
        cmd[1:1] = ["-fsanitize=address,undefined", "-fno-sanitize-recover=undefined", "-fno-omit-frame-pointer"]
    cmd[1:1] = os.environ.get("FWI_EMU_EXTRA", "").split()     # e.g. -DFWI_SELF_CHECK
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("emulation build failed:\n" + r.stdout + r.stderr)
    os.replace(EMU_LIB + ".tmp", EMU_LIB)
    return EMU_LIB


if __name__ == "__main__":
    if "--emu" in sys.argv:
        print(build_emu(force="--force" in sys.argv))
    else:
        print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
