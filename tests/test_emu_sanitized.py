"""Memory safety of the CUDA kernels without a GPU.

The engine's own .cu source is compiled as C++ against csrc/cpu_emu.h
(every CUDA block runs on host threads, every device buffer is an exact-size
heap block, dynamic shared memory is exactly the launch's byte count) under
AddressSanitizer and UBSan.  One gradient per boundary condition then runs
through the C ABI of that build in a child process: any out-of-bounds access
in any kernel aborts it.  The results must also match the FP64 oracle to the
GPU parity tolerances, so the emulation runs the same arithmetic.

The children of all cases start together (the emulation spends most of its time
in barrier waits, so they share the host's cores well); each test waits for its
own.
"""
import json
import os
import shutil
import subprocess
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GRAD_TOL = 1e-4
SYN_TOL = 2e-5


def _sanitizer_libs():
    cxx = shutil.which(os.environ.get("CXX", "g++"))
    if not cxx:
        return None
    libs = []
    for name in ("libasan.so", "libubsan.so"):
        p = subprocess.run([cxx, f"-print-file-name={name}"], capture_output=True, text=True).stdout.strip()
        if not os.path.isabs(p) or not os.path.exists(p):
            return None
        libs.append(p)
    return libs


@pytest.fixture(scope="module")
def emu_lib():
    libs = _sanitizer_libs()
    if libs is None:
        pytest.skip("g++ with AddressSanitizer/UBSan runtimes not available")
    import build as B
    return B.build_emu(), libs


GRAD_CASES = [(1, 150, 90, 0, 0), (0, 130, 70, 0, 0), (1, 130, 70, 8, 4), (0, 150, 90, 32, 16),
              (1, 64, 44, 0, 0)]                     # the last: no interior tile
CASES = dict({f"grad-{fs}-{nx}-{nz}-{xs}-{zs}": ["emu_gradient_case.py", fs, 41, nx, nz, 0, 4, xs, zs]
              for fs, nx, nz, xs, zs in GRAD_CASES},
             checkpoints=["emu_gradient_case.py", 1, 41, 130, 70, 5],
             eighth=["emu_gradient_case.py", 0, 41, 130, 70, 5, 8],
             aux=["emu_aux_case.py"])


@pytest.fixture(scope="module")
def emu_runs(emu_lib, oracles):
    """Starts every case's child process; yields {case: Popen}.  Children still
    running when the module ends (after a failure) are killed."""
    lib, libs = emu_lib
    env = dict(os.environ, FWI_LIB=lib, LD_PRELOAD=" ".join(libs),
               ASAN_OPTIONS="detect_leaks=0:abort_on_error=1", UBSAN_OPTIONS="halt_on_error=1:print_stacktrace=1")
    procs = {name: subprocess.Popen([sys.executable, os.path.join(HERE, argv[0])] + [str(a) for a in argv[1:]],
                                    stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True, env=env)
             for name, argv in CASES.items()}
    yield procs
    for p in procs.values():
        if p.poll() is None:
            p.kill()
            p.wait()


def finish(procs, name, timeout=1500):
    """The case's exit status checked for sanitizer reports; its last stdout line."""
    out, err = procs[name].communicate(timeout=timeout)
    assert procs[name].returncode == 0, out[-2000:] + err[-6000:]
    assert "ERROR: AddressSanitizer" not in err and "runtime error" not in err, err[-6000:]
    return out.strip().splitlines()[-1]


# (free surface, nx, nz): 150 x 90 has full-width edge tiles; 130 x 70 leaves a
# last tile column under half a tile wide and a last tile row of a few rows,
# which exercises the skipped padding halves and rows.
# The last two cases also lay the tile grid elsewhere (fwi_tuning x_first /
# z_first shifted) with the other kernel variants, class order and serial launches.
@pytest.mark.parametrize("fs,nx,nz,xs,zs", GRAD_CASES)
def test_emulated_gradient_is_memory_safe_and_matches_oracle(emu_runs, fs, nx, nz, xs, zs):
    out = json.loads(finish(emu_runs, f"grad-{fs}-{nx}-{nz}-{xs}-{zs}"))
    assert out["syn_rel"] <= SYN_TOL, out
    assert abs(out["J"] - out["J64"]) <= 1e-5 * out["J64"], out
    assert out["grad_rel"] <= GRAD_TOL and out["obs_call_same"], out


def test_emulated_checkpointing_is_memory_safe(emu_runs):
    """The checkpointed backward (5 segments of 9 steps over records of 41,
    1 and 19 steps: restores, strip extraction, recompute, segments that
    shots end in): memory safe; FP32 checkpoints within the gradient
    tolerance of FP64 and within FP32 rounding of the strip ring's gradient
    (the rebuild restarts from recomputed fields at every segment, so the
    two differ in rounding only); FP16 checkpoints within 1e-3 of FP64 on
    this short record (BF16 and the full-size errors are measured on the
    GPU)."""
    out = json.loads(finish(emu_runs, "checkpoints"))
    assert out["grad_rel"] <= GRAD_TOL, out
    assert out["snap_f32_rel"] <= GRAD_TOL and out["snap_f32_vs_strips"] <= 1e-5, out
    assert out["snap_f16_rel"] <= 1e-3, out


def test_emulated_eighth_order_is_memory_safe(emu_runs):
    """The 8th-order kernels (fwi_kernels8.cuh) with CPML on all four sides,
    strips of 7 and the checkpointed backward in 5 segments: memory safe,
    seismograms and gradient within the parity tolerances of the 8th-order
    FP64 oracle, FP32 checkpoints within rounding of the strip ring."""
    out = json.loads(finish(emu_runs, "eighth"))
    assert out["syn_rel"] <= SYN_TOL and abs(out["J"] - out["J64"]) <= 1e-5 * out["J64"], out
    assert out["grad_rel"] <= GRAD_TOL and out["snap_f32_rel"] <= GRAD_TOL, out
    assert out["snap_f32_vs_strips"] <= 1e-5 and out["snap_f16_rel"] <= 1e-3, out


def test_emulated_aux_routines_are_memory_safe_and_match_oracle(emu_runs):
    """fwi_grad_precond / fwi_bandpass bit-identical to the oracle, fwi_xcorr1d
    and the XCORR gradient within tolerance (tests/aux_cases.py)."""
    assert finish(emu_runs, "aux") == "ok"

