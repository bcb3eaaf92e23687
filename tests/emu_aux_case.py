"""The routines around the gradient through the CPU emulation build of the
engine, checked against the aux oracle (tests/aux_cases.py); run by
test_emu_sanitized.py in a child process with AddressSanitizer and UBSan
preloaded and FWI_LIB pointing at libfwiemu.so.  Prints "ok" at the end.
With --engine it also runs the XCORR gradient through the engine (minutes
under emulation; the GPU tests run it on every GPU run)."""
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
for p in (HERE, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "fwi2dacoustic-mpi-lbfgs_gb300")):
    sys.path.insert(0, p)

import aux_cases as A          # noqa: E402
import fwigpu                  # noqa: E402
import oracle as O             # noqa: E402
from test_gpu_parity import Case  # noqa: E402

aux = O.AuxOracle()
A.check_precond(fwigpu, aux)
A.check_bandpass(fwigpu, aux)
A.check_xcorr(fwigpu, aux)
A.check_lbfgs(fwigpu, O, 3000)
# a short record: receivers near the sources so that no trace is all zeros
# (XCORR1D divides by the trace's correlation energy, as the reference does)
from conftest import ricker  # noqa: E402
import numpy as np           # noqa: E402
near = [(40, 1, np.arange(30, 52, 2), np.zeros(11, int), ricker(61, 0.001, 40.0)),
        (85, 12, np.arange(76, 96, 3), np.full(7, 9), ricker(61, 0.001, 35.0))]
if "--engine" in sys.argv:
    case = Case(O, 1, seed=31, nt=61, nx=130, nz=70, shots=near)
    case.vtrue = (case.vel * 1.08).astype("float32")
    A.check_engine_xcorr(fwigpu, aux, case)
print("ok")
