"""One gradient through the CPU emulation build of the engine, checked
against the FP64 oracle; run by test_emu_sanitized.py in a child process
with AddressSanitizer and UBSan preloaded and FWI_LIB pointing at
libfwiemu.so.  Prints one JSON line {J, J64, grad_rel, syn_rel}."""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
for p in (HERE, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "fwi2dacoustic-mpi-lbfgs_gb300")):
    sys.path.insert(0, p)

import oracle as O                         # noqa: E402
from test_gpu_parity import Case, rel      # noqa: E402


def main(fs, nt, nx=150, nz=90):
    o64 = O.Oracle("f64")
    case = Case(O, fs, seed=11 + fs, nt=nt, nx=nx, nz=nz)
    case.vtrue = (case.vel * 1.08).astype(np.float32)    # signal in the direct waves of a short record
    obs = case.oracle_obs(o64)
    e = case.engine()
    e.set_model(case.vel)
    syn = e.split(e.forward())
    syn_rel = max(rel(got, o64.forward(case.oracle_cfg_for(len(s.wav)), case.vel, s))
                  for s, got in zip(case.oshots, syn))
    e.set_observed(np.concatenate([o.ravel() for o in obs]))
    J, g = e.gradient()
    J64, g64 = 0.0, np.zeros_like(g)
    for s, ob in zip(case.oshots, obs):
        j, gg, _ = o64.gradient(case.oracle_cfg_for(len(s.wav)), case.vel, [s], [ob])
        J64 += j
        g64 += gg
    print(json.dumps({"J": J, "J64": J64, "grad_rel": rel(g, g64), "syn_rel": syn_rel}))


if __name__ == "__main__":
    main(*[int(a) for a in sys.argv[1:]])
