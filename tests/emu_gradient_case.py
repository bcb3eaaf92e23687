"""One gradient through the CPU emulation build of the engine, checked
against the FP64 oracle; run by test_emu_sanitized.py in a child process
with AddressSanitizer and UBSan preloaded and FWI_LIB pointing at
libfwiemu.so.  Arguments: free surface, nt, nx, nz [, nseg [, fd_order [,
x shift, z shift of the tile grid (fwi_tuning)]]].
Prints one JSON line {J, J64, grad_rel, syn_rel, obs_call_same} (the last:
fwi_gradient_obs returns fwi_gradient's result bit for bit).  With nseg > 0
the same gradient is also taken with checkpoints (FWI_STORE_SNAPSHOTS, nseg
segments) in FP32 and FP16 storage (BF16 shares
the FP16 path but for its rounding) and the line adds {snap_f32_rel,
snap_f16_rel} (against FP64) and snap_f32_vs_strips."""
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


def main(fs, nt, nx=150, nz=90, nseg=0, order=4, xshift=0, zshift=0):
    o64 = O.Oracle("f64")
    case = Case(O, fs, seed=11 + fs, nt=nt, nx=nx, nz=nz, order=order)
    case.vtrue = (case.vel * 1.08).astype(np.float32)    # signal in the direct waves of a short record
    obs = case.oracle_obs(o64)
    e = case.engine()
    if xshift or zshift:                 # another tile grid (fwi_tuning x_first / z_first)
        t = e.tuning()
        e.set_tuning({"x_first": t["x_first"] + xshift, "z_first": t["z_first"] + zshift,
                      "fwd_gen_blocks": 3, "bwd_int_blocks": 3, "class_order": 2, "serial": 1, "gen_grid": 3,
                      "bwd_zgen_blocks": 3})
        e.set_shots(case.eshots)
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
    flat = np.concatenate([o.ravel() for o in obs])
    J2, g2 = e.gradient(observed=flat.copy())            # fwi_gradient_obs: the same gradient
    out = {"J": J, "J64": J64, "grad_rel": rel(g, g64), "syn_rel": syn_rel,
           "obs_call_same": bool(J2 == J and np.array_equal(g2, g))}
    if nseg:
        import fwigpu
        for prec in ("f32", "f16"):
            c = case.ecfg
            cfg = fwigpu.make_config(c.nx, c.nz, c.dx, c.dz, c.dt, c.nt_max, npml=c.npml,
                                     free_surface=c.free_surface, jump=c.jump, store=fwigpu.STORE_SNAPSHOTS,
                                     snapshots=nseg, snap_precision=prec, fd_order=c.fd_order)
            with fwigpu.Engine(cfg) as es:
                es.set_shots(case.eshots)
                es.set_model(case.vel)
                es.set_observed(flat)
                Js, gs = es.gradient()
                st = es.stats()
            assert st["store"] == fwigpu.STORE_SNAPSHOTS and st["segments"] == nseg, st
            out[f"snap_{prec}_rel"] = rel(gs, g64)
            if prec == "f32":
                out["snap_f32_vs_strips"] = rel(gs, g)
    print(json.dumps(out))


if __name__ == "__main__":
    main(*[int(a) for a in sys.argv[1:]])
