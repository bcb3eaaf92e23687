"""Generate the golden fixtures from the reference's OWN kernels.

Run where the reference checkout is available (it is compiled by
``make -C oracle ref REF=<checkout>`` into ``oracle/_ref/libfwiref.so``):

    python tests/golden/make_golden.py [<reference checkout>]

Writes ``tests/golden/ref_kernels.npz``: outputs of cpml_coe, model_ext,
model_ext_fs_no, a_lap_opt_2d_pml (one step, with psi), a_lap_opt_2d,
write_bdr / write_bdr_fs_no, and a full forward + boundary-strip rebuild
(a_lap_opt_2d_pml + time_integral forward, read_bdr + a_lap_opt_2d +
time_integral backward, chunked through a temporary file) on a small free-surface
case.  The inputs are regenerated from the seeds stored alongside.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import oracle as O  # noqa: E402

SEED = 20241203


def case_inputs():
    """Deterministic inputs shared by the generator and the tests."""
    rng = np.random.default_rng(SEED)
    cfg = dict(nx=48, nz=40, npml=8, nt=241, dx=10.0, dz=10.0, dt=0.001, jump=2)
    vel = rng.uniform(1500.0, 3000.0, (cfg["nz"], cfg["nx"])).astype(np.float32)
    t = np.arange(cfg["nt"]) * cfg["dt"]
    f0 = 15.0
    tt = t - 1.2 / f0
    wav = ((1 - 2 * (np.pi * f0 * tt) ** 2) * np.exp(-(np.pi * f0 * tt) ** 2)).astype(np.float32)
    irx = np.arange(2, 46, 3).astype(np.int32)
    irz = np.ones_like(irx)
    irz[::4] = 5
    shot = dict(isx=24, isz=2, irx=irx, irz=irz, wav=wav)
    pnx = cfg["nx"] + 2 * cfg["npml"]
    p_fs = rng.standard_normal((cfg["nz"] + cfg["npml"], pnx)).astype(np.float32)
    p_nofs = rng.standard_normal((cfg["nz"] + 2 * cfg["npml"], pnx)).astype(np.float32)
    p_int = rng.standard_normal((cfg["nz"], cfg["nx"])).astype(np.float32)
    model = rng.uniform(1500.0, 4500.0, (30, 40)).astype(np.float32)
    steps = np.array([1, 2, 3, 60, 120, 200, 238, 239], np.int32)
    return cfg, vel, shot, p_fs, p_nofs, p_int, model, steps


def main(ref_dir: str) -> None:
    O.build(ref_dir, quiet=False)
    if not O.RefKernels.available():
        raise SystemExit("reference kernels not built")
    ref = O.RefKernels()
    o32 = O.Oracle("f32")
    cfg, vel, shot, p_fs, p_nofs, p_int, model, steps = case_inputs()
    c1 = O.make_config(free_surface=1, **cfg)
    c0 = O.make_config(free_surface=0, **cfg)
    out = {}
    for npml, d, dt in [(8, 10.0, 0.001), (20, 12.5, 0.0008)]:
        a, b = ref.cpml_coe(npml, d, dt)
        out[f"cpml_a_{npml}"], out[f"cpml_b_{npml}"] = a, b
    out["ext_fs1"] = ref.model_ext(model, 40 + 16, 30 + 8, 1)
    out["ext_fs0"] = ref.model_ext(model, 40 + 16, 30 + 16, 0)
    rng = np.random.default_rng(SEED + 1)
    psi = rng.standard_normal(o32.psi_len(c1)).astype(np.float32)
    out["op_psi_in"] = psi
    out["op_w"], out["op_psi_out"] = ref.apply_op(c1, p_fs, psi)
    out["int_ux"], out["int_vz"] = ref.apply_int(c1, p_int)
    out["strips_ud_fs1"], out["strips_lr_fs1"] = ref.strips_write(c1, p_fs)
    out["strips_ud_fs0"], out["strips_lr_fs0"] = ref.strips_write(c0, p_nofs)
    sh = O.Shot(**shot)
    syn, pf, pp, fs, rs = ref.forward(c1, vel, sh, nt_mem=241, steps=steps)
    out.update(fwd_syn=syn, fwd_pfin=pf, fwd_pprev=pp, fwd_snaps=fs, reb_snaps=rs, steps=steps)
    path = os.path.join(HERE, "ref_kernels.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
