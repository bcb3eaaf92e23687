"""Generate the golden fixtures from the reference's OWN kernels.

Run where the reference's sources are at hand: the checkout named by
``make -C oracle stage REF_CHECKOUT=<checkout>`` (which copies them, git-ignored,
into ``oracle/_ref/src``) is compiled by ``make -C oracle ref`` into
``oracle/_ref/libfwiref.so``:

    python tests/golden/make_golden.py [--aux]

Writes ``tests/golden/ref_kernels.npz``: outputs of cpml_coe, model_ext,
model_ext_fs_no, a_lap_opt_2d_pml (one step, with psi), a_lap_opt_2d,
write_bdr / write_bdr_fs_no, and a full forward + boundary-strip rebuild
(a_lap_opt_2d_pml + time_integral forward, read_bdr + a_lap_opt_2d +
time_integral backward, chunked through a temporary file) on a small free-surface
case, and ``tests/golden/ref_aux.npz``: outputs of grad_precond_new5,
sfbandpass, XCORR1D and of MBotOpt.c's L-BFGS run on the objective of
oracle/lbfgs_objective.h (``--aux`` writes only this file).  The inputs are
regenerated from the seeds stored alongside.
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


# (perc, rectx1, repeat1, rectx2, repeat2, alpha_grad) of the preconditioning cases
PRECOND_CASES = [(0.9, 5, 2, 3, 1, 1.5), (0.0, 1, 1, 7, 3, 2.0), (0.5, 11, 1, 2, 2, 0.3)]
# (dt, phase, nphi, nplo, fhi, flo) of the band-pass cases: zero-phase and
# minimum-phase, odd and even orders, low-cut only, high-cut only
BANDPASS_CASES = [(0.002, 0, 6, 6, 30.0, 3.0), (0.001, 1, 5, 3, 60.0, 5.0), (0.004, 0, 4, 4, 40.0, 0.0),
                  (0.004, 1, 1, 2, 200.0, 10.0)]
# (mode, offset min, offset max, traces) of the XCORR cases; mode 0 "middle",
# 1 "leading"; traces "pulse" (wavelets with lags of both signs) or "noise"
# (broadband traces that correlate at every lag: in "leading" mode the kept
# residual window holds no correlation peak of pulse-like traces)
XCORR_CASES = [(0, 50.0, 550.0, "pulse"), (1, 0.0, 1.0e9, "noise"), (0, 0.0, 1.0e9, "noise")]


LBFGS_SAMPLE = 997               # the L-BFGS fixture keeps every 997th entry of the final model


def aux_inputs():
    """Deterministic inputs of the preconditioning, band-pass and XCORR cases."""
    rng = np.random.default_rng(SEED + 7)
    grad = rng.standard_normal((37, 53)).astype(np.float32)
    bottom = rng.integers(0, 6, 53).astype(np.int32)
    traces = rng.standard_normal((9, 400)).astype(np.float32)
    nt, nr = 121, 7
    t = np.arange(nt)
    # obs and syn wavelets with lags of both signs, one trace 20x weaker
    # (skipped by the energy test) and offsets 0..600 m (two outside [50, 550])
    obs = np.stack([np.exp(-((t - 60 - 3 * i) / 6.0) ** 2) * np.cos(0.3 * (t - 60)) for i in range(nr)])
    syn = np.stack([1.2 * np.exp(-((t - 60 + 4 * (i - 3)) / 6.0) ** 2) * np.cos(0.3 * (t - 57)) for i in range(nr)])
    syn[5] *= 0.04
    obs, syn = obs.astype(np.float32), syn.astype(np.float32)
    sr = np.array([0.0, 0.0] + sum([[100.0 * i, 2.0] for i in range(nr)], []), np.float32)
    return grad, bottom, traces, obs, syn, sr


def xcorr_traces(kind):
    """(obs, syn, sr_xyz) of an XCORR case."""
    *_, obs, syn, sr = aux_inputs()
    if kind == "noise":
        rng = np.random.default_rng(SEED + 8)
        obs = rng.standard_normal(obs.shape).astype(np.float32)
        syn = (np.roll(obs, 2, axis=1) + 0.3 * rng.standard_normal(obs.shape)).astype(np.float32)
    return obs, syn, sr


def main_aux() -> None:
    if not O.RefAux.available():
        raise SystemExit("reference routines not built")
    ref = O.RefAux()
    grad, bottom, traces, obs, syn, sr = aux_inputs()
    out = {}
    for k, c in enumerate(PRECOND_CASES):
        out[f"precond_{k}"] = ref.grad_precond(grad, *c, bottom)
    for k, c in enumerate(BANDPASS_CASES):
        out[f"bandpass_{k}"] = ref.bandpass(traces, *c)
    for k, (mode, omin, omax, kind) in enumerate(XCORR_CASES):
        o, sy, s_r = xcorr_traces(kind)
        out[f"xcorr_mis_{k}"], out[f"xcorr_res_{k}"] = ref.xcorr1d(o, sy, s_r, omin, omax, mode, npad=5)
    # the reference's own MBotOpt.c on the objective of oracle/lbfgs_objective.h
    import tempfile
    with tempfile.TemporaryDirectory() as td:
        ftrace, x = O.run_reference_mbotopt(td)
    out["lbfgs_ftrace"] = ftrace.astype(np.float32)
    out["lbfgs_x_sample"] = x[::LBFGS_SAMPLE]
    out["lbfgs_x_sum"] = np.array([x.astype(np.float64).sum()])
    path = os.path.join(HERE, "ref_aux.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes")


def main() -> None:
    O.build(quiet=False)
    if not O.RefKernels.available():
        raise SystemExit("the reference's kernels are not built: stage the reference sources first "
                         "(make -C oracle stage REF_CHECKOUT=<checkout>)")
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


if __name__ == "__main__" and "--aux" in sys.argv:
    O.build(quiet=False)
    main_aux()
elif __name__ == "__main__":
    main()
