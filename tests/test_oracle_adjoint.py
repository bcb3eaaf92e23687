"""Pins the oracle's gradient definition (the reference has none: grad4_1shot
is declared at header.h:283 but never defined).

* transpose test of one CPML operator step with its psi memory, over several
  steps: <L x, y> == <x, L^T y> in FP64;
* adjoint of the whole time stepping: <F w, r> == <w, F^T r> where F maps the
  source wavelet to the seismogram;
* central finite differences of the L2 misfit along random perturbations;
* FP32 twin against FP64 twin (the benchmark spec's <= 1e-4 relative error).
"""
import numpy as np
import pytest

from conftest import ricker


def small_cfg(O, fs, nt=401, jump=2):
    return O.make_config(nx=40, nz=36, npml=8, nt=nt, dx=10.0, dz=10.0, dt=0.001, free_surface=fs, jump=jump)


def geometry(O, fs, wav):
    irx = np.arange(1, 39, 2)
    irz = np.full_like(irx, 0 if fs else 3)
    irz[::3] = 5
    return O.Shot(17, 2, irx, irz, wav)


@pytest.mark.parametrize("fs", [1, 0])
def test_operator_transpose(oracles, fs):
    O, _, o64 = oracles
    cfg = small_cfg(O, fs)
    pnx, pnz, _, _ = o64.grid(cfg)
    rng = np.random.default_rng(11 + fs)
    n = o64.psi_len(cfg)
    ps = [rng.standard_normal((pnz, pnx)) for _ in range(4)]
    qs = [rng.standard_normal((pnz, pnx)) for _ in range(4)]
    psi, ws = np.zeros(n), []
    for p in ps:
        w, psi = o64.apply_op(cfg, p, psi)
        ws.append(w)
    psib, pbs = np.zeros(n), [None] * 4
    for k in (3, 2, 1, 0):
        pbs[k], psib = o64.apply_op_t(cfg, qs[k], psib)
    lhs = sum((w * q).sum() for w, q in zip(ws, qs))
    rhs = sum((p * pb).sum() for p, pb in zip(ps, pbs))
    assert abs(lhs - rhs) <= 1e-12 * abs(lhs)


@pytest.mark.parametrize("fs", [1, 0])
def test_time_stepping_adjoint(oracles, fs):
    O, _, o64 = oracles
    cfg = small_cfg(O, fs, nt=121)
    rng = np.random.default_rng(21 + fs)
    vel = rng.uniform(1500, 3000, (cfg.nz, cfg.nx)).astype(np.float32)
    sh = geometry(O, fs, rng.standard_normal(cfg.nt).astype(np.float32))
    syn = o64.forward(cfg, vel, sh)
    res = rng.standard_normal(syn.shape)
    wb = o64.adjoint_wavelet(cfg, vel, sh, res)
    lhs, rhs = (syn * res).sum(), (sh.wav.astype(np.float64) * wb).sum()
    assert abs(lhs - rhs) <= 1e-12 * abs(lhs)


@pytest.mark.parametrize("fs", [1, 0])
def test_gradient_finite_differences(oracles, fs):
    O, o32, o64 = oracles
    cfg = small_cfg(O, fs)
    rng = np.random.default_rng(31 + fs)
    vel = rng.uniform(1500, 3000, (cfg.nz, cfg.nx)).astype(np.float32)
    vtrue = vel.copy()
    vtrue[8:16, 10:30] += 300.0
    sh = geometry(O, fs, ricker(cfg.nt, cfg.dt, 15.0))
    obs = o64.forward(cfg, vtrue, sh).astype(np.float32)
    J0, g, _ = o64.gradient(cfg, vel, [sh], [obs])
    assert J0 > 0
    # perturbations vanish on the outermost cells that model_ext copies into the CPML
    dv = np.zeros_like(vel)
    dv[1:-1, 1:-1] = rng.standard_normal((cfg.nz - 2, cfg.nx - 2))
    if fs:
        dv[0, 1:-1] = rng.standard_normal(cfg.nx - 2)
    for eps in (1.0, 0.1):
        vp = (vel + eps * dv).astype(np.float32)
        vm = (vel - eps * dv).astype(np.float32)
        jp, _, _ = o64.gradient(cfg, vp, [sh], [obs])
        jm, _, _ = o64.gradient(cfg, vm, [sh], [obs])
        fd = jp - jm
        an = (g * (vp.astype(np.float64) - vm)).sum()
        # limited by the FP32 rounding of K = v^2 dt^2 (about 6e-8 relative)
        assert abs(fd - an) <= 5e-4 * abs(an), (eps, fd, an)
    # the FP32 twin stays within the benchmark spec's 1e-4 of the FP64 twin
    J32, g32, _ = o32.gradient(cfg, vel, [sh], [obs])
    assert abs(J32 - J0) <= 1e-5 * J0
    assert np.linalg.norm(g32 - g) <= 1e-4 * np.linalg.norm(g)


def test_multi_shot_gradient_is_sum(oracles):
    O, _, o64 = oracles
    cfg = small_cfg(O, 1, nt=201)
    rng = np.random.default_rng(41)
    vel = rng.uniform(1500, 3000, (cfg.nz, cfg.nx)).astype(np.float32)
    shots = [geometry(O, 1, ricker(cfg.nt, cfg.dt, 12.0)),
             O.Shot(30, 1, np.arange(0, 40, 5), np.zeros(8, np.int32), ricker(cfg.nt, cfg.dt, 9.0))]
    obs = [np.zeros((s.nr, o64.nt0(cfg)), np.float32) for s in shots]
    J, g, _ = o64.gradient(cfg, vel, shots, obs)
    parts = [o64.gradient(cfg, vel, [s], [o]) for s, o in zip(shots, obs)]
    assert abs(J - sum(p[0] for p in parts)) <= 1e-12 * J
    assert np.allclose(g, parts[0][1] + parts[1][1], rtol=1e-12, atol=1e-30 + 1e-12 * np.abs(g).max())
