"""Pins the oracle's gradient definition (the reference has none: grad4_1shot
is declared at header.h:283 but never defined), for the reference's 4th
order and for the 8th-order extension (which the reference lacks, so these
tests are its only pin):

* transpose test of one CPML operator step with its psi memory, over several
  steps: <L x, y> == <x, L^T y> in FP64;
* adjoint of the whole time stepping: <F w, r> == <w, F^T r> where F maps the
  source wavelet to the seismogram;
* central finite differences of the L2 misfit along random perturbations;
* FP32 twin against FP64 twin (<= 1e-4 relative error, the FP32 gradient tolerance).
"""
import numpy as np
import pytest

from conftest import ricker


ORDERS = [(1, 4), (0, 4), (1, 8), (0, 8)]


def small_cfg(O, fs, nt=401, jump=2, order=4):
    return O.make_config(nx=40, nz=36, npml=8, nt=nt, dx=10.0, dz=10.0, dt=0.001, free_surface=fs, jump=jump,
                         fd_order=order)


def geometry(O, fs, wav):
    irx = np.arange(1, 39, 2)
    irz = np.full_like(irx, 0 if fs else 3)
    irz[::3] = 5
    return O.Shot(17, 2, irx, irz, wav)


@pytest.mark.parametrize("fs,order", ORDERS)
def test_operator_transpose(oracles, fs, order):
    O, _, o64 = oracles
    cfg = small_cfg(O, fs, order=order)
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


@pytest.mark.parametrize("fs,order", ORDERS)
def test_time_stepping_adjoint(oracles, fs, order):
    O, _, o64 = oracles
    cfg = small_cfg(O, fs, nt=121, order=order)
    rng = np.random.default_rng(21 + fs)
    vel = rng.uniform(1500, 3000, (cfg.nz, cfg.nx)).astype(np.float32)
    sh = geometry(O, fs, rng.standard_normal(cfg.nt).astype(np.float32))
    syn = o64.forward(cfg, vel, sh)
    res = rng.standard_normal(syn.shape)
    wb = o64.adjoint_wavelet(cfg, vel, sh, res)
    lhs, rhs = (syn * res).sum(), (sh.wav.astype(np.float64) * wb).sum()
    assert abs(lhs - rhs) <= 1e-12 * abs(lhs)


@pytest.mark.parametrize("fs,order", ORDERS)
def test_gradient_finite_differences(oracles, fs, order):
    O, o32, o64 = oracles
    cfg = small_cfg(O, fs, order=order)
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
    # the FP32 twin stays within 1e-4 (the FP32 gradient tolerance) of the FP64 twin
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


@pytest.mark.parametrize("fs,order", ORDERS)
def test_rebuild_reproduces_forward(oracles, fs, order):
    """The strip-based rebuild (interior operator + 2M-1 strips) retraces the
    forward field: the interior operator equals the padded one there."""
    O, _, o64 = oracles
    cfg = small_cfg(O, fs, nt=161, order=order)
    rng = np.random.default_rng(51 + fs + order)
    vel = rng.uniform(1500, 3000, (cfg.nz, cfg.nx)).astype(np.float32)
    sh = geometry(O, fs, ricker(cfg.nt, cfg.dt, 15.0))
    steps = [150, 90, 40, 5]
    fwd, reb = o64.probe(cfg, vel, sh, steps)
    _, _, x0, z0 = o64.grid(cfg)
    for k in range(len(steps)):
        f = fwd[k][z0:z0 + cfg.nz, x0:x0 + cfg.nx]
        assert np.abs(reb[k] - f).max() <= 1e-9 * np.abs(f).max(), (order, steps[k])


def test_eighth_order_is_more_accurate(oracles):
    """On a smooth field the 8th-order interior operator's error against the
    analytic Laplacian is far below the 4th-order pair's."""
    O, _, o64 = oracles
    errs = {}
    for order in (4, 8):
        cfg = small_cfg(O, 1, order=order)
        z, x = np.mgrid[0:cfg.nz, 0:cfg.nx] * 10.0
        k = 2 * np.pi / 120.0
        p = np.sin(k * x) * np.cos(0.7 * k * z)
        ux, vz = o64.apply_int(cfg, p)
        lap = -(k ** 2 + (0.7 * k) ** 2) * p
        c = (slice(8, cfg.nz - 8), slice(8, cfg.nx - 8))
        errs[order] = np.abs((ux + vz)[c] - lap[c]).max() / np.abs(lap[c]).max()
    assert errs[8] < 0.05 * errs[4], errs
