"""Checks of the device routines around the gradient against the aux oracle,
shared by the GPU tests (test_gpu_aux.py) and the sanitized CPU emulation
of the same kernels (test_emu_sanitized.py via emu_aux_case.py).

* fwi_grad_precond and fwi_bandpass: bit-identical to the oracle (which is
  bit-identical to the reference's grad_precond_new5 and sfbandpass).
* fwi_xcorr1d: misfit to XCORR_MISFIT_RTOL, residual to XCORR_RES_RTOL
  (relative L2), skipped traces identical.
* fwi_gradient with the XCORR misfit: its misfit equals the oracle's XCORR1D
  of the engine's own seismograms, and its gradient equals fwi_backward
  driven by the oracle's XCORR residual, both to GRAD_RTOL.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

import make_golden as G  # noqa: E402

XCORR_MISFIT_RTOL = 1e-4      # FP32 correlation sums in a different order
XCORR_RES_RTOL = 1e-4
GRAD_RTOL = 1e-4


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def check_precond(fwigpu, aux, big=False):
    grad, bottom, *_ = G.aux_inputs()
    cases = [(grad, bottom, c) for c in G.PRECOND_CASES]
    if big:
        rng = np.random.default_rng(21)
        g2 = (rng.standard_normal((560, 1700)) * 1e-3).astype(np.float32)
        b2 = rng.integers(0, 40, 1700).astype(np.int32)
        cases.append((g2, b2, (0.95, 20, 3, 15, 2, 1.0)))
    for g, b, c in cases:
        got = fwigpu.grad_precond(g, *c, b)
        want = aux.grad_precond(g, *c, b)
        assert np.array_equal(got, want), (c, np.abs(got - want).max())


def check_bandpass(fwigpu, aux, big=False):
    _, _, traces, *_ = G.aux_inputs()
    cases = [(traces, c) for c in G.BANDPASS_CASES]
    if big:
        rng = np.random.default_rng(22)
        cases.append((rng.standard_normal((1700, 2001)).astype(np.float32), (0.002, 0, 6, 6, 10.0, 3.0)))
    for tr, c in cases:
        got = fwigpu.bandpass(tr, *c)
        want = aux.bandpass(tr, *c)
        assert np.array_equal(got, want), (c, np.abs(got - want).max())


def check_xcorr(fwigpu, aux):
    for mode, omin, omax, kind in G.XCORR_CASES:
        obs, syn, sr = G.xcorr_traces(kind)
        for nt in (obs.shape[1], obs.shape[1] - 1):
            m1, r1 = fwigpu.xcorr1d(obs[:, :nt], syn[:, :nt], sr, omin, omax, mode)
            m2, r2 = aux.xcorr1d(obs[:, :nt], syn[:, :nt], sr, omin, omax, mode)
            assert np.allclose(m1, m2, rtol=XCORR_MISFIT_RTOL, atol=0), (mode, kind, nt, m1, m2)
            assert rel(r1, r2) <= XCORR_RES_RTOL, (mode, kind, nt, rel(r1, r2))
            assert np.array_equal(np.all(r1 == 0, axis=1), np.all(r2 == 0, axis=1))


def check_engine_xcorr(fwigpu, aux, case):
    """case: a test_gpu_parity.Case; observed data from its true model."""
    e = case.engine()
    try:
        e.set_model(case.vtrue)
        obs = e.split(e.forward())
        e.set_model(case.vel)
        syn = e.split(e.forward())
        e.set_observed(np.concatenate([o.ravel() for o in obs]))
        for mode in (fwigpu.XCORR_MIDDLE, fwigpu.XCORR_LEADING):
            e.set_misfit(fwigpu.MISFIT_XCORR, mode, 0.0, 1.0e9)
            J, g = e.gradient()
            mis, res = [], []
            for sh, o, s in zip(case.eshots, obs, syn):
                sr = np.concatenate([[sh.src_x, sh.src_z], np.asarray(sh.rec_xz, np.float64).ravel()]).astype(np.float32)
                m, r = aux.xcorr1d(o, s, sr, 0.0, 1.0e9, mode)
                mis.append(m)
                res.append(r)
            J_want = float(sum(float(m[1]) for m in mis))
            assert abs(J - J_want) <= XCORR_MISFIT_RTOL * abs(J_want), (mode, J, J_want)
            e.forward()                      # the gradient's backward pass consumed the forward state
            g_want = e.backward(np.concatenate([r.ravel() for r in res]))
            assert rel(g, g_want) <= GRAD_RTOL, (mode, rel(g, g_want))
        e.set_misfit(fwigpu.MISFIT_L2)
        J2, _ = e.gradient()
        want = 0.5 * sum(float(((s.astype(np.float64) - o) ** 2).sum()) for s, o in zip(syn, obs))
        assert abs(J2 - want) <= 1e-5 * want
    finally:
        e.close()


LBFGS_RTOL = 1e-9    # FP64 both sides; only the order of the dot-product sums differs


def check_lbfgs(fwigpu, O, n, **param):
    """The device optimizer, fed by the FP64 oracle's objective, takes the
    same trial points, objective values and termination as orc_lbfgs_run."""
    o64 = O.LbfgsOracle("f64")
    p = dict(O.LBFGS_DEFAULTS, **param)
    ret, ftrace, x_want = o64.run(n, max_evals=5000, **param)
    opt = fwigpu.Lbfgs(n, **p)
    try:
        x = o64.x0(n)
        f, g = o64.objective(x)
        got = [f]
        state = opt.begin(x, f, g)
        while state == fwigpu.LBFGS_EVALUATE and len(got) < 5000:
            f, g = o64.objective(x)
            got.append(f)
            state = opt.next(x, f, g)
        assert state == ret, (state, ret)
        assert len(got) == len(ftrace), (len(got), len(ftrace))
        # relative to the start value: near convergence f -> 0 and only its scale is meaningful
        assert np.allclose(got, ftrace, rtol=LBFGS_RTOL, atol=LBFGS_RTOL * abs(ftrace[0]))
        assert rel(x, x_want) <= LBFGS_RTOL
        assert opt.info()["evaluations"] == len(ftrace)
    finally:
        opt.close()
