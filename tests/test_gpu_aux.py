"""GPU parity of the routines around the gradient (tests/aux_cases.py):
gradient preconditioning and Butterworth band-pass bit-identical to the
oracle (and so to the reference), XCORR1D and the XCORR gradient within
tolerance, at test sizes and at the grid / trace sizes of the 560 x 1700,
4000-step workload."""
import numpy as np
import pytest

import aux_cases as A
from conftest import ricker

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def aux(oracles, engine_lib):
    return oracles[0].AuxOracle()


def test_grad_precond_bit_exact(aux):
    import fwigpu
    A.check_precond(fwigpu, aux, big=True)


def test_bandpass_bit_exact(aux):
    import fwigpu
    A.check_bandpass(fwigpu, aux, big=True)


def test_xcorr1d(aux):
    import fwigpu
    A.check_xcorr(fwigpu, aux)


def test_xcorr_long_traces(aux):
    """Traces as long as the 560 x 1700 workload's (nt0 = 2001), both slices,
    against the oracle."""
    import fwigpu
    rng = np.random.default_rng(23)
    nr, nt = 12, 2001
    obs = rng.standard_normal((nr, nt)).astype(np.float32)
    syn = (np.roll(obs, 5, axis=1) + 0.5 * rng.standard_normal((nr, nt))).astype(np.float32)
    sr = np.concatenate([[0, 0], np.stack([np.arange(nr) * 50.0, np.full(nr, 2.0)], 1).ravel()]).astype(np.float32)
    for mode in (0, 1):
        m1, r1 = fwigpu.xcorr1d(obs, syn, sr, 0.0, 1e9, mode)
        m2, r2 = aux.xcorr1d(obs, syn, sr, 0.0, 1e9, mode)
        assert np.allclose(m1, m2, rtol=A.XCORR_MISFIT_RTOL, atol=0), (m1, m2)
        assert A.rel(r1, r2) <= A.XCORR_RES_RTOL


def test_engine_gradient_with_xcorr(oracles, aux):
    import fwigpu
    from test_gpu_parity import Case
    O = oracles[0]
    near = [(50, 1, np.arange(30, 72, 2), np.zeros(21, int), ricker(301, 0.001, 15.0)),
            (100, 20, np.arange(80, 121, 4), np.full(11, 15), ricker(261, 0.001, 12.0))]
    case = Case(O, 1, seed=41, nx=150, nz=90, shots=near)
    A.check_engine_xcorr(fwigpu, aux, case)


def test_misfit_argument_errors(engine_lib):
    import fwigpu
    cfg = fwigpu.make_config(40, 30, 10.0, 10.0, 0.001, 101, npml=8)
    with fwigpu.Engine(cfg) as e:
        with pytest.raises(fwigpu.FwiError):
            e.set_misfit(7)
        with pytest.raises(fwigpu.FwiError):
            e.set_misfit(fwigpu.MISFIT_XCORR, 3)
    assert fwigpu.STATUS[fwigpu.load_library().fwi_bandpass(None, 10, 1, 0.001, 0, 4, 4, 30.0, 3.0, None)] == \
        "FWI_ERR_ARG"


def test_lbfgs_matches_oracle(oracles):
    """The reference's settings (8 iterations) and a run to convergence."""
    import fwigpu
    O = oracles[0]
    A.check_lbfgs(fwigpu, O, 20000)
    A.check_lbfgs(fwigpu, O, 5000, max_iterations=500)


def test_lbfgs_on_the_fwi_gradient(oracles):
    """L-BFGS iterations of FWI.  As in the reference, the objective is scaled
    so that the first step (0.8 along -g) moves the model by tens of m/s
    (grad_precond_new5's alpha_grad plays this role); the objective must
    decrease.  The device-gradient path (fwi_grad_device) hands out the same
    first trial point as a host gradient."""
    import fwigpu
    from test_gpu_parity import Case
    O = oracles[0]
    case = Case(O, 1, seed=51)
    e = case.engine()
    try:
        e.set_model(case.vtrue)
        obs = e.forward()
        e.set_observed(obs)
        x0 = case.vel.astype(np.float64).ravel().copy()

        e.set_model(case.vel)
        J0, g0 = e.gradient()
        scale = 50.0 / np.abs(g0).max()
        # device gradient pointer: first trial point x0 - 0.8 g0
        opt = fwigpu.Lbfgs(x0.size, max_iterations=3)
        xd = x0.copy()
        assert opt.begin(xd, J0, e.grad_device_ptr()) == fwigpu.LBFGS_EVALUATE
        assert np.allclose(xd, x0 - 0.8 * g0.ravel(), rtol=0, atol=1e-9 * np.abs(x0).max())
        opt.close()

        def evaluate(xv):
            e.set_model(xv.reshape(case.vel.shape).astype(np.float32))
            J, g = e.gradient()
            return scale * J, scale * g.ravel()

        opt = fwigpu.Lbfgs(x0.size, max_iterations=3)
        x = x0.copy()
        f, g = evaluate(x)
        evals = [f]
        state = opt.begin(x, f, g)
        while state == fwigpu.LBFGS_EVALUATE and len(evals) < 40:
            f, g = evaluate(x)
            evals.append(f)
            state = opt.next(x, f, g)
        assert state in (fwigpu.LBFGS_MAXITERATION, fwigpu.LBFGS_SUCCESS), (state, evals)
        assert evals[-1] < 0.9 * evals[0], evals
        opt.close()
    finally:
        e.close()
