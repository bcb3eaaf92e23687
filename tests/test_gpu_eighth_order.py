"""The 8th-order extension (fd_order 8) on the GPU against the 8th-order
CPU oracle, whose operator and adjoint are pinned by tests/test_oracle_adjoint.py
(the reference has no 8th-order code to pin against).

Tolerances as for the reference's 4th order: seismograms vs the FP32 oracle
<= 2e-5, misfit vs FP64 <= 1e-5, gradient vs FP64 <= 1e-4.  The 8th-order
inversion workload runs as configured: 201 x 401, nt 2000, 8 shots, 200 receivers, 8th order, one
gradient checked against the FP64 oracle, then 5 L-BFGS iterations on the
device (fwi_lbfgs_*) driven by the engine's gradients.
"""
import numpy as np
import pytest

from test_gpu_parity import Case, rel

pytestmark = pytest.mark.gpu

SYN_TOL = 2e-5
GRAD_TOL = 1e-4


def _fp64(case, o64, obs):
    J, g = 0.0, None
    for s, ob in zip(case.oshots, obs):
        j, gg, _ = o64.gradient(case.oracle_cfg_for(len(s.wav)), case.vel, [s], [ob])
        J += j
        g = gg if g is None else g + gg
    return J, g


@pytest.mark.parametrize("fs,nx,nz", [(1, 150, 90), (0, 150, 90), (1, 130, 70)])
def test_eighth_order_forward_and_gradient(engine_lib, oracles, fs, nx, nz):
    O, o32, o64 = oracles
    case = Case(O, fs, seed=61 + fs, nx=nx, nz=nz, order=8)
    obs = case.oracle_obs(o64)
    with case.engine() as e:
        e.set_model(case.vel)
        for s, got in zip(case.oshots, e.split(e.forward())):
            want = o32.forward(case.oracle_cfg_for(len(s.wav)), case.vel, s)
            assert rel(got, want) <= SYN_TOL, rel(got, want)
        e.set_observed(np.concatenate([o.ravel() for o in obs]))
        J, g = e.gradient()
    J64, g64 = _fp64(case, o64, obs)
    assert abs(J - J64) <= 1e-5 * J64, (J, J64)
    assert rel(g, g64) <= GRAD_TOL, rel(g, g64)


def test_eighth_order_modes_agree(engine_lib, oracles):
    """Batched, graph-replayed and plain per-shot gradients are bit-identical;
    FP32 checkpoints agree with the strip ring to FP32 rounding."""
    import fwigpu
    O, _, o64 = oracles
    case = Case(O, 1, seed=65, nt=201, order=8)
    flat = np.concatenate([o.ravel() for o in case.oracle_obs(o64)])
    out = []
    c = case.ecfg
    for kw in (dict(use_graph=0), dict(use_graph=1), dict(plain_per_shot=1),
               dict(store=fwigpu.STORE_SNAPSHOTS, snapshots=6)):
        cfg = fwigpu.make_config(c.nx, c.nz, c.dx, c.dz, c.dt, c.nt_max, npml=c.npml, free_surface=1, jump=c.jump,
                                 fd_order=8, **kw)
        with fwigpu.Engine(cfg) as e:
            e.set_shots(case.eshots)
            e.set_model(case.vel)
            e.set_observed(flat)
            out.append(e.gradient())
    for J, g in out[1:3]:
        assert J == out[0][0] and np.array_equal(g, out[0][1])
    assert out[3][0] == out[0][0] and rel(out[3][1], out[0][1]) <= 1e-5


def test_c1_as_configured(engine_lib, oracles):
    import fwigpu
    import workloads
    O, o32, o64 = oracles
    cfgkw, vtrue, vstart, shots = workloads.build("c1")
    cases = []
    for sh in shots:
        isx, isz = o64.cell_of(sh.src_x, sh.src_z, cfgkw["dx"], cfgkw["dz"])
        cells = [o64.cell_of(float(x), float(z), cfgkw["dx"], cfgkw["dz"]) for x, z in sh.rec_xz]
        ocfg = O.make_config(nx=cfgkw["nx"], nz=cfgkw["nz"], npml=cfgkw["npml"], nt=sh.nt, dx=cfgkw["dx"],
                             dz=cfgkw["dz"], dt=cfgkw["dt"], free_surface=1, jump=cfgkw["jump"], fd_order=8)
        cases.append((ocfg, O.Shot(isx, isz, [c[0] for c in cells], [c[1] for c in cells], sh.wavelet)))
    obs = [o64.forward(c, vtrue, s).astype(np.float32) for c, s in cases]
    with fwigpu.Engine(fwigpu.make_config(**cfgkw, fd_order=8, use_graph=1)) as e:
        e.set_shots(shots)
        e.set_model(vstart)
        for (c, s), got in zip(cases[:2], e.split(e.forward())[:2]):
            assert rel(got, o32.forward(c, vstart, s)) <= SYN_TOL
        e.set_observed(np.concatenate([o.ravel() for o in obs]))
        J, g = e.gradient()
        J64, g64 = 0.0, np.zeros_like(g)
        for (c, s), ob in zip(cases, obs):
            j, gg, _ = o64.gradient(c, vstart, [s], [ob])
            J64 += j
            g64 += gg
        assert abs(J - J64) <= 1e-5 * J64, (J, J64)
        assert rel(g, g64) <= GRAD_TOL, rel(g, g64)

        # 5 L-BFGS iterations (MBotOpt's line search on the device); the
        # objective is scaled so that the first step moves the model by tens
        # of m/s, as grad_precond_new5's alpha_grad does in the reference
        scale = 40.0 / np.abs(g).max()

        def evaluate(xv):
            e.set_model(xv.reshape(vstart.shape).astype(np.float32))
            Jx, gx = e.gradient()
            return scale * Jx, scale * gx.ravel()

        x = vstart.astype(np.float64).ravel().copy()
        f, gr = evaluate(x)
        opt = fwigpu.Lbfgs(x.size, max_iterations=5)
        evals = [f]
        state = opt.begin(x, f, gr)
        while state == fwigpu.LBFGS_EVALUATE and len(evals) < 60:
            f, gr = evaluate(x)
            evals.append(f)
            state = opt.next(x, f, gr)
        it = opt.info()["iteration"]
        opt.close()
    assert state == fwigpu.LBFGS_MAXITERATION and it >= 5, (state, it, evals)
    assert evals[-1] < 0.8 * evals[0], evals
    assert np.isfinite(x).all()
