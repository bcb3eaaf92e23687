"""GPU parity: the engine (through its C ABI) against the CPU oracle.

Tolerances (FP32 stencils on both sides; the GPU contracts a*b+c into FMA,
the oracle does not, so results agree to rounding, not bit for bit):
  * seismograms vs the FP32 oracle: relative L2 error <= 2e-5 per shot;
  * misfit vs the FP64 oracle: relative error <= 1e-5;
  * gradient vs the FP64 oracle: relative L2 error <= 1e-4 (the project's
    FP32 gradient tolerance), and vs the FP32 oracle the same bound.
"""
import numpy as np
import pytest

from conftest import ricker

pytestmark = pytest.mark.gpu

SYN_TOL = 2e-5
GRAD_TOL = 1e-4


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


class Case:
    """One small problem expressed both for the oracle (cell indices) and for
    the engine (metres, converted by fwi_2d.c:363-371's rounding)."""

    def __init__(self, O, fs, nx=150, nz=90, npml=10, nt=301, jump=2, dx=10.0, dz=10.0, dt=0.001, seed=0,
                 shots=None, order=4):
        import fwigpu
        self.O, self.fs = O, fs
        self.dx, self.dz = dx, dz
        rng = np.random.default_rng(seed)
        self.vel = rng.uniform(1500.0, 3200.0, (nz, nx)).astype(np.float32)
        self.vel = (0.5 * self.vel + 0.5 * np.linspace(1600, 3000, nz)[:, None]).astype(np.float32)
        self.vtrue = self.vel.copy()
        self.vtrue[nz // 6:nz // 6 + 10, nx // 4:3 * nx // 4] += 250.0
        self.order = order
        self.ocfg = O.make_config(nx=nx, nz=nz, npml=npml, nt=nt, dx=dx, dz=dz, dt=dt, free_surface=fs, jump=jump,
                                  fd_order=order)
        self.shot_specs = shots or self.default_shots(rng, nx, nz, nt, jump, dt)
        self.oshots = []
        self.eshots = []
        for (isx, isz, irx, irz, wav) in self.shot_specs:
            self.oshots.append(O.Shot(isx, isz, irx, irz, wav))
            rec = np.stack([np.asarray(irx) * dx + 0.1 * dx, np.asarray(irz) * dz + 0.4 * dz], axis=1)
            self.eshots.append(fwigpu.ShotSpec(isx * dx + 0.1 * dx, isz * dz + 0.4 * dz, rec, wav))
        nt_max = max(len(s[4]) for s in self.shot_specs)
        self.ecfg = fwigpu.make_config(nx, nz, dx, dz, dt, nt_max, npml=npml, free_surface=fs, jump=jump,
                                       fd_order=order)

    @staticmethod
    def default_shots(rng, nx, nz, nt, jump, dt):
        shots = []
        # surface shot, dense surface spread with four receivers in one cell
        irx = np.concatenate([np.arange(0, nx, 2), [7, 7, 7, 7]])
        shots.append((nx // 3, 1, irx, np.zeros_like(irx), ricker(nt, dt, 15.0)))
        # buried source inside the rebuilt interior, sparse receivers on all edges
        irx = np.array([0, nx - 1, 5, nx // 2, nx - 3, 2, 60])
        irz = np.array([4, 10, nz - 1, nz - 1, 0, 2, 40])
        nt2 = nt - 2 * jump * 10
        shots.append((nx // 2 + 3, nz // 4, irx, irz, ricker(nt2, dt, 12.0)))
        # short record near the right edge
        irx = np.arange(nx - 40, nx, 3)
        nt3 = (nt // 2 - 1) // jump * jump + 1
        shots.append((nx - 5, 2, irx, np.ones_like(irx), ricker(nt3, dt, 18.0)))
        return shots

    def oracle_cfg_for(self, nt):
        O = self.O
        c = self.ocfg
        return O.make_config(nx=c.nx, nz=c.nz, npml=c.npml, nt=nt, dx=c.dx, dz=c.dz, dt=c.dt,
                             free_surface=c.free_surface, jump=c.jump, fd_order=c.fd_order)

    def engine(self):
        import fwigpu
        e = fwigpu.Engine(self.ecfg)
        e.set_shots(self.eshots)
        return e

    def oracle_obs(self, o):
        return [o.forward(self.oracle_cfg_for(len(s.wav)), self.vtrue, s).astype(np.float32) for s in self.oshots]


@pytest.fixture(scope="module")
def lib(engine_lib):
    return engine_lib


@pytest.mark.parametrize("fs", [1, 0])
def test_forward_seismograms(lib, oracles, fs):
    O, o32, _ = oracles
    case = Case(O, fs, seed=1 + fs)
    e = case.engine()
    e.set_model(case.vel)
    syn = e.split(e.forward())
    for s, got in zip(case.oshots, syn):
        want = o32.forward(case.oracle_cfg_for(len(s.wav)), case.vel, s)
        assert got.shape == want.shape
        assert rel(got, want) <= SYN_TOL, rel(got, want)


# 150 x 90: full-width edge tiles; 130 x 70: a last tile column under half a
# tile wide and a last tile row of a few rows (partial general tiles); 64 x 44:
# no interior tile at all, every tile takes the general path.
@pytest.mark.parametrize("fs,nx,nz", [(1, 150, 90), (0, 150, 90), (1, 130, 70), (0, 130, 70),
                                      (1, 64, 44), (0, 64, 44)])
def test_gradient_against_fp64_oracle(lib, oracles, fs, nx, nz):
    O, o32, o64 = oracles
    case = Case(O, fs, seed=3 + fs, nx=nx, nz=nz)
    obs = case.oracle_obs(o64)
    e = case.engine()
    e.set_model(case.vel)
    e.set_observed(np.concatenate([o.ravel() for o in obs]))
    J, g = e.gradient()
    energy = 0.5 * sum(float((o.astype(np.float64) ** 2).sum()) for o in obs)
    assert J > 1e-3 * energy          # the residual is signal, not rounding noise
    J64, g64 = 0.0, np.zeros_like(g)
    for s, ob in zip(case.oshots, obs):
        j, gg, _ = o64.gradient(case.oracle_cfg_for(len(s.wav)), case.vel, [s], [ob])
        J64 += j
        g64 += gg
    assert abs(J - J64) <= 1e-5 * J64, (J, J64)
    assert rel(g, g64) <= GRAD_TOL, rel(g, g64)
    # the FP32 oracle sees the same rounding class
    g32 = sum(o32.gradient(case.oracle_cfg_for(len(s.wav)), case.vel, [s], [ob])[1]
              for s, ob in zip(case.oshots, obs))
    assert rel(g, g32) <= GRAD_TOL
    st = e.stats()
    assert st["launches"] > 0 and st["ms_forward"] > 0 and st["ms_backward"] > 0


def test_backward_half_with_given_residual(lib, oracles):
    O, _, o64 = oracles
    case = Case(O, 1, seed=7)
    rng = np.random.default_rng(8)
    e = case.engine()
    e.set_model(case.vel)
    syn = e.forward()
    res = rng.standard_normal(syn.size).astype(np.float32) * 1e-2
    g = e.backward(res)
    parts = e.split(res)
    g64 = sum(o64.backward(case.oracle_cfg_for(len(s.wav)), case.vel, s, r.astype(np.float64))
              for s, r in zip(case.oshots, parts))
    assert rel(g, g64) <= GRAD_TOL, rel(g, g64)


def test_batched_equals_one_shot_at_a_time(lib, oracles):
    O, _, o64 = oracles
    case = Case(O, 1, seed=9)
    obs = case.oracle_obs(o64)
    flat = np.concatenate([o.ravel() for o in obs])
    e = case.engine()
    e.set_model(case.vel)
    e.set_observed(flat)
    J, g = e.gradient()
    syn_b = e.split(e.forward())
    import fwigpu
    Js, gs = 0.0, np.zeros_like(g)
    for spec, ob, sb in zip(case.eshots, obs, syn_b):
        cfg = fwigpu.make_config(case.ecfg.nx, case.ecfg.nz, case.dx, case.dz, case.ecfg.dt, spec.nt,
                                 npml=case.ecfg.npml, free_surface=1, jump=case.ecfg.jump)
        with fwigpu.Engine(cfg) as one:
            one.set_shots([spec])
            one.set_model(case.vel)
            assert np.array_equal(one.forward().reshape(sb.shape), sb)   # shots are independent
            one.set_observed(ob)
            j, gg = one.gradient()
        Js += j
        gs += gg
    assert abs(J - Js) <= 1e-12 * J
    assert np.allclose(g, gs, rtol=1e-9, atol=1e-12 * np.abs(g).max())


def test_minimal_record_beside_a_long_one(lib, oracles):
    """A shot of 2 * jump + 1 steps (two trace samples) batched with one of
    261 steps: the active-prefix launches drop it after its last step."""
    O, _, o64 = oracles
    base = Case(O, 1, seed=5)
    short = base.shot_specs[0][:4] + (ricker(2 * base.ecfg.jump + 1, base.ecfg.dt, 15.0),)
    case = Case(O, 1, seed=5, shots=[short, base.shot_specs[1]])
    assert [len(s.wav) for s in case.oshots] == [5, 261]
    obs = case.oracle_obs(o64)
    e = case.engine()
    e.set_model(case.vel)
    e.set_observed(np.concatenate([o.ravel() for o in obs]))
    J, g = e.gradient()
    J64, g64 = 0.0, np.zeros_like(g)
    for s, ob in zip(case.oshots, obs):
        j, gg, _ = o64.gradient(case.oracle_cfg_for(len(s.wav)), case.vel, [s], [ob])
        J64 += j
        g64 += gg
    assert abs(J - J64) <= 1e-5 * J64, (J, J64)
    assert rel(g, g64) <= GRAD_TOL, rel(g, g64)


def test_shot_without_receivers_adds_nothing(lib, oracles):
    """A shot with no receivers is accepted, has no traces and no residual, so
    a batch that adds one returns the other shot's misfit and gradient bit for
    bit."""
    import fwigpu
    O, _, o64 = oracles
    case = Case(O, 1, seed=5)
    obs = case.oracle_obs(o64)
    spec = case.eshots[0]
    silent = fwigpu.ShotSpec(spec.src_x + 200.0, spec.src_z, np.zeros((0, 2), np.float32), spec.wavelet)
    out = []
    with case.engine() as e:
        for shots in ([spec], [spec, silent]):
            e.set_shots(shots)
            e.set_model(case.vel)
            e.set_observed(obs[0].ravel())
            out.append(e.gradient())
    (J1, g1), (J2, g2) = out
    assert J1 == J2 and np.array_equal(g1, g2)


def test_repeated_gradients_are_deterministic(lib, oracles):
    O, _, o64 = oracles
    case = Case(O, 0, seed=11, nt=201)
    obs = case.oracle_obs(o64)
    e = case.engine()
    e.set_model(case.vel)
    e.set_observed(np.concatenate([o.ravel() for o in obs]))
    J1, g1 = e.gradient()
    J2, g2 = e.gradient()
    assert J1 == J2 and np.array_equal(g1, g2)


def test_error_paths(lib, oracles):
    import fwigpu
    O, _, _ = oracles
    case = Case(O, 1, seed=12, nt=101)
    e = case.engine()
    with pytest.raises(fwigpu.FwiError) as ei:
        e.backward(np.zeros(e.nsamples, np.float32))
    assert ei.value.status == -5                    # FWI_ERR_STATE
    bad = case.vel.copy()
    bad[3, 4] = np.nan
    with pytest.raises(fwigpu.FwiError) as ei:
        e.set_model(bad)
    assert ei.value.status == -7                    # FWI_ERR_NONFINITE
    with pytest.raises(fwigpu.FwiError) as ei:
        e.set_model(case.vel * 10.0)
    assert ei.value.status == -6                    # FWI_ERR_CFL
    outside = fwigpu.ShotSpec(10.0, 10.0, np.array([[1e6, 2.0]]), ricker(101, 0.001, 10.0))
    with pytest.raises(fwigpu.FwiError) as ei:
        e.set_shots([outside])
    assert ei.value.status == -2                    # FWI_ERR_GEOMETRY
    longer = fwigpu.ShotSpec(10.0, 10.0, np.array([[20.0, 2.0]]), ricker(500, 0.001, 10.0))
    with pytest.raises(fwigpu.FwiError) as ei:
        e.set_shots([longer])
    assert ei.value.status == -1                    # nt > nt_max
    with pytest.raises(fwigpu.FwiError) as ei:
        e.set_shots([])
    assert ei.value.status == -1                    # no shots
    with pytest.raises(fwigpu.FwiError) as ei:
        e.set_shots([case.eshots[0]] * 65536)
    assert ei.value.status == -1                    # more shots than the launch grid's z extent
    # the context stays usable after rejected calls
    e.set_shots(case.eshots)
    e.set_model(case.vel)
    assert np.isfinite(e.forward()).all()


def test_graph_replay_and_plain_mode_match_direct(lib, oracles):
    import fwigpu
    O, _, o64 = oracles
    case = Case(O, 1, seed=13, nt=201)
    flat = np.concatenate([o.ravel() for o in case.oracle_obs(o64)])
    out = []
    for graph, plain in [(0, 0), (1, 0), (0, 1)]:
        c = case.ecfg
        cfg = fwigpu.make_config(c.nx, c.nz, c.dx, c.dz, c.dt, c.nt_max, npml=c.npml, free_surface=c.free_surface,
                                 jump=c.jump, use_graph=graph, plain_per_shot=plain)
        with fwigpu.Engine(cfg) as e:
            e.set_shots(case.eshots)
            e.set_model(case.vel)
            e.set_observed(flat)
            J1, g1 = e.gradient()
            e.set_model(case.vel * 1.01)     # a graph replay must see the new model
            J2, g2 = e.gradient()
            e.set_model(case.vel)
            J3, g3 = e.gradient()
            st = e.stats()
        assert J1 == J3 and np.array_equal(g1, g3) and J2 != J1
        assert st["ms_forward"] > 0 and st["ms_backward"] > 0 and st["launches"] > 0
        out.append((J1, g1, J2, g2))
    for J1, g1, J2, g2 in out[1:]:        # every shot is computed identically in every mode
        assert J1 == out[0][0] and np.array_equal(g1, out[0][1])
        assert J2 == out[0][2] and np.array_equal(g2, out[0][3])
