"""Checkpointed backward (FWI_STORE_SNAPSHOTS) on the GPU against the FP64
oracle and against the strip ring (FWI_STORE_STRIPS).

Both storages solve the same discrete problem; they differ in where the
backward gets the forward field from (the strips of every step, or a
checkpoint per time segment plus a recompute of the segment), so:
  * the forward pass, the traces and the misfit are identical;
  * FP32 checkpoints: gradient within 1e-4 of FP64 and within FP32 rounding
    (1e-5) of the strip ring's gradient;
  * FP16 / BF16 checkpoints (p^{t_a} and p^{t_a} - p^{t_a-1}, each with an
    absmax scale): gradient within 1e-3 / 6e-3 of FP64 on these short
    records (301 steps in 18 segments; every segment restores a rounded state);
  * batched, plain per-shot and graph-replayed checkpointed gradients are
    bit-identical;
  * FWI_STORE_AUTO keeps the strip ring when the budget allows and falls
    back to checkpoints (or FWI_ERR_NOMEM) when it does not;
  * on the full grids of the two checkpointing workloads (2000 x 6000, dx 5 m,
    dt 0.5 ms and 800 x 2400, dx 10 m, dt 1 ms; 2 shots, 801 / 1001 steps in
    round(sqrt(nt)) segments), where the FP64 oracle would take minutes, the
    storages are compared with each other: identical traces and misfit, and
    the checkpointed gradients within FULL_TOL of the strip ring's (measured
    2.4e-6 / 4.6e-4 / 3.1e-3 on the larger grid, FP32 / FP16 / BF16).
"""
import numpy as np
import pytest

from test_gpu_parity import Case, rel

pytestmark = pytest.mark.gpu

GRAD_TOL = 1e-4
SNAP_TOL = {"f32": 1e-4, "f16": 1e-3, "bf16": 6e-3}
FULL_TOL = {"f32": 1e-5, "f16": 2e-3, "bf16": 1.5e-2}


def _engine(case, **kw):
    import fwigpu
    c = case.ecfg
    cfg = fwigpu.make_config(c.nx, c.nz, c.dx, c.dz, c.dt, c.nt_max, npml=c.npml, free_surface=c.free_surface,
                             jump=c.jump, **kw)
    e = fwigpu.Engine(cfg)
    e.set_shots(case.eshots)
    return e


def _fp64(case, o64, obs):
    J64, g64 = 0.0, None
    for s, ob in zip(case.oshots, obs):
        j, gg, _ = o64.gradient(case.oracle_cfg_for(len(s.wav)), case.vel, [s], [ob])
        J64 += j
        g64 = gg if g64 is None else g64 + gg
    return J64, g64


@pytest.mark.parametrize("fs", [1, 0])
def test_checkpointed_gradient_against_fp64_and_strips(engine_lib, oracles, fs):
    import fwigpu
    O, _, o64 = oracles
    case = Case(O, fs, seed=31 + fs)
    obs = case.oracle_obs(o64)
    flat = np.concatenate([o.ravel() for o in obs])
    J64, g64 = _fp64(case, o64, obs)
    with _engine(case, store=fwigpu.STORE_STRIPS) as e:
        e.set_model(case.vel)
        e.set_observed(flat)
        J, g = e.gradient()
        assert e.stats()["store"] == fwigpu.STORE_STRIPS
    assert rel(g, g64) <= GRAD_TOL
    for prec in ("f32", "f16", "bf16"):
        with _engine(case, store=fwigpu.STORE_SNAPSHOTS, snap_precision=prec) as e:
            e.set_model(case.vel)
            e.set_observed(flat)
            Js, gs = e.gradient()
            st = e.stats()
        assert st["store"] == fwigpu.STORE_SNAPSHOTS and st["segments"] == int(np.ceil(np.sqrt(case.ecfg.nt_max)))
        assert Js == J                                        # the forward pass is the same
        assert rel(gs, g64) <= SNAP_TOL[prec], (prec, rel(gs, g64))
        if prec == "f32":
            assert rel(gs, g) <= 1e-5, rel(gs, g)


def test_checkpointed_modes_are_bit_identical(engine_lib, oracles):
    import fwigpu
    O, _, o64 = oracles
    case = Case(O, 1, seed=35, nt=201)
    flat = np.concatenate([o.ravel() for o in case.oracle_obs(o64)])
    out = []
    for graph, plain in [(0, 0), (1, 0), (0, 1)]:
        with _engine(case, store=fwigpu.STORE_SNAPSHOTS, snapshots=7, snap_precision="f16", use_graph=graph,
                     plain_per_shot=plain) as e:
            e.set_model(case.vel)
            e.set_observed(flat)
            J1, g1 = e.gradient()
            J2, g2 = e.gradient()
        assert J1 == J2 and np.array_equal(g1, g2)
        out.append((J1, g1))
    for J, g in out[1:]:
        assert J == out[0][0] and np.array_equal(g, out[0][1])


def test_auto_storage_follows_the_budget(engine_lib, oracles):
    import fwigpu
    O, _, o64 = oracles
    case = Case(O, 1, seed=37, nx=96, nz=64, nt=1201)
    flat = np.concatenate([o.ravel() for o in case.oracle_obs(o64)])
    res = {}
    for budget in (64, 8):
        with _engine(case, store=fwigpu.STORE_AUTO, hbm_budget_mb=budget) as e:
            st = e.stats()
            e.set_model(case.vel)
            e.set_observed(flat)
            res[budget] = (st, e.gradient())
    assert res[64][0]["store"] == fwigpu.STORE_STRIPS
    st8 = res[8][0]
    assert st8["store"] == fwigpu.STORE_SNAPSHOTS and st8["store_bytes"] < res[64][0]["store_bytes"] / 2, st8
    assert res[8][1][0] == res[64][1][0] and rel(res[8][1][1], res[64][1][1]) <= 1e-5
    with pytest.raises(fwigpu.FwiError) as ei:
        _engine(case, store=fwigpu.STORE_AUTO, hbm_budget_mb=1)
    assert ei.value.status == -3                              # FWI_ERR_NOMEM


@pytest.mark.parametrize("name,nt", [("c4", 801), ("c5", 1001)])
def test_checkpoints_against_strips_on_full_grids(engine_lib, name, nt):
    import fwigpu
    import workloads
    cfgkw, vtrue, vstart, shots = workloads.build(name, nshots=2, nt=nt)
    assert (cfgkw["nz"], cfgkw["nx"]) == {"c4": (2000, 6000), "c5": (800, 2400)}[name]
    v0 = (0.95 * vstart).astype(np.float32)            # residuals of the order of the data
    nseg = int(round(np.sqrt(nt)))
    with fwigpu.Engine(fwigpu.make_config(**cfgkw, store=fwigpu.STORE_STRIPS)) as e:
        e.set_shots(shots)
        e.set_model(vtrue)
        obs = e.forward().copy()
        e.set_model(v0)
        e.set_observed(obs)
        J, g = e.gradient()
        syn = e.forward().copy()
        assert e.stats()["store"] == fwigpu.STORE_STRIPS
    for prec in ("f32", "f16", "bf16"):
        cfg = fwigpu.make_config(**cfgkw, store=fwigpu.STORE_SNAPSHOTS, snapshots=nseg, snap_precision=prec)
        with fwigpu.Engine(cfg) as e:
            e.set_shots(shots)
            e.set_model(v0)
            e.set_observed(obs)
            Js, gs = e.gradient()
            st = e.stats()
            assert np.array_equal(e.forward(), syn)
        assert st["store"] == fwigpu.STORE_SNAPSHOTS and st["segments"] == nseg, st
        assert Js == J, (prec, Js, J)
        assert rel(gs, g) <= FULL_TOL[prec], (prec, rel(gs, g))
