"""Launch tuning (fwi_set_tuning, fwi_time_steps) and the autotuner.

* The kernel variants (register budgets for 3 or 4 general blocks per SM, 4
  or 6 interior forward blocks, 3 or 4 interior backward blocks), the class
  order, serial launches and the looping general grids (gen_grid) run the
  same arithmetic per cell: the gradient is bit-identical to the default's.
* Another tile grid (x_first / z_first) moves cells between the interior
  and the general kernels, whose x stencils differ in their rounding: the
  gradient stays within the parity tolerance of the FP64 oracle.
* Values outside the lists are rejected; fwi_time_steps reports positive
  per-step times; the autotuner keeps the fastest candidate, writes its cache,
  and a second engine of the same shape takes the cached tuning.
"""
import numpy as np
import pytest

from test_gpu_parity import Case, rel

pytestmark = pytest.mark.gpu

GRAD_TOL = 1e-4


def _grad(case, flat, tuning=None):
    e = case.engine()
    try:
        if tuning:
            e.set_tuning(tuning)
            if not e.shots:
                e.set_shots(case.eshots)
        e.set_model(case.vel)
        e.set_observed(flat)
        return e.gradient(), e.tuning()
    finally:
        e.close()


def test_kernel_variants_are_bit_identical(engine_lib, oracles):
    O, _, o64 = oracles
    case = Case(O, 1, seed=71, nt=201)
    flat = np.concatenate([o.ravel() for o in case.oracle_obs(o64)])
    (J0, g0), t0 = _grad(case, flat)
    assert (t0["fwd_gen_blocks"], t0["bwd_gen_blocks"], t0["fwd_int_blocks"], t0["bwd_int_blocks"],
            t0["class_order"], t0["serial"], t0["priority"], t0["gen_grid"], t0["bwd_zgen_blocks"]) == \
        (4, 3, 6, 4, 1, 2, 1, 1, 4)
    assert t0["x_first"] % 4 == 0
    for tuning in ({"fwd_gen_blocks": 3, "bwd_gen_blocks": 4, "bwd_zgen_blocks": 3},
                   {"fwd_int_blocks": 4, "bwd_int_blocks": 3},
                   {"class_order": 2}, {"serial": 1}, {"priority": 2}, {"gen_grid": 2}, {"gen_grid": 5}):
        (J, g), t = _grad(case, flat, tuning)
        assert all(t[k] == v for k, v in tuning.items())
        assert J == J0 and np.array_equal(g, g0), tuning


@pytest.mark.parametrize("fs", [1, 0])
def test_other_tile_grids_stay_within_tolerance(engine_lib, oracles, fs):
    O, _, o64 = oracles
    case = Case(O, fs, seed=73 + fs)
    obs = case.oracle_obs(o64)
    flat = np.concatenate([o.ravel() for o in obs])
    J64, g64 = 0.0, None
    for s, ob in zip(case.oshots, obs):
        j, gg, _ = o64.gradient(case.oracle_cfg_for(len(s.wav)), case.vel, [s], [ob])
        J64 += j
        g64 = gg if g64 is None else g64 + gg
    (_, g0), t0 = _grad(case, flat)
    for dx, dz in ((8, 4), (16, 8), (32, 16)):
        (J, g), t = _grad(case, flat, {"x_first": t0["x_first"] + dx, "z_first": t0["z_first"] + dz})
        assert (t["x_first"], t["z_first"]) == (t0["x_first"] + dx, t0["z_first"] + dz)
        assert abs(J - J64) <= 1e-5 * J64
        assert rel(g, g64) <= GRAD_TOL, (dx, dz, rel(g, g64))
        assert rel(g, g0) <= GRAD_TOL             # both sit within rounding of FP64


def test_tuning_rejects_bad_values(engine_lib, oracles):
    import fwigpu
    O, _, _ = oracles
    case = Case(O, 1, seed=75, nt=101)
    with case.engine() as e:
        t0 = e.tuning()
        for bad in ({"fwd_gen_blocks": 5}, {"fwd_int_blocks": 5}, {"bwd_int_blocks": 2}, {"class_order": 3},
                    {"serial": 3}, {"priority": 3}, {"gen_grid": 6}, {"gen_grid": -1}, {"bwd_zgen_blocks": 5},
                    {"x_first": t0["x_first"] - 4},
                    {"x_first": t0["x_first"] + 2},
                    {"z_first": t0["z_first"] + 1}, {"x_first": 100000}):
            with pytest.raises(fwigpu.FwiError) as ei:
                e.set_tuning(bad)
            assert ei.value.status == -1, bad
        assert e.tuning() == t0                   # a rejected call changes nothing
        with pytest.raises(fwigpu.FwiError) as ei:
            e.time_steps(4)                       # no model yet
        assert ei.value.status == -5


def test_autotune_and_cache(engine_lib, oracles, tmp_path):
    import fwigpu
    import tuning
    O, _, o64 = oracles
    case = Case(O, 1, seed=77, nt=201)
    cache = str(tmp_path / "tuning.json")
    with case.engine() as e:
        e.set_model(case.vel)
        f, b = e.time_steps(8)
        assert f > 0 and b > 0
        out = tuning.autotune(e, case.eshots, case.vel, steps=6, cache=cache)
        assert not out["cached"] and out["ms_step"] <= out["default_ms_step"]
        assert len(out["trials"]) >= 10 and e.tuning() == out["tuning"]
        assert e.shots and np.isfinite(e.forward()).all()   # shots and model set again
    with case.engine() as e2:
        again = tuning.autotune(e2, case.eshots, case.vel, steps=6, cache=cache)
        assert again["cached"] and e2.tuning() == out["tuning"]
        e2.set_observed(np.concatenate([o.ravel() for o in case.oracle_obs(o64)]))
        J, g = e2.gradient()
        assert np.isfinite(g).all() and J > 0
    assert fwigpu.FwiTuning.KEYS == tuple(out["tuning"].keys())
