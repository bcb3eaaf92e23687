"""fwi_gradient_obs: the observed traces uploaded on a copy stream beside the
forward phase, in the same call as the gradient.

* Its misfit and gradient equal fwi_set_observed + fwi_gradient bit for bit,
  from pageable and from page-locked host memory, with graphs and without.
* The traces stay set: a following fwi_gradient returns the same result.
* Other traces in a later call replace the earlier ones: the result equals
  the direct path's on those traces.
* Before fwi_set_model it fails with FWI_ERR_STATE and changes nothing.
"""
import numpy as np
import pytest

from test_gpu_parity import Case

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("use_graph", [1, 0])
def test_gradient_obs_matches_set_observed(engine_lib, oracles, use_graph):
    import fwigpu
    import torch
    O, _, o64 = oracles
    case = Case(O, 1, seed=81, nt=301)
    flat = np.concatenate([o.ravel() for o in case.oracle_obs(o64)])
    other = (flat * np.float32(0.75)).astype(np.float32)
    pageable = np.empty_like(flat)
    pinned = torch.empty(flat.size, dtype=torch.float32, pin_memory=True).numpy()
    c = case.ecfg
    cfg = fwigpu.make_config(c.nx, c.nz, c.dx, c.dz, c.dt, c.nt_max, npml=c.npml, free_surface=c.free_surface,
                             jump=c.jump, use_graph=use_graph)
    with fwigpu.Engine(cfg) as e:
        e.set_shots(case.eshots)
        e.set_model(case.vel)
        e.set_observed(flat)
        J0, g0 = e.gradient()
        e.set_observed(other)
        J1, g1 = e.gradient()
        assert J1 != J0
        for obs in (pageable, pinned):
            obs[:] = flat
            J, g = e.gradient(observed=obs)
            assert J == J0 and np.array_equal(g, g0)
            J, g = e.gradient()                       # the traces stay set
            assert J == J0 and np.array_equal(g, g0)
            obs[:] = other
            J, g = e.gradient(observed=obs)           # and are replaced by the next call's
            assert J == J1 and np.array_equal(g, g1)
        pinned[:] = flat
        J, _ = e.gradient(keep_on_device=True, observed=pinned)
        assert J == J0


def test_gradient_obs_needs_a_model(engine_lib, oracles):
    import fwigpu
    O, _, o64 = oracles
    case = Case(O, 1, seed=83, nt=101)
    flat = np.concatenate([o.ravel() for o in case.oracle_obs(o64)])
    with case.engine() as e:
        with pytest.raises(fwigpu.FwiError) as ei:
            e.gradient(observed=flat)
        assert ei.value.status == -5
        e.set_model(case.vel)
        J, g = e.gradient(observed=flat)
        assert J > 0 and np.isfinite(g).all()
