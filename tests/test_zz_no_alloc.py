"""The allocation-free misfit entry point, fwi_l2_misfit_noalloc.

It is meant for callers that cannot call cudaMalloc, because their device
memory belongs to another allocator or because an allocation would stall
them.  Here the device buffers come from torch's allocator, standing in for
such a caller.  The entry point is checked through the C ABI against the
misfit that the existing entry point fwi_gradient computes on the same
traces, on two calls in a row with different inputs, and on its size limit.
This file is collected last, so a failure here comes after every other test.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import ricker

pytestmark = pytest.mark.gpu

MISFIT_RTOL = 1e-12      # same FP64 sums of the same FP32 squares, different order


def _dev(t):
    return C.c_void_p(t.data_ptr())


def test_noalloc_misfit_matches_fwi_gradient(engine_lib):
    torch = pytest.importorskip("torch")
    import fwigpu

    lib = engine_lib
    lib.fwi_l2_misfit_noalloc.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p,
                                          C.c_void_p]
    lib.fwi_l2_misfit_noalloc.restype = C.c_int
    nx, nz, nt, dx, dt = 96, 64, 201, 10.0, 0.001
    rng = np.random.default_rng(3)
    vel = (np.linspace(1600.0, 2800.0, nz)[:, None] + rng.uniform(-80, 80, (nz, nx))).astype(np.float32)
    rec = np.stack([np.arange(0, nx, 2) * dx + 1.0, np.full(nx // 2, 2.0)], axis=1)
    shots = [fwigpu.ShotSpec(sx * dx + 1.0, 14.0, rec, ricker(nt, dt, 15.0)) for sx in (20, 48, 75)]
    cfg = fwigpu.make_config(nx, nz, dx, dx, dt, nt, npml=10, jump=1)
    with fwigpu.Engine(cfg) as e:
        e.set_shots(shots)
        vtrue = vel.copy()
        vtrue[10:16, 20:70] += 150.0
        e.set_model(vtrue)
        obs_a = e.forward()
        e.set_model(vel)
        syn = e.forward()
        ntr, ns = sum(s.nr for s in shots), nt
        dev = torch.device("cuda", 0)
        syn_d = torch.from_numpy(syn).to(dev)
        res_d = torch.empty_like(syn_d)
        mis_d = torch.zeros(2, dtype=torch.float64, device=dev)
        stream = torch.cuda.current_stream(dev)
        for obs in (obs_a, (0.5 * obs_a + 1e-3 * rng.standard_normal(obs_a.size)).astype(np.float32)):
            e.set_observed(obs)
            J_ref, _ = e.gradient()                       # the existing entry point's misfit
            obs_d = torch.from_numpy(obs).to(dev)
            st = lib.fwi_l2_misfit_noalloc(_dev(syn_d), _dev(obs_d), _dev(res_d), ntr, ns, _dev(mis_d),
                                           C.c_void_p(stream.cuda_stream))
            assert st == 0
            torch.cuda.synchronize(dev)
            mis = mis_d.cpu().numpy()
            assert mis[0] == mis[1]
            assert abs(mis[1] - J_ref) <= MISFIT_RTOL * J_ref, (mis[1], J_ref)
            assert np.array_equal(res_d.cpu().numpy(), syn - obs)
        # beyond the scratch: rejected before any GPU work
        big = fwigpu.STATUS.get(lib.fwi_l2_misfit_noalloc(_dev(syn_d), _dev(obs_d), _dev(res_d), 65537, 1,
                                                          _dev(mis_d), None))
        assert big == "FWI_ERR_ARG"
