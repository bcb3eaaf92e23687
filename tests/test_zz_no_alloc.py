"""The allocation-free misfit entry point, fwi_l2_misfit_noalloc.

It is meant for callers that cannot call cudaMalloc, because their device
memory belongs to another allocator or because an allocation would stall
them.  Here the device buffers come from torch's allocator, standing in for
such a caller.  The entry point is checked through the C ABI on two calls in
a row with different inputs: against the misfit that the existing entry
point fwi_gradient computes on the same traces, against an FP64 numpy sum
of the squared residual, and (the residual) against numpy exactly.  It is
also run at its size limit, FWI_NOALLOC_MAX_TRACES = 65536 traces, and one
trace beyond it.  This file is collected last, so a failure here comes after
every other test.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import ricker

pytestmark = pytest.mark.gpu

MISFIT_RTOL = 1e-12      # FP64 sums of the same FP32 squares, in another order
MAX_TRACES = 65536


def _dev(t):
    return C.c_void_p(t.data_ptr())


def _np_misfit(syn, obs):
    r = syn.astype(np.float32) - obs.astype(np.float32)         # the FP32 residual, as the kernel forms it
    return 0.5 * np.sum(r.astype(np.float64) ** 2), r


def _bind(lib):
    lib.fwi_l2_misfit_noalloc.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p,
                                          C.c_void_p]
    lib.fwi_l2_misfit_noalloc.restype = C.c_int
    return lib.fwi_l2_misfit_noalloc


def test_noalloc_misfit_matches_fwi_gradient(engine_lib):
    torch = pytest.importorskip("torch")
    import fwigpu

    call = _bind(engine_lib)
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
            J_np, r_np = _np_misfit(syn, obs)
            obs_d = torch.from_numpy(obs).to(dev)
            st = call(_dev(syn_d), _dev(obs_d), _dev(res_d), ntr, ns, _dev(mis_d), C.c_void_p(stream.cuda_stream))
            assert st == 0
            torch.cuda.synchronize(dev)
            mis = mis_d.cpu().numpy()
            assert mis[0] == mis[1]
            assert abs(mis[1] - J_np) <= MISFIT_RTOL * J_np, (mis[1], J_np)
            assert abs(mis[1] - J_ref) <= MISFIT_RTOL * J_ref, (mis[1], J_ref)
            assert np.array_equal(res_d.cpu().numpy(), r_np)
        # beyond the scratch: rejected before any GPU work
        big = fwigpu.STATUS.get(call(_dev(syn_d), _dev(obs_d), _dev(res_d), MAX_TRACES + 1, 1, _dev(mis_d), None))
        assert big == "FWI_ERR_ARG"


def test_noalloc_misfit_at_its_trace_limit(engine_lib):
    """Exactly FWI_NOALLOC_MAX_TRACES traces, the largest count that must
    work, twice in a row; the second call reads scratch the first one wrote."""
    torch = pytest.importorskip("torch")
    call = _bind(engine_lib)
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(5)
    for ns in (1, 3):
        syn = rng.standard_normal(MAX_TRACES * ns).astype(np.float32)
        obs = rng.standard_normal(MAX_TRACES * ns).astype(np.float32)
        syn_d, obs_d = torch.from_numpy(syn).to(dev), torch.from_numpy(obs).to(dev)
        res_d = torch.empty_like(syn_d)
        mis_d = torch.full((2,), -1.0, dtype=torch.float64, device=dev)
        assert call(_dev(syn_d), _dev(obs_d), _dev(res_d), MAX_TRACES, ns, _dev(mis_d), None) == 0
        torch.cuda.synchronize(dev)
        J_np, r_np = _np_misfit(syn, obs)
        mis = mis_d.cpu().numpy()
        assert mis[0] == mis[1] and abs(mis[1] - J_np) <= MISFIT_RTOL * J_np, (mis, J_np)
        assert np.array_equal(res_d.cpu().numpy(), r_np)
