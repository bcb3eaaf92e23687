"""Shot-parallel gradients on two ranks (gloo, CPU): each rank computes the
FP64 oracle gradient of its cost-balanced share of the shots, the ranks sum
gradient and misfit with allreduce_gradient, and the result equals the
gradient of all shots in one process."""
import os
import socket

import numpy as np
import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_partition_is_balanced_and_complete():
    import shots_parallel as SP
    rng = np.random.default_rng(0)
    costs = list(rng.integers(3000, 6001, 256))            # uneven record lengths, 256 shots
    for world in (1, 2, 3, 8):
        parts = [SP.partition_shots(costs, world, r) for r in range(world)]
        assert sorted(i for p in parts for i in p) == list(range(len(costs)))
        loads = [sum(costs[i] for i in p) for p in parts]
        assert max(loads) - min(loads) <= max(costs)
    with pytest.raises(ValueError):
        SP.partition_shots(costs, 2, 2)


def _rank_main(rank, world, port, out_dir):
    import sys
    here = os.path.dirname(os.path.abspath(__file__))
    root = os.path.dirname(here)
    for p in (here, os.path.join(root, "oracle"), os.path.join(root, "fwi2dacoustic-mpi-lbfgs_gb300")):
        sys.path.insert(0, p)
    import torch
    import torch.distributed as dist
    import oracle as O
    import shots_parallel as SP
    from test_gpu_parity import Case
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    o64 = O.Oracle("f64")
    case = Case(O, 1, seed=7, nx=90, nz=50, npml=8, nt=121)
    costs = [len(s.wav) for s in case.oshots]
    mine = SP.partition_shots(costs, world, rank)
    grad = torch.zeros(50 * 90, dtype=torch.float64)
    mis = torch.zeros(2, dtype=torch.float64)
    for i in mine:
        s = case.oshots[i]
        obs = o64.forward(case.oracle_cfg_for(len(s.wav)), case.vtrue, s)
        j, g, _ = o64.gradient(case.oracle_cfg_for(len(s.wav)), case.vel, [s], [obs])
        grad += torch.from_numpy(np.ascontiguousarray(g, np.float64).ravel())
        mis += j
    SP.allreduce_gradient(grad, mis)
    np.save(os.path.join(out_dir, f"rank{rank}.npy"), np.concatenate([mis.numpy(), grad.numpy()]))
    dist.destroy_process_group()


def test_two_ranks_sum_to_the_single_process_gradient(oracles, tmp_path):
    import torch.multiprocessing as mp
    O = oracles[0]
    from test_gpu_parity import Case
    port = _free_port()
    mp.start_processes(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, start_method="spawn", join=True)
    r0, r1 = np.load(tmp_path / "rank0.npy"), np.load(tmp_path / "rank1.npy")
    assert np.array_equal(r0, r1)                            # every rank holds the same sum
    o64 = O.Oracle("f64")
    case = Case(O, 1, seed=7, nx=90, nz=50, npml=8, nt=121)
    J, g = 0.0, 0.0
    for s in case.oshots:
        obs = o64.forward(case.oracle_cfg_for(len(s.wav)), case.vtrue, s)
        j, gg, _ = o64.gradient(case.oracle_cfg_for(len(s.wav)), case.vel, [s], [obs])
        J, g = J + j, g + gg
    assert abs(r0[0] - J) <= 1e-12 * abs(J)
    assert np.allclose(r0[2:], np.asarray(g).ravel(), rtol=1e-12, atol=1e-12 * np.abs(g).max())
