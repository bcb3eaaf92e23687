"""Shot-parallel gradients over several processes (one per GPU).

Shots are independent, so the only exchange per gradient is the sum of the
ranks' FP64 gradients [nz][nx] and of their two misfit values -- the
reduction the reference leaves to its missing grad4_1shot driver after each
rank's shot (MBotOpt.c:51-55, 98-102).  Ranks run with torch.distributed
(NCCL between GPUs; gloo on CPU tensors for tests).

* ``partition_shots``: a deterministic cost-balanced split of the shots
  (cost = time steps), so that uneven record lengths do not leave ranks
  idle;
* ``allreduce_gradient``: the FP64 sum of gradient and misfit over ranks,
  in place, on whatever device the tensors live (a device gradient can be
  wrapped without a copy with ``device_tensor``).
"""
from __future__ import annotations

import heapq


def partition_shots(costs, world: int, rank: int) -> list[int]:
    """Indices of the shots rank `rank` of `world` owns: longest first, each
    to the currently least-loaded rank (ties to the lower rank), so every
    rank computes the same assignment."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank must be in [0, world)")
    order = sorted(range(len(costs)), key=lambda i: (-costs[i], i))
    heap = [(0, r) for r in range(world)]
    mine = []
    for i in order:
        load, r = heapq.heappop(heap)
        if r == rank:
            mine.append(i)
        heapq.heappush(heap, (load + costs[i], r))
    return sorted(mine)


def device_tensor(ptr: int, n: int, device):
    """A torch float64 tensor of n values at device pointer ptr (for example
    Engine.grad_device_ptr()), without a copy."""
    import torch

    class _View:
        def __init__(self):
            self.__cuda_array_interface__ = {"shape": (n,), "typestr": "<f8", "data": (ptr, False), "version": 2}

    return torch.as_tensor(_View(), device=device)


def allreduce_gradient(grad, misfit, group=None):
    """Sums grad (float64 tensor) and misfit (float64 tensor of 2) over the
    ranks of `group`, in place; returns (grad, misfit)."""
    import torch
    import torch.distributed as dist

    if grad.dtype != torch.float64 or misfit.dtype != torch.float64:
        raise TypeError("the shot reduction is FP64")
    dist.all_reduce(grad, op=dist.ReduceOp.SUM, group=group)
    dist.all_reduce(misfit, op=dist.ReduceOp.SUM, group=group)
    return grad, misfit
