"""Sharding of the tracking path over several GPUs (one process per GPU).

Particles are independent, so the tracking path needs no collective on its
data path: each rank advances its own contiguous slice of the particles (or
its own set of whole ensembles) on its own GPU with the snapshot buffers
replicated, and results meet only where the caller asks for them on one
rank (``gather_rows``).  The density passes are the one real exchange: a
Gaussian KDE on a fixed grid is a sum over particles, so each rank evaluates
its slice and one float64 all-reduce of the grid combines them
(``allreduce_sum``); SPH needs every particle near each query, so the
positions are all-gathered first (``gather_rows`` to every rank).

The helpers take an initialised ``torch.distributed`` process group; with
one process they reduce to the single-GPU path.
"""
from __future__ import annotations

from typing import Callable, List, Sequence, Tuple

import numpy as np


def _dist():
    import torch.distributed as dist
    return dist


def world_and_rank() -> Tuple[int, int]:
    dist = _dist()
    if dist.is_available() and dist.is_initialized():
        return dist.get_world_size(), dist.get_rank()
    return 1, 0


def shard_bounds(n: int, rank: int, world: int) -> Tuple[int, int]:
    """Contiguous slice [lo, hi) of n particles for ``rank``; the first
    n % world ranks take one particle more."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside a world of {world}")
    base, extra = divmod(int(n), world)
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def shard_ensembles(sizes: Sequence[int], world: int) -> List[List[int]]:
    """Whole ensembles per rank, balanced by particle count: largest first,
    each to the rank with the fewest particles so far (ties to the lower
    rank); every rank's list is returned in ascending ensemble order."""
    load = [0] * world
    out: List[List[int]] = [[] for _ in range(world)]
    for e in sorted(range(len(sizes)), key=lambda i: (-int(sizes[i]), i)):
        r = min(range(world), key=lambda q: (load[q], q))
        out[r].append(e)
        load[r] += int(sizes[e])
    return [sorted(v) for v in out]


def collective_device():
    """Where the process group's collectives take their tensors: this rank's
    current CUDA device under NCCL (which rejects host tensors), the host
    under gloo."""
    import torch
    dist = _dist()
    if dist.is_available() and dist.is_initialized() and str(dist.get_backend()).lower() == "nccl":
        return torch.device("cuda", torch.cuda.current_device())
    return torch.device("cpu")


def gather_rows(local, n_total: int, to_all: bool = False):
    """Concatenate every rank's (n_r, k) rows in rank order (the layout
    ``shard_bounds`` produced) on rank 0, or on every rank with ``to_all``.
    Other ranks get None unless ``to_all``.  The rows travel on the process
    group's device (``collective_device``) and come back there."""
    import torch
    dist = _dist()
    world, rank = world_and_rank()
    if world == 1:
        return local
    local = torch.as_tensor(local).to(collective_device())
    counts = [shard_bounds(n_total, r, world) for r in range(world)]
    lo, hi = counts[rank]
    if local.shape[0] != hi - lo:
        raise ValueError(f"rank {rank} holds {local.shape[0]} rows; its slice of {n_total} is {hi - lo}")
    width = max(hi - lo for lo, hi in counts)
    pad = torch.zeros((width,) + tuple(local.shape[1:]), dtype=local.dtype, device=local.device)
    pad[: local.shape[0]] = local
    parts = [torch.empty_like(pad) for _ in range(world)]
    dist.all_gather(parts, pad)
    if not to_all and rank != 0:
        return None
    return torch.cat([p[: hi - lo] for p, (lo, hi) in zip(parts, counts)], dim=0)


def allreduce_sum(t):
    """In-place float64 sum over ranks (the KDE grid reduction)."""
    import torch
    dist = _dist()
    world, _ = world_and_rank()
    if world == 1:
        return t
    acc = t.to(device=collective_device(), dtype=torch.float64)
    dist.all_reduce(acc, op=dist.ReduceOp.SUM)
    t.copy_(acc.to(device=t.device, dtype=t.dtype))
    return t


def gather_all(local, group=None):
    """Every rank's rows (any count per rank) on every rank, in rank order:
    the SPH exchange, where each query needs every particle near it."""
    import torch
    dist = _dist()
    local = torch.as_tensor(local)
    world = dist.get_world_size(group)
    if world == 1:
        return local
    dev = collective_device()
    x = local.to(dev)
    n = torch.tensor([x.shape[0]], dtype=torch.int64, device=dev)
    counts = [torch.zeros_like(n) for _ in range(world)]
    dist.all_gather(counts, n, group=group)
    counts = [int(c.item()) for c in counts]
    width = max(max(counts), 1)
    pad = torch.zeros((width,) + tuple(x.shape[1:]), dtype=x.dtype, device=dev)
    pad[: x.shape[0]] = x
    parts = [torch.empty_like(pad) for _ in range(world)]
    dist.all_gather(parts, pad, group=group)
    return torch.cat([p[:c] for p, c in zip(parts, counts)], dim=0).to(local.device)


def global_stats(P, group=None):
    """Count, mean, unbiased variance, minimum and maximum per column of the
    rows spread over the ranks (float64 sums, one all-reduce each): what the
    KDE bandwidth rules and the grid bounds need of all particles."""
    import torch
    dist = _dist()
    x = torch.as_tensor(P).double()
    dev = collective_device()
    s = torch.cat([torch.tensor([float(x.shape[0])], dtype=torch.float64), x.sum(0).cpu(),
                   (x * x).sum(0).cpu()]).to(dev)
    lo = x.min(0).values.cpu().to(dev) if x.shape[0] else torch.full((x.shape[1],), float("inf"), device=dev,
                                                                         dtype=torch.float64)
    hi = x.max(0).values.cpu().to(dev) if x.shape[0] else torch.full((x.shape[1],), float("-inf"), device=dev,
                                                                         dtype=torch.float64)
    if dist.get_world_size(group) > 1:
        dist.all_reduce(s, op=dist.ReduceOp.SUM, group=group)
        dist.all_reduce(lo, op=dist.ReduceOp.MIN, group=group)
        dist.all_reduce(hi, op=dist.ReduceOp.MAX, group=group)
    s = s.cpu().numpy()
    d = x.shape[1]
    n = s[0]
    mean = s[1:1 + d] / n
    var = (s[1 + d:] - n * mean * mean) / max(n - 1.0, 1.0)
    return int(n), mean, var, lo.cpu().numpy(), hi.cpu().numpy()


def allreduce_array(a, group=None):
    """Float64 sum over ranks of a host or device array (the KDE grid)."""
    import torch
    dist = _dist()
    if dist.get_world_size(group) == 1:
        return a
    is_np = isinstance(a, np.ndarray)
    t = torch.as_tensor(np.ascontiguousarray(a) if is_np else a)
    acc = t.to(device=collective_device(), dtype=torch.float64)
    dist.all_reduce(acc, op=dist.ReduceOp.SUM, group=group)
    return acc.cpu().numpy() if is_np else acc.to(device=t.device)


def track_sharded(run: Callable, x0: np.ndarray, to_all: bool = False):
    """Advance this rank's slice of ``x0`` with ``run`` (a function from a
    (n_r, 3) float32 array to its final positions, e.g. a tracker's
    ``track_particles(...).positions[-1]``) and gather the final positions of
    all particles in the original order."""
    import torch
    world, rank = world_and_rank()
    lo, hi = shard_bounds(len(x0), rank, world)
    local = torch.as_tensor(np.ascontiguousarray(run(x0[lo:hi])))
    out = gather_rows(local, len(x0), to_all=to_all)
    return None if out is None else out.cpu().numpy()


__all__ = ["world_and_rank", "shard_bounds", "shard_ensembles", "collective_device", "gather_rows", "allreduce_sum",
           "gather_all", "global_stats", "allreduce_array", "track_sharded"]
