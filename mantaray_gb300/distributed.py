"""Several GPUs: one process per GPU, rays sharded by contiguous ranges.

Rays are independent (the reference maps them in parallel with no exchange,
src/ray.rs:98-127), so a multi-GPU job splits the initial states into one
contiguous range per rank, traces each range on its own GPU with no
collective in the data path, and gathers only results: trajectories or end
states to rank 0, and timing / counters by max / sum.  These helpers hold
that host-side logic; they work over any torch.distributed backend (NCCL
between GPUs, gloo on CPU).
"""

from __future__ import annotations

import numpy as np


def _dist():
    import torch.distributed as dist

    return dist


def shard_range(n: int, rank: int, world: int) -> tuple[int, int]:
    """[start, stop) of rank's rays: contiguous, sizes differing by at most one."""
    if world < 1 or not (0 <= rank < world):
        raise ValueError("need 0 <= rank < world")
    base, extra = divmod(int(n), world)
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def _device():
    import torch

    dist = _dist()
    if dist.get_backend() == "nccl":
        return torch.device("cuda", torch.cuda.current_device())
    return torch.device("cpu")


def reduce_scalar(value: float, op: str = "max") -> float:
    """value reduced over all ranks ("max" or "sum"), returned on every rank."""
    import torch

    dist = _dist()
    t = torch.tensor([float(value)], dtype=torch.float64, device=_device())
    dist.all_reduce(t, op=dist.ReduceOp.MAX if op == "max" else dist.ReduceOp.SUM)
    return float(t.item())


def gather_rays(local: np.ndarray, n_total: int, dst: int = 0):
    """Concatenates every rank's shard along the last (ray) axis in rank
    order; returns the full array on rank `dst` and None elsewhere.  Shards
    are padded to the largest shard for the collective (all_gather, which
    every backend has) and trimmed after."""
    import torch

    dist = _dist()
    world, rank = dist.get_world_size(), dist.get_rank()
    local = np.ascontiguousarray(local)
    sizes = [shard_range(n_total, r, world) for r in range(world)]
    width = max(b - a for a, b in sizes)
    if local.shape[-1] != sizes[rank][1] - sizes[rank][0]:
        raise ValueError("local shard does not match shard_range")
    pad = np.full(local.shape[:-1] + (width,), np.nan, dtype=np.float64)
    pad[..., : local.shape[-1]] = local
    t = torch.from_numpy(pad).to(_device())
    parts = [torch.empty_like(t) for _ in range(world)]
    dist.all_gather(parts, t)
    if rank != dst:
        return None
    out = [p.cpu().numpy()[..., : b - a] for p, (a, b) in zip(parts, sizes)]
    return np.concatenate(out, axis=-1).astype(local.dtype, copy=False)


def allreduce_node_gradients(*grads):
    """Sums node-gradient arrays (torch tensors, e.g. the adjoint's depth, u
    and v gradients of each rank's ray shard) over all ranks, in place: the
    one exchange a sharded gradient needs (the per-ray work is independent,
    the grid is shared).  Returns the tensors."""
    dist = _dist()
    for g in grads:
        dist.all_reduce(g, op=dist.ReduceOp.SUM)
    return grads
