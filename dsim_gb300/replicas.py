"""Replicas across GPUs: the path's multi-GPU form.

Spins are independent, so a job is split by spin ranges over one process per
GPU; each shard runs the whole step loop on its own GPU with no exchange, and
the only communication is one sum of the FP64 signal sums {sum m cos(phi),
sum m sin(phi), n} per compartment at readout (the reference keeps all spins
on one device and reduces on the host, dSim3/src/spinSystem.cpp:1452-1500).
A shard sets its first spin's global index as its Philox spin base, so the
union of the shards draws exactly what one GPU running all spins draws.
"""
import numpy as np


def shard(n_total, rank, world):
    """[lo, hi) of the spins rank `rank` of `world` simulates (contiguous, sizes differ by <= 1)."""
    base, extra = divmod(n_total, world)
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def combine_sums(local, group=None):
    """Sum the (5, 3) FP64 signal sums of every rank (torch.distributed, any
    backend whose CPU tensors all_reduce: gloo here)."""
    import torch
    import torch.distributed as dist
    t = torch.from_numpy(np.ascontiguousarray(local, np.float64).reshape(-1).copy())
    if dist.is_available() and dist.is_initialized() and dist.get_world_size(group) > 1:
        dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return t.numpy().reshape(np.shape(local))


def max_time(seconds, group=None):
    """The slowest rank's time (the job's wall time)."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(seconds)], dtype=torch.float64)
    if dist.is_available() and dist.is_initialized() and dist.get_world_size(group) > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())


def signal(sums):
    """S = |X + iY| / n per row of the combined sums."""
    s = np.asarray(sums, np.float64).reshape(-1, 3)
    out = np.zeros(len(s))
    nz = s[:, 2] > 0
    out[nz] = np.hypot(s[nz, 0], s[nz, 1]) / s[nz, 2]
    return out
