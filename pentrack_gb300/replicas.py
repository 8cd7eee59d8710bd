"""Replica sharding over ranks (one process per GPU).

Particles never interact (the reference scales by disjoint job arrays), so
rank r tracks the id range [r * n, (r + 1) * n) with no data-path collective;
the Philox stream is keyed by the global particle id, so every particle's
result is independent of the partition.  The only cross-rank steps are the
measurement reduction (max device time, summed particle-seconds) and the
host-side concatenation of end states."""
import numpy as np


def shard(n_per_rank, rank):
    """First global particle id and count of `rank`'s share."""
    return rank * n_per_rank, n_per_rank


def reduce_timing(device_s, particle_seconds, device=None):
    """(max over ranks of the device time, sum of particle-seconds)."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([device_s], dtype=torch.float64, device=device)
    p = torch.tensor([particle_seconds], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(p, op=dist.ReduceOp.SUM)
    return float(t[0]), float(p[0])


def gather_states(parts, dst=0):
    """Concatenate every rank's particle set on rank `dst` (None elsewhere)."""
    import torch.distributed as dist
    world = dist.get_world_size()
    objs = [None] * world
    payload = {k: getattr(parts, k) for k in ("id", "t", "y", "spin", "stop_id", "n_hit")}
    dist.all_gather_object(objs, payload)
    if dist.get_rank() != dst:
        return None
    out = {}
    for k in payload:
        axis = 1 if objs[0][k].ndim == 2 else 0
        out[k] = np.concatenate([o[k] for o in objs], axis=axis)
    return out
