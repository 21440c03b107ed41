"""Sharding of independent systems across ranks, one process per GPU.

The batched solve and the adjoint batch consist of independent systems, so a
multi-GPU run partitions the systems and each rank solves its share with no
collective on the data path; only the small per-system outputs a caller asks
for (INFO, or solutions for a check) come back to rank 0 on the host.

The partition balances the LU work: systems are taken in decreasing order of
their cost 2/3 n^3 + 2 n^2 nrhs and each goes to the rank with the least work
so far (longest-processing-time-first), which keeps the most loaded rank
within one system's cost of the mean.  Ties go to the lower rank, so every
rank computes the same partition from the same sizes without communicating.
"""
import numpy as np


def system_cost(ns, nrhs=None):
    """Flops of one LU solve per system: 2/3 n^3 + 2 n^2 nrhs."""
    ns = np.asarray(ns, dtype=np.float64)
    r = np.ones_like(ns) if nrhs is None else np.asarray(nrhs, dtype=np.float64)
    return 2.0 / 3.0 * ns ** 3 + 2.0 * ns ** 2 * r


def partition_by_cost(ns, nrhs=None, world=1):
    """Split system indices 0..len(ns)-1 over `world` ranks: a list of
    `world` sorted index arrays, disjoint and covering every system."""
    if world < 1:
        raise ValueError("world must be at least 1")
    cost = system_cost(ns, nrhs)
    order = np.argsort(-cost, kind="stable")
    load = np.zeros(world)
    owner = np.empty(len(cost), dtype=np.int64)
    for i in order:
        r = int(np.argmin(load))          # first minimum: ties to the lower rank
        owner[i] = r
        load[r] += cost[i]
    return [np.flatnonzero(owner == r) for r in range(world)]


def gather_to_root(local_idx, local_values, n_total, group=None):
    """Host-side gather of per-system values (one entry per local system, in
    the order of `local_idx`) into a list ordered by global system index on
    rank 0; other ranks get None.  Uses torch.distributed.gather_object, so it
    works with the gloo and NCCL backends alike."""
    import torch.distributed as dist
    rank = dist.get_rank(group)
    world = dist.get_world_size(group)
    payload = (np.asarray(local_idx, dtype=np.int64).tolist(), list(local_values))
    parts = [None] * world if rank == 0 else None
    dist.gather_object(payload, parts, dst=0, group=group)
    if rank != 0:
        return None
    out = [None] * n_total
    for idx, vals in parts:
        for i, v in zip(idx, vals):
            if out[i] is not None:
                raise RuntimeError(f"system {i} returned by two ranks")
            out[i] = v
    missing = [i for i, v in enumerate(out) if v is None]
    if missing:
        raise RuntimeError(f"{len(missing)} systems returned by no rank (first {missing[0]})")
    return out
