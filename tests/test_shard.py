"""Sharding of independent systems across ranks (lapack_gb300/shard.py), on
the CPU: the cost-balanced partition, and a world-size-2 run over the gloo
backend in which each rank solves its share of an uneven batch (with the
oracle standing in for a GPU) and rank 0 gathers INFO and the solutions,
compared with the same batch solved in one process."""
import os
import socket

import numpy as np
import pytest

import oracle
from lapack_gb300 import shard


def _batch(count=37, seed=11):
    """Uneven systems n in [2, 40], nrhs in {1, 2, 4}; system 5 singular."""
    rng = np.random.default_rng(seed)
    ns = rng.integers(2, 41, count)
    nrhs = rng.choice([1, 2, 4], count)
    systems = []
    for i, (n, r) in enumerate(zip(ns, nrhs)):
        a = rng.standard_normal((n, n)) + (n if i % 2 == 0 else 0) * np.eye(n)
        if i == 5:
            a[:, 1] = 0.0
        systems.append((a, rng.standard_normal((n, r))))
    return ns, nrhs, systems


def test_partition_is_complete_disjoint_balanced_and_deterministic():
    rng = np.random.default_rng(0)
    ns = rng.integers(8, 513, 2000)
    nrhs = rng.choice([1, 2, 4], 2000)
    cost = shard.system_cost(ns, nrhs)
    for world in (1, 2, 3, 8):
        parts = shard.partition_by_cost(ns, nrhs, world)
        assert len(parts) == world
        assert np.array_equal(np.sort(np.concatenate(parts)), np.arange(len(ns)))
        loads = np.array([cost[p].sum() for p in parts])
        assert loads.max() - loads.min() <= cost.max()
        again = shard.partition_by_cost(ns, nrhs, world)
        assert all(np.array_equal(x, y) for x, y in zip(parts, again))
    assert np.array_equal(shard.partition_by_cost(ns, nrhs, 1)[0], np.arange(len(ns)))
    with pytest.raises(ValueError):
        shard.partition_by_cost(ns, nrhs, 0)


def _worker(rank, world, port, out_path):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ns, nrhs, systems = _batch()
        mine = shard.partition_by_cost(ns, nrhs, world)[rank]
        local = []
        for i in mine:
            _, _, x, info = oracle.gesv(*systems[i])
            local.append((int(info), np.asarray(x)))
        out = shard.gather_to_root(mine, local, len(ns))
        if rank == 0:
            np.savez(out_path, info=np.array([o[0] for o in out]),
                     x=np.concatenate([o[1].ravel() for o in out]),
                     counts=np.array([len(m) for m in shard.partition_by_cost(ns, nrhs, world)]))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


@pytest.mark.timeout(300)
def test_gloo_world2_sharded_batch_matches_one_process(tmp_path):
    import torch.multiprocessing as mp
    out = str(tmp_path / "gathered.npz")
    mp.spawn(_worker, args=(2, _free_port(), out), nprocs=2, join=True)
    got = np.load(out)
    ns, nrhs, systems = _batch()
    want_info, want_x = [], []
    for a, b in systems:
        _, _, x, info = oracle.gesv(a, b)
        want_info.append(info)
        want_x.append(np.asarray(x).ravel())
    assert np.array_equal(got["info"], want_info) and want_info[5] > 0
    assert got["x"].tobytes() == np.concatenate(want_x).tobytes()
    assert got["counts"].min() > 0 and got["counts"].sum() == len(ns)
