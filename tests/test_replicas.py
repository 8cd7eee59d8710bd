"""Replica sharding across ranks, on CPU with the gloo backend (world size 2):
the id ranges tile the global set, initial states do not depend on the
partition (Philox keyed by global id), the timing reduction is max/sum, and
the host-side gather reassembles the global set in id order."""
import os
import socket

import numpy as np
import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, n, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from pentrack_gb300 import replicas, workloads
        first, cnt = replicas.shard(n, rank)
        _, _, parts = workloads.field_storage(n=cnt, first_id=first)
        parts.stop_id[:] = -1 - rank
        tmax, ps = replicas.reduce_timing(1.0 + rank, 10.0 * (rank + 1))
        g = replicas.gather_states(parts)
        if rank == 0:
            q.put({"tmax": tmax, "ps": ps, "gathered": g})
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_partition_and_reduce():
    pytest.importorskip("torch.distributed")
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    n, world, port = 300, 2, _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, n, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res["tmax"] == 2.0 and res["ps"] == 30.0
    from pentrack_gb300 import workloads
    _, _, ref = workloads.field_storage(n=n * world, first_id=0)
    g = res["gathered"]
    assert np.array_equal(g["id"], ref.id)
    assert np.array_equal(g["y"], ref.y)
    assert np.array_equal(g["spin"], ref.spin)
    assert np.array_equal(g["stop_id"], np.repeat([-1, -2], n))
