"""Multi-process host logic of the replica path, world size 2 on gloo (CPU):
disjoint balanced sharding, max-time reduction and statistics gathering."""

import os
import socket

import pytest

from sph_seepage_flows_gb300.replicas import shard_balanced


def test_shard_balanced_covers_every_item_once():
    sizes = [60000, 2000, 35000, 8000, 8000, 12000, 41000]
    parts = shard_balanced(sizes, 3)
    flat = sorted(i for p in parts for i in p)
    assert flat == list(range(len(sizes)))
    loads = [sum(sizes[i] for i in p) for p in parts]
    assert max(loads) - min(loads) <= max(sizes)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, sizes, q):
    import torch.distributed as dist

    from sph_seepage_flows_gb300 import replicas
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    mine = replicas.shard_balanced(sizes, world)[rank]
    local_particles = sum(sizes[i] for i in mine)
    t = replicas.reduce_timing(0.5 + rank)
    stats = replicas.gather_stats({"rank": rank, "scenes": mine, "particles": local_particles})
    if rank == 0:
        q.put((t, stats))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_gloo_replicas():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    sizes = [5000, 9000, 3000, 12000, 7000]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, sizes, q)) for r in range(2)]
    for p in procs:
        p.start()
    t, stats = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert t == pytest.approx(1.5)
    assert [s["rank"] for s in stats] == [0, 1]
    seen = sorted(i for s in stats for i in s["scenes"])
    assert seen == list(range(len(sizes)))
    assert sum(s["particles"] for s in stats) == sum(sizes)
