"""Scene sharding for runs on several GPUs (one process per GPU).

The substep has no data-path exchange between independent scenes, so N GPUs
run N independent replicas or disjoint subsets of a scene list; ranks only
meet for a barrier and for reducing timings and statistics (torch.distributed,
NCCL on GPUs, gloo on CPU).
"""

from __future__ import annotations


def shard_balanced(sizes, world: int) -> list:
    """Assign items to ranks, largest first, each to the least-loaded rank
    (ties to the lowest rank). Returns one list of item indices per rank."""
    order = sorted(range(len(sizes)), key=lambda i: (-sizes[i], i))
    load = [0] * world
    out = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        out[r].append(i)
        load[r] += sizes[i]
    return [sorted(x) for x in out]


def local_scenes(scenes, rank: int, world: int):
    """The scenes of this rank under shard_balanced (by particle count)."""
    idx = shard_balanced([s.n for s in scenes], world)[rank]
    return [scenes[i] for i in idx], idx


def reduce_timing(elapsed_s: float, device=None) -> float:
    """Max over ranks of a wall/device time (the whole-job time)."""
    import torch
    import torch.distributed as dist
    if not dist.is_initialized() or dist.get_world_size() == 1:
        return float(elapsed_s)
    t = torch.tensor([float(elapsed_s)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def gather_stats(stats: dict) -> list:
    """All ranks' statistics dicts, in rank order."""
    import torch.distributed as dist
    if not dist.is_initialized() or dist.get_world_size() == 1:
        return [stats]
    out = [None] * dist.get_world_size()
    dist.all_gather_object(out, stats)
    return out
