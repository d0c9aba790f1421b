"""Sharding of a lidar scan across GPUs (one process per GPU, torch.distributed for the host side).

Rays are independent, so a scan shards by contiguous beam ranges (or whole sensors / requests) with
the scene replicated on every GPU; no traversal data crosses GPUs. The only exchange is for
compaction: every shard keeps its hit points in beam order, and the global output offset of shard r
is the exclusive prefix sum of the shards' hit counts, obtained with one all-gather of one int64 per
rank. Concatenating the shards' compacted points at those offsets gives exactly the compaction of
the whole scan (compaction is order preserving and shards are contiguous in beam order).

The reference (RobotecGPULidar) runs on one GPU and has no distributed layer; this module is the
host-side plan for running its lidar path on several GPUs.
"""
from __future__ import annotations

import numpy as np


def shard_range(n_units: int, world: int, rank: int) -> tuple[int, int]:
    """Contiguous [start, end) of `n_units` for `rank` of `world`; sizes differ by at most one."""
    if world <= 0 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside world of size {world}")
    base, extra = divmod(n_units, world)
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def sensor_assignment(sensor_beams, world: int) -> list[list[int]]:
    """Whole sensors per rank (greedy largest-first onto the least-loaded rank), for batched frames
    whose sensors should not be split."""
    loads = [0] * world
    out = [[] for _ in range(world)]
    for i in sorted(range(len(sensor_beams)), key=lambda k: -sensor_beams[k]):
        r = int(np.argmin(loads))
        out[r].append(i)
        loads[r] += int(sensor_beams[i])
    return [sorted(x) for x in out]


def exclusive_offsets(local_count: int, group=None) -> tuple[int, int]:
    """(offset of this rank's compacted points in the global output, global count): one all-gather
    of one int64 per rank."""
    import torch
    import torch.distributed as dist

    world = dist.get_world_size(group)
    t = torch.tensor([int(local_count)], dtype=torch.int64)
    got = [torch.zeros(1, dtype=torch.int64) for _ in range(world)]
    dist.all_gather(got, t, group=group)
    counts = [int(x.item()) for x in got]
    rank = dist.get_rank(group)
    return sum(counts[:rank]), sum(counts)


def place(global_buffer: np.ndarray, offset: int, local: np.ndarray) -> None:
    """Writes this shard's compacted points at its global offset."""
    global_buffer[offset : offset + len(local)] = local
