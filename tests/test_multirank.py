"""Multi-GPU sharding logic (robotecgpulidar_gb300/shard.py) on CPU: shard ranges and sensor
assignment, and a two-rank gloo run whose compacted shards, placed at the offsets from the one
all-gather of counts, reproduce the unsharded compaction exactly."""
import os
import socket
import subprocess
import sys

import numpy as np
import pytest

from robotecgpulidar_gb300 import shard

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("n,world", [(0, 2), (1, 2), (7, 3), (4096, 2), (262144, 8), (5, 8)])
def test_shard_ranges_partition_the_units(n, world):
    ranges = [shard.shard_range(n, world, r) for r in range(world)]
    assert ranges[0][0] == 0 and ranges[-1][1] == n
    assert all(a[1] == b[0] for a, b in zip(ranges, ranges[1:]))
    sizes = [e - s for s, e in ranges]
    assert max(sizes) - min(sizes) <= 1


def test_shard_range_rejects_bad_rank():
    with pytest.raises(ValueError):
        shard.shard_range(10, 2, 2)


def test_sensor_assignment_covers_and_balances():
    beams = [28800, 32768, 131072, 262144, 76800] * 13
    parts = shard.sensor_assignment(beams, 4)
    assert sorted(i for p in parts for i in p) == list(range(len(beams)))
    loads = [sum(beams[i] for i in p) for p in parts]
    assert max(loads) - min(loads) <= max(beams)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_rank_sharded_compaction_equals_unsharded(tmp_path, oracle):
    from robotecgpulidar_gb300 import rgl, scenes

    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2", "--master-addr", "127.0.0.1",
           "--master-port", str(_free_port()), os.path.join(ROOT, "tests", "shard_worker.py"), str(tmp_path)]
    env = dict(os.environ, OMP_NUM_THREADS="1")
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    parts = [np.load(tmp_path / f"rank{k}.npz") for k in range(2)]
    total = int(parts[0]["total"])
    assert total == int(parts[1]["total"])
    assert int(parts[0]["offset"]) == 0 and int(parts[1]["offset"]) == len(parts[0]["dist"])
    xyz = np.zeros((total, 3), np.float32)
    dist = np.zeros(total, np.float32)
    for p in parts:
        shard.place(xyz, int(p["offset"]), p["xyz"])
        shard.place(dist, int(p["offset"]), p["dist"])
    full = oracle.OracleScene(scenes.plain_scene()).raytrace(scenes.lidar_rays(16, 256), ray_transform=scenes.translation(0, 0, 1.8),
                                                             ranges=[[0.1, 100.0]], return_mode=rgl.RGL_RETURN_FIRST, threads=2)
    keep = full["is_hit"] != 0
    assert np.array_equal(xyz, full["xyz"][keep]) and np.array_equal(dist, full["distance"][keep])
