"""One rank of the two-rank sharding test (launched by tests/test_multirank.py through
torch.distributed.run with the gloo backend): casts its beam shard of a lidar scan with the CPU
oracle, compacts by is-hit, takes its global offset from the one all-gather of counts and writes
its part of the global output to <out_dir>/rank<r>.npz."""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def main(out_dir):
    import torch.distributed as dist

    import pyoracle
    from robotecgpulidar_gb300 import rgl, scenes, shard

    dist.init_process_group("gloo")
    rank, world = dist.get_rank(), dist.get_world_size()
    rays = scenes.lidar_rays(16, 256)
    lo, hi = shard.shard_range(rays.shape[0], world, rank)
    osc = pyoracle.OracleScene(scenes.plain_scene())
    res = osc.raytrace(rays[lo:hi], ray_transform=scenes.translation(0, 0, 1.8), ranges=[[0.1, 100.0]],
                       return_mode=rgl.RGL_RETURN_FIRST, threads=2)
    keep = res["is_hit"] != 0
    xyz, dist_ = res["xyz"][keep], res["distance"][keep]
    offset, total = shard.exclusive_offsets(int(keep.sum()))
    np.savez(os.path.join(out_dir, f"rank{rank}.npz"), xyz=xyz, dist=dist_, offset=offset, total=total, lo=lo, hi=hi)
    dist.barrier()
    dist.destroy_process_group()


if __name__ == "__main__":
    main(sys.argv[1])
