"""CPU tests of the library's BVH build and traversal logic: tests/cpp/bvh_harness.cpp runs the same
host/device functions the CUDA kernels wrap (LBVH, 8-wide collapse with verified 8-bit quantisation,
two-level watertight closest-hit traversal) serially on the host; results must agree with the FP64
oracle (hit/miss and entity exact off the oracle's ambiguity band, distance within 1e-5 relative)."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from robotecgpulidar_gb300 import scenes

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "bvh_harness.cpp")
OUT = os.path.join(ROOT, "tests", "cpp", "_build", "libbvh_harness.so")


@pytest.fixture(scope="module")
def harness():
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    if not os.path.exists(OUT) or os.path.getmtime(OUT) < max(
        os.path.getmtime(p) for p in [SRC] + [os.path.join(ROOT, "robotecgpulidar_gb300", "csrc", f)
                                            for f in ("bvh_core.hpp", "trace_core.hpp", "rgl_math.hpp", "device_types.hpp")]
    ):
        cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
        subprocess.run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off",
                        "-I", os.path.join(ROOT, "robotecgpulidar_gb300", "csrc"), "-I", os.path.join(cuda, "include"),
                        "-o", OUT, SRC], check=True)
    return C.CDLL(OUT)


def cast(h, scene, rays, tmax):
    ms = scene.meshes
    vp = (C.c_void_p * len(ms))(*[m.vertices.ctypes.data for m in ms])
    ip = (C.c_void_p * len(ms))(*[m.indices.ctypes.data for m in ms])
    nv = np.array([m.vertices.shape[0] for m in ms], np.int32)
    nt = np.array([m.indices.shape[0] for m in ms], np.int32)
    im = np.array([e.mesh for e in scene.entities], np.int32)
    tf = np.ascontiguousarray(np.stack([e.transform for e in scene.entities]).astype(np.float32))
    ids = np.array([e.entity_id for e in scene.entities], np.int32)
    o = rays[:, :, 3]
    d = (rays[:, :, 2] + rays[:, :, 3]) - rays[:, :, 3]
    wr = np.ascontiguousarray(np.concatenate([o, d, np.full((len(o), 1), tmax, np.float32)], axis=1).astype(np.float32))
    n = wr.shape[0]
    t = np.zeros(n, np.float32)
    inst = np.zeros(n, np.int32)
    prim = np.zeros(n, np.int32)
    p = lambda a: a.ctypes.data_as(C.c_void_p)
    r = h.harness_cast(len(ms), vp, p(nv), ip, p(nt), len(scene.entities), p(im), p(tf), p(ids), n, p(wr), p(t), p(inst), p(prim))
    assert r >= 0, "traversal stack overflow"
    return t, inst, np.linalg.norm(d.astype(np.float64), axis=1), ids


@pytest.mark.parametrize("which", ["plain", "million"])
def test_harness_matches_oracle(harness, oracle, which):
    if which == "plain":
        scene, rays, pose = scenes.plain_scene(), scenes.lidar_rays(32, 1024), scenes.translation(0, 0, 1.8)
    else:
        scene, rays, pose = scenes.million_scene(), scenes.lidar_rays(64, 256), scenes.translation(0, 0, 8.0)
    world = oracle.transform_rays(pose, rays)
    t, inst, dlen, ids = cast(harness, scene, world, 100.0)
    o = oracle.OracleScene(scene).raytrace(rays, ray_transform=pose, ranges=[[0.0, 100.0]])
    amb = o["ambiguous"] != 0
    hit = inst >= 0
    ent = np.where(hit, ids[np.maximum(inst, 0)], 0)
    mism = (hit != (o["is_hit"] == 1)) | (ent != o["entity_id"])
    assert not (mism & ~amb).any()
    both = hit & (o["is_hit"] == 1) & ~amb
    rel = np.abs(t[both] * dlen[both] - o["distance"][both]) / o["distance"][both]
    assert rel.max() <= 1e-5


def test_harness_single_triangle_and_degenerate(harness):
    tri = scenes.Mesh(np.array([[-1, -1, 5], [1, -1, 5], [0, 1, 5]], np.float32), np.array([[0, 1, 2]], np.int32))
    sc = scenes.Scene([tri], [scenes.Entity(0, scenes.translation(0, 0, 0), 7)])
    rays = np.stack([scenes.translation(0, 0, 0), scenes.translation(5, 5, 0)])
    t, inst, dlen, _ = cast(harness, sc, rays, 100.0)
    assert inst[0] == 0 and t[0] == np.float32(5.0)
    assert inst[1] == -1


def test_axis_parallel_rays_stay_cheap(harness):
    """Rays with exact-zero direction components (azimuth 0/90/180/270 deg, vertical rays) must not
    degrade into visiting the whole BVH: the slab test keeps such axes exact."""
    scene = scenes.million_scene()
    rays = scenes.lidar_rays(16, 4)  # azimuths 0, 90, 180, 270 deg
    straight_down = scenes.rotation_xyz(np.pi, 0, 0)  # local +Z -> world -Z
    rays = np.concatenate([rays, straight_down[None]])
    rays[:, :, 3] = (0.0, 0.0, 6.0)
    cast(harness, scene, rays, 100.0)
    assert harness.harness_max_node_visits() < 3000
