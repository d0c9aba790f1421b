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


def load_harness():
    """Builds tests/cpp/bvh_harness.cpp (when older than its sources) and loads it."""
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


@pytest.fixture(scope="module")
def harness():
    return load_harness()


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


def cast_world(h, scene, o, d, tmax, group=0):
    """Casts world rays (origin o[i], direction d[i]) with the harness; group > 0 walks groups of that
    many consecutive rays (shared origin) as packets."""
    ms = scene.meshes
    vp = (C.c_void_p * len(ms))(*[m.vertices.ctypes.data for m in ms])
    ip = (C.c_void_p * len(ms))(*[m.indices.ctypes.data for m in ms])
    nv = np.array([m.vertices.shape[0] for m in ms], np.int32)
    nt = np.array([m.indices.shape[0] for m in ms], np.int32)
    im = np.array([e.mesh for e in scene.entities], np.int32)
    tf = np.ascontiguousarray(np.stack([e.transform for e in scene.entities]).astype(np.float32))
    ids = np.array([e.entity_id for e in scene.entities], np.int32)
    wr = np.ascontiguousarray(np.concatenate([o, d, np.full((len(o), 1), tmax)], axis=1).astype(np.float32))
    n = wr.shape[0]
    t, inst, prim = np.zeros(n, np.float32), np.zeros(n, np.int32), np.zeros(n, np.int32)
    p = lambda a: a.ctypes.data_as(C.c_void_p)
    h.harness_set_packet_group(group)
    try:
        r = h.harness_cast(len(ms), vp, p(nv), ip, p(nt), len(scene.entities), p(im), p(tf), p(ids), n, p(wr), p(t), p(inst), p(prim))
    finally:
        h.harness_set_packet_group(0)
    assert r >= 0, "traversal stack overflow"
    return t, inst, prim


def beams_with_subrays(n_beams, group, spread_rad, seed):
    """n_beams beams from one sensor position, each with `group` sub-rays within spread_rad of the
    beam direction; sub-rays of a beam share the origin bit for bit."""
    rng = np.random.default_rng(seed)
    o = np.repeat(rng.uniform(-20, 20, size=(n_beams, 3)).astype(np.float32) * np.float32([1, 1, 0.1]) + np.float32([0, 0, 4]), group, 0)
    az = rng.uniform(-np.pi, np.pi, n_beams)
    el = rng.uniform(-0.5, 0.2, n_beams)
    d0 = np.stack([np.cos(el) * np.cos(az), np.cos(el) * np.sin(az), np.sin(el)], 1)
    jit = rng.normal(size=(n_beams, group, 3)) * spread_rad
    jit[:, 0] = 0.0
    d = (d0[:, None, :] + jit).reshape(-1, 3).astype(np.float32)
    return o, d


@pytest.mark.parametrize("group,spread", [(5, 0.0017), (5, 0.3), (3, 0.0017), (8, 0.5), (7, 0.002), (1, 0.0)])
def test_packets_equal_single_rays_bit_for_bit(harness, group, spread):
    """A beam's sub-rays walked together (the packet kernel) hit exactly what each ray hits alone:
    same t bits, instance and triangle, including mixed-octant packets (wide spreads) and packets
    with unused slots (3 of 4, 7 of 8)."""
    scene = scenes.million_scene(seed=7, instances=24, spheres=3, cells=96, extent=80.0)
    o, d = beams_with_subrays(2000, group, spread, seed=group * 100 + int(spread * 1000))
    single = cast_world(harness, scene, o, d, 60.0)
    packet = cast_world(harness, scene, o, d, 60.0, group=group)
    assert np.array_equal(single[0].view(np.uint32), packet[0].view(np.uint32))
    assert np.array_equal(single[1], packet[1])
    assert np.array_equal(single[2], packet[2])
    assert (single[1] >= 0).mean() > 0.3


def test_packets_resolve_ties_like_single_rays(harness):
    """Rays straight down onto shared terrain vertices hit several triangles at the same t; the
    closest-hit order (t, then instance, then triangle) picks the same one in both traversals."""
    scene = scenes.plain_scene()
    xs = np.arange(-10.0, 10.0, 2.0, dtype=np.float32)
    pts = np.array([(x, y, 30.0) for x in xs for y in xs], np.float32)
    group = 4
    o = np.repeat(pts, group, 0)
    d = np.tile(np.array([[0, 0, -1], [1e-3, 0, -1], [0, -1e-3, -1], [0, 0, -1]], np.float32), (len(pts), 1))
    single = cast_world(harness, scene, o, d, 100.0)
    packet = cast_world(harness, scene, o, d, 100.0, group=group)
    assert np.array_equal(single[0].view(np.uint32), packet[0].view(np.uint32))
    assert np.array_equal(single[1], packet[1]) and np.array_equal(single[2], packet[2])
