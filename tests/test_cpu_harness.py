"""CPU tests of the library's BVH build and traversal logic: tests/cpp/bvh_harness.cpp runs the same
host/device functions the CUDA kernels wrap (LBVH, 8-wide collapse with verified 8-bit quantisation,
two-level watertight closest-hit traversal) serially on the host; results must agree with the FP64
oracle (hit/miss and entity exact off the oracle's ambiguity band, distance within 1e-5 relative)."""
import ctypes as C
import math
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
                                            for f in ("bvh_core.hpp", "trace_core.hpp", "rgl_math.hpp", "device_types.hpp", "wave_split.hpp")]
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


def warp_lane_use(work_per_beam, order, beams_per_warp=6, lanes=32):
    """Share of a warp's lane slots doing work when `beams_per_warp` beams of `work_per_beam.shape[1]`
    sub-rays (one lane each) run until the warp's longest ray ends, beams taken in `order`."""
    w = work_per_beam[order]
    m = (len(w) // beams_per_warp) * beams_per_warp
    g = w[:m].reshape(-1, beams_per_warp * w.shape[1])
    return g.sum() / (lanes * g.max(axis=1)).sum()


def test_scan_row_order_groups_similar_work(harness):
    """Beams of one elevation at neighbouring azimuths do similar traversal work, so the scan-row
    visiting order (elevation, then azimuth: the graph runs' default) keeps more of a warp's lanes busy
    than a spinning lidar's given order (one azimuth's channels from the ground to the sky). Work per
    ray is the host traversal's node visits plus triangle tests; 5 sub-rays per beam on a ring of
    0.1 degrees, 6 beams per warp, as the device runs them."""
    scene = scenes.million_scene()
    pose = scenes.translation(0, 0, 6.0)
    world = np.einsum("ij,njk->nik", pose[:, :3].astype(np.float64), scenes.lidar_rays(64, 512).astype(np.float64))
    world[:, :, 3] += pose[:, 3]
    o = world[:, :, 3]
    d = world[:, :, 2] / np.linalg.norm(world[:, :, 2], axis=1, keepdims=True)
    a = np.where(np.abs(d[:, 2:3]) < 0.9, np.array([[0.0, 0.0, 1.0]]), np.array([[1.0, 0.0, 0.0]]))
    u = np.cross(d, a)
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    v = np.cross(d, u)
    half = math.radians(0.1)
    subs = [d] + [d + half * (math.cos(2 * math.pi * k / 4) * u + math.sin(2 * math.pi * k / 4) * v) for k in range(4)]
    n = len(d)
    rays = np.zeros((n * 5, 3, 4), np.float32)
    rays[:, :, 3] = np.repeat(o, 5, axis=0)
    rays[:, :, 2] = np.stack(subs, axis=1).reshape(-1, 3)
    cast(harness, scene, rays, 100.0)
    visits = np.zeros(n * 5, np.int32)
    tris = np.zeros(n * 5, np.int32)
    harness.harness_ray_work(visits.ctypes.data_as(C.c_void_p), tris.ctypes.data_as(C.c_void_p), n * 5)
    work = (visits + tris).reshape(n, 5)
    assert work.min() > 0
    # Scan-row key: sine of the elevation (11 bits), then a pseudo-angle of the azimuth (11 bits).
    l1 = np.abs(d[:, 0]) + np.abs(d[:, 1])
    pa = np.where(l1 > 0, 1.0 - d[:, 0] / np.maximum(l1, 1e-30), 0.0)
    az = np.where(d[:, 1] < 0, -pa, pa)
    q = lambda c: np.clip((c * 2048).astype(np.int64), 0, 2047)
    key = (q(d[:, 2] * 0.5 + 0.5) << 11) | q(az * 0.25 + 0.5)
    given = warp_lane_use(work, np.arange(n))
    rows = warp_lane_use(work, np.argsort(key, kind="stable"))
    assert rows > given + 0.03, (given, rows)


def split_waves(h, rays, waves):
    r = np.ascontiguousarray(rays, np.int64)
    out = np.zeros(len(r) + 2, np.int32)
    w = h.harness_split_waves(r.ctypes.data_as(C.c_void_p), len(r), waves, out.ctypes.data_as(C.c_void_p))
    return [int(x) for x in out[:w + 1]]


def test_wave_cut_of_batched_frames(harness):
    """Batched frames cut their sensors, in order, into contiguous waves of about equal rays; never more
    waves than sensors, none empty, and a heavy sensor closes its wave early."""
    assert split_waves(harness, [100] * 8, 4) == [0, 2, 4, 6, 8]
    assert split_waves(harness, [100] * 8, 1) == [0, 8]
    assert split_waves(harness, [100] * 3, 9) == [0, 1, 2, 3]  # capped at the sensor count
    assert split_waves(harness, [1000, 1, 1, 1, 1, 1], 3) == [0, 1, 2, 6]  # the heavy first sensor alone
    assert split_waves(harness, [1, 1, 1, 1, 1, 1000], 3) == [0, 4, 5, 6]  # later waves keep a sensor each
    assert split_waves(harness, [0, 0, 0, 0], 2) == [0, 1, 4]
    rng = np.random.default_rng(4)
    for _ in range(200):
        n = int(rng.integers(1, 40))
        rays = rng.integers(1, 1 << 20, size=n)
        W = int(rng.integers(1, 20))
        first = split_waves(harness, rays, W)
        waves = min(W, n)
        assert first[0] == 0 and first[-1] == n and len(first) - 1 == waves
        assert all(b > a for a, b in zip(first, first[1:]))
        # Each wave but the last ends once its running total reaches its share, or when exactly one
        # sensor is left for each later wave.
        cum = np.cumsum(rays)
        for w, end in enumerate(first[1:-1]):
            assert cum[end - 1] * waves >= cum[-1] * (w + 1) or n - end == waves - (w + 1)
