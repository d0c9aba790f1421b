"""CPU tests: the oracle against the reference's own known answers, Philox known-answer vectors and
the semantics it restates. No GPU needed."""
import json
import math
import os

import numpy as np
import pytest

from robotecgpulidar_gb300 import rgl, scenes

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_values.json")))
CUBE = scenes.cube_mesh(1.0)


def cube_world(oracle, transforms, ids=None):
    s = oracle.OracleScene()
    m = s.add_mesh(CUBE.vertices, CUBE.indices)
    for k, tf in enumerate(transforms):
        s.add_instance(m, tf, rgl.RGL_DEFAULT_ENTITY_ID if ids is None or ids[k] is None else ids[k])
    s.build()
    return s


@pytest.mark.parametrize("z", GOLD["distance_field_cube_z"])
def test_distance_to_cube_face_is_exact(oracle, z):
    z = np.float32(z)
    o = cube_world(oracle, [scenes.translation(0, 0, z)]).raytrace([scenes.translation(0, 0, 0)], ranges=[[0, z + 10]])
    assert o["distance"][0] == np.float32(z - np.float32(1.0))
    assert np.float32(np.linalg.norm(o["xyz"][0])) == o["distance"][0]


def test_origin_on_face_and_inside(oracle):
    o = cube_world(oracle, [scenes.translation(0, 0, 1.0)]).raytrace([scenes.translation(0, 0, 0)], ranges=[[0, 11]])
    assert o["distance"][0] == 2.0
    z = np.float32(-0.001)
    o = cube_world(oracle, [scenes.translation(0, 0, z)]).raytrace([scenes.translation(0, 0, 0)], ranges=[[0, 10]])
    assert o["distance"][0] == np.float32(np.float32(1.0) + z)


@pytest.mark.parametrize("z", GOLD["distance_field_cube_z"])
def test_range_gating(oracle, z):
    z = np.float32(z)
    w = cube_world(oracle, [scenes.translation(0, 0, z)])
    assert np.isinf(w.raytrace([scenes.translation(0, 0, 0)], ranges=[[0, z - 2]])["distance"][0])
    assert np.isinf(w.raytrace([scenes.translation(0, 0, 0)], ranges=[[z + 2, z + 3]])["distance"][0])
    w2 = cube_world(oracle, [scenes.translation(0, 0, z), scenes.translation(0, 0, z + 10)])
    out = w2.raytrace([scenes.translation(0, 0, 0)], ranges=[[z + 2, z + 12]])
    assert np.isinf(out["distance"][0]) and out["is_hit"][0] == 0


def test_nonhit_xyz_rule(oracle):
    w = cube_world(oracle, [scenes.translation(0, 0, 0)])
    rays = scenes.lidar_rays(7, 12, -90, 90)
    out = w.raytrace(rays, ranges=[[2.0, 3.0]], near=12.34, far=0.0)
    assert np.all(out["is_hit"] == 0) and np.all(out["distance"] == np.float32(12.34))
    d = rays[:, :, 2].astype(np.float64)
    assert np.allclose(out["xyz"], d / np.linalg.norm(d, axis=1, keepdims=True) * 12.34, atol=1e-5)
    far = cube_world(oracle, []).raytrace(rays[:3], near=0.0, far=13.24)
    assert np.all(far["distance"] == np.float32(13.24))
    inf = cube_world(oracle, []).raytrace([scenes.translation(0, 0, 0)])
    assert np.isinf(inf["distance"][0]) and np.all(np.isfinite(inf["xyz"][0][:2]))  # NaN components -> 0


def test_entity_id_and_default(oracle):
    w = cube_world(oracle, [scenes.translation(6, -5, 0), scenes.translation(6, 0, 0), scenes.translation(6, 5, 0)], [1, 2, None])
    out = w.raytrace(scenes.lidar_rays(50, 500, -90, 90))
    hit = out["is_hit"] == 1
    y = out["xyz"][:, 1]
    assert np.all(out["entity_id"][~hit] == 0)
    assert np.all(out["entity_id"][hit & (y < -2.5)] == 1)
    assert np.all(out["entity_id"][hit & (y > 2.5)] == rgl.RGL_DEFAULT_ENTITY_ID)


def test_readme_example(oracle):
    out = cube_world(oracle, [scenes.translation(0, 0, 5)]).raytrace([scenes.translation(0, 0, 0)])
    assert out["xyz"][0, 2] == GOLD["readme_hit_z"]


def test_mat3x4_multiplication_gold(oracle):
    g = GOLD["mat3x4_mul"]
    lhs = np.array(g["lhs"], np.float32).reshape(3, 4)
    rhs = np.array(g["rhs"], np.float32).reshape(1, 3, 4)
    assert np.array_equal(oracle.transform_rays(lhs, rhs)[0].ravel(), np.array(g["gold"], np.float32))


def test_philox_known_answers(oracle):
    # Known-answer vectors of Philox4x32-10 published with Random123 (Salmon et al., SC'11).
    kat = [
        ((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
        ((0xFFFFFFFF,) * 4, (0xFFFFFFFF, 0xFFFFFFFF), (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
        ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
         (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
    ]
    for ctr, key, want in kat:
        assert tuple(int(x) for x in oracle.philox(ctr, key)) == want


def test_normals_are_standard(oracle):
    from scipy import stats

    n = oracle.normals(1234, 3, 0, 200000)
    assert abs(n.mean()) < 0.01 and abs(n.std() - 1.0) < 0.01
    assert stats.kstest(n, "norm").pvalue > 1e-3
    assert not np.array_equal(n, oracle.normals(1234, 3, 1, 200000))


def test_distance_noise_statistics(oracle):
    # Reference DistanceFieldTest.cpp:278-327: mean shift and sigma = base + rise * d within 0.002.
    g = GOLD["distance_noise"]
    n = 100000
    d0 = 3.0
    xyz = np.tile(np.array([[0, 0, d0]], np.float32), (n, 1))
    dist = np.full(n, d0, np.float32)
    eye = np.eye(4)[:3]
    ox, od = oracle.noise_distance(eye, g["mean"], g["st_dev"], g["st_dev_per_meter"], 99, 0, xyz, dist)
    assert abs(od.mean() - (d0 + g["mean"])) < GOLD["noise_epsilon"]
    assert abs(od.std() - (g["st_dev"] + d0 * g["st_dev_per_meter"])) < GOLD["noise_epsilon"]
    assert np.allclose(np.linalg.norm(ox, axis=1), od, atol=2e-6)


def test_angular_hitpoint_noise_keeps_range(oracle):
    n = 20000
    rng = np.random.default_rng(3)
    xyz = rng.normal(size=(n, 3)).astype(np.float32) * 10
    look = oracle.inv34(scenes.trs((1, 2, 3), (0.1, 0.2, 0.3)))
    ox, od = oracle.noise_angular_hitpoint(look, 0.0, math.radians(1.0), rgl.RGL_AXIS_Z, 5, 0, xyz)
    local = (oracle.mat4(look) @ np.c_[xyz, np.ones(n)].T).T[:, :3]
    assert np.allclose(np.linalg.norm(local, axis=1), od, rtol=1e-5)


@pytest.mark.parametrize("n", GOLD["point_counts"])
def test_compaction_semantics(oracle, n):
    rng = np.random.default_rng(n)
    flags = rng.integers(0, 2, n).astype(np.int32)
    xyz = rng.normal(size=(n, 3)).astype(np.float32)
    out = oracle.compact(flags, xyz)
    assert np.array_equal(out, xyz[flags != 0])
    assert oracle.compact(np.zeros(n, np.int32), xyz).shape[0] == 0


def test_format_semantics(oracle):
    n = 5
    xyz = np.arange(15, dtype=np.float32).reshape(5, 3)
    d = np.arange(5, dtype=np.float32)
    out = oracle.format_points([xyz, None, d], [12, 4, 4], n).reshape(n, 20)
    assert np.array_equal(out[:, :12].copy().view(np.float32), xyz)
    assert np.array_equal(out[:, 16:].copy().view(np.float32).ravel(), d)


def test_beam_sample_pattern(oracle):
    t = oracle.beam_samples(math.radians(0.2), math.radians(0.2), 3, 19)
    assert t.shape[0] == 58
    assert np.array_equal(t[0], scenes.translation(0, 0, 0))
    # Outer ring at the full half-divergence, layer 2 at one third of it.
    z = t[:, :, 2].astype(np.float64)
    ang = np.degrees(np.arcsin(np.hypot(z[:, 0], z[:, 1])))
    assert np.allclose(ang[1:20], 0.1, atol=1e-4)
    assert np.allclose(ang[39:58], 0.1 / 3, atol=1e-4)
    assert oracle.beam_samples(0.0, 0.0, 3, 19).shape[0] == 1
    assert oracle.beam_samples(math.radians(0.2), math.radians(0.2), 1, 4).shape[0] == 5
