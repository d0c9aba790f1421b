"""Point nodes through the C API on the GPU against the oracle.

Compaction and format must be bit-exact (reference CompactByFieldPointsNodeTest.cpp:86-177,
FormatPointsNodeTest.cpp:79-334); transforms bit-exact (same float operation order as the reference's
Mat3x4f); noise value-by-value against the oracle's Philox/Box-Muller restatement within 1e-5
(relative to the coordinate magnitude), reproducible for a fixed seed, and statistically matching
the reference's own noise tests (DistanceFieldTest.cpp:278-327, mean and sigma within 0.002).
"""
import ctypes as C
import json
import math
import os

import numpy as np
import pytest

from robotecgpulidar_gb300 import scenes

pytestmark = pytest.mark.gpu
GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_values.json")))


def point_cloud(rgl, n, hits, rng):
    """AoS point array with XYZ, PADDING_32, IS_HIT, DISTANCE, ENTITY_ID fields."""
    fields = [rgl.RGL_FIELD_XYZ_VEC3_F32, rgl.RGL_FIELD_PADDING_32, rgl.RGL_FIELD_IS_HIT_I32, rgl.RGL_FIELD_DISTANCE_F32,
              rgl.RGL_FIELD_ENTITY_ID_I32]
    dt = np.dtype([("xyz", np.float32, 3), ("pad", np.uint32), ("hit", np.int32), ("dist", np.float32), ("ent", np.int32)])
    a = np.zeros(n, dt)
    a["xyz"] = rng.normal(size=(n, 3)).astype(np.float32) * 20
    a["pad"] = 0xDEADBEEF
    a["hit"] = hits
    a["dist"] = np.linalg.norm(a["xyz"], axis=1)
    a["ent"] = rng.integers(1, 1000, n)
    node = rgl.node()
    rgl.points_from_array(node, a, n, fields)
    return node, a


@pytest.mark.parametrize("n", GOLD["point_counts"])
@pytest.mark.parametrize("kind", ["none", "all", "random"])
def test_compaction_matches_oracle(rgl, oracle, n, kind):
    rng = np.random.default_rng(n)
    hits = {"none": np.zeros(n), "all": np.ones(n), "random": rng.integers(0, 2, n)}[kind].astype(np.int32)
    src, a = point_cloud(rgl, n, hits, rng)
    cmp = rgl.node()
    rgl.points_compact_by_field(cmp)
    rgl.add_child(src, cmp)
    rgl.graph_run(src)
    cnt, size = rgl.result_size(cmp, rgl.RGL_FIELD_XYZ_VEC3_F32)
    assert cnt == int(hits.sum()) and size == 12
    assert np.array_equal(rgl.result(cmp, rgl.RGL_FIELD_XYZ_VEC3_F32), oracle.compact(hits, a["xyz"]))
    assert np.array_equal(rgl.result(cmp, rgl.RGL_FIELD_ENTITY_ID_I32), oracle.compact(hits, a["ent"]))
    assert np.array_equal(rgl.result(cmp, rgl.RGL_FIELD_DISTANCE_F32), oracle.compact(hits, a["dist"]))


def test_compaction_leaves_caller_buffer_untouched_when_empty(rgl):
    src, _ = point_cloud(rgl, 100, np.zeros(100, np.int32), np.random.default_rng(0))
    cmp = rgl.node()
    rgl.points_compact_by_field(cmp)
    rgl.add_child(src, cmp)
    rgl.graph_run(src)
    out = np.array([[2, 3, 5], [7, 11, 13], [17, 19, 23]], np.float32)
    keep = out.copy()
    assert rgl.result_size(cmp, rgl.RGL_FIELD_XYZ_VEC3_F32) == (0, 12)
    rgl.check(rgl.lib().rgl_graph_get_result_data(cmp, rgl.RGL_FIELD_XYZ_VEC3_F32, rgl.ptr(out)))
    assert np.array_equal(out, keep)


@pytest.mark.parametrize("n", GOLD["point_counts"])
def test_chained_compactions(rgl, oracle, n):
    rng = np.random.default_rng(n + 1)
    hits = rng.integers(0, 2, n).astype(np.int32)
    src, a = point_cloud(rgl, n, hits, rng)
    nodes = [rgl.node() for _ in range(GOLD["chained_compactions"])]
    for nd in nodes:
        rgl.points_compact_by_field(nd)
    rgl.chain(src, *nodes)
    rgl.graph_run(src)
    assert np.array_equal(rgl.result(nodes[-1], rgl.RGL_FIELD_XYZ_VEC3_F32), oracle.compact(hits, a["xyz"]))


def test_compaction_requires_is_hit(rgl):
    dt = np.dtype([("xyz", np.float32, 3)])
    a = np.zeros(10, dt)
    src = rgl.node()
    rgl.points_from_array(src, a, 10, [rgl.RGL_FIELD_XYZ_VEC3_F32])
    cmp = rgl.node()
    rgl.points_compact_by_field(cmp)
    rgl.add_child(src, cmp)
    assert rgl.lib().rgl_graph_run(src) == rgl.RGL_INVALID_PIPELINE
    assert "IS_HIT_I32" in rgl.last_error()


@pytest.mark.parametrize("n", GOLD["point_counts"])
def test_format_matches_oracle(rgl, oracle, n):
    rng = np.random.default_rng(n + 2)
    src, a = point_cloud(rgl, n, np.ones(n, np.int32), rng)
    fmt_fields = [rgl.RGL_FIELD_XYZ_VEC3_F32, rgl.RGL_FIELD_DISTANCE_F32, rgl.RGL_FIELD_PADDING_16, rgl.RGL_FIELD_ENTITY_ID_I32,
                  rgl.RGL_FIELD_XYZ_VEC3_F32, rgl.RGL_FIELD_PADDING_8]
    fmt = rgl.node()
    rgl.points_format(fmt, fmt_fields)
    rgl.add_child(src, fmt)
    rgl.graph_run(src)
    cnt, size = rgl.result_size(fmt, rgl.RGL_FIELD_DYNAMIC_FORMAT)
    assert cnt == n and size == 12 + 4 + 2 + 4 + 12 + 1
    got = rgl.result_bytes(fmt, rgl.RGL_FIELD_DYNAMIC_FORMAT).reshape(n, size)
    exp = oracle.format_points([a["xyz"], a["dist"], None, a["ent"], a["xyz"], None], [12, 4, 2, 4, 12, 1], n).reshape(n, size)
    data_cols = np.r_[0:16, 18:34]
    assert np.array_equal(got[:, data_cols], exp[:, data_cols])


def test_format_after_compaction_word_aligned(rgl, oracle):
    n = 20000
    rng = np.random.default_rng(9)
    hits = rng.integers(0, 2, n).astype(np.int32)
    src, a = point_cloud(rgl, n, hits, rng)
    cmp, fmt = rgl.node(), rgl.node()
    rgl.points_compact_by_field(cmp)
    rgl.points_format(fmt, [rgl.RGL_FIELD_XYZ_VEC3_F32, rgl.RGL_FIELD_DISTANCE_F32, rgl.RGL_FIELD_ENTITY_ID_I32])
    rgl.chain(src, cmp, fmt)
    rgl.graph_run(src)
    k = int(hits.sum())
    got = rgl.result_bytes(fmt, rgl.RGL_FIELD_DYNAMIC_FORMAT)
    exp = oracle.format_points([oracle.compact(hits, a["xyz"]), oracle.compact(hits, a["dist"]), oracle.compact(hits, a["ent"])],
                               [12, 4, 4], k)
    assert np.array_equal(got, exp)


def test_format_rejects_dynamic_format(rgl):
    f = np.array([rgl.RGL_FIELD_DYNAMIC_FORMAT], np.int32)
    n = rgl.node()
    assert rgl.lib().rgl_node_points_format(C.byref(n), rgl.ptr(f), 1) == rgl.RGL_INVALID_ARGUMENT
    assert "RGL_FIELD_DYNAMIC_FORMAT" in rgl.last_error()


def test_points_transform_bit_exact(rgl, oracle):
    n = 20000
    src, a = point_cloud(rgl, n, np.ones(n, np.int32), np.random.default_rng(3))
    tf = scenes.trs((1.5, -2.0, 0.25), (0.3, -0.2, 1.1), (1.0, 1.0, 1.0))
    node = rgl.node()
    rgl.points_transform(node, tf)
    rgl.add_child(src, node)
    rgl.graph_run(src)
    assert np.array_equal(rgl.result(node, rgl.RGL_FIELD_XYZ_VEC3_F32), oracle.transform_points(tf, a["xyz"]))


def _noise_graph(rgl, kind, n, seed, frame=0, look=None):
    rng = np.random.default_rng(4)
    src, a = point_cloud(rgl, n, np.ones(n, np.int32), rng)
    chain = [src]
    tf_node = None
    if look is not None:
        tf_node = rgl.node()
        rgl.points_transform(tf_node, look)
        chain.append(tf_node)
    node = rgl.node()
    lib = rgl.lib()
    if kind == "angular":
        rgl.check(lib.rgl_node_gaussian_noise_angular_hitpoint(C.byref(node), 0.01, math.radians(2.0), rgl.RGL_AXIS_Z))
    else:
        rgl.check(lib.rgl_node_gaussian_noise_distance(C.byref(node), 0.1, 0.02, 0.001))
    rgl.set_noise_seed(node, seed, frame)
    chain.append(node)
    rgl.chain(*chain)
    return chain[0], node, a


@pytest.mark.parametrize("kind", ["angular", "distance"])
def test_noise_matches_oracle_and_is_reproducible(rgl, oracle, kind):
    n = 20000
    look = scenes.trs((3.0, 1.0, -2.0), (0.2, 0.1, -0.4))
    src, node, a = _noise_graph(rgl, kind, n, seed=1234, look=look)
    rgl.graph_run(src)
    xyz1 = rgl.result(node, rgl.RGL_FIELD_XYZ_VEC3_F32)
    d1 = rgl.result(node, rgl.RGL_FIELD_DISTANCE_F32)
    # frame advanced: different noise
    rgl.graph_run(src)
    xyz2 = rgl.result(node, rgl.RGL_FIELD_XYZ_VEC3_F32)
    assert not np.array_equal(xyz1, xyz2)
    # reset seed/frame: identical bits
    rgl.set_noise_seed(node, 1234, 0)
    rgl.graph_run(src)
    assert np.array_equal(rgl.result(node, rgl.RGL_FIELD_XYZ_VEC3_F32), xyz1)
    # oracle: the input points went through the transform node, whose frame L = tf^-1
    tin = oracle.transform_points(look, a["xyz"])
    L = oracle.inv34(look)
    if kind == "angular":
        ex, ed = oracle.noise_angular_hitpoint(L, 0.01, math.radians(2.0), rgl.RGL_AXIS_Z, 1234, 0, tin)
    else:
        ex, ed = oracle.noise_distance(L, 0.1, 0.02, 0.001, 1234, 0, tin, a["dist"])
    scale = np.maximum(np.abs(ex).max(axis=1), 1.0)
    assert (np.abs(xyz1 - ex).max(axis=1) <= 1e-5 * scale).all()
    assert np.allclose(d1, ed, rtol=1e-5, atol=1e-5)


def test_distance_noise_statistics_match_reference_test(rgl):
    # DistanceFieldTest.cpp:278-327: 100k rays at a cube 3 m away; mean and sigma within 0.002.
    g = GOLD["distance_noise"]
    cube = scenes.cube_mesh(1.0)
    m = rgl.mesh_create(cube.vertices, cube.indices)
    e = rgl.entity_create(m)
    rgl.entity_set_transform(e, scenes.translation(0, 0, 4.0))
    n_rays, n_rng, n_rt, n_noise, n_y = (rgl.node() for _ in range(5))
    rgl.rays_from_mat3x4f(n_rays, np.tile(scenes.translation(0, 0, 0), (100000, 1, 1)))
    rgl.rays_set_range(n_rng, [[0.0, 14.0]])
    rgl.raytrace(n_rt)
    rgl.check(rgl.lib().rgl_node_gaussian_noise_distance(C.byref(n_noise), g["mean"], g["st_dev"], g["st_dev_per_meter"]))
    rgl.points_yield(n_y, [rgl.RGL_FIELD_DISTANCE_F32, rgl.RGL_FIELD_XYZ_VEC3_F32])
    rgl.chain(n_rays, n_rng, n_rt, n_noise, n_y)
    rgl.graph_run(n_rays)
    d = rgl.result(n_y, rgl.RGL_FIELD_DISTANCE_F32).astype(np.float64)
    xyz = rgl.result(n_y, rgl.RGL_FIELD_XYZ_VEC3_F32)
    assert abs(d.mean() - (3.0 + g["mean"])) < GOLD["noise_epsilon"]
    assert abs(d.std() - (3.0 * g["st_dev_per_meter"] + g["st_dev"])) < GOLD["noise_epsilon"]
    assert np.allclose(np.linalg.norm(xyz, axis=1), d, atol=2e-6 * 4)
    from scipy import stats

    z = (d - (3.0 + g["mean"])) / (3.0 * g["st_dev_per_meter"] + g["st_dev"])
    assert stats.kstest(z, "norm").pvalue > 1e-4


def test_angular_ray_noise_matches_oracle_and_is_reproducible(rgl, oracle):
    """rgl_node_gaussian_noise_angular_ray (reference gaussianNoiseKernels.cu:20-29): every ray is
    rotated about the axis of the sensor frame L = (cumulative ray transform)^-1 by mean + sigma * n,
    out = L^-1 R L ray. The oracle applies its FP64 Philox restatement to the same rays and casts
    them; the GPU result must agree within the parity bounds (a wrong draw moves a hit by metres, far
    beyond them) and reproduce bit for bit for the same seed and frame."""
    import accuracy

    scene = scenes.plain_scene()
    rgl.spawn_scene(scene)
    rays = scenes.lidar_rays(32, 512)
    pose = scenes.trs((3.0, -4.0, 1.8), (0.0, 0.0, 0.6))
    mean, sigma = 0.01, math.radians(2.0)
    n = {k: rgl.node() for k in ("rays", "pose", "noise", "range", "trace", "out")}
    rgl.rays_from_mat3x4f(n["rays"], rays)
    rgl.rays_transform(n["pose"], pose)
    rgl.check(rgl.lib().rgl_node_gaussian_noise_angular_ray(C.byref(n["noise"]), mean, sigma, rgl.RGL_AXIS_Z))
    rgl.set_noise_seed(n["noise"], 1234)
    rgl.rays_set_range(n["range"], [[0.1, 100.0]])
    rgl.raytrace(n["trace"])
    fields = [rgl.RGL_FIELD_XYZ_VEC3_F32, rgl.RGL_FIELD_DISTANCE_F32, rgl.RGL_FIELD_ENTITY_ID_I32, rgl.RGL_FIELD_IS_HIT_I32,
              rgl.RGL_FIELD_RETURN_TYPE_U8]
    rgl.points_yield(n["out"], fields)
    rgl.chain(n["rays"], n["pose"], n["noise"], n["range"], n["trace"], n["out"])
    rgl.graph_run(n["rays"])
    got = {f: rgl.result(n["out"], f) for f in fields}
    world = oracle.transform_rays(pose, rays)
    noisy = oracle.noise_angular_ray(oracle.inv34(pose), mean, sigma, rgl.RGL_AXIS_Z, 1234, 0, world)
    exp = oracle.OracleScene(scene).raytrace(noisy, ranges=[[0.1, 100.0]])
    stats, _ = accuracy.evaluate(rgl, got, exp)
    assert stats["mismatches_outside_ambiguity_band"] == 0, stats.get("mismatch_examples")
    assert stats["nonhit_distances_exact"]
    # The draw is computed in FP32 here and in FP64 by the oracle, so each cast ray differs from the
    # oracle's by about 1e-7 rad; a hit at grazing angle g moves along the ray by that times 1/sin(g).
    # Distances must agree within 1e-5 plus 1e-6 / sin(g), sin(g) = cos(incident angle).
    both = (got[rgl.RGL_FIELD_IS_HIT_I32] == 1) & (exp["is_hit"] == 1) & (exp["ambiguous"] == 0)
    de = exp["distance"][both].astype(np.float64)
    rel = np.abs(got[rgl.RGL_FIELD_DISTANCE_F32][both] - de) / de
    graze = np.maximum(np.cos(exp["incident_angle"][both].astype(np.float64)), 1e-3)
    assert (rel <= 1e-5 + 1e-6 / graze).all(), f"max rel {rel.max()}"
    assert np.median(rel) < 1e-6
    assert got[rgl.RGL_FIELD_IS_HIT_I32].sum() > 5000
    # The draw differs from the noiseless scan, advances with the frame and repeats for the same seed.
    clean = oracle.OracleScene(scene).raytrace(world, ranges=[[0.1, 100.0]])
    assert np.abs(got[rgl.RGL_FIELD_DISTANCE_F32] - clean["distance"])[(clean["is_hit"] == 1) & (exp["is_hit"] == 1)].max() > 0.1
    rgl.graph_run(n["rays"])
    second = rgl.result(n["out"], rgl.RGL_FIELD_XYZ_VEC3_F32)
    assert not np.array_equal(second, got[rgl.RGL_FIELD_XYZ_VEC3_F32])
    rgl.set_noise_seed(n["noise"], 1234, 0)
    rgl.graph_run(n["rays"])
    assert np.array_equal(rgl.result(n["out"], rgl.RGL_FIELD_XYZ_VEC3_F32), got[rgl.RGL_FIELD_XYZ_VEC3_F32])


@pytest.mark.parametrize("kind", ["angular_ray", "angular_hitpoint"])
def test_angular_noise_statistics_match_reference_stress_test(rgl, kind):
    """Restates reference test/src/graph/gaussianStressTest.cpp:97-148: 100,000 identical rays from
    (0, 0, 1) along +Z at a cube whose face is 3 m ahead, angular noise (mean 0.1 rad, sigma 0.01 rad
    about Y) on the rays before the raytrace or on the hit points after it, points taken back into the
    lidar frame. The angle atan2(z, x) of each point is pi/2 - (rotation), so its mean and sigma must
    match within 0.002 (the reference's epsilon), the distance field must equal |xyz| within 2e-6
    relative per metre, and a KS test must accept the normal shape. Four runs (frames) instead of
    256."""
    from scipy import stats

    cube = scenes.cube_mesh(1.0)
    e = rgl.entity_create(rgl.mesh_create(cube.vertices, cube.indices))
    rgl.entity_set_transform(e, scenes.translation(0, 0, 5))
    lidar = scenes.translation(0, 0, 1)
    mean, sigma = 0.1, 0.01
    lib = rgl.lib()
    n = {k: rgl.node() for k in ("rays", "pose", "noise", "trace", "back", "out")}
    rgl.rays_from_mat3x4f(n["rays"], np.tile(scenes.translation(0, 0, 0), (100000, 1, 1)))
    rgl.rays_transform(n["pose"], lidar)
    rgl.raytrace(n["trace"])
    rgl.points_transform(n["back"], oracle_free_inverse(lidar))
    rgl.points_yield(n["out"], [rgl.RGL_FIELD_XYZ_VEC3_F32, rgl.RGL_FIELD_DISTANCE_F32])
    if kind == "angular_ray":
        rgl.check(lib.rgl_node_gaussian_noise_angular_ray(C.byref(n["noise"]), mean, sigma, rgl.RGL_AXIS_Y))
        rgl.chain(n["rays"], n["pose"], n["noise"], n["trace"], n["back"], n["out"])
    else:
        rgl.check(lib.rgl_node_gaussian_noise_angular_hitpoint(C.byref(n["noise"]), mean, sigma, rgl.RGL_AXIS_Y))
        rgl.chain(n["rays"], n["pose"], n["trace"], n["noise"], n["back"], n["out"])
    rgl.set_noise_seed(n["noise"], 2024)
    expected_mean = math.atan2(3.0 * math.cos(mean), 3.0 * math.sin(mean))
    for _ in range(4):
        rgl.graph_run(n["rays"])
        xyz = rgl.result(n["out"], rgl.RGL_FIELD_XYZ_VEC3_F32).astype(np.float64)
        d = rgl.result(n["out"], rgl.RGL_FIELD_DISTANCE_F32).astype(np.float64)
        assert np.all(np.abs(np.linalg.norm(xyz, axis=1) - d) <= 2e-6 * np.maximum(d, 1.0))
        ang = np.arctan2(xyz[:, 2], xyz[:, 0])
        assert abs(ang.mean() - expected_mean) < 0.002
        assert abs(ang.std() - sigma) < 0.002
        assert stats.kstest((ang - expected_mean) / sigma, "norm").pvalue > 1e-4


def oracle_free_inverse(m34):
    """Inverse of a rigid 3x4 pose, in float64 then float32 (test helper, no oracle involved)."""
    m = np.vstack([np.asarray(m34, np.float64), [0, 0, 0, 1]])
    return np.ascontiguousarray(np.linalg.inv(m)[:3].astype(np.float32))
