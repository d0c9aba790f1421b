"""Whole lidar pipelines through the C API on the GPU, against the oracle.

Config 1 (plain scene, 64x2048 beams): raytrace -> angular hit-point noise (sigma 0.05 deg about the
sensor up axis) -> distance noise (0.02 m + 0.001 d) -> transform into a world frame by a random rigid
pose -> compaction by is-hit -> format [XYZ f32, distance f32, entity id i32]. The raytrace stage is
compared with the oracle's raytrace; the post-raytrace chain is replayed by the oracle on the GPU's own
raytrace output, so the chain is checked value by value (entity ids and counts exact, XYZ and distance
within 1e-5 of the coordinate magnitude).
"""
import ctypes as C
import math

import numpy as np
import pytest

from robotecgpulidar_gb300 import scenes

pytestmark = pytest.mark.gpu

SIGMA = math.radians(0.05)


def test_config1_pipeline(rgl, oracle):
    scene = scenes.plain_scene()
    rays = scenes.lidar_rays(64, 2048)
    pose = scenes.translation(0, 0, 1.8)
    rng = np.random.default_rng(1)
    world = scenes.trs(rng.uniform(-50, 50, 3), rng.uniform(-np.pi, np.pi, 3))
    rgl.spawn_scene(scene)
    lib = rgl.lib()
    n = {k: rgl.node() for k in ("rays", "pose", "range", "trace", "y", "ang", "dist", "tf", "cmp", "fmt")}
    rgl.rays_from_mat3x4f(n["rays"], rays)
    rgl.rays_transform(n["pose"], pose)
    rgl.rays_set_range(n["range"], [[0.1, 100.0]])
    rgl.raytrace(n["trace"])
    yf = [rgl.RGL_FIELD_XYZ_VEC3_F32, rgl.RGL_FIELD_DISTANCE_F32, rgl.RGL_FIELD_ENTITY_ID_I32, rgl.RGL_FIELD_IS_HIT_I32]
    rgl.points_yield(n["y"], yf)
    rgl.check(lib.rgl_node_gaussian_noise_angular_hitpoint(C.byref(n["ang"]), 0.0, SIGMA, rgl.RGL_AXIS_Z))
    rgl.check(lib.rgl_node_gaussian_noise_distance(C.byref(n["dist"]), 0.0, 0.02, 0.001))
    rgl.set_noise_seed(n["ang"], 1234)
    rgl.set_noise_seed(n["dist"], 1234)
    rgl.points_transform(n["tf"], world)
    rgl.points_compact_by_field(n["cmp"])
    ff = [rgl.RGL_FIELD_XYZ_VEC3_F32, rgl.RGL_FIELD_DISTANCE_F32, rgl.RGL_FIELD_ENTITY_ID_I32]
    rgl.points_format(n["fmt"], ff)
    rgl.chain(n["rays"], n["pose"], n["range"], n["trace"], n["y"], n["ang"], n["dist"], n["tf"], n["cmp"], n["fmt"])
    rgl.graph_run(n["rays"])

    # raytrace stage vs oracle
    got = {f: rgl.result(n["y"], f) for f in yf}
    exp = oracle.OracleScene(scene).raytrace(rays, ray_transform=pose, ranges=[[0.1, 100.0]])
    amb = exp["ambiguous"] != 0
    mism = (got[rgl.RGL_FIELD_IS_HIT_I32] != exp["is_hit"]) | (got[rgl.RGL_FIELD_ENTITY_ID_I32] != exp["entity_id"])
    assert not (mism & ~amb).any()

    # post-raytrace chain replayed by the oracle on the GPU's raytrace output
    xyz0 = got[rgl.RGL_FIELD_XYZ_VEC3_F32]
    d0 = got[rgl.RGL_FIELD_DISTANCE_F32]
    L = oracle.inv34(pose)  # raytrace look-at frame: inverse of the cumulative ray transform
    xyz1, d1 = oracle.noise_angular_hitpoint(L, 0.0, SIGMA, rgl.RGL_AXIS_Z, 1234, 0, xyz0)
    xyz2, d2 = oracle.noise_distance(L, 0.0, 0.02, 0.001, 1234, 0, xyz1, d1)
    xyz3 = oracle.transform_points(world, xyz2)
    hit = got[rgl.RGL_FIELD_IS_HIT_I32]
    cnt, size = rgl.result_size(n["fmt"], rgl.RGL_FIELD_DYNAMIC_FORMAT)
    assert size == 20 and cnt == int(hit.sum())
    raw = rgl.result_bytes(n["fmt"], rgl.RGL_FIELD_DYNAMIC_FORMAT).reshape(cnt, 20)
    gx = raw[:, :12].copy().view(np.float32).reshape(cnt, 3)
    gd = raw[:, 12:16].copy().view(np.float32).ravel()
    ge = raw[:, 16:20].copy().view(np.int32).ravel()
    ex = oracle.compact(hit, xyz3)
    ed = oracle.compact(hit, d2)
    ee = oracle.compact(hit, got[rgl.RGL_FIELD_ENTITY_ID_I32])
    assert np.array_equal(ge, ee)
    scale = np.maximum(np.abs(ex).max(axis=1), 1.0)
    assert (np.abs(gx - ex).max(axis=1) <= 1e-5 * scale).all()
    assert np.allclose(gd, ed, rtol=1e-5, atol=1e-5)
    # noise actually applied: distances moved with the configured spread
    moved = oracle.compact(hit, d2 - d0)
    assert 0.01 < np.std(moved) < 0.2


def test_second_run_advances_noise_and_reset_reproduces(rgl):
    cube = scenes.cube_mesh()
    e = rgl.entity_create(rgl.mesh_create(cube.vertices, cube.indices))
    rgl.entity_set_transform(e, scenes.translation(0, 0, 10))
    n_rays, n_rt, n_noise = rgl.node(), rgl.node(), rgl.node()
    rgl.rays_from_mat3x4f(n_rays, np.tile(scenes.translation(0, 0, 0), (1000, 1, 1)))
    rgl.raytrace(n_rt)
    rgl.check(rgl.lib().rgl_node_gaussian_noise_distance(C.byref(n_noise), 0.0, 0.05, 0.0))
    y = rgl.points_yield(rgl.node(), [rgl.RGL_FIELD_DISTANCE_F32])
    rgl.chain(n_rays, n_rt, n_noise, y)
    rgl.set_noise_seed(n_noise, 77)
    rgl.graph_run(n_rays)
    a = rgl.result(y, rgl.RGL_FIELD_DISTANCE_F32)
    rgl.graph_run(n_rays)
    b = rgl.result(y, rgl.RGL_FIELD_DISTANCE_F32)
    rgl.set_noise_seed(n_noise, 77)
    rgl.graph_run(n_rays)
    c = rgl.result(y, rgl.RGL_FIELD_DISTANCE_F32)
    assert not np.array_equal(a, b) and np.array_equal(a, c)


def build_scene_now(rgl):
    """Runs a one-ray raytrace so the scene's acceleration structures (built on the device, with their
    own kernel launches) exist before launch counts are compared."""
    n_rays, n_rt = rgl.node(), rgl.node()
    rgl.rays_from_mat3x4f(n_rays, [scenes.translation(0, 0, 0)])
    rgl.raytrace(n_rt)
    rgl.chain(n_rays, n_rt)
    rgl.graph_run(n_rays)
    rgl.check(rgl.lib().rgl_gb300_graph_sync(n_rays))
    rgl.check(rgl.lib().rgl_graph_destroy(n_rays))


def test_folded_sensor_transform_equals_separate_kernel(rgl):
    """A rays transform whose only consumer is the raytrace is applied in the traversal prologue (no
    transform kernel); with a second consumer it runs as its own kernel. Both give the same bytes."""
    scene = scenes.million_scene(seed=6, instances=10, spheres=2, cells=48, extent=90.0)
    rgl.spawn_scene(scene)
    rays = scenes.lidar_rays(32, 256)
    pose = scenes.trs((3.0, -4.0, 5.0), (0.02, -0.03, 0.7))
    fields = [rgl.RGL_FIELD_XYZ_VEC3_F32, rgl.RGL_FIELD_DISTANCE_F32, rgl.RGL_FIELD_ENTITY_ID_I32, rgl.RGL_FIELD_AZIMUTH_F32]

    def graph(extra_consumer):
        n = {k: rgl.node() for k in ("rays", "pose", "range", "trace", "out")}
        rgl.rays_from_mat3x4f(n["rays"], rays)
        rgl.rays_transform(n["pose"], pose)
        rgl.rays_set_range(n["range"], [[0.1, 80.0]])
        rgl.raytrace(n["trace"])
        rgl.points_yield(n["out"], fields)
        rgl.chain(n["rays"], n["pose"], n["range"], n["trace"], n["out"])
        if extra_consumer:
            n["trace2"] = rgl.node()
            rgl.raytrace(n["trace2"])
            rgl.add_child(n["pose"], n["trace2"])
        return n

    build_scene_now(rgl)
    a, b = graph(False), graph(True)
    l0 = rgl.kernel_launch_count()
    rgl.graph_run(a["rays"])
    ra = {f: rgl.result_bytes(a["out"], f).tobytes() for f in fields}
    l1 = rgl.kernel_launch_count()
    rgl.graph_run(b["rays"])
    rb = {f: rgl.result_bytes(b["out"], f).tobytes() for f in fields}
    l2 = rgl.kernel_launch_count()
    assert ra == rb
    assert (l1 - l0) < (l2 - l1)  # the folded graph launches no transform kernel
    # A new pose reaches the folded traversal without a new capture.
    pose2 = scenes.trs((1.0, 2.0, 4.0), (0.0, 0.0, -0.4))
    rgl.rays_transform(a["pose"], pose2)
    rgl.rays_transform(b["pose"], pose2)
    rgl.graph_run(a["rays"])
    rgl.graph_run(b["rays"])
    assert {f: rgl.result_bytes(a["out"], f).tobytes() for f in fields} == {f: rgl.result_bytes(b["out"], f).tobytes() for f in fields}


def test_point_chain_absorbed_by_compaction(rgl):
    """Noise and transform nodes that feed only a compaction run inside its pass, on the kept points;
    with a second consumer on the chain nothing is absorbed and each node runs its own kernel. Both give
    the same bytes, and so do an absorbed node's own fields when asked for after the run."""
    scene = scenes.million_scene(seed=6, instances=10, spheres=2, cells=48, extent=90.0)
    rgl.spawn_scene(scene)
    rays = scenes.lidar_rays(32, 256)
    lib = rgl.lib()
    XYZ, DIST = rgl.RGL_FIELD_XYZ_VEC3_F32, rgl.RGL_FIELD_DISTANCE_F32
    fields = [XYZ, DIST, rgl.RGL_FIELD_ENTITY_ID_I32]

    def graph(extra_consumer):
        n = {k: rgl.node() for k in ("rays", "range", "trace", "ang", "dist", "tf", "cmp", "out")}
        rgl.rays_from_mat3x4f(n["rays"], rays)
        rgl.rays_set_range(n["range"], [[0.1, 80.0]])
        rgl.raytrace(n["trace"])
        rgl.check(lib.rgl_node_gaussian_noise_angular_hitpoint(C.byref(n["ang"]), 0.0, SIGMA, rgl.RGL_AXIS_Z))
        rgl.check(lib.rgl_node_gaussian_noise_distance(C.byref(n["dist"]), 0.0, 0.02, 0.001))
        rgl.set_noise_seed(n["ang"], 77)
        rgl.set_noise_seed(n["dist"], 78)
        rgl.points_transform(n["tf"], scenes.trs((1.0, 2.0, 3.0), (0.1, 0.2, 0.3)))
        rgl.points_compact_by_field(n["cmp"])
        rgl.points_yield(n["out"], fields)
        rgl.chain(n["rays"], n["range"], n["trace"], n["ang"], n["dist"], n["tf"], n["cmp"], n["out"])
        if extra_consumer:
            n["y2"] = rgl.node()
            rgl.points_yield(n["y2"], [XYZ])
            rgl.add_child(n["tf"], n["y2"])
        return n

    build_scene_now(rgl)
    a, b = graph(False), graph(True)
    l0 = rgl.kernel_launch_count()
    rgl.graph_run(a["rays"])
    ra = {f: rgl.result_bytes(a["out"], f).tobytes() for f in fields}
    l1 = rgl.kernel_launch_count()
    rgl.graph_run(b["rays"])
    rb = {f: rgl.result_bytes(b["out"], f).tobytes() for f in fields}
    l2 = rgl.kernel_launch_count()
    assert ra == rb
    assert (l2 - l1) - (l1 - l0) == 3  # the absorbed graph launches no noise or transform kernel
    # An absorbed node's own output, computed on demand, equals the one its kernel wrote in the run.
    for f in (XYZ, DIST):
        assert rgl.result_bytes(a["dist"], f).tobytes() == rgl.result_bytes(b["dist"], f).tobytes()
    assert rgl.result_bytes(a["tf"], XYZ).tobytes() == rgl.result_bytes(b["tf"], XYZ).tobytes()


def test_run_timing_covers_the_captured_run(rgl):
    """With timing on, a graph run reports the device time of the whole run and of its traversal: both
    positive, the traversal within the run, for captured runs (events recorded inside the CUDA graph)
    and for eager ones; turning timing on after a capture re-captures the run."""
    scene = scenes.million_scene(seed=6, instances=10, spheres=2, cells=48, extent=90.0)
    rgl.spawn_scene(scene)
    lib = rgl.lib()
    n = {k: rgl.node() for k in ("rays", "pose", "trace", "cmp", "out")}
    rgl.rays_from_mat3x4f(n["rays"], scenes.lidar_rays(32, 512))
    rgl.rays_transform(n["pose"], scenes.translation(0, 0, 3.0))
    rgl.raytrace(n["trace"])
    rgl.points_compact_by_field(n["cmp"])
    rgl.points_yield(n["out"], [rgl.RGL_FIELD_XYZ_VEC3_F32])
    rgl.chain(n["rays"], n["pose"], n["trace"], n["cmp"], n["out"])
    run_ms, trace_ms = C.c_float(), C.c_float()
    try:
        rgl.graph_run(n["rays"])  # captured without timing
        rgl.check(lib.rgl_gb300_configure_timing(True))
        for graphs in (True, False):
            rgl.check(lib.rgl_gb300_configure_cuda_graphs(graphs))
            for _ in range(3):
                rgl.graph_run(n["rays"])
                rgl.check(lib.rgl_gb300_graph_get_timing(n["rays"], C.byref(run_ms), C.byref(trace_ms)))
                assert 0.0 < trace_ms.value <= run_ms.value < 50.0
    finally:
        rgl.check(lib.rgl_gb300_configure_timing(False))
        rgl.check(lib.rgl_gb300_configure_cuda_graphs(True))
