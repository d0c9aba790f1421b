"""Graph runs executed as captured CUDA graphs: replays give bit-identical results to direct enqueue
(noise frames keep advancing between replays), and a run is re-captured exactly when a node's kernel
parameters or buffers change."""
import ctypes as C
import math

import numpy as np
import pytest

from robotecgpulidar_gb300 import scenes

pytestmark = pytest.mark.gpu


def build(rgl):
    rgl.spawn_scene(scenes.plain_scene())
    lib = rgl.lib()
    n = {k: rgl.node() for k in ("rays", "pose", "trace", "ang", "dist", "cmp", "y")}
    rgl.rays_from_mat3x4f(n["rays"], scenes.lidar_rays(32, 512))
    rgl.rays_transform(n["pose"], scenes.translation(0, 0, 1.8))
    rgl.raytrace(n["trace"])
    rgl.check(lib.rgl_node_gaussian_noise_angular_hitpoint(C.byref(n["ang"]), 0.0, math.radians(0.5), rgl.RGL_AXIS_Z))
    rgl.check(lib.rgl_node_gaussian_noise_distance(C.byref(n["dist"]), 0.0, 0.02, 0.001))
    rgl.set_noise_seed(n["ang"], 5)
    rgl.set_noise_seed(n["dist"], 6)
    rgl.points_compact_by_field(n["cmp"])
    rgl.points_yield(n["y"], [rgl.RGL_FIELD_XYZ_VEC3_F32, rgl.RGL_FIELD_DISTANCE_F32, rgl.RGL_FIELD_ENTITY_ID_I32])
    rgl.chain(n["rays"], n["pose"], n["trace"], n["ang"], n["dist"], n["cmp"], n["y"])
    return n


def runs(rgl, n, k):
    out = []
    for _ in range(k):
        rgl.graph_run(n["rays"])
        out.append((rgl.result(n["y"], rgl.RGL_FIELD_XYZ_VEC3_F32), rgl.result(n["y"], rgl.RGL_FIELD_DISTANCE_F32)))
    return out


def stats(rgl, node):
    c, r = C.c_int64(), C.c_int64()
    rgl.check(rgl.lib().rgl_gb300_graph_get_capture_stats(node, C.byref(c), C.byref(r)))
    return c.value, r.value


def test_replay_matches_direct_enqueue(rgl):
    lib = rgl.lib()
    rgl.check(lib.rgl_gb300_configure_cuda_graphs(False))
    try:
        direct = runs(rgl, build(rgl), 4)
    finally:
        rgl.check(lib.rgl_gb300_configure_cuda_graphs(True))
    rgl.cleanup()
    n = build(rgl)
    graphed = runs(rgl, n, 4)
    captures, replays = stats(rgl, n["rays"])
    assert captures == 1 and replays == 3
    for (x0, d0), (x1, d1) in zip(direct, graphed):
        assert np.array_equal(x0, x1) and np.array_equal(d0, d1)
    assert not np.array_equal(graphed[0][1], graphed[1][1])  # frames advance across replays


def test_recapture_only_on_parameter_changes(rgl):
    n = build(rgl)
    runs(rgl, n, 2)
    assert stats(rgl, n["rays"]) == (1, 1)
    # Same-size ray upload: contents only, the capture stays valid.
    rgl.rays_from_mat3x4f(n["rays"], scenes.lidar_rays(32, 512))
    runs(rgl, n, 1)
    assert stats(rgl, n["rays"]) == (1, 2)
    # Changing a kernel parameter re-captures once.
    rgl.check(rgl.lib().rgl_node_raytrace_configure_non_hits(n["trace"], 1.0, 2.0))
    runs(rgl, n, 2)
    assert stats(rgl, n["rays"]) == (2, 3)
    # A scene change is applied outside the captured work and needs no re-capture.
    cube = scenes.cube_mesh()
    e = rgl.entity_create(rgl.mesh_create(cube.vertices, cube.indices))
    rgl.entity_set_transform(e, scenes.translation(5, 0, 2))
    rgl.graph_run(n["rays"])
    assert stats(rgl, n["rays"]) == (2, 4)
    assert (rgl.result(n["y"], rgl.RGL_FIELD_ENTITY_ID_I32) == rgl.RGL_DEFAULT_ENTITY_ID).any()  # the new cube is hit
    # A different ray count moves buffers: re-captured.
    rgl.rays_from_mat3x4f(n["rays"], scenes.lidar_rays(32, 1024))
    runs(rgl, n, 1)
    assert stats(rgl, n["rays"])[0] == 3


def test_on_demand_compaction_after_replay_is_fresh(rgl):
    """A field nobody downstream declared is compacted when it is first read after a run; a replayed
    run must not serve the previous run's copy (the per-run state is reset outside the capture)."""
    rgl.spawn_scene(scenes.plain_scene())
    n = {k: rgl.node() for k in ("rays", "pose", "trace", "cmp", "y", "side")}
    rgl.rays_from_mat3x4f(n["rays"], scenes.lidar_rays(16, 256))
    rgl.rays_transform(n["pose"], scenes.translation(0, 0, 1.8))
    rgl.raytrace(n["trace"])
    rgl.points_compact_by_field(n["cmp"])
    rgl.points_yield(n["y"], [rgl.RGL_FIELD_XYZ_VEC3_F32])
    # DISTANCE is requested on a sibling branch, so the raytrace node computes it while nothing below
    # the compaction declares it: reading it from the compaction node compacts it on demand.
    rgl.points_yield(n["side"], [rgl.RGL_FIELD_DISTANCE_F32])
    rgl.chain(n["rays"], n["pose"], n["trace"], n["cmp"], n["y"])
    rgl.add_child(n["trace"], n["side"])
    origin = np.array([0.0, 0.0, 1.8])
    seen = []
    # Same ray count, new directions: content-only updates. The first on-demand read allocates the
    # field's buffer, which re-captures the next run once; the last two runs are replays.
    for lo, hi in ((-25.0, 15.0), (-12.0, -2.0), (-25.0, 15.0), (-12.0, -2.0)):
        rgl.rays_from_mat3x4f(n["rays"], scenes.lidar_rays(16, 256, lo, hi))
        rgl.graph_run(n["rays"])
        xyz = rgl.result(n["y"], rgl.RGL_FIELD_XYZ_VEC3_F32)
        dist = rgl.result(n["cmp"], rgl.RGL_FIELD_DISTANCE_F32)  # compacted on demand
        assert dist.shape[0] == xyz.shape[0]
        assert np.allclose(np.linalg.norm(xyz - origin, axis=1), dist, rtol=1e-5, atol=1e-4)
        seen.append(dist)
    assert stats(rgl, n["rays"]) == (2, 2)
    assert not np.array_equal(seen[2], seen[3]) and np.array_equal(seen[0], seen[2])


def test_moving_sensor_replays_one_capture(rgl):
    """A new sensor pose every run (rgl_node_rays_transform) and a reseeded noise node are staged
    per run: the run is captured once and replayed, with results equal to direct enqueue."""
    lib = rgl.lib()

    def frames(n):
        out = []
        for k in range(4):
            rgl.rays_transform(n["pose"], scenes.trs((k * 3.0, -k * 2.0, 1.8 + 0.2 * k), (0.0, 0.0, 0.3 * k)))
            rgl.set_noise_seed(n["ang"], 40 + k, k)
            rgl.graph_run(n["rays"])
            out.append((rgl.result(n["y"], rgl.RGL_FIELD_XYZ_VEC3_F32), rgl.result(n["y"], rgl.RGL_FIELD_DISTANCE_F32)))
        return out

    rgl.check(lib.rgl_gb300_configure_cuda_graphs(False))
    try:
        direct = frames(build(rgl))
    finally:
        rgl.check(lib.rgl_gb300_configure_cuda_graphs(True))
    rgl.cleanup()
    n = build(rgl)
    graphed = frames(n)
    assert stats(rgl, n["rays"]) == (1, 3)
    for (x0, d0), (x1, d1) in zip(direct, graphed):
        assert np.array_equal(x0, x1) and np.array_equal(d0, d1)
    assert not np.array_equal(graphed[0][0], graphed[1][0])
