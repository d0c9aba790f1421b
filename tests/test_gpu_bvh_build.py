"""Mesh BLAS builders on the GPU (rgl_gb300_configure_blas_builder).

The default builder computes the binned SAH topology on the device (csrc/sah.cu) with the host
builder's arithmetic, so the device tree is the host tree: same wide-node count and bytes, and every
raytrace output byte-identical to a scene built by the host builder. Cases cover the level loop
(meshes above 2,048 triangles), the block and warp phases, one- and two-triangle meshes, coincident
centroids (middle splits) and a random triangle soup. The device LBVH builder is checked against the
oracle. Reference: OptiX builds the GAS on the device (src/scene/GASBuilder.hpp:31-100).
"""
import ctypes as C
import math
import time

import numpy as np
import pytest

from robotecgpulidar_gb300 import scenes

pytestmark = pytest.mark.gpu

DEVICE_SAH, HOST_SAH, DEVICE_LBVH = 0, 1, 2


def soup_mesh(n, seed, extent=20.0, size=1.5):
    rng = np.random.default_rng(seed)
    c = rng.uniform(-extent, extent, size=(n, 3)).astype(np.float32)
    v = (c[:, None, :] + rng.uniform(-size, size, size=(n, 3, 3))).astype(np.float32).reshape(-1, 3)
    return scenes.Mesh(v, np.arange(3 * n, dtype=np.int32).reshape(n, 3))


def stacked_mesh(copies):
    """`copies` copies of one triangle (all centroids coincide: every split is a middle split)."""
    tri = np.array([[-3, -3, 0], [3, -3, 0], [0, 3, 0]], np.float32)
    v = np.tile(tri, (copies, 1))
    return scenes.Mesh(v, np.arange(3 * copies, dtype=np.int32).reshape(copies, 3))


def single_entity(mesh, tf=None):
    s = scenes.Scene()
    s.meshes.append(mesh)
    s.entities.append(scenes.Entity(0, tf if tf is not None else scenes.translation(0, 0, 8.0), 5))
    return s


CASES = {
    "plain_20k": lambda: scenes.plain_scene(),
    "million": lambda: scenes.million_scene(),
    "one_triangle": lambda: single_entity(soup_mesh(1, 1, extent=0.5, size=3.0)),
    "two_triangles": lambda: single_entity(soup_mesh(2, 2, extent=1.0, size=3.0)),
    "soup_33": lambda: single_entity(soup_mesh(33, 3, extent=4.0)),
    "soup_2049": lambda: single_entity(soup_mesh(2049, 4)),
    "soup_70000": lambda: single_entity(soup_mesh(70000, 5, extent=60.0, size=0.8)),
    "stacked_3000": lambda: single_entity(stacked_mesh(3000)),
}


def scan(rgl, scene, builder):
    """Builds `scene` with `builder` and casts a dense scan around and below the sensor; returns the
    raytrace fields (bytes), the BLAS node bytes and the number of BLAS builds it took."""
    lib = rgl.lib()
    rgl.check(lib.rgl_gb300_configure_blas_builder(builder))
    b0, ms0 = C.c_int64(), C.c_double()
    rgl.check(lib.rgl_gb300_get_blas_build_stats(C.byref(b0), C.byref(ms0)))
    rgl.spawn_scene(scene)
    fields = [rgl.RGL_FIELD_XYZ_VEC3_F32, rgl.RGL_FIELD_DISTANCE_F32, rgl.RGL_FIELD_ENTITY_ID_I32, rgl.RGL_FIELD_IS_HIT_I32]
    n = {k: rgl.node() for k in ("rays", "pose", "trace", "out")}
    rgl.rays_from_mat3x4f(n["rays"], scenes.lidar_rays(64, 1024, -89.0, 60.0))
    rgl.rays_transform(n["pose"], scenes.translation(0.5, 0.25, 12.0))
    rgl.raytrace(n["trace"])
    rgl.points_yield(n["out"], fields)
    rgl.chain(n["rays"], n["pose"], n["trace"], n["out"])
    rgl.graph_run(n["rays"])
    out = {f: rgl.result_bytes(n["out"], f).tobytes() for f in fields}
    nb, tb, ni = C.c_int64(), C.c_int64(), C.c_int32()
    rgl.check(lib.rgl_gb300_scene_get_stats(C.byref(nb), C.byref(tb), C.byref(ni)))
    b1, ms1 = C.c_int64(), C.c_double()
    rgl.check(lib.rgl_gb300_get_blas_build_stats(C.byref(b1), C.byref(ms1)))
    hits = int(np.frombuffer(out[rgl.RGL_FIELD_IS_HIT_I32], np.int32).sum())
    rgl.check(lib.rgl_cleanup())
    rgl.check(lib.rgl_configure_logging(rgl.RGL_LOG_LEVEL_OFF, None, False))
    return out, nb.value, b1.value - b0.value, ms1.value - ms0.value, hits


@pytest.mark.parametrize("case", list(CASES))
def test_device_sah_tree_equals_host_tree(rgl, case):
    scene = CASES[case]()
    try:
        host, host_nodes, host_builds, host_ms, hits = scan(rgl, scene, HOST_SAH)
        dev, dev_nodes, dev_builds, dev_ms, _ = scan(rgl, scene, DEVICE_SAH)
    finally:
        rgl.check(rgl.lib().rgl_gb300_configure_blas_builder(DEVICE_SAH))
    assert host_builds == dev_builds == len(scene.meshes)
    assert hits > 0
    assert dev_nodes == host_nodes, "device and host SAH trees differ in size"
    for f in host:
        assert dev[f] == host[f], f"field {f} differs between the device and host SAH builds"
    print(f"{case}: {sum(m.triangle_count for m in scene.meshes)} triangles, node bytes {dev_nodes}, "
          f"build device {dev_ms:.1f} ms / host {host_ms:.1f} ms")


def test_device_lbvh_builder_matches_oracle(rgl, oracle):
    scene = scenes.million_scene(seed=3, instances=30, spheres=3, cells=128, extent=150.0)
    rays, pose = scenes.lidar_rays(32, 512), scenes.translation(2.0, -3.0, 6.0)
    try:
        rgl.check(rgl.lib().rgl_gb300_configure_blas_builder(DEVICE_LBVH))
        rgl.spawn_scene(scene)
        fields = [rgl.RGL_FIELD_DISTANCE_F32, rgl.RGL_FIELD_ENTITY_ID_I32, rgl.RGL_FIELD_IS_HIT_I32]
        n = {k: rgl.node() for k in ("rays", "pose", "range", "trace", "out")}
        rgl.rays_from_mat3x4f(n["rays"], rays)
        rgl.rays_transform(n["pose"], pose)
        rgl.rays_set_range(n["range"], [[0.1, 100.0]])
        rgl.raytrace(n["trace"])
        rgl.points_yield(n["out"], fields)
        rgl.chain(n["rays"], n["pose"], n["range"], n["trace"], n["out"])
        rgl.graph_run(n["rays"])
        got = {f: rgl.result(n["out"], f) for f in fields}
    finally:
        rgl.check(rgl.lib().rgl_gb300_configure_blas_builder(DEVICE_SAH))
    exp = oracle.OracleScene(scene).raytrace(rays, ray_transform=pose, ranges=[[0.1, 100.0]])
    amb = exp["ambiguous"] != 0
    mism = (got[rgl.RGL_FIELD_IS_HIT_I32] != exp["is_hit"]) | (got[rgl.RGL_FIELD_ENTITY_ID_I32] != exp["entity_id"])
    assert not (mism & ~amb).any()
    both = (got[rgl.RGL_FIELD_IS_HIT_I32] == 1) & (exp["is_hit"] == 1) & ~amb
    rel = np.abs(got[rgl.RGL_FIELD_DISTANCE_F32][both] - exp["distance"][both]) / exp["distance"][both]
    assert rel.max() <= 1e-5


def test_builder_argument_check(rgl):
    assert rgl.lib().rgl_gb300_configure_blas_builder(7) == rgl.RGL_INVALID_ARGUMENT
    assert "builder" in rgl.last_error()


def test_serving_scene_build_time(rgl):
    """Device build of the 4M-triangle serving scene (9 meshes, 2.0 M unique triangles) completes and
    its time is reported; the host build of the same trees is timed beside it for the record."""
    scene = scenes.serving_scene(4_000_000, 13)
    t0 = time.perf_counter()
    _, nodes, builds, dev_ms, hits = scan(rgl, scene, DEVICE_SAH)
    wall = time.perf_counter() - t0
    assert builds == len(scene.meshes) and nodes > 0 and hits > 0
    print(f"4M serving scene: {sum(m.triangle_count for m in scene.meshes)} unique triangles, "
          f"device BLAS builds {dev_ms:.1f} ms (scan wall {wall:.2f} s)")
