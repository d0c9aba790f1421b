"""Hit-point velocities and velocity distortion (reference src/gpu/optixPrograms.cu:60-70,169-212;
src/scene/Entity.cpp:35-81; src/scene/Scene.hpp:60-67), compared with the oracle's FP64 restatements
(pyoracle.hit_velocities, pyoracle.distort_rays)."""
import ctypes as C
import math

import numpy as np
import pytest

from robotecgpulidar_gb300 import scenes

pytestmark = pytest.mark.gpu

VEL_FIELDS = lambda rgl: [rgl.RGL_FIELD_XYZ_VEC3_F32, rgl.RGL_FIELD_IS_HIT_I32, rgl.RGL_FIELD_ENTITY_ID_I32,
                          rgl.RGL_FIELD_ABSOLUTE_VELOCITY_VEC3_F32, rgl.RGL_FIELD_RELATIVE_VELOCITY_VEC3_F32,
                          rgl.RGL_FIELD_RADIAL_SPEED_F32, rgl.RGL_FIELD_DISTANCE_F32]


def vec3(v):
    return (C.c_float * 3)(*v)


def sensor_graph(rgl, rays, pose, fields, lin=(0, 0, 0), ang=(0, 0, 0), offsets=None, distortion=False):
    lib = rgl.lib()
    n = {k: rgl.node() for k in ("rays", "pose", "trace", "out")}
    rgl.rays_from_mat3x4f(n["rays"], rays)
    rgl.rays_transform(n["pose"], pose)
    chain = [n["rays"], n["pose"]]
    if offsets is not None:
        n["off"] = rgl.node()
        o = np.ascontiguousarray(offsets, np.float32)
        rgl.check(lib.rgl_node_rays_set_time_offsets(C.byref(n["off"]), rgl.ptr(o), len(o)))
        chain.append(n["off"])
    rgl.raytrace(n["trace"])
    rgl.check(lib.rgl_node_raytrace_configure_velocity(n["trace"], vec3(lin), vec3(ang)))
    rgl.check(lib.rgl_node_raytrace_configure_distortion(n["trace"], distortion))
    rgl.points_yield(n["out"], fields)
    rgl.chain(*chain, n["trace"], n["out"])
    return n


def test_velocities_of_moving_and_static_entities(rgl, oracle):
    lib = rgl.lib()
    cube = scenes.cube_mesh(1.0)
    m = rgl.mesh_create(cube.vertices, cube.indices)
    moving, static = rgl.entity_create(m), rgl.entity_create(m)
    rgl.entity_set_id(moving, 1)
    rgl.entity_set_id(static, 2)
    t0 = scenes.trs((6.0, -1.5, 0.0), (0.0, 0.0, 0.1))
    ts = scenes.trs((5.0, 2.5, 0.3), (0.0, 0.0, 0.0))
    t1 = scenes.trs((6.5, -1.4, 0.2), (0.0, 0.05, 0.18))
    rgl.check(lib.rgl_scene_set_time(None, 1_000_000_000))
    rgl.entity_set_transform(moving, t0)
    rgl.entity_set_transform(static, ts)
    rgl.check(lib.rgl_scene_set_time(None, 1_100_000_000))
    rgl.entity_set_transform(moving, t1)
    rays = scenes.lidar_rays(24, 360)
    pose = scenes.trs((0.0, 0.0, 0.3), (0.0, 0.0, 0.05))
    lin, ang = (1.0, 0.5, -0.2), (0.0, 0.1, 0.3)
    n = sensor_graph(rgl, rays, pose, VEL_FIELDS(rgl), lin, ang)
    rgl.graph_run(n["rays"])
    got = {f: rgl.result(n["out"], f) for f in VEL_FIELDS(rgl)}
    scene = scenes.Scene([cube], [scenes.Entity(0, t1, 1), scenes.Entity(0, ts, 2)])
    exp = oracle.OracleScene(scene).raytrace(rays, ray_transform=pose)
    hit = (got[rgl.RGL_FIELD_IS_HIT_I32] == 1) & (exp["is_hit"] == 1) & (exp["ambiguous"] == 0)
    assert hit.sum() > 100
    ent = exp["entity_id"][hit]
    assert np.array_equal(got[rgl.RGL_FIELD_ENTITY_ID_I32][hit], ent)
    now = [t1 if e == 1 else ts for e in ent]
    prev = [t0 if e == 1 else ts for e in ent]
    absv, rel, radial = oracle.hit_velocities(exp["xyz"][hit], now, prev, 0.1, pose, lin, ang)
    g_abs = got[rgl.RGL_FIELD_ABSOLUTE_VELOCITY_VEC3_F32][hit]
    g_rel = got[rgl.RGL_FIELD_RELATIVE_VELOCITY_VEC3_F32][hit]
    g_rad = got[rgl.RGL_FIELD_RADIAL_SPEED_F32][hit]
    assert np.abs(g_abs - absv).max() <= 2e-3
    assert np.abs(g_rel - rel).max() <= 2e-3
    assert np.abs(g_rad - radial).max() <= 2e-3
    # The static entity (pose set once) does not move; the moving one does.
    assert np.all(g_abs[ent == 2] == 0.0) and (np.linalg.norm(g_abs[ent == 1], axis=1) > 1.0).all()
    # Non-hits: NaN velocities, zero radial speed.
    miss = got[rgl.RGL_FIELD_IS_HIT_I32] == 0
    assert miss.any() and np.isnan(got[rgl.RGL_FIELD_ABSOLUTE_VELOCITY_VEC3_F32][miss]).all()
    assert np.isnan(got[rgl.RGL_FIELD_RELATIVE_VELOCITY_VEC3_F32][miss]).all()
    assert not got[rgl.RGL_FIELD_RADIAL_SPEED_F32][miss].any()


def test_velocities_without_a_time_step_are_nan(rgl):
    cube = scenes.cube_mesh(1.0)
    e = rgl.entity_create(rgl.mesh_create(cube.vertices, cube.indices))
    rgl.entity_set_transform(e, scenes.translation(0, 0, 5))
    n = sensor_graph(rgl, [scenes.translation(0, 0, 0)], scenes.translation(0, 0, 0), VEL_FIELDS(rgl), (1, 0, 0), (0, 0, 1))
    rgl.graph_run(n["rays"])
    assert rgl.result(n["out"], rgl.RGL_FIELD_IS_HIT_I32)[0] == 1
    assert np.isnan(rgl.result(n["out"], rgl.RGL_FIELD_ABSOLUTE_VELOCITY_VEC3_F32)).all()
    assert np.isnan(rgl.result(n["out"], rgl.RGL_FIELD_RADIAL_SPEED_F32)).all()


def test_velocity_distortion_matches_oracle(rgl, oracle):
    """Each ray is cast from where the moving sensor is at its time offset; XYZ keeps the undistorted
    ray (origin + direction * distance), time stamps carry the offset."""
    lib = rgl.lib()
    box = scenes.cube_mesh(12.0)
    e = rgl.entity_create(rgl.mesh_create(box.vertices, box.indices))
    rgl.entity_set_transform(e, scenes.translation(0, 0, 0))
    rgl.check(lib.rgl_scene_set_time(None, 5_000_000_000))
    rays = scenes.lidar_rays(8, 90)
    pose = scenes.trs((1.0, -2.0, 0.5), (0.0, 0.0, 0.4))
    offsets = np.arange(len(rays), dtype=np.float32) * 0.1  # ms
    lin, ang = (8.0, -3.0, 0.5), (0.2, -0.1, 0.6)
    fields = [rgl.RGL_FIELD_DISTANCE_F32, rgl.RGL_FIELD_XYZ_VEC3_F32, rgl.RGL_FIELD_IS_HIT_I32, rgl.RGL_FIELD_TIME_STAMP_F64,
              rgl.RGL_FIELD_TIME_STAMP_U32]
    n = sensor_graph(rgl, rays, pose, fields, lin, ang, offsets=offsets, distortion=True)
    rgl.graph_run(n["rays"])
    got = {f: rgl.result(n["out"], f) for f in fields}
    world = oracle.transform_rays(pose, rays)
    distorted = oracle.distort_rays(world, pose, offsets, lin, ang)
    scene = scenes.Scene([box], [scenes.Entity(0, scenes.translation(0, 0, 0), 0)])
    exp = oracle.OracleScene(scene).raytrace(distorted)
    ok = exp["ambiguous"] == 0
    assert (got[rgl.RGL_FIELD_IS_HIT_I32][ok] == 1).all()
    d = got[rgl.RGL_FIELD_DISTANCE_F32].astype(np.float64)
    assert (np.abs(d[ok] - exp["distance"][ok]) / exp["distance"][ok]).max() <= 1e-5
    # Without distortion the distances differ (the sensor moves up to 7 cm during the scan).
    plain = oracle.OracleScene(scene).raytrace(world)
    assert np.abs(d - plain["distance"]).max() > 1e-3
    o = world[:, :, 3].astype(np.float64)
    dirs = world[:, :, 2].astype(np.float64)
    xyz = o + dirs / np.linalg.norm(dirs, axis=1, keepdims=True) * d[:, None]
    assert np.abs(got[rgl.RGL_FIELD_XYZ_VEC3_F32] - xyz).max() <= 1e-4
    assert np.array_equal(got[rgl.RGL_FIELD_TIME_STAMP_F64], (offsets * np.float32(1e-3)).astype(np.float64))
    assert np.array_equal(got[rgl.RGL_FIELD_TIME_STAMP_U32], (offsets * np.float32(1e6)).astype(np.uint32))


def test_distortion_needs_time_offsets(rgl):
    n = sensor_graph(rgl, scenes.lidar_rays(2, 4), scenes.translation(0, 0, 0), [rgl.RGL_FIELD_DISTANCE_F32], distortion=True)
    with pytest.raises(rgl.RGLError) as e:
        rgl.graph_run(n["rays"])
    assert e.value.status == rgl.RGL_INVALID_PIPELINE and "cannot get time offsets" in str(e.value)
