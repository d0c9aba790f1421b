"""Mesh animation of entities (reference src/scene/animator/*, src/gpu/sceneKernels.cu,
src/scene/Entity.cpp:83-118): external vertex animation and skeleton skinning rebuild the entity's own
BLAS; hits match the oracle on the animated geometry; hit velocities include the vertices' motion."""
import ctypes as C

import numpy as np
import pytest

from robotecgpulidar_gb300 import scenes

pytestmark = pytest.mark.gpu


def grid_mesh(n=8, size=4.0):
    xs = np.linspace(-size / 2, size / 2, n + 1)
    v = np.array([(x, y, 0.0) for y in xs for x in xs], np.float32)
    idx = []
    for j in range(n):
        for i in range(n):
            a = j * (n + 1) + i
            idx += [(a, a + 1, a + n + 2), (a, a + n + 2, a + n + 1)]
    return scenes.Mesh(v, np.array(idx, np.int32))


def down_rays(n=16, size=3.5, z=20.0):
    xs = np.linspace(-size / 2, size / 2, n)
    down = scenes.rotation_xyz(np.pi, 0, 0)
    out = []
    for y in xs:
        for x in xs:
            m = down.copy()
            m[:, 3] = (x, y, z)
            out.append(m)
    return np.stack(out)


def trace(rgl, rays, fields):
    n = {k: rgl.node() for k in ("rays", "trace", "out")}
    rgl.rays_from_mat3x4f(n["rays"], rays)
    rgl.raytrace(n["trace"])
    rgl.points_yield(n["out"], fields)
    rgl.chain(n["rays"], n["trace"], n["out"])
    rgl.graph_run(n["rays"])
    out = {f: rgl.result(n["out"], f) for f in fields}
    rgl.check(rgl.lib().rgl_graph_destroy(n["rays"]))
    return out


def vec3_array(v):
    return np.ascontiguousarray(v, np.float32)


def test_external_animation_moves_the_geometry(rgl, oracle):
    g = grid_mesh()
    m = rgl.mesh_create(g.vertices, g.indices)
    e = rgl.entity_create(m)
    tf = scenes.trs((0.3, -0.2, 2.0), (0.0, 0.0, 0.4))
    rgl.entity_set_transform(e, tf)
    rays = down_rays()
    f = [rgl.RGL_FIELD_DISTANCE_F32, rgl.RGL_FIELD_IS_HIT_I32]
    flat = trace(rgl, rays, f)
    assert np.allclose(flat[rgl.RGL_FIELD_DISTANCE_F32][flat[rgl.RGL_FIELD_IS_HIT_I32] == 1], 18.0, atol=1e-4)
    moved = g.vertices.copy()
    moved[:, 2] = 0.4 * np.sin(moved[:, 0]) * np.cos(0.7 * moved[:, 1])
    rgl.check(rgl.lib().rgl_entity_apply_external_animation(e, rgl.ptr(vec3_array(moved)), len(moved)))
    got = trace(rgl, rays, f)
    exp = oracle.OracleScene(scenes.Scene([scenes.Mesh(moved, g.indices)], [scenes.Entity(0, tf, 1)])).raytrace(rays)
    ok = exp["ambiguous"] == 0
    assert np.array_equal(got[rgl.RGL_FIELD_IS_HIT_I32][ok], exp["is_hit"][ok])
    both = ok & (exp["is_hit"] == 1)
    assert both.sum() > 100
    rel = np.abs(got[rgl.RGL_FIELD_DISTANCE_F32][both] - exp["distance"][both]) / exp["distance"][both]
    assert rel.max() <= 1e-5
    # Other entities of the mesh keep the mesh's own vertices.
    e2 = rgl.entity_create(m)
    rgl.entity_set_transform(e2, scenes.translation(10.0, 0.0, 2.0))
    r2 = rays.copy()
    r2[:, 0, 3] += 10.0
    other = trace(rgl, r2, f)
    assert np.allclose(other[rgl.RGL_FIELD_DISTANCE_F32][other[rgl.RGL_FIELD_IS_HIT_I32] == 1], 18.0, atol=1e-4)
    bad = rgl.lib().rgl_entity_apply_external_animation(e, rgl.ptr(vec3_array(moved[:-1])), len(moved) - 1)
    assert bad == rgl.RGL_INVALID_ARGUMENT and "vertex counts do not match" in rgl.last_error()


def skin_setup(rgl, g):
    """Two bones: vertices with x > 0 follow bone 1, the others bone 0 (blended near x = 0)."""
    n = len(g.vertices)
    w = np.zeros(n, dtype=[("w", "<f4", 4), ("b", "<i4", 4)])
    t = np.clip(g.vertices[:, 0] + 0.5, 0.0, 1.0)
    w["w"][:, 0] = 1.0 - t
    w["w"][:, 1] = t
    w["b"][:, 0] = 0
    w["b"][:, 1] = 1
    restposes = np.stack([scenes.translation(0, 0, 0), scenes.translation(0, 0, 0)]).astype(np.float32)
    return w, restposes


def test_skeleton_animation_matches_oracle(rgl, oracle):
    lib = rgl.lib()
    g = grid_mesh()
    m = rgl.mesh_create(g.vertices, g.indices)
    e = rgl.entity_create(m)
    tf = scenes.translation(0.0, 0.0, 1.0)
    rgl.entity_set_transform(e, tf)
    pose = np.stack([scenes.translation(0, 0, 0), scenes.trs((0.0, 0.0, 0.8), (0.0, -0.3, 0.0))]).astype(np.float32)
    st = lib.rgl_entity_set_pose_world(e, rgl.ptr(pose), 2)
    assert st == rgl.RGL_INVALID_ARGUMENT and "has no bone weights" in rgl.last_error()
    w, restposes = skin_setup(rgl, g)
    rgl.check(lib.rgl_mesh_set_bone_weights(m, rgl.ptr(w), len(w)))
    assert lib.rgl_mesh_set_bone_weights(m, rgl.ptr(w), len(w) - 1) == rgl.RGL_INVALID_ARGUMENT
    rgl.check(lib.rgl_mesh_set_restposes(m, rgl.ptr(restposes), 2))
    assert lib.rgl_entity_set_pose_world(e, rgl.ptr(pose), 1) == rgl.RGL_INVALID_ARGUMENT
    rgl.check(lib.rgl_entity_set_pose_world(e, rgl.ptr(pose), 2))
    skinned = oracle.skinned_vertices(g.vertices, w["w"], w["b"], pose, restposes)
    rays = down_rays()
    f = [rgl.RGL_FIELD_DISTANCE_F32, rgl.RGL_FIELD_IS_HIT_I32]
    got = trace(rgl, rays, f)
    exp = oracle.OracleScene(scenes.Scene([scenes.Mesh(skinned, g.indices)], [scenes.Entity(0, tf, 1)])).raytrace(rays)
    ok = (exp["ambiguous"] == 0) & (exp["is_hit"] == 1)
    assert ok.sum() > 100 and (got[rgl.RGL_FIELD_IS_HIT_I32][ok] == 1).all()
    rel = np.abs(got[rgl.RGL_FIELD_DISTANCE_F32][ok] - exp["distance"][ok]) / exp["distance"][ok]
    assert rel.max() <= 1e-5


def test_bone_outside_the_pose_raises_the_kernel_flag(rgl):
    """A weighted bone index beyond the pose is found by the skinning kernel, which raises its error
    flag (a slot in mapped host memory); the call fails with the reference's kind of error, and once
    the weights are fixed the same pose applies."""
    lib = rgl.lib()
    g = grid_mesh()
    m = rgl.mesh_create(g.vertices, g.indices)
    e = rgl.entity_create(m)
    w, restposes = skin_setup(rgl, g)
    w["b"][::7, 1] = 5  # bone 5 of a two-bone pose
    w["w"][::7, 0] = 0.5
    w["w"][::7, 1] = 0.5
    rgl.check(lib.rgl_mesh_set_bone_weights(m, rgl.ptr(w), len(w)))
    rgl.check(lib.rgl_mesh_set_restposes(m, rgl.ptr(restposes), 2))
    pose = np.stack([scenes.translation(0, 0, 0), scenes.trs((0.0, 0.0, 0.8), (0.0, -0.3, 0.0))]).astype(np.float32)
    st = lib.rgl_entity_set_pose_world(e, rgl.ptr(pose), 2)
    assert st == rgl.RGL_INVALID_ARGUMENT and "outside the pose" in rgl.last_error()
    w_ok, _ = skin_setup(rgl, g)
    rgl.check(lib.rgl_mesh_set_bone_weights(m, rgl.ptr(w_ok), len(w_ok)))
    rgl.check(lib.rgl_entity_set_pose_world(e, rgl.ptr(pose), 2))


def test_hit_velocity_of_animated_vertices(rgl, oracle):
    lib = rgl.lib()
    g = grid_mesh()
    m = rgl.mesh_create(g.vertices, g.indices)
    e = rgl.entity_create(m)
    tf = scenes.trs((0.0, 0.0, 1.0), (0.0, 0.0, 0.5))
    rgl.check(lib.rgl_scene_set_time(None, 2_000_000_000))
    rgl.entity_set_transform(e, tf)
    v0 = g.vertices.copy()
    rgl.check(lib.rgl_entity_apply_external_animation(e, rgl.ptr(vec3_array(v0)), len(v0)))
    rgl.check(lib.rgl_scene_set_time(None, 2_050_000_000))
    v1 = v0.copy()
    v1[:, 2] += 0.1 * (1.0 + v1[:, 0])  # a tilt: the displacement varies over the surface
    v1[:, 0] += 0.05
    rgl.check(lib.rgl_entity_apply_external_animation(e, rgl.ptr(vec3_array(v1)), len(v1)))
    rays = down_rays(n=8, size=3.0)
    f = [rgl.RGL_FIELD_XYZ_VEC3_F32, rgl.RGL_FIELD_IS_HIT_I32, rgl.RGL_FIELD_ABSOLUTE_VELOCITY_VEC3_F32]
    got = trace(rgl, rays, f)
    scene = scenes.Scene([scenes.Mesh(v1, g.indices)], [scenes.Entity(0, tf, 1)])
    osc = oracle.OracleScene(scene)
    exp = osc.raytrace(rays)
    checked = 0
    for i in np.nonzero((exp["is_hit"] == 1) & (exp["ambiguous"] == 0))[0]:
        # The hit triangle: the one containing the hit point's (x, y) in the entity frame.
        p = (np.linalg.inv(oracle.mat4(tf)) @ np.append(exp["xyz"][i].astype(np.float64), 1.0))[:3]
        for tri in g.indices:
            a, b, c = (v1[k].astype(np.float64) for k in tri)
            n = np.cross(b - a, c - a)
            u = np.dot(np.cross(p - a, c - a), n) / np.dot(n, n)
            w = np.dot(np.cross(b - a, p - a), n) / np.dot(n, n)
            if min(u, w, 1 - u - w) > 1e-3:
                vel = oracle.animation_velocity(exp["xyz"][i], tf, [v1[k] for k in tri], [v1[k] - v0[k] for k in tri], 0.05)
                assert np.abs(got[rgl.RGL_FIELD_ABSOLUTE_VELOCITY_VEC3_F32][i] - vel).max() <= 2e-3
                checked += 1
                break
    assert checked > 20
