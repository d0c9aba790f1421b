"""C API boundary behaviour on the GPU build: status codes and error messages as the reference tests
assert them (test/include/helpers/commonHelpers.hpp:14-30; node tests' invalid-argument cases),
handle validation, the create-or-modify idiom, graph links and priorities
(reference src/graph/Node.cpp:23-215, test/src/graph/setPriorityTest.cpp, addChildTest.cpp)."""
import ctypes as C

import numpy as np
import pytest

from robotecgpulidar_gb300 import scenes

pytestmark = pytest.mark.gpu


def status(rgl, name, *args):
    return rgl.call(name, *args)


def test_version_and_extensions(rgl):
    a, b, c = C.c_int32(), C.c_int32(), C.c_int32()
    rgl.check(rgl.lib().rgl_get_version_info(C.byref(a), C.byref(b), C.byref(c)))
    assert (a.value, b.value, c.value) == (0, 19, 0)
    av = C.c_int32(7)
    rgl.check(rgl.lib().rgl_get_extension_info(0, C.byref(av)))
    assert av.value == 0
    assert rgl.lib().rgl_get_extension_info(99, C.byref(av)) == rgl.RGL_INVALID_ARGUMENT


@pytest.mark.parametrize("call,args,expr", [
    ("rgl_node_raytrace", (None, None), "node != nullptr"),
    ("rgl_node_points_compact_by_field", (None, 4), "node != nullptr"),
    ("rgl_node_raytrace_configure_non_hits", (None, 0.0, 0.0), "node != nullptr"),
    ("rgl_node_raytrace_configure_distortion", (None, False), "node != nullptr"),
    ("rgl_graph_run", (None,), "raw_node != nullptr"),
    ("rgl_mesh_create", (None, None, 0, None, 0), "out_mesh != nullptr"),
])
def test_invalid_argument_messages(rgl, call, args, expr):
    assert status(rgl, call, *args) == rgl.RGL_INVALID_ARGUMENT
    msg = rgl.last_error()
    assert "Invalid argument" in msg and expr in msg


def test_invalid_object_message(rgl):
    assert rgl.lib().rgl_node_raytrace_configure_non_hits(C.c_void_p(0x1234), 0.0, 0.0) == rgl.RGL_INVALID_API_OBJECT
    msg = rgl.last_error()
    assert "Object does not exist: " in msg and "Node 0x1234" in msg


def test_velocity_argument_checks(rgl):
    n = rgl.raytrace(rgl.node())
    v = np.array([1.0, 2.0, 3.0], np.float32)
    assert rgl.lib().rgl_node_raytrace_configure_velocity(n, None, None) == rgl.RGL_INVALID_ARGUMENT
    assert "linear_velocity != nullptr" in rgl.last_error()
    assert rgl.lib().rgl_node_raytrace_configure_velocity(n, rgl.ptr(v), None) == rgl.RGL_INVALID_ARGUMENT
    assert "angular_velocity != nullptr" in rgl.last_error()
    rgl.check(rgl.lib().rgl_node_raytrace_configure_velocity(n, rgl.ptr(v), rgl.ptr(v)))


def test_create_or_modify_and_type_mismatch(rgl):
    n = rgl.node()
    rgl.raytrace(n)
    first = n.value
    rgl.raytrace(n)
    assert n.value == first
    r = np.array([[0.0, 1.0]], np.float32)
    assert rgl.lib().rgl_node_rays_set_range(C.byref(n), rgl.ptr(r), 1) == rgl.RGL_INVALID_API_OBJECT
    assert "type mismatch" in rgl.last_error()


def test_range_validation(rgl):
    n = rgl.node()
    for bad, msg in (([[np.nan, 1.0]], "range must be a number"), ([[2.0, 1.0]], "minimum range must be lower"),
                     ([[-1.0, 1.0]], "must not be negative")):
        r = np.array(bad, np.float32)
        assert rgl.lib().rgl_node_rays_set_range(C.byref(n), rgl.ptr(r), 1) == rgl.RGL_INVALID_ARGUMENT
        assert msg in rgl.last_error()


def test_pipeline_errors(rgl):
    cmp = rgl.points_compact_by_field(rgl.node())
    assert rgl.lib().rgl_graph_run(cmp) == rgl.RGL_INVALID_PIPELINE
    assert "looked for" in rgl.last_error() and "IPointsNode" in rgl.last_error()
    rays = rgl.rays_from_mat3x4f(rgl.node(), [scenes.translation(0, 0, 0)])
    cmp2 = rgl.points_compact_by_field(rgl.node())
    rgl.add_child(rays, cmp2)
    assert rgl.lib().rgl_graph_run(cmp2) == rgl.RGL_INVALID_PIPELINE


def test_ranges_must_match_rays(rgl):
    rays = rgl.rays_from_mat3x4f(rgl.node(), np.tile(scenes.translation(0, 0, 0), (3, 1, 1)))
    rng = rgl.rays_set_range(rgl.node(), [[0, 1], [0, 2]])
    rt = rgl.raytrace(rgl.node())
    rgl.chain(rays, rng, rt)
    assert rgl.lib().rgl_graph_run(rays) == rgl.RGL_INVALID_PIPELINE
    assert "ranges doesn't match number of rays" in rgl.last_error()


def test_results_before_run(rgl):
    rt = rgl.raytrace(rgl.node())
    cnt = C.c_int32()
    assert rgl.lib().rgl_graph_get_result_size(rt, rgl.RGL_FIELD_XYZ_VEC3_F32, C.byref(cnt), None) == rgl.RGL_INVALID_PIPELINE


def test_missing_field(rgl):
    rays = rgl.rays_from_mat3x4f(rgl.node(), [scenes.translation(0, 0, 0)])
    rt = rgl.raytrace(rgl.node())
    y = rgl.points_yield(rgl.node(), [rgl.RGL_FIELD_XYZ_VEC3_F32])
    rgl.chain(rays, rt, y)
    rgl.graph_run(rays)
    buf = np.zeros(4, np.float32)
    assert rgl.lib().rgl_graph_get_result_data(y, rgl.RGL_FIELD_DISTANCE_F32, rgl.ptr(buf)) == rgl.RGL_INVALID_PIPELINE
    assert "does not provide field" in rgl.last_error()


def test_add_child_twice_and_remove(rgl):
    a = rgl.rays_from_mat3x4f(rgl.node(), [scenes.translation(0, 0, 0)])
    b = rgl.raytrace(rgl.node())
    rgl.add_child(a, b)
    assert rgl.lib().rgl_graph_node_add_child(a, b) == rgl.RGL_INVALID_PIPELINE
    assert "twice" in rgl.last_error()
    assert rgl.lib().rgl_graph_node_add_child(a, a) == rgl.RGL_INVALID_ARGUMENT
    rgl.check(rgl.lib().rgl_graph_node_remove_child(a, b))
    assert rgl.lib().rgl_graph_node_remove_child(a, b) == rgl.RGL_INVALID_PIPELINE


def test_priorities_propagate(rgl):
    a = rgl.rays_from_mat3x4f(rgl.node(), [scenes.translation(0, 0, 0)])
    b = rgl.raytrace(rgl.node())
    c = rgl.points_yield(rgl.node(), [rgl.RGL_FIELD_XYZ_VEC3_F32])
    rgl.chain(a, b, c)
    rgl.check(rgl.lib().rgl_graph_node_set_priority(c, 5))
    p = C.c_int32()
    rgl.check(rgl.lib().rgl_graph_node_get_priority(a, C.byref(p)))
    assert p.value == 5
    assert rgl.lib().rgl_graph_node_set_priority(b, 1) == rgl.RGL_INVALID_PIPELINE


def test_alive_and_destroy(rgl):
    cube = scenes.cube_mesh()
    m = rgl.mesh_create(cube.vertices, cube.indices)
    e = rgl.entity_create(m)
    alive = C.c_bool()
    rgl.check(rgl.lib().rgl_entity_is_alive(e, C.byref(alive)))
    assert alive.value
    rgl.check(rgl.lib().rgl_entity_destroy(e))
    rgl.check(rgl.lib().rgl_entity_is_alive(e, C.byref(alive)))
    assert not alive.value
    rgl.check(rgl.lib().rgl_mesh_destroy(m))
    assert rgl.lib().rgl_mesh_destroy(m) == rgl.RGL_INVALID_API_OBJECT
    n = rgl.raytrace(rgl.node())
    rgl.check(rgl.lib().rgl_graph_destroy(n))
    rgl.check(rgl.lib().rgl_node_is_alive(n, C.byref(alive)))
    assert not alive.value


def test_entity_id_limit(rgl):
    cube = scenes.cube_mesh()
    e = rgl.entity_create(rgl.mesh_create(cube.vertices, cube.indices))
    assert rgl.lib().rgl_entity_set_id(e, 1 << 28) == rgl.RGL_INVALID_ARGUMENT
    assert rgl.lib().rgl_entity_set_id(e, 0) == rgl.RGL_INVALID_ARGUMENT
    rgl.check(rgl.lib().rgl_entity_set_id(e, (1 << 28) - 1))


def test_not_implemented_calls_are_recoverable(rgl):
    n = rgl.node()
    f = C.c_float(1.0)
    assert rgl.lib().rgl_node_points_radar_track_objects(C.byref(n), f, f, f, f, f, f, f) == rgl.RGL_NOT_IMPLEMENTED
    # the library keeps working afterwards
    rgl.raytrace(rgl.node())


def test_scene_mutation_between_runs(rgl):
    """Pose changes after a run refit the TLAS; the next run sees the new pose."""
    cube = scenes.cube_mesh()
    m = rgl.mesh_create(cube.vertices, cube.indices)
    e = rgl.entity_create(m)
    rgl.entity_set_transform(e, scenes.translation(0, 0, 5))
    rays = rgl.rays_from_mat3x4f(rgl.node(), [scenes.translation(0, 0, 0)])
    rt = rgl.raytrace(rgl.node())
    rgl.chain(rays, rt)
    # Without downstream consumers a raytrace node computes XYZ only (reference RaytraceNode.cpp:165-191).
    z = lambda: rgl.result(rt, rgl.RGL_FIELD_XYZ_VEC3_F32)[0, 2]
    rgl.graph_run(rays)
    assert z() == np.float32(4.0)
    rgl.entity_set_transform(e, scenes.translation(0, 0, 9))
    rgl.graph_run(rays)
    assert z() == np.float32(8.0)
    e2 = rgl.entity_create(m)
    rgl.entity_set_transform(e2, scenes.translation(0, 0, 3))
    rgl.graph_run(rays)
    assert z() == np.float32(2.0)
    rgl.check(rgl.lib().rgl_entity_destroy(e2))
    rgl.graph_run(rays)
    assert z() == np.float32(8.0)
