"""Raytrace node through the C API on the GPU, against the reference's known answers and the oracle.

Known-answer cases restate reference test/src/graph/DistanceFieldTest.cpp:86-276,
test/src/graph/nodes/RaytraceNodeTest.cpp:109-273, test/src/apiReadmeExample.cpp:19-55 and
test/src/scene/entityIdTest.cpp:28-95 (golden values in tests/golden/reference_values.json).
Tolerances: hit/miss and entity id exact except on rays the oracle flags as ambiguous (within 1e-6
relative of an edge or range bound), distance within 1e-5 relative, XYZ within 1e-5 of the
coordinate magnitude.
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
F = None  # filled lazily with the rgl module


def cube_scene(rgl, transforms, ids=None):
    cube = scenes.cube_mesh(1.0)
    ents = []
    for k, tf in enumerate(transforms):
        m = rgl.mesh_create(cube.vertices, cube.indices)
        e = rgl.entity_create(m)
        rgl.entity_set_transform(e, tf)
        if ids is not None and ids[k] is not None:
            rgl.entity_set_id(e, ids[k])
        ents.append(e)
    return ents


def run_yield(rgl, rays, ranges=None, fields=None, configure=None):
    fields = fields or [rgl.RGL_FIELD_DISTANCE_F32, rgl.RGL_FIELD_XYZ_VEC3_F32]
    n_rays, n_rng, n_rt, n_y = rgl.node(), rgl.node(), rgl.node(), rgl.node()
    rgl.rays_from_mat3x4f(n_rays, rays)
    chain = [n_rays]
    if ranges is not None:
        rgl.rays_set_range(n_rng, ranges)
        chain.append(n_rng)
    rgl.raytrace(n_rt)
    if configure:
        configure(n_rt)
    rgl.points_yield(n_y, fields)
    chain += [n_rt, n_y]
    rgl.chain(*chain)
    rgl.graph_run(n_rays)
    return {f: rgl.result(n_y, f) for f in fields}


@pytest.mark.parametrize("z", GOLD["distance_field_cube_z"])
def test_distance_single_object_exact(rgl, z):
    cube_scene(rgl, [scenes.translation(0, 0, np.float32(z))])
    out = run_yield(rgl, [scenes.translation(0, 0, 0)], [[0.0, np.float32(z) + 10.0]])
    d = out[rgl.RGL_FIELD_DISTANCE_F32][0]
    xyz = out[rgl.RGL_FIELD_XYZ_VEC3_F32][0]
    assert d == np.float32(np.float32(z) - np.float32(1.0))
    assert d == np.float32(np.sqrt(np.float32(xyz @ xyz)))


def test_distance_origin_on_cube_face(rgl):
    cube_scene(rgl, [scenes.translation(0, 0, 1.0)])
    out = run_yield(rgl, [scenes.translation(0, 0, 0)], [[0.0, 11.0]])
    assert out[rgl.RGL_FIELD_DISTANCE_F32][0] == np.float32(2.0)


def test_distance_origin_inside_cube(rgl):
    z = np.float32(-0.001)
    cube_scene(rgl, [scenes.translation(0, 0, z)])
    out = run_yield(rgl, [scenes.translation(0, 0, 0)], [[0.0, z + 10.0]])
    assert out[rgl.RGL_FIELD_DISTANCE_F32][0] == np.float32(np.float32(1.0) + z)


def test_nonhit_off_path_is_infinite(rgl):
    cube_scene(rgl, [scenes.translation(0, 55.5, 0)])
    rays = [scenes.translation(0, 0, 0), scenes.rotation_xyz(math.pi, 0, 0)]
    out = run_yield(rgl, rays, [[0.0, 10000.0]])
    assert np.all(np.isinf(out[rgl.RGL_FIELD_DISTANCE_F32]))
    assert np.all(out[rgl.RGL_FIELD_DISTANCE_F32] > 0)


@pytest.mark.parametrize("z", GOLD["distance_field_cube_z"])
def test_out_of_max_range(rgl, z):
    z = np.float32(z)
    cube_scene(rgl, [scenes.translation(0, 0, z)])
    out = run_yield(rgl, [scenes.translation(0, 0, 0)], [[0.0, z - 1.0 - 1.0]])
    assert np.isinf(out[rgl.RGL_FIELD_DISTANCE_F32][0])


@pytest.mark.parametrize("z", GOLD["distance_field_cube_z"])
def test_out_of_min_range(rgl, z):
    z = np.float32(z)
    cube_scene(rgl, [scenes.translation(0, 0, z)])
    out = run_yield(rgl, [scenes.translation(0, 0, 0)], [[z + 1.0 + 1.0, z + 1.0 + 2.0]])
    assert np.isinf(out[rgl.RGL_FIELD_DISTANCE_F32][0])


@pytest.mark.parametrize("z", GOLD["distance_field_cube_z"])
def test_object_in_range_behind_object_below_min_range(rgl, z):
    z = np.float32(z)
    cube_scene(rgl, [scenes.translation(0, 0, z), scenes.translation(0, 0, z + 10.0)])
    out = run_yield(rgl, [scenes.translation(0, 0, 0)], [[z + 1.0 + 1.0, z + 10.0 + 1.0 + 1.0]])
    assert np.isinf(out[rgl.RGL_FIELD_DISTANCE_F32][0])


def test_distance_from_ray_beginning(rgl):
    cube_scene(rgl, [scenes.translation(0, 0, 10.0)])
    a = run_yield(rgl, [scenes.translation(0, 0, 0)], [[0.0, 20.0]])[rgl.RGL_FIELD_DISTANCE_F32][0]
    b = run_yield(rgl, [scenes.translation(0, 0, 5.0)], [[0.0, 20.0]])
    assert a == np.float32(9.0)
    assert b[rgl.RGL_FIELD_DISTANCE_F32][0] == np.float32(4.0)
    assert a - b[rgl.RGL_FIELD_DISTANCE_F32][0] == np.float32(5.0)


@pytest.mark.parametrize("z", GOLD["distance_field_cube_z"])
def test_various_angles(rgl, z):
    z = np.float32(z)
    cube_scene(rgl, [scenes.translation(0, 0, z)])
    max_angle = math.atan(1.0 / (float(z) - 1.0))
    angles = np.random.default_rng(7).uniform(-max_angle, max_angle, 100)
    rays = np.stack([scenes.rotation_xyz(a, 0, 0) for a in angles])
    out = run_yield(rgl, rays, [[0.0, z + 10.0]])
    d = out[rgl.RGL_FIELD_DISTANCE_F32]
    expected = (float(z) - 1.0) / np.cos(angles)
    assert np.allclose(np.linalg.norm(out[rgl.RGL_FIELD_XYZ_VEC3_F32], axis=1), d, atol=GOLD["distance_field_epsilon"])
    assert np.allclose(expected, d, atol=GOLD["distance_field_epsilon"])


def test_readme_example(rgl):
    cube_scene(rgl, [scenes.translation(0, 0, 5.0)])
    n_rays, n_rt = rgl.node(), rgl.node()
    rgl.rays_from_mat3x4f(n_rays, [scenes.translation(0, 0, 0)])
    rgl.raytrace(n_rt)
    rgl.chain(n_rays, n_rt)
    rgl.graph_run(n_rt)
    xyz = rgl.result(n_rt, rgl.RGL_FIELD_XYZ_VEC3_F32)
    assert xyz.shape == (1, 3)
    assert xyz[0, 2] == pytest.approx(GOLD["readme_hit_z"], rel=1e-6)


def test_entity_ids(rgl, oracle):
    tfs = [scenes.translation(6, -5, 0), scenes.translation(6, 0, 0), scenes.translation(6, 5, 0)]
    cube_scene(rgl, tfs, ids=[1, 2, None])
    rays = scenes.lidar_rays(50, 500, -90.0, 90.0)
    out = run_yield(rgl, rays, None, [rgl.RGL_FIELD_XYZ_VEC3_F32, rgl.RGL_FIELD_ENTITY_ID_I32, rgl.RGL_FIELD_IS_HIT_I32])
    hit = out[rgl.RGL_FIELD_IS_HIT_I32] == 1
    ids = out[rgl.RGL_FIELD_ENTITY_ID_I32]
    y = out[rgl.RGL_FIELD_XYZ_VEC3_F32][:, 1]
    assert hit.sum() > 100
    assert np.all(ids[~hit] == rgl.RGL_ENTITY_INVALID_ID)
    assert np.all(ids[hit & (y < -2.5)] == 1)
    assert np.all(ids[hit & (y > -2.5) & (y < 2.5)] == 2)
    assert np.all(ids[hit & (y > 2.5)] == rgl.RGL_DEFAULT_ENTITY_ID)


def test_non_hits_configuration(rgl):
    cube_scene(rgl, [scenes.translation(0, 0, 0)])
    rays = scenes.lidar_rays(7, 12, -90.0, 90.0)
    fields = [rgl.RGL_FIELD_XYZ_VEC3_F32, rgl.RGL_FIELD_IS_HIT_I32, rgl.RGL_FIELD_DISTANCE_F32]
    # Near non-hit: every ray hits the cube below min range.
    out = run_yield(rgl, rays, [[2.0, 3.0]], fields,
                    configure=lambda n: rgl.check(rgl.lib().rgl_node_raytrace_configure_non_hits(n, 12.34, 0.0)))
    assert np.all(out[rgl.RGL_FIELD_IS_HIT_I32] == 0)
    assert np.all(out[rgl.RGL_FIELD_DISTANCE_F32] == np.float32(12.34))
    dirs = rays[:, :, 2].astype(np.float64)
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    assert np.allclose(out[rgl.RGL_FIELD_XYZ_VEC3_F32], dirs * 12.34, atol=1e-5)


def _parity(rgl, oracle, scene, rays, pose, ranges, mode, h_div=0.0, v_div=0.0, layers=3, vertices=19,
            default_intensity=0.0, extra_fields=()):
    rgl.spawn_scene(scene)
    fields = [rgl.RGL_FIELD_XYZ_VEC3_F32, rgl.RGL_FIELD_DISTANCE_F32, rgl.RGL_FIELD_ENTITY_ID_I32,
              rgl.RGL_FIELD_IS_HIT_I32, rgl.RGL_FIELD_RETURN_TYPE_U8, *extra_fields]
    n_rays, n_tf, n_rng, n_rt, n_y = (rgl.node() for _ in range(5))
    rgl.rays_from_mat3x4f(n_rays, rays)
    rgl.rays_transform(n_tf, pose)
    rgl.rays_set_range(n_rng, ranges)
    rgl.raytrace(n_rt)
    lib = rgl.lib()
    rgl.check(lib.rgl_node_raytrace_configure_return_mode(n_rt, mode))
    if h_div > 0:
        rgl.check(lib.rgl_node_raytrace_configure_beam_divergence(n_rt, h_div, v_div))
        rgl.configure_beam_samples(n_rt, layers, vertices)
    if default_intensity > 0:
        rgl.check(lib.rgl_node_raytrace_configure_default_intensity(n_rt, default_intensity))
    rgl.points_yield(n_y, fields)
    rgl.chain(n_rays, n_tf, n_rng, n_rt, n_y)
    rgl.graph_run(n_rays)
    got = {f: rgl.result(n_y, f) for f in fields}
    osc = oracle.OracleScene(scene)
    exp = osc.raytrace(rays, ray_transform=pose, ranges=ranges, return_mode=mode, h_div=h_div, v_div=v_div,
                       layers=layers, vertices=vertices, default_intensity=default_intensity)
    return got, exp


def _check(rgl, got, exp, min_agreement=0.99999):
    amb = exp["ambiguous"] != 0
    hit_g, hit_e = got[rgl.RGL_FIELD_IS_HIT_I32], exp["is_hit"]
    ent_g, ent_e = got[rgl.RGL_FIELD_ENTITY_ID_I32], exp["entity_id"]
    mism = (hit_g != hit_e) | (ent_g != ent_e)
    assert not (mism & ~amb).any(), f"{int((mism & ~amb).sum())} non-ambiguous mismatches"
    assert 1.0 - mism.mean() >= min_agreement, f"agreement {1.0 - mism.mean()}"
    assert np.all(got[rgl.RGL_FIELD_RETURN_TYPE_U8] == exp["return_type"])
    both = (hit_g == 1) & (hit_e == 1) & ~amb
    dg, de = got[rgl.RGL_FIELD_DISTANCE_F32][both], exp["distance"][both]
    rel = np.abs(dg.astype(np.float64) - de) / np.maximum(np.abs(de), 1e-6)
    assert rel.max(initial=0.0) <= 1e-5, f"max rel distance error {rel.max()}"
    xg, xe = got[rgl.RGL_FIELD_XYZ_VEC3_F32][both], exp["xyz"][both]
    scale = np.maximum(np.abs(xe).max(axis=1), 1.0)
    assert (np.abs(xg - xe).max(axis=1, initial=0.0) <= 1e-5 * scale * 4).all()
    # Non-hits: distances and XYZ follow the non-hit rule exactly.
    nh = (hit_g == 0) & (hit_e == 0)
    assert np.array_equal(got[rgl.RGL_FIELD_DISTANCE_F32][nh], exp["distance"][nh])
    return rel


def test_parity_plain_scene_first_return(rgl, oracle):
    got, exp = _parity(rgl, oracle, scenes.plain_scene(), scenes.lidar_rays(32, 1024), scenes.translation(0, 0, 1.8),
                       [[0.1, 100.0]], rgl.RGL_RETURN_FIRST)
    _check(rgl, got, exp)


@pytest.mark.parametrize("mode_name", ["RGL_RETURN_FIRST_LAST", "RGL_RETURN_LAST", "RGL_RETURN_STRONGEST",
                                       "RGL_RETURN_FIRST_SECOND", "RGL_RETURN_LAST_STRONGEST",
                                       "RGL_RETURN_STRONGEST_SECOND_STRONGEST", "RGL_RETURN_SECOND"])
def test_parity_return_modes_reference_pattern(rgl, oracle, mode_name):
    mode = getattr(rgl, mode_name)
    got, exp = _parity(rgl, oracle, scenes.plain_scene(), scenes.lidar_rays(16, 256), scenes.translation(0, 0, 1.8),
                       [[0.1, 100.0]], mode, h_div=math.radians(2.0), v_div=math.radians(1.0), default_intensity=100.0,
                       extra_fields=[rgl.RGL_FIELD_INTENSITY_F32])
    _check(rgl, got, exp)


def test_parity_million_scene_dual_return_5_subrays(rgl, oracle):
    got, exp = _parity(rgl, oracle, scenes.million_scene(), scenes.lidar_rays(32, 512), scenes.translation(0, 0, 8.0),
                       [[0.1, 100.0]], rgl.RGL_RETURN_FIRST_LAST, h_div=math.radians(0.2), v_div=math.radians(0.2),
                       layers=1, vertices=4)
    _check(rgl, got, exp)


@pytest.mark.parametrize("layers,vertices", [(1, 4), (1, 7), (1, 2)])
def test_union_and_single_ray_traversals_agree(rgl, layers, vertices):
    """Lane groups (a beam's sub-rays on adjacent lanes walking the union of their nodes) and one lane
    per beam (each sub-ray alone) give byte-identical points: the closest-hit order does not depend on
    the traversal."""
    scene = scenes.million_scene(seed=3, instances=30, spheres=3, cells=128, extent=150.0)
    rgl.spawn_scene(scene)
    n = {k: rgl.node() for k in ("rays", "pose", "trace", "out")}
    rgl.rays_from_mat3x4f(n["rays"], scenes.lidar_rays(32, 360))
    rgl.rays_transform(n["pose"], scenes.translation(3.0, -2.0, 6.0))
    rgl.raytrace(n["trace"])
    lib = rgl.lib()
    rgl.check(lib.rgl_node_raytrace_configure_return_mode(n["trace"], rgl.RGL_RETURN_FIRST_LAST))
    rgl.check(lib.rgl_node_raytrace_configure_beam_divergence(n["trace"], math.radians(0.4), math.radians(0.4)))
    rgl.configure_beam_samples(n["trace"], layers, vertices)
    fields = [rgl.RGL_FIELD_XYZ_VEC3_F32, rgl.RGL_FIELD_DISTANCE_F32, rgl.RGL_FIELD_ENTITY_ID_I32, rgl.RGL_FIELD_IS_HIT_I32,
              rgl.RGL_FIELD_NORMAL_VEC3_F32]
    rgl.points_yield(n["out"], fields)
    rgl.chain(n["rays"], n["pose"], n["trace"], n["out"])
    got = {}
    for packing, regs, order in ((0, 80, 0), (1, 128, 0), (0, 96, 1), (1, 64, 2), (0, 128, 1), (1, 128, 1), (0, 128, 3), (1, 96, 3)):
        rgl.check(lib.rgl_gb300_configure_trace_schedule(256, packing, 1, regs))
        rgl.check(lib.rgl_gb300_configure_trace_order(order))
        rgl.graph_run(n["rays"])
        got[(packing, regs, order)] = {f: rgl.result_bytes(n["out"], f).tobytes() for f in fields}
    rgl.check(lib.rgl_gb300_configure_trace_schedule(256, 0, 1, 128))  # back to the default
    rgl.check(lib.rgl_gb300_configure_trace_order(3))
    ref = got[(1, 128, 0)]
    for k, v in got.items():
        assert v == ref, f"schedule {k} differs from single-ray traversal in the given order"


def test_kept_beam_order_after_new_ray_contents(rgl):
    """A graph run keeps its beam order (sorted directions of the rays it first cast) when new rays of
    the same count arrive: the order is then stale but still a permutation, and the points equal a run
    in the given order."""
    scene = scenes.million_scene(seed=3, instances=30, spheres=3, cells=128, extent=150.0)
    rgl.spawn_scene(scene)
    lib = rgl.lib()
    n = {k: rgl.node() for k in ("rays", "pose", "trace", "out")}
    first = scenes.lidar_rays(32, 360)
    rgl.rays_from_mat3x4f(n["rays"], first)
    rgl.rays_transform(n["pose"], scenes.translation(3.0, -2.0, 6.0))
    rgl.raytrace(n["trace"])
    rgl.check(lib.rgl_node_raytrace_configure_return_mode(n["trace"], rgl.RGL_RETURN_FIRST_LAST))
    fields = [rgl.RGL_FIELD_XYZ_VEC3_F32, rgl.RGL_FIELD_DISTANCE_F32, rgl.RGL_FIELD_ENTITY_ID_I32, rgl.RGL_FIELD_IS_HIT_I32]
    rgl.points_yield(n["out"], fields)
    rgl.chain(n["rays"], n["pose"], n["trace"], n["out"])
    rng = np.random.default_rng(12)
    second = first[rng.permutation(first.shape[0])]  # same count, other beams at every index
    got = {}
    try:
        for order in (1, 2, 3, 0):
            rgl.check(lib.rgl_gb300_configure_trace_order(order))
            rgl.rays_from_mat3x4f(n["rays"], first)
            rgl.graph_run(n["rays"])
            rgl.rays_from_mat3x4f(n["rays"], second)
            rgl.graph_run(n["rays"])
            got[order] = {f: rgl.result_bytes(n["out"], f).tobytes() for f in fields}
    finally:
        rgl.check(lib.rgl_gb300_configure_trace_order(3))
    for order in (1, 2, 3):
        assert got[order] == got[0], f"order {order} kept over new ray contents differs from the given order"


def _beam_field_graph(rgl, rays, pose, fields, ring_ids=None, offsets=None):
    n = {k: rgl.node() for k in ("rays", "pose", "trace", "out")}
    rgl.rays_from_mat3x4f(n["rays"], rays)
    rgl.rays_transform(n["pose"], pose)
    chain = [n["rays"], n["pose"]]
    lib = rgl.lib()
    if ring_ids is not None:
        n["ring"] = rgl.node()
        ids = np.ascontiguousarray(ring_ids, dtype=np.int32)
        rgl.check(lib.rgl_node_rays_set_ring_ids(C.byref(n["ring"]), rgl.ptr(ids), len(ids)))
        chain.append(n["ring"])
    if offsets is not None:
        n["off"] = rgl.node()
        o = np.ascontiguousarray(offsets, dtype=np.float32)
        rgl.check(lib.rgl_node_rays_set_time_offsets(C.byref(n["off"]), rgl.ptr(o), len(o)))
        chain.append(n["off"])
    rgl.raytrace(n["trace"])
    rgl.points_yield(n["out"], fields)
    rgl.chain(*chain, n["trace"], n["out"])
    return n


def test_azimuth_elevation_ring_ids_match_oracle(rgl, oracle):
    """Fields a beam's returns share (reference optixPrograms.cu:288-326): azimuth and elevation of the
    sensor-frame ray pose, ring id = ids[beam % count], time stamps 0 without velocity distortion."""
    cube = scenes.cube_mesh(2.0)
    e = rgl.entity_create(rgl.mesh_create(cube.vertices, cube.indices))
    rgl.entity_set_transform(e, scenes.translation(0, 0, 5))
    rays = scenes.lidar_rays(16, 90)
    pose = scenes.trs((1.0, -2.0, 0.5), (0.1, -0.2, 0.7))
    ids = np.arange(16, dtype=np.int32) * 7 + 70000  # wraps in uint16
    fields = [rgl.RGL_FIELD_AZIMUTH_F32, rgl.RGL_FIELD_ELEVATION_F32, rgl.RGL_FIELD_RING_ID_U16, rgl.RGL_FIELD_TIME_STAMP_U32,
              rgl.RGL_FIELD_RAY_IDX_U32]
    n = _beam_field_graph(rgl, rays, pose, fields, ring_ids=ids)
    rgl.check(rgl.lib().rgl_node_raytrace_configure_return_mode(n["trace"], rgl.RGL_RETURN_FIRST_LAST))
    rgl.graph_run(n["rays"])
    world = oracle.transform_rays(pose, rays)
    exp = oracle.beam_shared_fields(world, pose, return_count=2, ring_ids=ids)
    az, el = rgl.result(n["out"], rgl.RGL_FIELD_AZIMUTH_F32), rgl.result(n["out"], rgl.RGL_FIELD_ELEVATION_F32)
    assert az.shape == (2 * len(rays),)
    assert np.abs(az - exp["azimuth"]).max() <= 1e-5
    assert np.abs(el - exp["elevation"]).max() <= 1e-5
    assert np.array_equal(rgl.result(n["out"], rgl.RGL_FIELD_RING_ID_U16), exp["ring_id"])
    assert not rgl.result(n["out"], rgl.RGL_FIELD_TIME_STAMP_U32).any()
    assert np.array_equal(rgl.result(n["out"], rgl.RGL_FIELD_RAY_IDX_U32), np.repeat(np.arange(len(rays), dtype=np.uint32), 2))


def test_beam_field_pipeline_errors(rgl):
    rays = scenes.lidar_rays(4, 10)
    n = _beam_field_graph(rgl, rays, scenes.translation(0, 0, 0), [rgl.RGL_FIELD_RING_ID_U16])
    with pytest.raises(rgl.RGLError) as e:
        rgl.graph_run(n["rays"])
    assert e.value.status == rgl.RGL_INVALID_PIPELINE and "cannot get ring ids" in str(e.value)
    n = _beam_field_graph(rgl, rays, scenes.translation(0, 0, 0), [rgl.RGL_FIELD_RING_ID_U16], ring_ids=np.arange(3))
    with pytest.raises(rgl.RGLError) as e:
        rgl.graph_run(n["rays"])
    assert e.value.status == rgl.RGL_INVALID_PIPELINE and "ring ids doesn't match number of rays" in str(e.value)
    n = _beam_field_graph(rgl, rays, scenes.translation(0, 0, 0), [rgl.RGL_FIELD_DISTANCE_F32], offsets=np.zeros(7))
    with pytest.raises(rgl.RGLError) as e:
        rgl.graph_run(n["rays"])
    assert e.value.status == rgl.RGL_INVALID_PIPELINE and "time offsets don't match number of rays" in str(e.value)
    n = _beam_field_graph(rgl, rays, scenes.translation(0, 0, 0), [rgl.RGL_FIELD_TIME_STAMP_F64], offsets=np.zeros(40))
    with pytest.raises(rgl.RGLError) as e:
        rgl.graph_run(n["rays"])
    assert e.value.status == rgl.RGL_INVALID_PIPELINE and "cannot get time from scene" in str(e.value)
    rgl.check(rgl.lib().rgl_scene_set_time(None, 1_000_000))
    rgl.graph_run(n["rays"])
    assert not rgl.result(n["out"], rgl.RGL_FIELD_TIME_STAMP_F64).any()


def test_laser_retro_of_hit_entity(rgl, oracle):
    scene = scenes.million_scene(seed=4, instances=10, spheres=2, cells=32, extent=60.0)
    _, ents = rgl.spawn_scene(scene)
    retro = {e.entity_id: 0.05 * (k + 1) for k, e in enumerate(scene.entities)}
    for h, e in zip(ents, scene.entities):
        rgl.check(rgl.lib().rgl_entity_set_laser_retro(h, retro[e.entity_id]))
    rays = scenes.lidar_rays(32, 256)
    pose = scenes.translation(0, 0, 6.0)
    n = _beam_field_graph(rgl, rays, pose, [rgl.RGL_FIELD_LASER_RETRO_F32, rgl.RGL_FIELD_ENTITY_ID_I32, rgl.RGL_FIELD_IS_HIT_I32])
    rgl.graph_run(n["rays"])
    got = rgl.result(n["out"], rgl.RGL_FIELD_LASER_RETRO_F32)
    ent = rgl.result(n["out"], rgl.RGL_FIELD_ENTITY_ID_I32)
    hit = rgl.result(n["out"], rgl.RGL_FIELD_IS_HIT_I32) == 1
    exp = oracle.OracleScene(scene).raytrace(rays, ray_transform=pose, ranges=[[0.0, 1e30]])
    ok = ~(exp["ambiguous"] != 0)
    assert np.array_equal(ent[ok], exp["entity_id"][ok])
    want = np.array([retro.get(int(x), 0.0) for x in exp["entity_id"]], np.float32)
    assert np.array_equal(got[ok & hit], want[ok & hit])
    assert not got[~hit].any()
    # A new value reaches the next run (on the entity hit most often).
    ids, counts = np.unique(ent[hit], return_counts=True)
    top = int(ids[np.argmax(counts)])
    k = [e.entity_id for e in scene.entities].index(top)
    rgl.check(rgl.lib().rgl_entity_set_laser_retro(ents[k], 0.9))
    rgl.graph_run(n["rays"])
    got2 = rgl.result(n["out"], rgl.RGL_FIELD_LASER_RETRO_F32)
    sel = (rgl.result(n["out"], rgl.RGL_FIELD_ENTITY_ID_I32) == top) & hit
    assert sel.any() and np.all(got2[sel] == np.float32(0.9))
    assert np.array_equal(got2[hit & ~sel], got[hit & ~sel])


def test_normal_and_incident_angle_match_oracle(rgl, oracle):
    """Hit normal and incident angle of the selected sample (reference optixPrograms.cu:138-150: the
    normalised cross product of the world-space edges AB and AC, acos(|normal . ray direction|); NaN for
    non-hits, nodeKernels.cu:196-201) against the oracle's FP64 values, on rotated, scaled and one
    mirrored instance with FIRST_LAST over 5 sub-rays. The GPU forms the world vertices and the cross
    product in FP32 as the reference does; with vertex coordinates up to 60 m and edges down to 3 cm
    that is about 4e-6 m of rounding per coordinate, 1.3e-4 relative to an edge, so components and
    cosines are held to 1e-3."""
    scene = scenes.million_scene(seed=4, instances=10, spheres=2, cells=32, extent=60.0)
    scene.entities.append(scenes.Entity(1, scenes.trs((10.0, 5.0, 5.0), (0.3, -0.2, 0.5), (-2.0, 2.0, 2.0)), 99))
    rgl.spawn_scene(scene)
    rays = scenes.lidar_rays(32, 256)
    pose = scenes.translation(20.0, 0.0, 7.0)
    fields = [rgl.RGL_FIELD_NORMAL_VEC3_F32, rgl.RGL_FIELD_INCIDENT_ANGLE_F32, rgl.RGL_FIELD_ENTITY_ID_I32, rgl.RGL_FIELD_IS_HIT_I32,
              rgl.RGL_FIELD_DISTANCE_F32]
    n = {k: rgl.node() for k in ("rays", "pose", "trace", "out")}
    rgl.rays_from_mat3x4f(n["rays"], rays)
    rgl.rays_transform(n["pose"], pose)
    rgl.raytrace(n["trace"])
    lib = rgl.lib()
    rgl.check(lib.rgl_node_raytrace_configure_return_mode(n["trace"], rgl.RGL_RETURN_FIRST_LAST))
    rgl.check(lib.rgl_node_raytrace_configure_beam_divergence(n["trace"], math.radians(0.3), math.radians(0.3)))
    rgl.configure_beam_samples(n["trace"], 1, 4)
    rgl.points_yield(n["out"], fields)
    rgl.chain(n["rays"], n["pose"], n["trace"], n["out"])
    rgl.graph_run(n["rays"])
    got = {f: rgl.result(n["out"], f) for f in fields}
    exp = oracle.OracleScene(scene).raytrace(rays, ray_transform=pose, return_mode=rgl.RGL_RETURN_FIRST_LAST,
                                             h_div=math.radians(0.3), v_div=math.radians(0.3), layers=1, vertices=4)
    hit = got[rgl.RGL_FIELD_IS_HIT_I32] == 1
    # Beams whose hit samples on different triangles tie in distance within the unresolved band may
    # select another triangle of the same entity (same distance and entity, another normal).
    ok = hit & (exp["is_hit"] == 1) & (exp["ambiguous"] == 0) & (exp["triangle_tie"] == 0)
    ok &= got[rgl.RGL_FIELD_ENTITY_ID_I32] == exp["entity_id"]
    assert ok.sum() > 3000 and (got[rgl.RGL_FIELD_ENTITY_ID_I32][ok] == 99).sum() > 100
    gn, en = got[rgl.RGL_FIELD_NORMAL_VEC3_F32][ok], exp["normal"][ok]
    assert np.abs(np.linalg.norm(gn, axis=1) - 1.0).max() <= 1e-5
    assert np.abs(gn - en).max() <= 1e-3
    ga, ea = got[rgl.RGL_FIELD_INCIDENT_ANGLE_F32][ok], exp["incident_angle"][ok]
    assert np.abs(np.cos(ga.astype(np.float64)) - np.cos(ea.astype(np.float64))).max() <= 1e-3
    assert np.all((ga >= 0.0) & (ga <= np.float32(math.pi / 2) + 1e-6))
    # Non-hits carry NaN normals and angles, as the reference writes them.
    assert np.isnan(got[rgl.RGL_FIELD_NORMAL_VEC3_F32][~hit]).all()
    assert np.isnan(got[rgl.RGL_FIELD_INCIDENT_ANGLE_F32][~hit]).all()


def test_ray_mask_skips_masked_rays(rgl):
    """Masked rays are not cast: their beams return the far non-hit (reference optixPrograms.cu:55-58);
    the other beams are unchanged."""
    scene = scenes.million_scene(seed=2, instances=8, spheres=2, cells=32, extent=60.0)
    rgl.spawn_scene(scene)
    rays = scenes.lidar_rays(16, 128)
    fields = [rgl.RGL_FIELD_DISTANCE_F32, rgl.RGL_FIELD_IS_HIT_I32, rgl.RGL_FIELD_XYZ_VEC3_F32]
    n = _beam_field_graph(rgl, rays, scenes.translation(0, 0, 6.0), fields)
    lib = rgl.lib()
    rgl.check(lib.rgl_node_raytrace_configure_non_hits(n["trace"], 0.5, 77.0))
    rgl.graph_run(n["rays"])
    full = {f: rgl.result(n["out"], f) for f in fields}
    mask = (np.arange(len(rays)) % 3 != 0).astype(np.int8)
    rgl.check(lib.rgl_node_raytrace_configure_mask(n["trace"], rgl.ptr(mask), len(mask)))
    rgl.graph_run(n["rays"])
    got = {f: rgl.result(n["out"], f) for f in fields}
    on = mask == 1
    for f in fields:
        assert np.array_equal(got[f][on], full[f][on])
    assert not got[rgl.RGL_FIELD_IS_HIT_I32][~on].any()
    assert np.all(got[rgl.RGL_FIELD_DISTANCE_F32][~on] == np.float32(77.0))
    assert (full[rgl.RGL_FIELD_IS_HIT_I32][~on] == 1).any()
    short = np.ones(len(rays) - 1, np.int8)
    rgl.check(lib.rgl_node_raytrace_configure_mask(n["trace"], rgl.ptr(short), len(short)))
    with pytest.raises(rgl.RGLError) as e:
        rgl.graph_run(n["rays"])
    assert e.value.status == rgl.RGL_INVALID_PIPELINE and "Mask size does not match the number of rays" in str(e.value)


def test_ground_filter_flags_non_ground_points(rgl):
    """IS_GROUND_I32 = angle(normal, up) > threshold (reference nodeKernels.cu:322-332); compacting by
    it keeps the points off the ground: here the wall, not the floor."""
    floor = scenes.Mesh(np.array([[-50, -50, 0], [50, -50, 0], [50, 50, 0], [-50, 50, 0]], np.float32),
                        np.array([[0, 1, 2], [0, 2, 3]], np.int32))
    wall = scenes.Mesh(np.array([[8, -50, -1], [8, 50, -1], [8, 50, 30], [8, -50, 30]], np.float32),
                       np.array([[0, 1, 2], [0, 2, 3]], np.int32))
    rgl.spawn_scene(scenes.Scene([floor, wall], [scenes.Entity(0, scenes.translation(0, 0, 0), 1),
                                                 scenes.Entity(1, scenes.translation(0, 0, 0), 2)]))
    n = {k: rgl.node() for k in ("rays", "pose", "trace", "ground", "cmp", "out", "all")}
    rgl.rays_from_mat3x4f(n["rays"], scenes.lidar_rays(16, 180))
    rgl.rays_transform(n["pose"], scenes.translation(0, 0, 2.0))
    rgl.raytrace(n["trace"])
    up = np.array([0, 0, 1], np.float32)
    rgl.check(rgl.lib().rgl_node_points_filter_ground(C.byref(n["ground"]), rgl.ptr(up), 0.1))
    rgl.points_compact_by_field(n["cmp"], rgl.RGL_FIELD_IS_GROUND_I32)
    rgl.points_yield(n["out"], [rgl.RGL_FIELD_XYZ_VEC3_F32, rgl.RGL_FIELD_ENTITY_ID_I32])
    rgl.points_yield(n["all"], [rgl.RGL_FIELD_IS_GROUND_I32, rgl.RGL_FIELD_ENTITY_ID_I32, rgl.RGL_FIELD_IS_HIT_I32])
    rgl.chain(n["rays"], n["pose"], n["trace"], n["ground"], n["cmp"], n["out"])
    rgl.add_child(n["ground"], n["all"])
    rgl.graph_run(n["rays"])
    flags = rgl.result(n["all"], rgl.RGL_FIELD_IS_GROUND_I32)
    ent = rgl.result(n["all"], rgl.RGL_FIELD_ENTITY_ID_I32)
    hit = rgl.result(n["all"], rgl.RGL_FIELD_IS_HIT_I32) == 1
    assert (hit & (ent == 1)).any() and (hit & (ent == 2)).any()
    assert np.all(flags[hit & (ent == 1)] == 0) and np.all(flags[hit & (ent == 2)] == 1)
    kept = rgl.result(n["out"], rgl.RGL_FIELD_ENTITY_ID_I32)
    assert len(kept) == int(flags.sum()) and np.all(kept[kept != 0] == 2)


def test_intensity_texture(rgl):
    """Intensity = texel at the hit's interpolated texture coordinates (point sampling, wrap) times
    |cos| of the incidence (reference optixPrograms.cu:151-167); entities without a texture keep the
    default intensity."""
    lib = rgl.lib()
    quad = scenes.Mesh(np.array([[0, 0, 0], [4, 0, 0], [4, 4, 0], [0, 4, 0]], np.float32), np.array([[0, 1, 2], [0, 2, 3]], np.int32))
    m = rgl.mesh_create(quad.vertices, quad.indices)
    uv = np.array([[0, 0], [1, 0], [1, 1], [0, 1]], np.float32)
    rgl.check(lib.rgl_mesh_set_texture_coords(m, rgl.ptr(uv), 4))
    assert lib.rgl_mesh_set_texture_coords(m, rgl.ptr(uv), 3) == rgl.RGL_INVALID_ARGUMENT
    texels = (np.arange(16, dtype=np.uint8) * 13 + 7).reshape(4, 4)  # row = v, column = u
    tex = C.c_void_p()
    rgl.check(lib.rgl_texture_create(C.byref(tex), rgl.ptr(np.ascontiguousarray(texels)), 4, 4))
    textured, plain = rgl.entity_create(m), rgl.entity_create(m)
    rgl.entity_set_transform(textured, scenes.translation(0, 0, 0))
    rgl.entity_set_transform(plain, scenes.translation(10, 0, 0))
    rgl.check(lib.rgl_entity_set_intensity_texture(textured, tex))
    down = scenes.rotation_xyz(np.pi, 0, 0)
    rays, expect = [], []
    for j in range(4):
        for i in range(4):
            r = down.copy()
            r[:, 3] = (i + 0.5, j + 0.5, 5.0)
            rays.append(r)
            expect.append(float(texels[j, i]))
    r = down.copy()
    r[:, 3] = (12.0, 2.0, 5.0)
    rays.append(r)
    expect.append(3.0)
    n = {k: rgl.node() for k in ("rays", "trace", "out")}
    rgl.rays_from_mat3x4f(n["rays"], np.stack(rays))
    rgl.raytrace(n["trace"])
    rgl.check(lib.rgl_node_raytrace_configure_default_intensity(n["trace"], 3.0))
    rgl.points_yield(n["out"], [rgl.RGL_FIELD_INTENSITY_F32, rgl.RGL_FIELD_IS_HIT_I32])
    rgl.chain(n["rays"], n["trace"], n["out"])
    rgl.graph_run(n["rays"])
    assert (rgl.result(n["out"], rgl.RGL_FIELD_IS_HIT_I32) == 1).all()
    assert np.array_equal(rgl.result(n["out"], rgl.RGL_FIELD_INTENSITY_F32), np.array(expect, np.float32))
