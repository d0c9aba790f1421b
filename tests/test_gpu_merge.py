"""Spatial and temporal merge of point clouds (reference src/graph/SpatialMergePointsNode.cpp:18-82,
TemporalMergePointsNode.cpp:18-48; tests test/src/graph/nodes/SpatialMergePointsNodeTest.cpp and
TemporalMergePointsNodeTest.cpp): the merged cloud is the inputs' clouds concatenated in link order
(spatial) or in run order (temporal), byte for byte."""
import math

import numpy as np
import pytest

from robotecgpulidar_gb300 import scenes

pytestmark = pytest.mark.gpu


def cube_scene(rgl):
    cube = scenes.cube_mesh(2.0)
    m = rgl.mesh_create(cube.vertices, cube.indices)
    e = rgl.entity_create(m)
    rgl.entity_set_transform(e, scenes.translation(4, 0, 0))  # beside the sensors: some beams miss
    rgl.entity_set_id(e, 7)


def sensor_branch(rgl, yaw_deg, compact):
    rays = scenes.lidar_rays(24, 180)
    n = {k: rgl.node() for k in ("rays", "pose", "trace")}
    rgl.rays_from_mat3x4f(n["rays"], rays)
    rgl.rays_transform(n["pose"], scenes.trs((0.0, 0.0, 0.0), (0.0, 0.0, math.radians(yaw_deg))))
    rgl.raytrace(n["trace"])
    rgl.chain(n["rays"], n["pose"], n["trace"])
    last = n["trace"]
    if compact:
        n["cmp"] = rgl.node()
        rgl.points_compact_by_field(n["cmp"])
        rgl.add_child(last, n["cmp"])
        last = n["cmp"]
    n["last"] = last
    return n


FIELDS_OF = lambda rgl: [rgl.RGL_FIELD_XYZ_VEC3_F32, rgl.RGL_FIELD_DISTANCE_F32, rgl.RGL_FIELD_ENTITY_ID_I32]


@pytest.mark.parametrize("compact", [False, True])
def test_spatial_merge_of_sensors_is_the_concatenation(rgl, compact):
    cube_scene(rgl)
    fields = FIELDS_OF(rgl)
    branches = [sensor_branch(rgl, yaw, compact) for yaw in (0, 20, 40, 200)]
    merge = rgl.node()
    rgl.points_spatial_merge(merge, fields)
    ys = []
    for b in branches:
        rgl.add_child(b["last"], merge)
        y = rgl.node()
        rgl.points_yield(y, fields)
        rgl.add_child(b["last"], y)
        ys.append(y)
    out = rgl.node()
    rgl.points_yield(out, fields)
    rgl.add_child(merge, out)
    rgl.graph_run(merge)
    for f in fields:
        parts = [rgl.result_bytes(y, f) for y in ys]
        assert np.array_equal(rgl.result_bytes(merge, f), np.concatenate(parts))
        assert np.array_equal(rgl.result_bytes(out, f), np.concatenate(parts))
    n_merged = rgl.result_size(merge, rgl.RGL_FIELD_XYZ_VEC3_F32)[0]
    assert n_merged == sum(rgl.result_size(y, rgl.RGL_FIELD_XYZ_VEC3_F32)[0] for y in ys)
    if compact:
        assert 0 < n_merged < 4 * 24 * 180
    # A second run (replayed capture) with a moved sensor merges the new clouds.
    rgl.rays_transform(branches[1]["pose"], scenes.trs((0.3, 0.0, 0.0), (0.0, 0.0, 0.5)))
    rgl.graph_run(merge)
    for f in fields:
        assert np.array_equal(rgl.result_bytes(merge, f), np.concatenate([rgl.result_bytes(y, f) for y in ys]))


def test_spatial_merge_of_arrays_with_narrow_fields(rgl):
    """Static-count inputs and 1-, 2- and 8-byte fields (byte, half-word and word copies)."""
    fields = [rgl.RGL_FIELD_XYZ_VEC3_F32, rgl.RGL_FIELD_INTENSITY_U8, rgl.RGL_FIELD_RING_ID_U16, rgl.RGL_FIELD_TIME_STAMP_F64]
    rng = np.random.default_rng(3)
    dt = np.dtype([("xyz", "<f4", 3), ("i", "u1"), ("ring", "<u2"), ("t", "<f8")])
    arrays = []
    nodes = []
    for n in (1, 4099, 37):
        a = np.zeros(n, dtype=dt)
        a["xyz"] = rng.normal(size=(n, 3))
        a["i"] = rng.integers(0, 256, n)
        a["ring"] = rng.integers(0, 65536, n)
        a["t"] = rng.normal(size=n)
        arrays.append(a)
        node = rgl.node()
        rgl.points_from_array(node, a.view(np.uint8), n, fields)
        nodes.append(node)
    merge = rgl.node()
    rgl.points_spatial_merge(merge, fields[::-1] + [rgl.RGL_FIELD_PADDING_32])
    for node in nodes:
        rgl.add_child(node, merge)
    rgl.graph_run(merge)
    allp = np.concatenate(arrays)
    assert np.array_equal(rgl.result(merge, rgl.RGL_FIELD_XYZ_VEC3_F32), allp["xyz"])
    assert np.array_equal(rgl.result(merge, rgl.RGL_FIELD_INTENSITY_U8), allp["i"])
    assert np.array_equal(rgl.result(merge, rgl.RGL_FIELD_RING_ID_U16), allp["ring"])
    assert np.array_equal(rgl.result(merge, rgl.RGL_FIELD_TIME_STAMP_F64), allp["t"])


def test_spatial_merge_pipeline_errors(rgl):
    fields = [rgl.RGL_FIELD_XYZ_VEC3_F32, rgl.RGL_FIELD_DISTANCE_F32]
    a = np.zeros((5, 3), np.float32)
    src = rgl.node()
    rgl.points_from_array(src, a.view(np.uint8), 5, [rgl.RGL_FIELD_XYZ_VEC3_F32])
    merge = rgl.node()
    rgl.points_spatial_merge(merge, [rgl.RGL_FIELD_XYZ_VEC3_F32])
    rgl.add_child(src, merge)
    with pytest.raises(rgl.RGLError) as e:
        rgl.graph_run(merge)
    assert e.value.status == rgl.RGL_INVALID_PIPELINE and "requires >= 2 input nodes, found 1" in str(e.value)
    src2 = rgl.node()
    rgl.points_from_array(src2, a.view(np.uint8), 5, [rgl.RGL_FIELD_XYZ_VEC3_F32])
    rgl.add_child(src2, merge)
    rgl.points_spatial_merge(merge, fields)
    with pytest.raises(rgl.RGLError) as e:
        rgl.graph_run(merge)
    assert e.value.status == rgl.RGL_INVALID_PIPELINE and "does not have required field" in str(e.value)


def test_temporal_merge_accumulates_runs_until_reset(rgl):
    cube_scene(rgl)
    fields = FIELDS_OF(rgl)
    b = sensor_branch(rgl, 0, True)
    tm, y = rgl.node(), rgl.node()
    rgl.points_temporal_merge(tm, fields)
    rgl.points_yield(y, fields)
    rgl.add_child(b["last"], tm)
    rgl.add_child(b["last"], y)
    runs = []
    for k in range(5):
        rgl.rays_transform(b["pose"], scenes.trs((0.1 * k, 0.0, 0.0), (0.0, 0.0, 0.3 * k)))
        rgl.graph_run(b["rays"])
        runs.append({f: rgl.result_bytes(y, f) for f in fields})
        for f in fields:
            assert np.array_equal(rgl.result_bytes(tm, f), np.concatenate([r[f] for r in runs]))
    # Setting the fields again starts a new accumulation.
    rgl.points_temporal_merge(tm, fields[:2])
    rgl.graph_run(b["rays"])
    assert np.array_equal(rgl.result_bytes(tm, rgl.RGL_FIELD_DISTANCE_F32), rgl.result_bytes(y, rgl.RGL_FIELD_DISTANCE_F32))
    with pytest.raises(rgl.RGLError) as e:
        rgl.result_bytes(tm, rgl.RGL_FIELD_ENTITY_ID_I32)
    assert e.value.status == rgl.RGL_INVALID_PIPELINE
