"""Batched multi-sensor frames (rgl_gb300_batch_*) on the GPU.

The property under test: after a batched frame, every graph's results are byte-identical to what a
run of that graph alone (rgl_graph_run) writes, whatever the traversal schedule; entity re-poses
between frames reach the traversal through the refit captured into the frame; and one sensor of a
batch agrees with the FP64 oracle within the tolerances of the single-sensor parity tests.
"""
import ctypes as C
import math

import numpy as np
import pytest

from robotecgpulidar_gb300 import scenes

pytestmark = pytest.mark.gpu

SEED = 77


def small_multi_entity_scene():
    """Terrain (64x64 cells over 120 m) + 12 posed icospheres of 2 meshes: 28,672 triangles."""
    return scenes.million_scene(seed=5, instances=12, spheres=2, cells=64, extent=120.0)


# Per-sensor configurations: pattern, return mode, sub-ray pattern (layers, vertices) or None for no
# divergence, extra fields, noise, compaction, format.
SENSORS = [
    dict(rays=("lidar", 8, 360), mode="RGL_RETURN_FIRST", samples=None, extra=[], noise=False, compact=True, fmt=False),
    dict(rays=("lidar", 16, 256), mode="RGL_RETURN_FIRST_LAST", samples=(1, 4), extra=[], noise=True, compact=True, fmt=False),
    dict(rays=("grid", 24, 64), mode="RGL_RETURN_LAST", samples=(2, 6), extra=[], noise=True, compact=False, fmt=True),
    dict(rays=("lidar", 32, 128), mode="RGL_RETURN_FIRST_LAST", samples=(3, 19), extra=[], noise=False, compact=True, fmt=False),
    dict(rays=("lidar", 4, 100), mode="RGL_RETURN_STRONGEST", samples=(1, 4), extra=["RGL_FIELD_INTENSITY_F32"], noise=False,
         compact=False, fmt=False),
    dict(rays=("grid", 10, 40), mode="RGL_RETURN_FIRST", samples=None, extra=["RGL_FIELD_NORMAL_VEC3_F32"], noise=False, compact=False,
         fmt=False),
]


def pattern_rays(p):
    if p[0] == "grid":
        return scenes.solid_state_rays(p[1], p[2])
    return scenes.lidar_rays(p[1], p[2])


def sensor_pose(k):
    rng = np.random.default_rng(100 + k)
    x, y = rng.uniform(-40, 40, size=2)
    return scenes.trs((x, y, 4.0 + k * 0.5), (0.0, 0.0, rng.uniform(-math.pi, math.pi)))


def make_graph(rgl, cfg, pose):
    lib = rgl.lib()
    n = {k: rgl.node() for k in ("rays", "pose", "range", "trace", "ang", "dist", "compact", "fmt", "out")}
    rgl.rays_from_mat3x4f(n["rays"], pattern_rays(cfg["rays"]))
    rgl.rays_transform(n["pose"], pose)
    rgl.rays_set_range(n["range"], [[0.1, 90.0]])
    rgl.raytrace(n["trace"])
    rgl.check(lib.rgl_node_raytrace_configure_return_mode(n["trace"], getattr(rgl, cfg["mode"])))
    if cfg["samples"] is not None:
        rgl.check(lib.rgl_node_raytrace_configure_beam_divergence(n["trace"], math.radians(0.4), math.radians(0.3)))
        rgl.configure_beam_samples(n["trace"], *cfg["samples"])
    if cfg["extra"]:
        rgl.check(lib.rgl_node_raytrace_configure_default_intensity(n["trace"], 100.0))
    chain = [n["rays"], n["pose"], n["range"], n["trace"]]
    if cfg["noise"]:
        rgl.check(lib.rgl_node_gaussian_noise_angular_hitpoint(C.byref(n["ang"]), 0.0, math.radians(0.05), rgl.RGL_AXIS_Z))
        rgl.check(lib.rgl_node_gaussian_noise_distance(C.byref(n["dist"]), 0.0, 0.02, 0.001))
        chain += [n["ang"], n["dist"]]
    if cfg["compact"]:
        rgl.points_compact_by_field(n["compact"])
        chain.append(n["compact"])
    fields = [rgl.RGL_FIELD_XYZ_VEC3_F32, rgl.RGL_FIELD_DISTANCE_F32, rgl.RGL_FIELD_ENTITY_ID_I32, rgl.RGL_FIELD_IS_HIT_I32,
              rgl.RGL_FIELD_RETURN_TYPE_U8] + [getattr(rgl, f) for f in cfg["extra"]]
    if cfg["fmt"]:
        rgl.points_format(n["fmt"], fields)
        chain.append(n["fmt"])
    rgl.points_yield(n["out"], fields)
    chain.append(n["out"])
    rgl.chain(*chain)
    n["fields"] = fields
    n["cfg"] = cfg
    return n


def reseed(rgl, graphs, frame=0):
    for g in graphs:
        if g["cfg"]["noise"]:
            rgl.set_noise_seed(g["ang"], SEED, frame)
            rgl.set_noise_seed(g["dist"], SEED + 1, frame)


def collect(rgl, g):
    out = {f: rgl.result_bytes(g["out"], f).tobytes() for f in g["fields"]}
    if g["cfg"]["fmt"]:
        out["fmt"] = rgl.result_bytes(g["fmt"], rgl.RGL_FIELD_DYNAMIC_FORMAT).tobytes()
    return out


def solo_results(rgl, graphs, frame=0):
    reseed(rgl, graphs, frame)
    res = []
    for g in graphs:
        rgl.graph_run(g["rays"])
        res.append(collect(rgl, g))
    return res


def assert_same(rgl, batched, solo):
    for k, (b, s) in enumerate(zip(batched, solo)):
        for f in s:
            assert b[f] == s[f], f"sensor {k} field {f}: batched result differs from its solo run"


def build_batch(rgl, scene=None):
    scene = scene or small_multi_entity_scene()
    _, ents = rgl.spawn_scene(scene)
    graphs = [make_graph(rgl, cfg, sensor_pose(k)) for k, cfg in enumerate(SENSORS)]
    batch = rgl.batch_create([g["rays"] for g in graphs])
    return scene, ents, graphs, batch


SCHEDULES = [
    dict(autotune=True),
    dict(autotune=False, block=64, packing=1, order=1, chunk=1, regs=128),
    dict(autotune=False, block=256, packing=0, order=2, chunk=4, regs=96),
    dict(autotune=False, block=128, packing=0, order=0, chunk=8, regs=128),
    dict(autotune=False, block=128, packing=1, order=2, chunk=2, regs=96),
    dict(autotune=False, block=256, packing=0, order=3, chunk=1, regs=128),
]


@pytest.mark.parametrize("sched", SCHEDULES, ids=lambda s: "auto" if s["autotune"] else
                         f"b{s['block']}-p{s['packing']}-o{s['order']}-c{s['chunk']}-r{s['regs']}")
def test_batched_frame_equals_solo_runs(rgl, sched):
    _, _, graphs, batch = build_batch(rgl)
    rgl.batch_configure_schedule(batch, **sched)
    reseed(rgl, graphs)
    rgl.batch_run(batch)
    batched = [collect(rgl, g) for g in graphs]
    st = rgl.batch_stats(batch)
    assert st["beams"] == sum(pattern_rays(c["rays"]).shape[0] for c in SENSORS)
    assert st["frame_ms"] > 0 and st["trace_ms"] > 0
    tuning = rgl.batch_tuning(batch)
    if sched["autotune"]:
        assert st["tunings"] == 1
        # Every stage is recorded; the kept schedule is the fastest candidate tried.
        assert len(tuning) >= 14 and all(ms > 0 for _, ms in tuning)
        assert {(s["packing"], s["order"]) for s, _ in tuning[:8]} == {(p, o) for p in (0, 1) for o in (0, 1, 2, 3)}
        assert rgl.batch_schedule(batch) == min(tuning, key=lambda c: c[1])[0]
    else:
        assert tuning == []
        assert rgl.batch_schedule(batch) == {k: v for k, v in sched.items() if k != "autotune"}
    assert_same(rgl, batched, solo_results(rgl, graphs))
    rgl.batch_destroy(batch)


MIXED_SCHEDULES = [
    dict(autotune=False, block=256, packing=0, order=1, chunk=1, regs=80),
    dict(autotune=False, block=128, packing=1, order=0, chunk=2, regs=96),
    dict(autotune=False, block=64, packing=0, order=2, chunk=4, regs=64),
]


@pytest.mark.parametrize("sched", MIXED_SCHEDULES, ids=lambda s: f"b{s['block']}-p{s['packing']}-o{s['order']}-c{s['chunk']}-r{s['regs']}")
def test_mixed_sample_counts_batch_equals_solo_runs(rgl, sched):
    """Sensors of 1 and 5 samples in one launch (lane groups of 1 and 5 lanes walking the scene
    together, or one lane per beam) write what their solo runs write."""
    scene = small_multi_entity_scene()
    rgl.spawn_scene(scene)
    cfgs = [SENSORS[k] for k in (0, 1, 4, 5)]
    graphs = [make_graph(rgl, cfg, sensor_pose(k)) for k, cfg in enumerate(cfgs)]
    batch = rgl.batch_create([g["rays"] for g in graphs])
    rgl.batch_configure_schedule(batch, **sched)
    reseed(rgl, graphs)
    rgl.batch_run(batch)
    batched = [collect(rgl, g) for g in graphs]
    assert_same(rgl, batched, solo_results(rgl, graphs))
    rgl.batch_destroy(batch)


@pytest.mark.parametrize("waves", [1, 2, 3, 6, 9])
def test_waves_equal_solo_runs(rgl, waves):
    """A frame cut into waves (one traversal launch and one set of later nodes per wave; each graph's
    results readable when its wave ends) writes what the solo runs write, over re-posed frames; the
    wave count is capped by the number of graphs."""
    scene, ents, graphs, batch = build_batch(rgl)
    rgl.batch_configure_schedule(batch, autotune=False, block=128, packing=0, order=1, chunk=1, regs=128)
    rgl.batch_configure_waves(batch, waves)
    assert rgl.batch_waves(batch) == 0
    rng = np.random.default_rng(31)
    captures = []
    for frame in range(3):
        if frame > 0:
            for i, tf in scenes.repose(scene, 0.25, rng):
                rgl.entity_set_transform(ents[i], tf)
        reseed(rgl, graphs, frame)
        rgl.batch_run(batch)
        # Read in batch order right away: the first graphs' reads overlap the later waves.
        batched = [collect(rgl, g) for g in graphs]
        assert rgl.batch_waves(batch) == min(waves, len(graphs))
        st = rgl.batch_stats(batch)
        captures.append(st["captures"])
        assert st["trace_ms"] > 0 and st["frame_ms"] >= st["trace_ms"]
        assert_same(rgl, batched, solo_results(rgl, graphs, frame))
    assert captures[2] == captures[1]  # re-posed frames replay the captured waves
    rgl.batch_destroy(batch)


def test_waves_without_cuda_graphs_equal_solo_runs(rgl):
    """With CUDA graphs off the frame's work is enqueued directly (waves, side stream, events as in the
    captured frame) and writes the same points."""
    lib = rgl.lib()
    rgl.check(lib.rgl_gb300_configure_cuda_graphs(False))
    try:
        scene, ents, graphs, batch = build_batch(rgl)
        rgl.batch_configure_schedule(batch, autotune=False, block=256, packing=1, order=2, chunk=1, regs=128)
        rgl.batch_configure_waves(batch, 3)
        rng = np.random.default_rng(5)
        for frame in range(2):
            if frame > 0:
                for i, tf in scenes.repose(scene, 0.25, rng):
                    rgl.entity_set_transform(ents[i], tf)
            reseed(rgl, graphs, frame)
            rgl.batch_run(batch)
            batched = [collect(rgl, g) for g in graphs]
            assert rgl.batch_waves(batch) == 3
            assert_same(rgl, batched, solo_results(rgl, graphs, frame))
        assert rgl.batch_stats(batch)["captures"] == 0
        rgl.batch_destroy(batch)
    finally:
        rgl.check(lib.rgl_gb300_configure_cuda_graphs(True))


def test_automatic_waves_follow_the_ray_count(rgl):
    """0 waves: one wave per 2 Mi traced rays, at most 16; this batch traces far fewer rays."""
    _, _, graphs, batch = build_batch(rgl)
    rgl.batch_configure_schedule(batch, autotune=False)
    rgl.batch_run(batch)
    assert rgl.batch_waves(batch) == 1
    rgl.batch_configure_waves(batch, 4)
    reseed(rgl, graphs)
    rgl.batch_run(batch)
    assert rgl.batch_waves(batch) == 4
    batched = [collect(rgl, g) for g in graphs]
    assert rgl.batch_stats(batch)["captures"] == 2  # a new wave cut is a new capture
    assert_same(rgl, batched, solo_results(rgl, graphs))
    rgl.batch_destroy(batch)


def test_repose_frames_equal_solo_runs(rgl):
    scene, ents, graphs, batch = build_batch(rgl)
    rng = np.random.default_rng(9)
    for frame in range(4):
        if frame > 0:
            for i, tf in scenes.repose(scene, 0.25, rng):
                rgl.entity_set_transform(ents[i], tf)
        reseed(rgl, graphs, frame)
        rgl.batch_run(batch)
        batched = [collect(rgl, g) for g in graphs]
        assert_same(rgl, batched, solo_results(rgl, graphs, frame))
    rgl.batch_destroy(batch)


def test_repose_reaches_traversal_without_recapture(rgl, oracle):
    """Only the frame's captured refit updates the TLAS here: the oracle sees the new poses, and the
    batch replays its first capture."""
    from test_gpu_raytrace import _check

    scene = small_multi_entity_scene()
    _, ents = rgl.spawn_scene(scene)
    cfg = dict(rays=("lidar", 32, 512), mode="RGL_RETURN_FIRST", samples=None, extra=[], noise=False, compact=False, fmt=False)
    pose = scenes.trs((0.0, 0.0, 5.0), (0.0, 0.0, 0.3))
    graphs = [make_graph(rgl, cfg, pose), make_graph(rgl, SENSORS[1], sensor_pose(1))]
    batch = rgl.batch_create([g["rays"] for g in graphs])
    rng = np.random.default_rng(11)
    for frame in range(3):
        if frame > 0:
            # Move spheres into the sensor's view so a stale TLAS would miss them.
            for i, tf in scenes.repose(scene, 0.5, rng, extent=40.0):
                rgl.entity_set_transform(ents[i], tf)
        rgl.batch_run(batch)
        got = {f: rgl.result(graphs[0]["out"], f) for f in graphs[0]["fields"]}
        exp = oracle.OracleScene(scene).raytrace(pattern_rays(cfg["rays"]), ray_transform=pose, ranges=[[0.1, 90.0]],
                                                 return_mode=rgl.RGL_RETURN_FIRST)
        _check(rgl, got, exp)
    st = rgl.batch_stats(batch)
    assert (st["captures"], st["replays"]) == (1, 2)
    rgl.batch_destroy(batch)


def test_batch_validation_follows_graph_edits(rgl):
    """Frames that only re-pose entities keep the graphs' last validation; any other API call may edit
    a graph, so the next frame validates again and reports what the edit broke."""
    scene, ents, graphs, batch = build_batch(rgl)
    rgl.batch_configure_schedule(batch, autotune=False)
    reseed(rgl, graphs)
    rgl.batch_run(batch)
    rng = np.random.default_rng(21)
    for i, tf in scenes.repose(scene, 0.25, rng):
        rgl.entity_set_transform(ents[i], tf)
    rgl.batch_run(batch)  # nothing but poses changed since the last frame (the noise frame advanced to 1)
    batched = [collect(rgl, g) for g in graphs]
    assert_same(rgl, batched, solo_results(rgl, graphs, frame=1))
    # Two ranges for a pattern of many rays: the graph no longer validates.
    rgl.rays_set_range(graphs[1]["range"], [[0.1, 90.0], [0.1, 90.0]])
    with pytest.raises(rgl.RGLError) as e:
        rgl.batch_run(batch)
    assert e.value.status == rgl.RGL_INVALID_PIPELINE
    assert "doesn't match number of rays" in str(e.value)
    rgl.rays_set_range(graphs[1]["range"], [[0.1, 90.0]])
    reseed(rgl, graphs)
    rgl.batch_run(batch)
    batched = [collect(rgl, g) for g in graphs]
    assert_same(rgl, batched, solo_results(rgl, graphs))
    rgl.batch_destroy(batch)


def test_batch_recaptures_on_structure_change(rgl):
    scene, ents, graphs, batch = build_batch(rgl)
    rgl.batch_configure_schedule(batch, autotune=False)
    rgl.batch_run(batch)
    rgl.batch_run(batch)
    assert (rgl.batch_stats(batch)["captures"], rgl.batch_stats(batch)["replays"]) == (1, 1)
    # A new entity changes the TLAS topology: rebuilt outside the capture, then recaptured.
    cube = scenes.cube_mesh(2.0)
    e = rgl.entity_create(rgl.mesh_create(cube.vertices, cube.indices))
    rgl.entity_set_transform(e, scenes.translation(0, 0, 3))
    rgl.batch_run(batch)
    assert rgl.batch_stats(batch)["captures"] == 2
    # A new ray count changes the batch shape: recaptured (and the job table rebuilt).
    rgl.rays_from_mat3x4f(graphs[0]["rays"], scenes.lidar_rays(8, 100))
    reseed(rgl, graphs)
    rgl.batch_run(batch)
    batched = [collect(rgl, g) for g in graphs]
    assert rgl.batch_stats(batch)["captures"] == 3
    assert_same(rgl, batched, solo_results(rgl, graphs))
    rgl.batch_destroy(batch)


def test_batch_rejects_graph_without_single_raytrace(rgl):
    n_rays, n_y = rgl.node(), rgl.node()
    rgl.rays_from_mat3x4f(n_rays, scenes.lidar_rays(2, 8))
    rgl.raytrace(n_y)
    b = rgl.batch_create([n_rays])  # the rays node alone: no raytrace node in its graph
    with pytest.raises(rgl.RGLError) as e:
        rgl.batch_run(b)
    assert "exactly one RaytraceNode" in str(e.value)
    rgl.batch_destroy(b)


def test_batch_api_argument_checks(rgl):
    lib = rgl.lib()
    b = C.c_void_p()
    assert lib.rgl_gb300_batch_create(C.byref(b), None, 1) == rgl.RGL_INVALID_ARGUMENT
    arr = (C.c_void_p * 1)(None)
    assert lib.rgl_gb300_batch_create(C.byref(b), arr, 1) == rgl.RGL_INVALID_ARGUMENT
    assert lib.rgl_gb300_batch_configure_waves(C.c_void_p(0x1234), 2) == rgl.RGL_INVALID_API_OBJECT
    assert lib.rgl_gb300_batch_configure_waves(None, 2) == rgl.RGL_INVALID_ARGUMENT
    assert lib.rgl_gb300_batch_run(C.c_void_p(0x1234)) == rgl.RGL_INVALID_API_OBJECT
    assert "Object does not exist: Batch" in rgl.last_error()
