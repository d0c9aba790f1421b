"""Accuracy of every benchmarked configuration against the FP64 oracle, at the benchmarked sizes.

Each test runs the configuration's graph through the C API (the raytrace output read by a yield
before the point nodes) and the oracle on the same seeded scene, rays and poses, asserts the parity
bounds (tests/accuracy.py) and records agreement, ambiguous points and the maximum / p99 relative
distance error of the configuration:
  config0  plain scene (20,768 triangles), 32x1024 beams, first return, sensor at (0, 0, 1.8) m;
  config1  plain scene, 64x2048 beams, then angular + distance noise, world transform, compaction
           and format (the point chain replayed by the oracle on the GPU's raytrace output);
  config2  1M-triangle scene, 128x2048 beams, FIRST_LAST, 0.2 deg divergence in 5 sub-rays, sensor
           at (0, 0, 6) m, then the noise chain and compaction, exactly the single-sensor benchmark;
  config2_58  the same scan with the reference's 58-sample divergence pattern;
  config3  the 64-sensor batched frame on the 1M-triangle scene, before and after re-posing 20 % of
           the entities (the refit inside the captured frame);
  config4  requests of the serving fleet over the four resident scenes (0.2M-4M triangles), served
           by the continuous-batching server: each served result equals the plain graph's compacted
           result byte for byte, and the plain graph's raytrace output is compared with the oracle.
"""
import ctypes as C
import math

import numpy as np
import pytest

import accuracy
from robotecgpulidar_gb300 import scenes

pytestmark = pytest.mark.gpu

RANGE = [[0.1, 100.0]]
SIGMA = math.radians(0.05)
DIV = math.radians(0.2)


def raytrace_fields(rgl):
    return [rgl.RGL_FIELD_XYZ_VEC3_F32, rgl.RGL_FIELD_DISTANCE_F32, rgl.RGL_FIELD_ENTITY_ID_I32, rgl.RGL_FIELD_IS_HIT_I32,
            rgl.RGL_FIELD_RETURN_TYPE_U8]


def sensor_graph(rgl, rays, pose, mode, samples=None, noise=False, world=None, fmt=False, seed=1234):
    """rays -> pose -> range -> raytrace -> yield(raytrace fields) [-> noise -> transform -> compact
    -> yield / format]; the same nodes as the benchmark's sensor graph plus the raytrace yield."""
    lib = rgl.lib()
    n = {k: rgl.node() for k in ("rays", "pose", "range", "trace", "y", "ang", "dist", "tf", "cmp", "out", "fmt")}
    rgl.rays_from_mat3x4f(n["rays"], rays)
    rgl.rays_transform(n["pose"], pose)
    rgl.rays_set_range(n["range"], RANGE)
    rgl.raytrace(n["trace"])
    rgl.check(lib.rgl_node_raytrace_configure_return_mode(n["trace"], mode))
    if samples is not None:
        rgl.check(lib.rgl_node_raytrace_configure_beam_divergence(n["trace"], DIV, DIV))
        rgl.configure_beam_samples(n["trace"], *samples)
    rgl.points_yield(n["y"], raytrace_fields(rgl))
    chain = [n["rays"], n["pose"], n["range"], n["trace"], n["y"]]
    if noise:
        rgl.check(lib.rgl_node_gaussian_noise_angular_hitpoint(C.byref(n["ang"]), 0.0, SIGMA, rgl.RGL_AXIS_Z))
        rgl.check(lib.rgl_node_gaussian_noise_distance(C.byref(n["dist"]), 0.0, 0.02, 0.001))
        rgl.set_noise_seed(n["ang"], seed)
        rgl.set_noise_seed(n["dist"], seed)
        chain += [n["ang"], n["dist"]]
        if world is not None:
            rgl.points_transform(n["tf"], world)
            chain.append(n["tf"])
        rgl.points_compact_by_field(n["cmp"])
        chain.append(n["cmp"])
        out = [rgl.RGL_FIELD_XYZ_VEC3_F32, rgl.RGL_FIELD_DISTANCE_F32, rgl.RGL_FIELD_ENTITY_ID_I32]
        if fmt:
            rgl.points_format(n["fmt"], out)
            chain.append(n["fmt"])
        else:
            rgl.points_yield(n["out"], out)
            chain.append(n["out"])
    rgl.chain(*chain)
    return n


def read_raytrace(rgl, n):
    return {f: rgl.result(n["y"], f) for f in raytrace_fields(rgl)}


def check_point_chain(rgl, oracle, n, got, pose, world, fmt, seed=1234):
    """The compacted, noised points against the oracle's replay of the chain on the GPU's own raytrace
    output: entity ids and count exact, XYZ within 1e-5 of the coordinate magnitude, distance within
    1e-5 relative. Returns the maximum and p99 relative error of XYZ and distance."""
    xyz0 = got[rgl.RGL_FIELD_XYZ_VEC3_F32]
    L = oracle.inv34(pose)
    xyz1, d1 = oracle.noise_angular_hitpoint(L, 0.0, SIGMA, rgl.RGL_AXIS_Z, seed, 0, xyz0)
    xyz2, d2 = oracle.noise_distance(L, 0.0, 0.02, 0.001, seed, 0, xyz1, d1)
    if world is not None:
        xyz2 = oracle.transform_points(world, xyz2)
    hit = got[rgl.RGL_FIELD_IS_HIT_I32]
    if fmt:
        cnt, size = rgl.result_size(n["fmt"], rgl.RGL_FIELD_DYNAMIC_FORMAT)
        assert size == 20
        raw = rgl.result_bytes(n["fmt"], rgl.RGL_FIELD_DYNAMIC_FORMAT).reshape(cnt, 20)
        gx = raw[:, :12].copy().view(np.float32).reshape(cnt, 3)
        gd = raw[:, 12:16].copy().view(np.float32).ravel()
        ge = raw[:, 16:20].copy().view(np.int32).ravel()
    else:
        gx = rgl.result(n["out"], rgl.RGL_FIELD_XYZ_VEC3_F32)
        gd = rgl.result(n["out"], rgl.RGL_FIELD_DISTANCE_F32)
        ge = rgl.result(n["out"], rgl.RGL_FIELD_ENTITY_ID_I32)
        cnt = gd.shape[0]
    assert cnt == int(hit.sum())
    ex, ed, ee = oracle.compact(hit, xyz2), oracle.compact(hit, d2), oracle.compact(hit, got[rgl.RGL_FIELD_ENTITY_ID_I32])
    assert np.array_equal(ge, ee)
    scale = np.maximum(np.abs(ex).max(axis=1), 1.0)
    xerr = np.abs(gx.astype(np.float64) - ex).max(axis=1) / scale
    derr = np.abs(gd.astype(np.float64) - ed) / np.maximum(np.abs(ed), 1e-6)
    assert xerr.max(initial=0.0) <= 1e-5 and derr.max(initial=0.0) <= 1e-5
    return {"chain_points": int(cnt), "chain_max_rel_xyz_error": float(xerr.max(initial=0.0)),
            "chain_p99_rel_xyz_error": float(np.quantile(xerr, 0.99)) if xerr.size else 0.0,
            "chain_max_rel_distance_error": float(derr.max(initial=0.0)),
            "chain_p99_rel_distance_error": float(np.quantile(derr, 0.99)) if derr.size else 0.0}


def test_accuracy_config0(rgl, oracle):
    scene, rays, pose = scenes.plain_scene(), scenes.lidar_rays(32, 1024), scenes.translation(0, 0, 1.8)
    rgl.spawn_scene(scene)
    n = sensor_graph(rgl, rays, pose, rgl.RGL_RETURN_FIRST)
    rgl.graph_run(n["rays"])
    got = read_raytrace(rgl, n)
    exp = oracle.OracleScene(scene).raytrace(rays, ray_transform=pose, ranges=RANGE)
    stats, _ = accuracy.evaluate(rgl, got, exp, beams=rays.shape[0], samples_per_beam=1)
    accuracy.record("config0", stats)
    accuracy.assert_within_bounds(stats)


def test_accuracy_config1(rgl, oracle):
    scene, rays, pose = scenes.plain_scene(), scenes.lidar_rays(64, 2048), scenes.translation(0, 0, 1.8)
    rng = np.random.default_rng(1)
    world = scenes.trs(rng.uniform(-50, 50, 3), rng.uniform(-np.pi, np.pi, 3))
    rgl.spawn_scene(scene)
    n = sensor_graph(rgl, rays, pose, rgl.RGL_RETURN_FIRST, noise=True, world=world, fmt=True)
    rgl.graph_run(n["rays"])
    got = read_raytrace(rgl, n)
    exp = oracle.OracleScene(scene).raytrace(rays, ray_transform=pose, ranges=RANGE)
    stats, _ = accuracy.evaluate(rgl, got, exp, beams=rays.shape[0], samples_per_beam=1)
    accuracy.record("config1", stats)
    accuracy.assert_within_bounds(stats)
    stats.update(check_point_chain(rgl, oracle, n, got, pose, world, fmt=True))
    accuracy.record("config1", stats)


@pytest.mark.parametrize("name,samples", [("config2", (1, 4)), ("config2_58", (3, 19))])
def test_accuracy_config2_full_scan(rgl, oracle, name, samples):
    scene, rays, pose = scenes.million_scene(), scenes.lidar_rays(128, 2048), scenes.translation(0.0, 0.0, 6.0)
    rgl.spawn_scene(scene)
    n = sensor_graph(rgl, rays, pose, rgl.RGL_RETURN_FIRST_LAST, samples=samples, noise=True)
    rgl.graph_run(n["rays"])
    got = read_raytrace(rgl, n)
    exp = oracle.OracleScene(scene).raytrace(rays, ray_transform=pose, ranges=RANGE, return_mode=rgl.RGL_RETURN_FIRST_LAST,
                                             h_div=DIV, v_div=DIV, layers=samples[0], vertices=samples[1])
    stats, _ = accuracy.evaluate(rgl, got, exp, beams=rays.shape[0], samples_per_beam=1 + samples[0] * samples[1],
                                 sensor_position_m=[0.0, 0.0, 6.0])
    accuracy.record(name, stats)
    accuracy.assert_within_bounds(stats)
    stats.update(check_point_chain(rgl, oracle, n, got, pose, None, fmt=False))
    accuracy.record(name, stats)


def test_accuracy_config3_batched_frame(rgl, oracle):
    scene = scenes.million_scene()
    _, ents = rgl.spawn_scene(scene)
    rig = scenes.sensor_rig(scene, 64, seed=4)
    graphs = [sensor_graph(rgl, s.rays(), s.pose, rgl.RGL_RETURN_FIRST_LAST, samples=(1, 4), noise=True) for s in rig]
    batch = rgl.batch_create([g["rays"] for g in graphs])
    osc = oracle.OracleScene(scene)
    rng = np.random.default_rng(6)
    frames = []
    for frame in range(2):
        if frame:
            for i, tf in scenes.repose(scene, 0.2, rng):
                rgl.entity_set_transform(ents[i], tf)
                osc.set_instance(i, tf, scene.entities[i].entity_id)
            osc.build()
        rgl.batch_run(batch)
        rgl.batch_stats(batch)
        tally = accuracy.Tally()
        for si, (s, g) in enumerate(zip(rig, graphs)):
            got = read_raytrace(rgl, g)
            exp = osc.raytrace(s.rays(), ray_transform=s.pose, ranges=RANGE, return_mode=rgl.RGL_RETURN_FIRST_LAST, h_div=DIV,
                               v_div=DIV, layers=1, vertices=4)
            tally.add(rgl, got, exp, tag=f"frame {frame} sensor {si} {s.pattern}")
        stats = tally.finish(sensors=len(rig), beams=sum(s.beam_count for s in rig), samples_per_beam=5,
                             frame="after 20 % re-pose" if frame else "first")
        frames.append(stats)
    rgl.batch_destroy(batch)
    accuracy.record("config3", {**frames[-1], "first_frame": frames[0]})
    for stats in frames:
        accuracy.assert_within_bounds(stats)


def test_accuracy_config4_served_requests(rgl, oracle):
    triangles = (200_000, 1_000_000, 2_000_000, 4_000_000)
    scene_objs = [scenes.serving_scene(t, 10 + k) for k, t in enumerate(triangles)]
    handles = []
    for sc in scene_objs:
        h = rgl.scene_create()
        rgl.spawn_scene_in(h, sc)
        handles.append(h)
    fleet = scenes.robot_fleet(scene_objs, 256, seed=5)
    oscs = [oracle.OracleScene(sc) for sc in scene_objs]
    picked = list(range(0, 256, 11))  # 24 robots spread over the fleet
    modes = (rgl.RGL_RETURN_FIRST, rgl.RGL_RETURN_FIRST_LAST)
    out_fields = [rgl.RGL_FIELD_XYZ_VEC3_F32, rgl.RGL_FIELD_DISTANCE_F32, rgl.RGL_FIELD_ENTITY_ID_I32]
    srv = rgl.Server(8 << 30, 2)
    tally = accuracy.Tally()
    try:
        reqs = []
        for j, k in enumerate(picked):
            r = fleet[k]
            pat = srv.add_pattern(scenes.lidar_rays(*r.pattern))
            reqs.append((k, modes[j % 2], srv.submit(handles[r.scene], pat, r.pose, modes[j % 2], *RANGE[0])))
        rays_total = 0
        for k, mode, q in reqs:
            assert srv.wait(q, 60000.0)
            r = fleet[k]
            rays = scenes.lidar_rays(*r.pattern)
            rays_total += rays.shape[0]
            served = {f: srv.result(q, f).tobytes() for f in out_fields}
            srv.release(q)
            n = {x: rgl.node() for x in ("rays", "pose", "range", "trace", "y", "cmp", "out")}
            rgl.rays_from_mat3x4f(n["rays"], rays)
            rgl.rays_transform(n["pose"], r.pose)
            rgl.rays_set_range(n["range"], RANGE)
            rgl.raytrace_in(n["trace"], handles[r.scene])
            rgl.check(rgl.lib().rgl_node_raytrace_configure_return_mode(n["trace"], mode))
            rgl.points_yield(n["y"], raytrace_fields(rgl))
            rgl.points_compact_by_field(n["cmp"])
            rgl.points_yield(n["out"], out_fields)
            rgl.chain(n["rays"], n["pose"], n["range"], n["trace"], n["y"], n["cmp"], n["out"])
            rgl.graph_run(n["rays"])
            assert {f: rgl.result_bytes(n["out"], f).tobytes() for f in out_fields} == served
            got = read_raytrace(rgl, n)
            exp = oscs[r.scene].raytrace(rays, ray_transform=r.pose, ranges=RANGE, return_mode=mode)
            tally.add(rgl, got, exp, tag=f"robot {k} scene {r.scene}")
            rgl.check(rgl.lib().rgl_graph_destroy(n["rays"]))
    finally:
        srv.destroy()
    stats = tally.finish(requests=len(picked), beams=rays_total, samples_per_beam=1, scenes_triangles=list(triangles))
    accuracy.record("config4", stats)
    accuracy.assert_within_bounds(stats)
