"""Resident scenes (rgl_gb300_scene_*) and the serving loop (rgl_gb300_server_*) on the GPU.

The serving property: a request's result is byte-identical whether it is served alone, in a mix of
concurrent requests coalesced into batches, or computed by the equivalent plain RGL graph
(rays_from_mat3x4f -> rays_transform -> rays_set_range -> raytrace -> compact_by_field -> yield).
"""
import ctypes as C
import math

import numpy as np
import pytest

from robotecgpulidar_gb300 import scenes

pytestmark = pytest.mark.gpu

FIELDS = None


def fields(rgl):
    return [rgl.RGL_FIELD_XYZ_VEC3_F32, rgl.RGL_FIELD_DISTANCE_F32, rgl.RGL_FIELD_ENTITY_ID_I32]


def two_scenes(rgl):
    a = scenes.million_scene(seed=5, instances=12, spheres=2, cells=64, extent=120.0)
    b = scenes.million_scene(seed=8, instances=20, spheres=2, cells=48, extent=100.0)
    meshes_a, _ = rgl.spawn_scene_in(sa := rgl.scene_create(), a)
    _, _ = rgl.spawn_scene_in(sb := rgl.scene_create(), b)
    return (sa, a), (sb, b)


PATTERNS = [("lidar", 16, 256), ("grid", 24, 64), ("lidar", 32, 512), ("lidar", 4, 90)]


def pattern_rays(p):
    return scenes.solid_state_rays(p[1], p[2]) if p[0] == "grid" else scenes.lidar_rays(p[1], p[2])


def pose(k):
    rng = np.random.default_rng(1000 + k)
    x, y = rng.uniform(-35, 35, size=2)
    return scenes.trs((x, y, rng.uniform(2.0, 6.0)), (0.0, 0.0, rng.uniform(-math.pi, math.pi)))


def served(rgl, srv, req):
    return {f: srv.result(req, f).tobytes() for f in fields(rgl)}


def plain_graph_result(rgl, scene, rays, tf, mode, rng_min, rng_max):
    n = {k: rgl.node() for k in ("rays", "pose", "range", "trace", "cmp", "out")}
    rgl.rays_from_mat3x4f(n["rays"], rays)
    rgl.rays_transform(n["pose"], tf)
    rgl.rays_set_range(n["range"], [[rng_min, rng_max]])
    rgl.raytrace_in(n["trace"], scene)
    rgl.check(rgl.lib().rgl_node_raytrace_configure_return_mode(n["trace"], mode))
    rgl.points_compact_by_field(n["cmp"])
    rgl.points_yield(n["out"], fields(rgl))
    rgl.chain(n["rays"], n["pose"], n["range"], n["trace"], n["cmp"], n["out"])
    rgl.graph_run(n["rays"])
    out = {f: rgl.result_bytes(n["out"], f).tobytes() for f in fields(rgl)}
    rgl.check(rgl.lib().rgl_graph_destroy(n["rays"]))
    return out


def test_request_alone_in_mix_and_plain_graph_agree(rgl):
    (sa, _), (sb, _) = two_scenes(rgl)
    srv = rgl.Server(8 << 30, 2)
    try:
        pats = [srv.add_pattern(pattern_rays(p)) for p in PATTERNS]
        probe = dict(scene=sa, pattern=pats[2], pose=pose(0), mode=rgl.RGL_RETURN_FIRST_LAST, lo=0.1, hi=80.0)

        def submit_probe():
            return srv.submit(probe["scene"], probe["pattern"], probe["pose"], probe["mode"], probe["lo"], probe["hi"])

        alone = submit_probe()
        assert srv.wait(alone)
        res_alone = served(rgl, srv, alone)
        assert len(res_alone[rgl.RGL_FIELD_DISTANCE_F32]) > 0
        srv.release(alone)
        b0 = srv.stats()["batches"]

        rng = np.random.default_rng(3)
        mix = []
        for k in range(60):
            if k == 30:
                mix.append(("probe", submit_probe()))
            sc = sa if rng.random() < 0.5 else sb
            mode = rgl.RGL_RETURN_FIRST if rng.random() < 0.5 else rgl.RGL_RETURN_FIRST_LAST
            mix.append(("other", srv.submit(sc, pats[int(rng.integers(0, len(pats)))], pose(k + 1), mode, 0.1, 90.0)))
        for _, req in mix:
            assert srv.wait(req, 20000.0)
        res_mix = served(rgl, srv, [r for t, r in mix if t == "probe"][0])
        st = srv.stats()
        # Continuous batching coalesced the mix: fewer batches than requests.
        assert st["batches"] - b0 < len(mix)
        assert st["completed"] == len(mix) + 1
        for _, req in mix:
            srv.release(req)
        assert res_mix == res_alone
        plain = plain_graph_result(rgl, probe["scene"], pattern_rays(PATTERNS[2]), probe["pose"], probe["mode"], probe["lo"], probe["hi"])
        assert plain == res_alone
    finally:
        srv.destroy()


def test_every_request_of_a_mix_equals_its_plain_graph(rgl):
    (sa, _), (sb, _) = two_scenes(rgl)
    srv = rgl.Server(8 << 30, 2)
    try:
        pats = [srv.add_pattern(pattern_rays(p)) for p in PATTERNS]
        specs = []
        rng = np.random.default_rng(4)
        for k in range(12):
            specs.append(dict(scene=sa if k % 2 == 0 else sb, p=int(rng.integers(0, len(pats))), pose=pose(50 + k),
                              mode=rgl.RGL_RETURN_FIRST if k % 3 else rgl.RGL_RETURN_FIRST_LAST, lo=0.1 * (k % 2), hi=60.0 + k))
        reqs = [srv.submit(s["scene"], pats[s["p"]], s["pose"], s["mode"], s["lo"], s["hi"]) for s in specs]
        for r in reqs:
            assert srv.wait(r, 20000.0)
        got = [served(rgl, srv, r) for r in reqs]
        for s, g in zip(specs, got):
            assert g == plain_graph_result(rgl, s["scene"], pattern_rays(PATTERNS[s["p"]]), s["pose"], s["mode"], s["lo"], s["hi"])
        q, t = srv.timing(reqs[-1])
        assert 0.0 <= q <= t
    finally:
        srv.destroy()


def test_admission_respects_hbm_budget(rgl):
    (sa, _), _ = two_scenes(rgl)
    rays = pattern_rays(PATTERNS[2])  # 16,384 beams
    per_request = rays.shape[0] * 2 * (24 + 20)  # dual return: raw + compacted bytes per point
    srv = rgl.Server(int(2.5 * per_request), 2)
    try:
        pat = srv.add_pattern(rays)
        reqs = [srv.submit(sa, pat, pose(k), rgl.RGL_RETURN_FIRST_LAST, 0.1, 90.0) for k in range(10)]
        for r in reqs:
            assert srv.wait(r, 20000.0)
            srv.release(r)  # frees the compacted result, so later requests fit
        st = srv.stats()
        assert st["completed"] == 10
        assert st["peak_reserved_bytes"] <= int(2.5 * per_request)
        assert st["batches"] >= 5  # at most two requests fit at a time
        # A request larger than the whole budget is refused at submission.
        big = srv.add_pattern(scenes.lidar_rays(64, 1024))
        with pytest.raises(rgl.RGLError) as e:
            srv.submit(sa, big, pose(0), rgl.RGL_RETURN_FIRST_LAST, 0.1, 90.0)
        assert e.value.status == rgl.RGL_INVALID_ARGUMENT
    finally:
        srv.destroy()


def test_server_argument_checks(rgl):
    srv = rgl.Server(1 << 30, 2)
    try:
        with pytest.raises(rgl.RGLError) as e:
            srv.submit(None, 7, pose(0), rgl.RGL_RETURN_FIRST)
        assert e.value.status == rgl.RGL_INVALID_ARGUMENT and "pattern 7" in str(e.value)
        lib = rgl.lib()
        assert lib.rgl_gb300_server_release(srv.h, 12345) == rgl.RGL_INVALID_API_OBJECT
        assert "Object does not exist: Request 12345" in rgl.last_error()
    finally:
        srv.destroy()


def test_resident_scenes_are_separate(rgl):
    cube = scenes.cube_mesh(1.0)
    m = rgl.mesh_create(cube.vertices, cube.indices)
    sa, sb = rgl.scene_create(), rgl.scene_create()
    ea = rgl.entity_create_in(sa, m)
    rgl.entity_set_transform(ea, scenes.translation(0, 0, 5))
    rgl.entity_set_id(ea, 11)
    eb = rgl.entity_create_in(sb, m)
    rgl.entity_set_transform(eb, scenes.translation(0, 0, 9))
    rgl.entity_set_id(eb, 22)

    def trace(scene):
        n_rays, n_rt, n_y = rgl.node(), rgl.node(), rgl.node()
        rgl.rays_from_mat3x4f(n_rays, [scenes.translation(0, 0, 0)])
        rgl.raytrace_in(n_rt, scene)
        rgl.points_yield(n_y, [rgl.RGL_FIELD_DISTANCE_F32, rgl.RGL_FIELD_ENTITY_ID_I32, rgl.RGL_FIELD_IS_HIT_I32])
        rgl.chain(n_rays, n_rt, n_y)
        rgl.graph_run(n_rays)
        return (rgl.result(n_y, rgl.RGL_FIELD_DISTANCE_F32)[0], rgl.result(n_y, rgl.RGL_FIELD_ENTITY_ID_I32)[0],
                rgl.result(n_y, rgl.RGL_FIELD_IS_HIT_I32)[0])

    assert trace(sa) == (4.0, 11, 1)
    assert trace(sb) == (8.0, 22, 1)
    assert trace(None)[2] == 0  # the default scene is empty
    rgl.scene_destroy(sb)
    assert rgl.lib().rgl_entity_set_id(eb, 3) == rgl.RGL_INVALID_API_OBJECT  # destroyed with its scene


def test_batch_over_two_scenes_equals_solo(rgl):
    from test_gpu_batch import assert_same, collect, make_graph, SENSORS

    (sa, _), (sb, _) = two_scenes(rgl)
    graphs = []
    for k, cfg in enumerate(SENSORS[:4]):
        g = make_graph(rgl, dict(cfg, noise=False), pose(200 + k))
        rgl.raytrace_in(g["trace"], sa if k % 2 == 0 else sb)
        graphs.append(g)
    batch = rgl.batch_create([g["rays"] for g in graphs])
    rgl.batch_run(batch)
    batched = [collect(rgl, g) for g in graphs]
    solo = []
    for g in graphs:
        rgl.graph_run(g["rays"])
        solo.append(collect(rgl, g))
    assert_same(rgl, batched, solo)
    rgl.batch_destroy(batch)


def test_batches_of_varying_size_complete_and_host_results_match(rgl):
    """Batches of 1, 60, 3 and 200 requests in turn (launch shapes that grow and shrink) all complete;
    the host-resident result equals the copied one."""
    (sa, _), (sb, _) = two_scenes(rgl)
    srv = rgl.Server(8 << 30, 2)
    try:
        pats = [srv.add_pattern(pattern_rays(p)) for p in PATTERNS]
        rng = np.random.default_rng(21)
        for wave in (1, 60, 3, 200):
            reqs = [srv.submit(sa if k % 2 else sb, pats[int(rng.integers(0, len(pats)))], pose(k), rgl.RGL_RETURN_FIRST_LAST, 0.1, 90.0)
                    for k in range(wave)]
            for r in reqs:
                assert srv.wait(r, 20000.0)
            r0 = reqs[-1]
            ptr, cnt = C.c_void_p(), C.c_int32()
            rgl.check(rgl.lib().rgl_gb300_server_get_result_host(srv.h, r0, rgl.RGL_FIELD_DISTANCE_F32, C.byref(ptr), C.byref(cnt)))
            host = np.ctypeslib.as_array(C.cast(ptr, C.POINTER(C.c_float)), shape=(cnt.value,)).copy() if cnt.value else np.zeros(0, np.float32)
            assert np.array_equal(host, srv.result(r0, rgl.RGL_FIELD_DISTANCE_F32))
            for r in reqs:
                srv.release(r)
        assert srv.stats()["failed"] == 0
        # Every retired batch was timed in its three phases on the device's clock.
        srv.drain()
        bt = srv.batch_times(reset=True)
        assert bt["batches"] == srv.stats()["batches"]
        assert bt["max_ms"]["trace"] > 0 and bt["max_ms"]["copies"] >= 0
        assert srv.batch_times()["batches"] == 0
    finally:
        srv.destroy()


def test_server_schedule_changes_speed_only(rgl):
    """Scan-row, natural and octahedral beam order, other block/register shapes and batches capped at
    a few thousand beams (every request its own batch) give byte-identical results."""
    (sa, _), (sb, _) = two_scenes(rgl)
    srv = rgl.Server(8 << 30, 2)
    try:
        pats = [srv.add_pattern(pattern_rays(p)) for p in PATTERNS]
        specs = [(sa if k % 2 else sb, pats[k % len(pats)], pose(300 + k), rgl.RGL_RETURN_FIRST_LAST if k % 3 else rgl.RGL_RETURN_FIRST)
                 for k in range(16)]
        runs = []
        for sched in (dict(), dict(order=0), dict(block=128, regs=64, chunk=4), dict(order=2, regs=128, max_batch_beams=4096),
                      dict(order=1, block=128)):
            srv.configure_schedule(**sched)
            reqs = [srv.submit(sc, p, tf, mode, 0.1, 90.0) for sc, p, tf, mode in specs]
            for r in reqs:
                assert srv.wait(r, 20000.0)
            runs.append([served(rgl, srv, r) for r in reqs])
            for r in reqs:
                srv.release(r)
        for other in runs[1:]:
            assert other == runs[0]
        with pytest.raises(rgl.RGLError) as e:
            srv.configure_schedule(block=96)
        assert e.value.status == rgl.RGL_INVALID_ARGUMENT
    finally:
        srv.destroy()
