#!/usr/bin/env python3
"""Benchmark of the lidar ray-casting hot path on the 1M-triangle scene.

Workload (one step = one lidar scan through the RGL C API): million-triangle scene (512x512-cell
value-noise terrain + 93 posed icosphere entities, 1,000,448 triangles), one sensor at (0, 0, 6) m,
128 channels x 2048 azimuth steps = 262,144 beams, dual return (first + last), 0.2 deg beam divergence
sampled by 5 sub-rays per beam (1,310,720 rays per scan), range [0.1, 100] m, angular hit-point noise
(sigma 0.05 deg about the sensor up axis) and distance noise (sigma 0.02 m + 0.001 d), Philox seed 1234,
then compaction by is-hit. Rays/s counts sub-rays.

Reported:
  value  device time of whole graph runs with inputs resident in HBM (CUDA events on the graph's
         stream), L2 flushed (256 MiB write) before every step;
  e2e    the same scans end to end through the C API from pinned host memory: ray upload
         (rgl_node_rays_from_mat3x4f), rgl_graph_run, result size and XYZ/distance/entity-id read-back;
  roofline  algorithmic bytes of the traversal kernel / its event-timed duration vs measured HBM peak;
  cpu_baseline  the FP64 CPU oracle casting the same scan on the host cores.
``--impl reference`` times the CPU implementation of the path (the oracle restatement; the reference's
OptiX build cannot be built or run here) on the same workload.
"""
from __future__ import annotations

import argparse
import gc
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Mrays/s at 1M-tri scene; p50/p99 scan latency, served vs plain, 1 GB300"
CHANNELS, AZIMUTHS, LAYERS, VERTICES = 128, 2048, 1, 4
SUBRAYS = 1 + LAYERS * VERTICES
SENSOR = (0.0, 0.0, 6.0)
RANGE = (0.1, 100.0)
DIVERGENCE_RAD = math.radians(0.2)
ANGULAR_SIGMA = math.radians(0.05)
SEED = 1234
L2_FLUSH_BYTES = 256 << 20


def workload_config():
    return {
        "workload": "1M-tri scene single sensor: 128x2048 beams, FIRST_LAST, 5 sub-rays/beam in 0.2 deg, "
                    "angular+distance noise, compaction by is-hit",
        "triangles": 1000448,
        "beams": CHANNELS * AZIMUTHS,
        "rays_per_step": CHANNELS * AZIMUTHS * SUBRAYS,
        "returns_per_beam": 2,
        "l2": "flushed (256 MiB write) before every timed step",
    }


def rank_info():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


class Clocks:
    """Samples nvidia-smi SM clocks and throttle reasons during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.path = None

    def start(self):
        """Starts sampling every 50 ms and returns once the first sample is written (at most 5 s)."""
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                                          "-lms", "50"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (FileNotFoundError, OSError):
            self.proc = None
            return
        t0 = time.perf_counter()
        while time.perf_counter() - t0 < 5.0 and os.path.getsize(self.path) == 0:
            time.sleep(0.02)

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx = float(p[2])
            except ValueError:
                continue
            for k, n in enumerate(names):
                if p[5 + k].lower() == "active":
                    reasons.add(n)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def build_sensor_graph(rgl, rays, pose):
    """One sensor's graph: rays -> pose -> range -> raytrace (FIRST_LAST, 0.2 deg divergence, 5 sub-rays)
    -> angular + distance noise -> compaction by is-hit -> yield."""
    import ctypes as C

    lib = rgl.lib()
    n = {k: rgl.node() for k in ("rays", "pose", "range", "trace", "ang", "dist", "compact", "out")}
    rgl.rays_from_mat3x4f(n["rays"], rays)
    rgl.rays_transform(n["pose"], pose)
    rgl.rays_set_range(n["range"], [RANGE])
    rgl.raytrace(n["trace"])
    rgl.check(lib.rgl_node_raytrace_configure_return_mode(n["trace"], rgl.RGL_RETURN_FIRST_LAST))
    rgl.check(lib.rgl_node_raytrace_configure_beam_divergence(n["trace"], DIVERGENCE_RAD, DIVERGENCE_RAD))
    rgl.configure_beam_samples(n["trace"], LAYERS, VERTICES)
    rgl.check(lib.rgl_node_gaussian_noise_angular_hitpoint(C.byref(n["ang"]), 0.0, ANGULAR_SIGMA, rgl.RGL_AXIS_Z))
    rgl.check(lib.rgl_node_gaussian_noise_distance(C.byref(n["dist"]), 0.0, 0.02, 0.001))
    rgl.set_noise_seed(n["ang"], SEED)
    rgl.set_noise_seed(n["dist"], SEED)
    rgl.points_compact_by_field(n["compact"])
    rgl.points_yield(n["out"], OUT_FIELDS)
    rgl.chain(n["rays"], n["pose"], n["range"], n["trace"], n["ang"], n["dist"], n["compact"], n["out"])
    return n


def build_pipeline(rgl, scene, rays):
    from robotecgpulidar_gb300 import scenes

    rgl.spawn_scene(scene)
    return build_sensor_graph(rgl, rays, scenes.translation(*SENSOR))


OUT_FIELDS = [1, 8, 7]  # XYZ_VEC3_F32, DISTANCE_F32, ENTITY_ID_I32 read back by the e2e loop


def cpu_baseline(scene, rays, seconds: float):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    from robotecgpulidar_gb300 import rgl, scenes

    t0 = time.perf_counter()
    osc = pyoracle.OracleScene(scene)
    build_s = time.perf_counter() - t0
    threads = os.cpu_count() or 1
    pose = scenes.translation(*SENSOR)
    n_rays = 0
    t0 = time.perf_counter()
    frames = 0
    while True:
        osc.raytrace(rays, ray_transform=pose, ranges=[RANGE], return_mode=rgl.RGL_RETURN_FIRST_LAST, h_div=DIVERGENCE_RAD,
                     v_div=DIVERGENCE_RAD, layers=LAYERS, vertices=VERTICES, threads=threads)
        n_rays += rays.shape[0] * SUBRAYS
        frames += 1
        if time.perf_counter() - t0 >= seconds:
            break
    dt = time.perf_counter() - t0
    return {"value": n_rays / dt / 1e6, "unit": "Mrays/s", "cores": threads, "kind": "port",
            "sample": f"{frames} full scans of the same workload (FP64 oracle caster, {threads} threads, "
                      f"{seconds:.0f} s budget); BVH build {build_s:.2f} s not included"}


def run_reference(args):
    rank, world, _ = rank_info()
    if rank != 0:
        return 0
    from robotecgpulidar_gb300 import scenes

    scene = scenes.million_scene()
    rays = scenes.lidar_rays(CHANNELS, AZIMUTHS)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    from robotecgpulidar_gb300 import rgl

    osc = pyoracle.OracleScene(scene)
    threads = os.cpu_count() or 1
    pose = scenes.translation(*SENSOR)
    # Each step casts a bounded sample (1/8 of the scan's beams) so the run ends within minutes.
    sample = rays[: rays.shape[0] // 8]

    def step():
        osc.raytrace(sample, ray_transform=pose, ranges=[RANGE], return_mode=rgl.RGL_RETURN_FIRST_LAST, h_div=DIVERGENCE_RAD,
                     v_div=DIVERGENCE_RAD, layers=LAYERS, vertices=VERTICES, threads=threads)

    for _ in range(args.warmup):
        step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step()
    dt = time.perf_counter() - t0
    value = args.steps * sample.shape[0] * SUBRAYS / dt / 1e6
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "Mrays/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": workload_config(),
            "cpu_baseline": {"value": value, "unit": "Mrays/s", "cores": threads, "kind": "port",
                             "sample": f"{sample.shape[0]} of {rays.shape[0]} beams x {SUBRAYS} sub-rays per step; FP64 CPU "
                                       "restatement of RGL's ray casting (the OptiX reference cannot be built: no OptiX SDK, "
                                       "no RT cores on GB300)"},
            "e2e": {"value": value, "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def run_ours(args):
    rank, world, local = rank_info()
    import torch

    dist = None
    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    from robotecgpulidar_gb300 import build as b

    b.build()
    from robotecgpulidar_gb300 import rgl, scenes
    import ctypes as C

    lib = rgl.lib()
    rgl.check(lib.rgl_configure_logging(rgl.RGL_LOG_LEVEL_OFF, None, False))
    rgl.check(lib.rgl_gb300_configure_blas_builder(BLAS_BUILDERS[args.blas_builder]))
    scene = scenes.million_scene()
    rays = scenes.lidar_rays(CHANNELS, AZIMUTHS)
    n_beams = rays.shape[0]
    rays_per_step = n_beams * SUBRAYS
    nodes = build_pipeline(rgl, scene, rays)
    rgl.check(lib.rgl_gb300_configure_timing(True))
    builds0 = blas_build_stats(rgl)

    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")

    def flush_l2():
        flush.zero_()
        torch.cuda.synchronize()

    run_ms, trace_ms = C.c_float(), C.c_float()
    # Clocks are sampled from before the warm-up to after the end-to-end loop: the timed region alone
    # is shorter than the sampling interval, so the window holds the same load around it (warm-up
    # extended to at least 0.5 s of back-to-back scans).
    clocks = Clocks(local)
    clocks.start()
    t_soak = time.perf_counter()
    k = 0
    while k < max(3, args.warmup) or time.perf_counter() - t_soak < 0.5:
        rgl.graph_run(nodes["rays"])
        rgl.check(lib.rgl_gb300_graph_sync(nodes["rays"]))
        k += 1
    builds1 = blas_build_stats(rgl)

    # ---- device-resident timed region
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    launches0 = rgl.kernel_launch_count()
    runs, traces = [], []
    t_wall = time.perf_counter()
    for _ in range(args.steps):
        flush_l2()
        rgl.graph_run(nodes["rays"])
        rgl.check(lib.rgl_gb300_graph_get_timing(nodes["rays"], C.byref(run_ms), C.byref(trace_ms)))
        runs.append(run_ms.value)
        traces.append(trace_ms.value)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t_wall
    launches = rgl.kernel_launch_count() - launches0
    total_ms = sum(runs)
    if dist:
        t = torch.tensor([total_ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    value = world * rays_per_step * args.steps / (total_ms / 1e3) / 1e6

    # ---- end-to-end through the C API from pinned host memory
    pinned_rays = torch.empty((n_beams, 12), dtype=torch.float32, pin_memory=True).numpy()
    pinned_rays[:] = rays.reshape(n_beams, 12)
    cap = n_beams * 2
    out_xyz = torch.empty((cap, 3), dtype=torch.float32, pin_memory=True).numpy()
    out_dist = torch.empty(cap, dtype=torch.float32, pin_memory=True).numpy()
    out_ent = torch.empty(cap, dtype=torch.int32, pin_memory=True).numpy()
    cnt, sz = C.c_int32(), C.c_int32()
    lat, d2h = [], []
    if dist:
        dist.barrier()
    for _ in range(args.steps):
        flush_l2()
        t0 = time.perf_counter()
        rgl.check(lib.rgl_node_rays_from_mat3x4f(C.byref(nodes["rays"]), rgl.ptr(pinned_rays), n_beams))
        rgl.check(lib.rgl_graph_run(nodes["rays"]))
        rgl.check(lib.rgl_graph_get_result_size(nodes["out"], rgl.RGL_FIELD_XYZ_VEC3_F32, C.byref(cnt), C.byref(sz)))
        for f, arr in ((rgl.RGL_FIELD_XYZ_VEC3_F32, out_xyz), (rgl.RGL_FIELD_DISTANCE_F32, out_dist),
                       (rgl.RGL_FIELD_ENTITY_ID_I32, out_ent)):
            rgl.check(lib.rgl_graph_get_result_data(nodes["out"], f, rgl.ptr(arr)))
        lat.append(time.perf_counter() - t0)
        d2h.append(cnt.value * (12 + 4 + 4))
    e2e_s = sum(lat)
    clk = clocks.stop()
    if clk is not None:
        clk["window"] = "warm-up (>= 0.5 s), timed and end-to-end loops of the same scan"
    if dist:
        t = torch.tensor([e2e_s], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())
    e2e_value = world * rays_per_step * args.steps / e2e_s / 1e6

    # ---- roofline of the traversal kernel (algorithmic bytes per launch)
    nb, tb, ni = C.c_int64(), C.c_int64(), C.c_int32()
    rgl.check(lib.rgl_gb300_scene_get_stats(C.byref(nb), C.byref(tb), C.byref(ni)))
    V = sum(m.vertices.shape[0] for m in scene.meshes)
    T = sum(m.indices.shape[0] for m in scene.meshes)
    per_beam = 48 + 2 * (12 + 4 + 4 + 4)  # ray pose read + 2 returns x (xyz, distance, entity id, is-hit)
    algo_bytes = n_beams * per_beam + 12 * V + 12 * T + nb.value
    trace_mean_ms = statistics.mean(traces)
    achieved = algo_bytes / (trace_mean_ms / 1e3) / 1e9
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    peak, peak_src = 6785.9, "fallback"
    if os.path.exists(peaks_path):
        peak, peak_src = float(json.load(open(peaks_path))["hbm_gbs"]), "measured"
    traffic, warp_insts = None, None
    tpath = os.path.join(ROOT, "profiles", "trace_kernel_traffic.json")
    if os.path.exists(tpath):
        prof = json.load(open(tpath))
        traffic = prof.get("dram_bytes_per_launch")
        warp_insts = prof.get("warp_instructions_per_launch")
    # The traversal is bound by instruction issue, not by bytes: its warp instructions per launch (ncu)
    # over the event-timed launch, against one warp instruction per clock on each of the SMs' 4
    # schedulers at the clock sampled during the run.
    issue = None
    if warp_insts:
        sms = torch.cuda.get_device_properties(local).multi_processor_count
        mhz = (clk or {}).get("sm_mhz") or (clk or {}).get("sm_max_mhz") or 2070.0
        issue_peak = sms * 4 * mhz * 1e6
        issue_achieved = warp_insts / (trace_mean_ms / 1e3)
        issue = {"achieved": issue_achieved, "peak": issue_peak, "unit": "warp instructions/s", "frac": issue_achieved / issue_peak,
                 "warp_instructions_per_launch": int(warp_insts), "sm_mhz": mhz}

    line = None
    if rank == 0:
        rays_cpu = None
        cpu = cpu_baseline(scene, rays, args.cpu_seconds) if world == 1 else None
        lat_ms = sorted(x * 1e3 for x in lat)
        line = {
            "metric": METRIC, "value": value, "unit": "Mrays/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic", "config": workload_config(),
            "e2e": {"value": e2e_value, "unit": "Mrays/s", "h2d_bytes_per_step": int(pinned_rays.nbytes),
                    "d2h_bytes_per_step": int(statistics.mean(d2h)),
                    "p50_ms": lat_ms[len(lat_ms) // 2], "p99_ms": lat_ms[min(len(lat_ms) - 1, int(0.99 * len(lat_ms)))]},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "traffic": traffic, "kernel": "kTraceBatch", "algorithmic_bytes_per_launch": int(algo_bytes),
                         "kernel_ms": trace_mean_ms, "peak_source": peak_src, "issue": issue},
            "cpu_baseline": cpu,
            "clocks": clk,
            "gpu_launches": int(launches),
            "scene_build": {"blas_builder": args.blas_builder, "meshes": builds1[0] - builds0[0],
                            "triangles": int(T), "blas_ms": builds1[1] - builds0[1]},
            "beams_per_s": world * n_beams * args.steps / (total_ms / 1e3),
            "wall_s_timed_region": wall,
        }
        print(json.dumps(line), flush=True)
    rgl.cleanup()
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    return 0


MULTI_SENSORS = 64
REPOSE_FRACTION = 0.2


def run_multi_sensor(args):
    """64 uneven sensors on the 1M-triangle scene, 20 % of the entities re-posed every frame. Times
    the batched frame (rgl_gb300_batch_run: one CUDA graph with the refit, every sensor's nodes and one
    persistent traversal launch per wave of sensors) against the plain loop of one rgl_graph_run per
    sensor graph, both over the same graphs and poses. Besides the device-only frame, both are timed
    end to end: run, then read every graph's XYZ, distance and entity id into pinned host buffers."""
    from robotecgpulidar_gb300 import build as b

    b.build()
    import ctypes as C

    import torch
    from robotecgpulidar_gb300 import rgl, scenes

    lib = rgl.lib()
    rgl.check(lib.rgl_configure_logging(rgl.RGL_LOG_LEVEL_OFF, None, False))
    scene = scenes.million_scene()
    _, ents = rgl.spawn_scene(scene)
    rig = scenes.sensor_rig(scene, MULTI_SENSORS, seed=4)
    graphs = [build_sensor_graph(rgl, s.rays(), s.pose) for s in rig]
    beams = sum(s.beam_count for s in rig)
    rays_per_frame = beams * SUBRAYS
    rng = np.random.default_rng(6)

    def repose():
        for i, tf in scenes.repose(scene, REPOSE_FRACTION, rng):
            rgl.entity_set_transform(ents[i], tf)

    def sync_all():
        for g in graphs:
            rgl.check(lib.rgl_gb300_graph_sync(g["rays"]))

    cnt, sz = C.c_int32(), C.c_int32()
    cap = max(s.beam_count for s in rig) * 2
    out_xyz = torch.empty((cap, 3), dtype=torch.float32, pin_memory=True).numpy()
    out_dist = torch.empty(cap, dtype=torch.float32, pin_memory=True).numpy()
    out_ent = torch.empty(cap, dtype=torch.int32, pin_memory=True).numpy()

    def read_results():
        total = 0
        for g in graphs:
            rgl.check(lib.rgl_graph_get_result_size(g["out"], rgl.RGL_FIELD_XYZ_VEC3_F32, C.byref(cnt), C.byref(sz)))
            for f, arr in ((rgl.RGL_FIELD_XYZ_VEC3_F32, out_xyz), (rgl.RGL_FIELD_DISTANCE_F32, out_dist),
                           (rgl.RGL_FIELD_ENTITY_ID_I32, out_ent)):
                rgl.check(lib.rgl_graph_get_result_data(g["out"], f, rgl.ptr(arr)))
            total += cnt.value * 20
        return total

    clocks = Clocks(0)
    clocks.start()
    # ---- batched frames
    batch = rgl.batch_create([g["rays"] for g in graphs])
    rgl.batch_configure_waves(batch, args.waves)
    t0 = time.perf_counter()
    repose()
    rgl.batch_run(batch)
    st = rgl.batch_stats(batch)
    first_frame_s = time.perf_counter() - t0
    for _ in range(max(3, args.warmup)):
        repose()
        rgl.batch_run(batch)
    rgl.batch_stats(batch)
    launches0 = rgl.kernel_launch_count()
    dev_ms, trace_ms, wall_b, call_b = [], [], [], []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        repose()
        t1 = time.perf_counter()
        rgl.batch_run(batch)
        call_b.append(time.perf_counter() - t1)
        st = rgl.batch_stats(batch)  # waits for the frame
        wall_b.append(time.perf_counter() - t0)
        dev_ms.append(st["frame_ms"])
        trace_ms.append(st["trace_ms"])
    launches = rgl.kernel_launch_count() - launches0
    e2e_b, d2h = [], []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        repose()
        rgl.batch_run(batch)
        d2h.append(read_results())
        e2e_b.append(time.perf_counter() - t0)
    sched = rgl.batch_schedule(batch)
    waves = rgl.batch_waves(batch)
    tuning = [dict(s, ms=round(ms, 4)) for s, ms in rgl.batch_tuning(batch)]
    st = rgl.batch_stats(batch)
    rgl.batch_destroy(batch)

    # ---- plain loop: one rgl_graph_run per sensor graph (each graph replays its own CUDA graph)
    for _ in range(max(3, args.warmup)):
        repose()
        for g in graphs:
            rgl.graph_run(g["rays"])
        sync_all()
    wall_p, e2e_p, call_p = [], [], []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        repose()
        t1 = time.perf_counter()
        for g in graphs:
            rgl.graph_run(g["rays"])
        call_p.append(time.perf_counter() - t1)
        sync_all()
        wall_p.append(time.perf_counter() - t0)
    for _ in range(args.steps):
        t0 = time.perf_counter()
        repose()
        for g in graphs:
            rgl.graph_run(g["rays"])
        read_results()
        e2e_p.append(time.perf_counter() - t0)
    clk = clocks.stop()
    if clk is not None:
        clk["window"] = "batched and plain frame loops"

    nb, tb, ni = C.c_int64(), C.c_int64(), C.c_int32()
    rgl.check(lib.rgl_gb300_scene_get_stats(C.byref(nb), C.byref(tb), C.byref(ni)))
    V = sum(m.vertices.shape[0] for m in scene.meshes)
    T = sum(m.indices.shape[0] for m in scene.meshes)
    algo_bytes = beams * (48 + 2 * (12 + 4 + 4 + 4)) + 12 * V + 12 * T + nb.value
    trace_mean = statistics.mean(trace_ms)
    achieved = algo_bytes / (trace_mean / 1e3) / 1e9
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    peak = float(json.load(open(peaks_path))["hbm_gbs"]) if os.path.exists(peaks_path) else 6785.9

    def mrays(sec_list):
        return rays_per_frame * len(sec_list) / sum(sec_list) / 1e6

    def pct(xs, q):
        xs = sorted(x * 1e3 for x in xs)
        return xs[min(len(xs) - 1, int(q * len(xs)))]

    line = {
        "metric": "Mrays/s, 64 uneven sensors per frame on the 1M-tri scene (batched vs plain loop), 1 GB300",
        "value": rays_per_frame * args.steps / (sum(dev_ms) / 1e3) / 1e6, "unit": "Mrays/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": statistics.mean(dev_ms), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "64 uneven sensors (16x1800, 32x1024, 64x2048, 128x2048, 120x640 grid; seed 4) on the 1M-tri "
                               "scene, FIRST_LAST, 5 sub-rays/beam in 0.2 deg, angular+distance noise, compaction by is-hit; "
                               "20% of entities re-posed every frame (TLAS refit inside the frame's CUDA graph)",
                   "triangles": 1000448, "sensors": MULTI_SENSORS, "beams_per_frame": beams, "rays_per_frame": rays_per_frame,
                   "l2": "inputs larger than L2 (%d MB of ray poses per frame)" % (beams * 48 >> 20)},
        "batched": {"device_mrays_s": rays_per_frame * args.steps / (sum(dev_ms) / 1e3) / 1e6, "wall_mrays_s": mrays(wall_b),
                    "frame_ms_p50": pct(wall_b, 0.5), "frame_ms_p99": pct(wall_b, 0.99), "device_frame_ms": statistics.mean(dev_ms),
                    "trace_ms": trace_mean, "e2e_mrays_s": mrays(e2e_b), "e2e_frame_ms_p50": pct(e2e_b, 0.5),
                    "e2e_frame_ms_p99": pct(e2e_b, 0.99), "schedule": sched, "tuning": tuning, "first_frame_s_incl_tuning": first_frame_s,
                    "host_run_call_ms_p50": pct(call_b, 0.5), "waves": waves, "captures": st["captures"], "replays": st["replays"], "tunings": st["tunings"]},
        "plain_loop": {"wall_mrays_s": mrays(wall_p), "frame_ms_p50": pct(wall_p, 0.5), "frame_ms_p99": pct(wall_p, 0.99),
                       "host_run_calls_ms_p50": pct(call_p, 0.5),
                       "e2e_mrays_s": mrays(e2e_p), "e2e_frame_ms_p50": pct(e2e_p, 0.5), "e2e_frame_ms_p99": pct(e2e_p, 0.99)},
        "speedup_wall": mrays(wall_b) / mrays(wall_p),
        "speedup_e2e": mrays(e2e_b) / mrays(e2e_p),
        "e2e": {"value": mrays(e2e_b), "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": int(statistics.mean(d2h))},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak, "traffic": None,
                     "kernel": "kTraceBatch", "algorithmic_bytes_per_frame": int(algo_bytes), "launches_per_frame": waves,
                     "kernel_ms": trace_mean},
        "clocks": clk,
        "gpu_launches": int(launches),
    }
    print(json.dumps(line), flush=True)
    rgl.cleanup()
    return 0


def run_small_config(args, which):
    """Config 0 (plain 20,768-tri scene, 32x1024 first return, yield XYZ/distance/entity id/is-hit,
    compaction) or config 1 (the same scene at 64x2048 with angular + distance noise, a transform into
    a random world frame, compaction and format [XYZ, distance, entity id]): device time of whole graph
    runs, end to end through the C API, and the FP64 oracle on the host cores."""
    from robotecgpulidar_gb300 import build as b

    b.build()
    import ctypes as C

    import torch
    from robotecgpulidar_gb300 import rgl, scenes

    lib = rgl.lib()
    rgl.check(lib.rgl_configure_logging(rgl.RGL_LOG_LEVEL_OFF, None, False))
    scene = scenes.plain_scene()
    rgl.spawn_scene(scene)
    ch, az = (32, 1024) if which == 0 else (64, 2048)
    rays = scenes.lidar_rays(ch, az)
    pose = scenes.translation(0, 0, 1.8)
    n = {k: rgl.node() for k in ("rays", "pose", "range", "trace", "ang", "dist", "tf", "cmp", "out")}
    rgl.rays_from_mat3x4f(n["rays"], rays)
    rgl.rays_transform(n["pose"], pose)
    rgl.rays_set_range(n["range"], [RANGE])
    rgl.raytrace(n["trace"])
    chain = [n["rays"], n["pose"], n["range"], n["trace"]]
    if which == 0:
        fields = [rgl.RGL_FIELD_XYZ_VEC3_F32, rgl.RGL_FIELD_DISTANCE_F32, rgl.RGL_FIELD_ENTITY_ID_I32, rgl.RGL_FIELD_IS_HIT_I32]
        rgl.points_compact_by_field(n["cmp"])
        rgl.points_yield(n["out"], fields)
        chain += [n["cmp"], n["out"]]
        read = [(f, 0) for f in fields]
    else:
        rgl.check(lib.rgl_node_gaussian_noise_angular_hitpoint(C.byref(n["ang"]), 0.0, ANGULAR_SIGMA, rgl.RGL_AXIS_Z))
        rgl.check(lib.rgl_node_gaussian_noise_distance(C.byref(n["dist"]), 0.0, 0.02, 0.001))
        rgl.set_noise_seed(n["ang"], SEED)
        rgl.set_noise_seed(n["dist"], SEED)
        rng = np.random.default_rng(1)
        rgl.points_transform(n["tf"], scenes.trs(rng.uniform(-50, 50, 3), rng.uniform(-np.pi, np.pi, 3)))
        rgl.points_compact_by_field(n["cmp"])
        rgl.points_format(n["out"], [rgl.RGL_FIELD_XYZ_VEC3_F32, rgl.RGL_FIELD_DISTANCE_F32, rgl.RGL_FIELD_ENTITY_ID_I32])
        chain += [n["ang"], n["dist"], n["tf"], n["cmp"], n["out"]]
        read = [(rgl.RGL_FIELD_DYNAMIC_FORMAT, 20)]
    rgl.chain(*chain)
    rgl.check(lib.rgl_gb300_configure_timing(True))
    run_ms, trace_ms = C.c_float(), C.c_float()
    for _ in range(max(3, args.warmup)):
        rgl.graph_run(n["rays"])
        rgl.check(lib.rgl_gb300_graph_sync(n["rays"]))
    runs, traces = [], []
    for _ in range(args.steps):
        rgl.graph_run(n["rays"])
        rgl.check(lib.rgl_gb300_graph_get_timing(n["rays"], C.byref(run_ms), C.byref(trace_ms)))
        runs.append(run_ms.value)
        traces.append(trace_ms.value)
    beams = rays.shape[0]
    pinned = torch.empty((beams, 12), dtype=torch.float32, pin_memory=True).numpy()
    pinned[:] = rays.reshape(beams, 12)
    out = torch.empty(beams * 32, dtype=torch.uint8, pin_memory=True).numpy()
    cnt, sz = C.c_int32(), C.c_int32()
    lat = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        rgl.check(lib.rgl_node_rays_from_mat3x4f(C.byref(n["rays"]), rgl.ptr(pinned), beams))
        rgl.check(lib.rgl_graph_run(n["rays"]))
        for f, _ in read:
            rgl.check(lib.rgl_graph_get_result_size(n["out"], f, C.byref(cnt), C.byref(sz)))
            rgl.check(lib.rgl_graph_get_result_data(n["out"], f, rgl.ptr(out)))
        lat.append(time.perf_counter() - t0)
    # CPU baseline: the FP64 oracle caster on all host cores, on the same scan.
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle

    osc = pyoracle.OracleScene(scene)
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    scans = 0
    while True:
        osc.raytrace(rays, ray_transform=pose, ranges=[RANGE], return_mode=rgl.RGL_RETURN_FIRST, threads=threads)
        scans += 1
        if time.perf_counter() - t0 >= args.cpu_seconds:
            break
    cpu = beams * scans / (time.perf_counter() - t0) / 1e6
    lat_ms = sorted(x * 1e3 for x in lat)
    line = {"metric": f"Mrays/s, config {which} (plain 20,768-tri scene, {ch}x{az} first return)", "unit": "Mrays/s",
            "value": beams * args.steps / (sum(runs) / 1e3) / 1e6, "ms_per_step": statistics.mean(runs), "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "dtype": "f32", "data": "synthetic",
            "trace_kernel_ms": statistics.mean(traces),
            "e2e": {"value": beams * args.steps / sum(lat) / 1e6, "unit": "Mrays/s", "p50_ms": lat_ms[len(lat_ms) // 2],
                    "p99_ms": lat_ms[min(len(lat_ms) - 1, int(0.99 * len(lat_ms)))]},
            "cpu_baseline": {"value": cpu, "unit": "Mrays/s", "cores": threads, "kind": "port",
                             "sample": f"{scans} full scans (raytrace stage only, FP64 oracle caster)"}}
    print(json.dumps(line), flush=True)
    rgl.cleanup()
    return 0


SERVE_SCENES = (200_000, 1_000_000, 2_000_000, 4_000_000)
SERVE_ROBOTS = 256
SERVE_BUDGET = 80 << 30


def run_serving(args):
    """Scan requests from 256 virtual robots arriving by a Poisson process over 4 resident scenes
    (0.2M/1M/2M/4M triangles), ray count log-uniform in [10k, 1M], FIRST or FIRST_LAST 50/50, range
    [0.1, 100] m, compaction by is-hit; results (XYZ, distance, entity id) read back into pinned host
    memory. Served: rgl_gb300_server_* (continuous batching under an 80 GB budget; results land in the
    server's pinned host memory). Plain: one rgl_graph_run per request on the robot's own graph, in
    arrival order, results copied with rgl_graph_get_result_data into pinned host buffers. Latency =
    arrival to results in host memory."""
    from robotecgpulidar_gb300 import build as b

    b.build()
    import ctypes as C

    import torch
    from robotecgpulidar_gb300 import rgl, scenes

    lib = rgl.lib()
    rgl.check(lib.rgl_configure_logging(rgl.RGL_LOG_LEVEL_OFF, None, False))
    scene_objs = [scenes.serving_scene(t, 10 + k) for k, t in enumerate(SERVE_SCENES)]
    handles = []
    for sc in scene_objs:
        h = rgl.scene_create()
        rgl.spawn_scene_in(h, sc)
        handles.append(h)
    fleet = scenes.robot_fleet(scene_objs, SERVE_ROBOTS, seed=5)
    rays_of = [scenes.lidar_rays(*r.pattern) for r in fleet]
    max_pts = max(r.rays for r in fleet) * 2
    out_xyz = torch.empty((max_pts, 3), dtype=torch.float32, pin_memory=True).numpy()
    out_dist = torch.empty(max_pts, dtype=torch.float32, pin_memory=True).numpy()
    out_ent = torch.empty(max_pts, dtype=torch.int32, pin_memory=True).numpy()
    outs = ((rgl.RGL_FIELD_XYZ_VEC3_F32, out_xyz), (rgl.RGL_FIELD_DISTANCE_F32, out_dist), (rgl.RGL_FIELD_ENTITY_ID_I32, out_ent))
    modes = (rgl.RGL_RETURN_FIRST, rgl.RGL_RETURN_FIRST_LAST)
    cnt, sz = C.c_int32(), C.c_int32()

    def make_trace(rate, seed):
        rng = np.random.default_rng(seed)
        t, arr = 0.0, []
        while True:
            t += rng.exponential(1.0 / rate)
            if t >= args.trace_seconds:
                break
            arr.append(t)
        n = len(arr)
        robots = rng.integers(0, SERVE_ROBOTS, size=n)
        mode = rng.integers(0, 2, size=n)
        poses = []
        for k in range(n):
            base = fleet[robots[k]].pose
            d = rng.uniform(-1.0, 1.0, size=2)
            poses.append(np.ascontiguousarray((scenes.translation(d[0], d[1], 0.0).astype(np.float64) @ np.vstack([base, [0, 0, 0, 1]]))[:3]
                                              .astype(np.float32)))
        return np.array(arr), robots, mode, poses

    def summarize(lat, rays_done, t_first, t_last, n_req, saturated):
        lat_ms = sorted(x * 1e3 for x in lat)
        span = max(t_last - t_first, 1e-9)
        return {"requests": n_req, "completed": len(lat), "mrays_s": rays_done / span / 1e6,
                "p50_ms": lat_ms[len(lat_ms) // 2] if lat_ms else None,
                "p99_ms": lat_ms[min(len(lat_ms) - 1, int(0.99 * len(lat_ms)))] if lat_ms else None,
                "max_ms": lat_ms[-1] if lat_ms else None, "over_20ms": sum(1 for x in lat_ms if x > 20.0), "saturated": saturated}

    failures = []
    host_ptr = C.c_void_p()

    def read_served(q):
        """Takes a served request's three result fields, already in the server's pinned host memory
        (the address and count of each); a failed request is recorded."""
        for f, _ in outs:
            if lib.rgl_gb300_server_get_result_host(srv.h, q, f, C.byref(host_ptr), C.byref(cnt)) != rgl.RGL_SUCCESS:
                failures.append(rgl.last_error())
                return

    # ---- served
    srv = rgl.Server(SERVE_BUDGET, 2)
    if args.max_batch_beams:
        srv.configure_schedule(max_batch_beams=args.max_batch_beams)
    pats = [srv.add_pattern(r) for r in rays_of]
    warm = [srv.submit(handles[fleet[k].scene], pats[k], fleet[k].pose, modes[k % 2], *RANGE) for k in range(SERVE_ROBOTS)]
    srv.drain()
    for q in warm:
        srv.release(q)
    served = {}
    # The client loops run without Python's cyclic garbage collector (collected once before), so its
    # pauses do not land in the measured latencies of either arm.
    gc.collect()
    gc.disable()
    for rate in args.rates:
        arr, robots, mode, poses = make_trace(rate, int(rate))
        st0 = srv.stats()
        srv.batch_times(reset=True)
        lat, rays_done, t_last, i, saturated = [], 0, 0.0, 0, False
        outstanding = {}
        t0 = time.perf_counter()
        while i < len(arr) or outstanding:
            now = time.perf_counter() - t0
            while i < len(arr) and arr[i] <= now:
                k = int(robots[i])
                q = srv.submit(handles[fleet[k].scene], pats[k], poses[i], modes[int(mode[i])], *RANGE)
                outstanding[q] = (arr[i], fleet[k].rays)
                i += 1
            if i < len(arr) and now - arr[i] > args.max_lag:
                saturated = True
                break
            # Wait for completions until the next arrival is due.
            wait_ms = 0.0 if i >= len(arr) and not outstanding else max(0.0, ((arr[i] if i < len(arr) else now + 1e-3) - now) * 1e3)
            done = srv.wait_completed(min(wait_ms, 1.0)) if outstanding else []
            for q in done:
                read_served(q)
                t_done = time.perf_counter() - t0
                a, nr = outstanding.pop(q)
                lat.append(t_done - a)
                rays_done += nr
                t_last = t_done
                srv.release(q)
        if saturated:
            srv.drain()
            for q in srv.take_completed():
                srv.release(q)
        st1 = srv.stats()
        res = summarize(lat, rays_done, 0.0, t_last, len(arr), saturated)
        res["device_busy_frac"] = (st1["device_us"] - st0["device_us"]) / 1e6 / max(t_last, 1e-9)
        res["batches"] = st1["batches"] - st0["batches"]
        res["mean_requests_per_batch"] = (st1["requests_in_batches"] - st0["requests_in_batches"]) / max(1, res["batches"])
        res["offered_mrays_s"] = sum(fleet[int(k)].rays for k in robots) / args.trace_seconds / 1e6
        res["batch_phases"] = srv.batch_times(reset=True)
        served[str(int(rate))] = res
    # Capacity: the same request mix submitted at once, results read as requests complete (three
    # times, to show the spread; the best run is reported).
    rng = np.random.default_rng(99)
    cap_robots = rng.integers(0, SERVE_ROBOTS, size=args.capacity_requests)
    cap_modes = rng.integers(0, 2, size=args.capacity_requests)
    cap_rays = int(sum(fleet[int(k)].rays for k in cap_robots))
    cap_runs = []
    for _ in range(3):
        clk = Clocks(0)
        clk.start()
        st0 = srv.stats()
        t0 = time.perf_counter()
        reqs = [srv.submit(handles[fleet[int(k)].scene], pats[int(k)], fleet[int(k)].pose, modes[int(m)], *RANGE)
                for k, m in zip(cap_robots, cap_modes)]
        left = set(reqs)
        while left:
            done = srv.wait_completed(1.0)
            for q in done:
                read_served(q)
                srv.release(q)
                left.discard(q)
        wall = time.perf_counter() - t0
        st1 = srv.stats()
        cap_runs.append({"mrays_s": cap_rays / wall / 1e6, "wall_s": wall, "device_s": (st1["device_us"] - st0["device_us"]) / 1e6,
                         "clocks": clk.stop(),
                         "batches": st1["batches"] - st0["batches"],
                         "requests_per_batch": (st1["requests_in_batches"] - st0["requests_in_batches"]) / max(1, st1["batches"] - st0["batches"])})
    best_cap = max(cap_runs, key=lambda c: c["mrays_s"])
    cap_wall = best_cap["wall_s"]
    served_capacity = best_cap["mrays_s"]
    served_device_s = best_cap["device_s"]
    gc.enable()
    peak_reserved = srv.stats()["peak_reserved_bytes"]
    srv.destroy()

    # ---- plain per-request loop: each robot has one graph per return mode
    graphs = {}
    for k, r in enumerate(fleet):
        for m in range(2):
            n = {x: rgl.node() for x in ("rays", "pose", "range", "trace", "cmp", "out")}
            rgl.rays_from_mat3x4f(n["rays"], rays_of[k])
            rgl.rays_transform(n["pose"], r.pose)
            rgl.rays_set_range(n["range"], [RANGE])
            rgl.raytrace_in(n["trace"], handles[r.scene])
            rgl.check(lib.rgl_node_raytrace_configure_return_mode(n["trace"], modes[m]))
            rgl.points_compact_by_field(n["cmp"])
            rgl.points_yield(n["out"], [f for f, _ in outs])
            rgl.chain(n["rays"], n["pose"], n["range"], n["trace"], n["cmp"], n["out"])
            rgl.graph_run(n["rays"])
            graphs[(k, m)] = n
    for n in graphs.values():
        rgl.check(lib.rgl_gb300_graph_sync(n["rays"]))
    plain = {}
    gc.collect()
    gc.disable()
    for rate in args.rates:
        arr, robots, mode, poses = make_trace(rate, int(rate))
        lat, rays_done, t_last, saturated = [], 0, 0.0, False
        t0 = time.perf_counter()
        for i in range(len(arr)):
            now = time.perf_counter() - t0
            if now - arr[i] > args.max_lag:
                saturated = True
                break
            while now < arr[i]:
                now = time.perf_counter() - t0
            k = int(robots[i])
            n = graphs[(k, int(mode[i]))]
            rgl.rays_transform(n["pose"], poses[i])
            rgl.check(lib.rgl_graph_run(n["rays"]))
            for f, buf in outs:
                rgl.check(lib.rgl_graph_get_result_size(n["out"], f, C.byref(cnt), C.byref(sz)))
                if cnt.value:
                    rgl.check(lib.rgl_graph_get_result_data(n["out"], f, rgl.ptr(buf)))
            t_last = time.perf_counter() - t0
            lat.append(t_last - arr[i])
            rays_done += fleet[k].rays
        plain[str(int(rate))] = summarize(lat, rays_done, 0.0, t_last, len(arr), saturated)

    t0 = time.perf_counter()
    for k, m in zip(cap_robots, cap_modes):
        n = graphs[(int(k), int(m))]
        rgl.rays_transform(n["pose"], fleet[int(k)].pose)
        rgl.check(lib.rgl_graph_run(n["rays"]))
        for f, buf in outs:
            rgl.check(lib.rgl_graph_get_result_size(n["out"], f, C.byref(cnt), C.byref(sz)))
            if cnt.value:
                rgl.check(lib.rgl_graph_get_result_data(n["out"], f, rgl.ptr(buf)))
    plain_capacity = cap_rays / (time.perf_counter() - t0) / 1e6
    gc.enable()

    top = str(int(max(args.rates)))
    line = {
        "metric": "Mrays/s and p50/p99 scan latency, served vs plain per-request rgl_graph_run loop, 1 GB300",
        "value": served[top]["mrays_s"], "unit": "Mrays/s", "n_gpus": 1, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "serving: 256 robots, Poisson arrivals, 4 resident scenes (0.2M/1M/2M/4M tris), rays/request "
                               "log-uniform [10k, 1M], FIRST or FIRST_LAST 50/50, compaction by is-hit, results read to pinned "
                               "host memory, 80 GB admission budget",
                   "trace_seconds": args.trace_seconds, "rates_per_s": args.rates, "max_lag_s": args.max_lag,
                   "scene_triangles": [s.triangle_count for s in scene_objs]},
        "served": served, "plain_loop": plain,
        "speedup_at_top_rate": served[top]["mrays_s"] / max(plain[top]["mrays_s"], 1e-9),
        "capacity": {"requests": args.capacity_requests, "rays": cap_rays, "served_mrays_s": served_capacity, "served_runs": cap_runs,
                     "served_device_busy_frac": served_device_s / cap_wall,
                     "served_device_mrays_s": cap_rays / max(served_device_s, 1e-9) / 1e6,
                     "plain_mrays_s": plain_capacity, "speedup": served_capacity / plain_capacity},
        "peak_reserved_bytes": peak_reserved,
        "served_failures": len(failures), "first_failure": failures[0] if failures else None,
    }
    print(json.dumps(line), flush=True)
    rgl.cleanup()
    return 0


BLAS_BUILDERS = {"device_sah": 0, "host_sah": 1, "device_lbvh": 2}


def blas_build_stats(rgl):
    import ctypes as C

    n, ms = C.c_int64(), C.c_double()
    rgl.check(rgl.lib().rgl_gb300_get_blas_build_stats(C.byref(n), C.byref(ms)))
    return n.value, ms.value


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--workload", choices=["single_sensor", "multi_sensor", "serving", "config0", "config1"], default="single_sensor",
                    help="single_sensor: the 1M-tri scan (the headline line); multi_sensor: 64 sensors, batched vs plain loop; "
                         "serving: Poisson scan requests, served vs plain loop")
    ap.add_argument("--rates", type=lambda v: [float(x) for x in v.split(",")], default=[100, 200, 500, 1000, 2000, 5000, 10000, 15000],
                    help="serving: request rates (per second) to sweep")
    ap.add_argument("--waves", type=int, default=0, help="multi_sensor: waves per batched frame (0: automatic)")
    ap.add_argument("--trace-seconds", type=float, default=30.0, help="serving: length of each arrival trace")
    ap.add_argument("--max-lag", type=float, default=5.0, help="serving: stop a trace once the loop lags arrivals by this much (s)")
    ap.add_argument("--max-batch-beams", type=int, default=0, help="serving: most beams per batch (0: the library's default)")
    ap.add_argument("--capacity-requests", type=int, default=2000, help="serving: requests of the all-at-once capacity run")
    ap.add_argument("--blas-builder", choices=list(BLAS_BUILDERS), default="device_sah",
                    help="mesh BLAS builder: binned SAH on the device (default), the same tree built on the host, or the device LBVH")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "multi_sensor":
        return run_multi_sensor(args)
    if args.workload == "serving":
        return run_serving(args)
    if args.workload in ("config0", "config1"):
        return run_small_config(args, int(args.workload[-1]))
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
