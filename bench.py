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
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (FileNotFoundError, OSError):
            self.proc = None

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


def build_pipeline(rgl, scene, rays):
    rgl.spawn_scene(scene)
    lib = rgl.lib()
    n = {k: rgl.node() for k in ("rays", "pose", "range", "trace", "ang", "dist", "compact", "out")}
    rgl.rays_from_mat3x4f(n["rays"], rays)
    from robotecgpulidar_gb300 import scenes

    rgl.rays_transform(n["pose"], scenes.translation(*SENSOR))
    rgl.rays_set_range(n["range"], [RANGE])
    rgl.raytrace(n["trace"])
    rgl.check(lib.rgl_node_raytrace_configure_return_mode(n["trace"], rgl.RGL_RETURN_FIRST_LAST))
    rgl.check(lib.rgl_node_raytrace_configure_beam_divergence(n["trace"], DIVERGENCE_RAD, DIVERGENCE_RAD))
    rgl.configure_beam_samples(n["trace"], LAYERS, VERTICES)
    import ctypes as C

    rgl.check(lib.rgl_node_gaussian_noise_angular_hitpoint(C.byref(n["ang"]), 0.0, ANGULAR_SIGMA, rgl.RGL_AXIS_Z))
    rgl.check(lib.rgl_node_gaussian_noise_distance(C.byref(n["dist"]), 0.0, 0.02, 0.001))
    rgl.set_noise_seed(n["ang"], SEED)
    rgl.set_noise_seed(n["dist"], SEED)
    rgl.points_compact_by_field(n["compact"])
    rgl.points_yield(n["out"], OUT_FIELDS)
    rgl.chain(n["rays"], n["pose"], n["range"], n["trace"], n["ang"], n["dist"], n["compact"], n["out"])
    return n


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
    scene = scenes.million_scene()
    rays = scenes.lidar_rays(CHANNELS, AZIMUTHS)
    n_beams = rays.shape[0]
    rays_per_step = n_beams * SUBRAYS
    nodes = build_pipeline(rgl, scene, rays)
    rgl.check(lib.rgl_gb300_configure_timing(True))

    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")

    def flush_l2():
        flush.zero_()
        torch.cuda.synchronize()

    run_ms, trace_ms = C.c_float(), C.c_float()
    for _ in range(max(3, args.warmup)):
        rgl.graph_run(nodes["rays"])
        rgl.check(lib.rgl_gb300_graph_sync(nodes["rays"]))

    # ---- device-resident timed region
    clocks = Clocks(local)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    launches0 = rgl.kernel_launch_count()
    clocks.start()
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
    clk = clocks.stop()
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
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "trace_kernel_traffic.json")
    if os.path.exists(tpath):
        traffic = json.load(open(tpath)).get("dram_bytes_per_launch")

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
                         "traffic": traffic, "kernel": "kTrace", "algorithmic_bytes_per_launch": int(algo_bytes),
                         "kernel_ms": trace_mean_ms, "peak_source": peak_src},
            "cpu_baseline": cpu,
            "clocks": clk,
            "gpu_launches": int(launches),
            "beams_per_s": world * n_beams * args.steps / (total_ms / 1e3),
            "wall_s_timed_region": wall,
        }
        print(json.dumps(line), flush=True)
    rgl.cleanup()
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
