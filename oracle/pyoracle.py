"""ctypes front-end of the CPU oracle (oracle/rgl_oracle.cpp) — TEST INFRASTRUCTURE ONLY.

Imported by the test-suite, by ``__graft_entry__.smoke()`` and by ``bench.py``'s CPU-baseline leg,
always as the checker; the product library never imports it.  ``build()`` compiles the oracle with
the committed Makefile (g++, ``-ffp-contract=off``).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "librgl_oracle.so")
_lib = None

F32P = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")


def build(force: bool = False) -> str:
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(
        os.path.join(_HERE, "rgl_oracle.cpp")
    ):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        l = C.CDLL(_LIB_PATH)
        l.orc_scene_create.restype = C.c_void_p
        l.orc_scene_destroy.argtypes = [C.c_void_p]
        l.orc_scene_add_mesh.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_int]
        l.orc_scene_add_instance.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_int]
        l.orc_scene_set_instance.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_int]
        l.orc_scene_build.argtypes = [C.c_void_p]
        l.orc_beam_samples.argtypes = [C.c_float, C.c_float, C.c_int, C.c_int, C.c_void_p]
        l.orc_raytrace.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_int32,
                                   C.c_float, C.c_float, C.c_int, C.c_int, C.c_float, C.c_float, C.c_float, C.c_int,
                                   C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        l.orc_transform_rays.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]
        l.orc_transform_points.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]
        l.orc_philox4x32_10.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        l.orc_normals.argtypes = [C.c_uint64, C.c_uint32, C.c_uint64, C.c_int, C.c_void_p]
        l.orc_noise_angular_hitpoint.argtypes = [C.c_void_p, C.c_float, C.c_float, C.c_int, C.c_uint64, C.c_uint64,
                                                 C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
        l.orc_noise_distance.argtypes = [C.c_void_p, C.c_float, C.c_float, C.c_float, C.c_uint64, C.c_uint64,
                                         C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
        l.orc_noise_angular_ray.argtypes = [C.c_void_p, C.c_float, C.c_float, C.c_int, C.c_uint64, C.c_uint64,
                                            C.c_void_p, C.c_int, C.c_void_p]
        l.orc_compact.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p]
        l.orc_compact.restype = C.c_int
        l.orc_format.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
        _lib = l
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class OracleScene:
    """World = instances of meshes, flattened to FP64 world triangles."""

    def __init__(self, scene=None):
        self._l = lib()
        self.h = self._l.orc_scene_create()
        self._keep = []
        if scene is not None:
            for m in scene.meshes:
                self.add_mesh(m.vertices, m.indices)
            for e in scene.entities:
                self.add_instance(e.mesh, e.transform, e.entity_id)
            self.build()

    def add_mesh(self, vertices, indices) -> int:
        v = np.ascontiguousarray(vertices, dtype=np.float32)
        i = np.ascontiguousarray(indices, dtype=np.int32)
        return self._l.orc_scene_add_mesh(self.h, _p(v), v.shape[0], _p(i), i.shape[0])

    def add_instance(self, mesh: int, transform, entity_id: int) -> int:
        t = np.ascontiguousarray(transform, dtype=np.float32).reshape(12)
        return self._l.orc_scene_add_instance(self.h, mesh, _p(t), int(entity_id))

    def set_instance(self, inst: int, transform, entity_id: int):
        t = np.ascontiguousarray(transform, dtype=np.float32).reshape(12)
        self._l.orc_scene_set_instance(self.h, inst, _p(t), int(entity_id))

    def build(self):
        self._l.orc_scene_build(self.h)

    def __del__(self):
        try:
            self._l.orc_scene_destroy(self.h)
        except Exception:
            pass

    def raytrace(self, rays, ray_transform=None, ranges=None, return_mode=None, h_div=0.0, v_div=0.0, layers=3,
                 vertices=19, near=float("inf"), far=float("inf"), default_intensity=0.0, threads=None):
        """RaytraceNode semantics. Returns dict of per-point arrays (returnCount * nRays points)."""
        from robotecgpulidar_gb300 import rgl  # enum values only

        if return_mode is None:
            return_mode = rgl.RGL_RETURN_FIRST
        rays = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 12)
        n = rays.shape[0]
        rc = (return_mode >> 24) & 0xFF
        npts = rc * n
        xyz = np.zeros((npts, 3), np.float32)
        dist = np.zeros(npts, np.float32)
        ent = np.zeros(npts, np.int32)
        hit = np.zeros(npts, np.int32)
        rtype = np.zeros(npts, np.uint8)
        inten = np.zeros(npts, np.float32)
        amb = np.zeros(npts, np.uint8)
        tf = None if ray_transform is None else np.ascontiguousarray(ray_transform, dtype=np.float32).reshape(12)
        rg = None if ranges is None else np.ascontiguousarray(ranges, dtype=np.float32).reshape(-1, 2)
        threads = threads or os.cpu_count() or 1
        ns = self._l.orc_raytrace(self.h, _p(rays), n, _p(tf), _p(rg), 0 if rg is None else rg.shape[0],
                                  int(np.int32(np.uint32(return_mode & 0xFFFFFFFF))), h_div, v_div, layers, vertices,
                                  near, far, default_intensity, threads, _p(xyz), _p(dist), _p(ent), _p(hit),
                                  _p(rtype), _p(inten), _p(amb))
        return {"xyz": xyz, "distance": dist, "entity_id": ent, "is_hit": hit, "return_type": rtype,
                "intensity": inten, "ambiguous": amb, "samples": ns}


def beam_samples(h_div, v_div, layers, vertices):
    out = np.zeros((1 + layers * vertices, 12), np.float32)
    n = lib().orc_beam_samples(h_div, v_div, layers, vertices, _p(out))
    return out[:n].reshape(n, 3, 4)


def philox(ctr, key):
    c = np.asarray(ctr, dtype=np.uint32)
    k = np.asarray(key, dtype=np.uint32)
    o = np.zeros(4, np.uint32)
    lib().orc_philox4x32_10(_p(c), _p(k), _p(o))
    return o


def normals(seed: int, kind: int, frame: int, n: int):
    out = np.zeros(n, np.float64)
    lib().orc_normals(seed, kind, frame, n, _p(out))
    return out


def transform_rays(tf, rays):
    rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 12)
    out = np.zeros_like(rays)
    lib().orc_transform_rays(_p(np.ascontiguousarray(tf, np.float32).reshape(12)), _p(rays), rays.shape[0], _p(out))
    return out.reshape(-1, 3, 4)


def transform_points(tf, xyz):
    xyz = np.ascontiguousarray(xyz, np.float32).reshape(-1, 3)
    out = np.zeros_like(xyz)
    lib().orc_transform_points(_p(np.ascontiguousarray(tf, np.float32).reshape(12)), _p(xyz), xyz.shape[0], _p(out))
    return out


def _frame64(look_at):
    return np.ascontiguousarray(np.asarray(look_at, dtype=np.float64).reshape(3, 4))


def noise_angular_hitpoint(look_at, mean, st_dev, axis, seed, frame, xyz, with_distance=True):
    xyz = np.ascontiguousarray(xyz, np.float32).reshape(-1, 3)
    ox = np.zeros_like(xyz)
    od = np.zeros(xyz.shape[0], np.float32) if with_distance else None
    lib().orc_noise_angular_hitpoint(_p(_frame64(look_at)), mean, st_dev, axis, seed, frame, _p(xyz), xyz.shape[0],
                                     _p(ox), _p(od))
    return ox, od


def noise_distance(look_at, mean, base, rise, seed, frame, xyz, dist):
    xyz = np.ascontiguousarray(xyz, np.float32).reshape(-1, 3)
    dist = np.ascontiguousarray(dist, np.float32)
    ox = np.zeros_like(xyz)
    od = np.zeros_like(dist)
    lib().orc_noise_distance(_p(_frame64(look_at)), mean, base, rise, seed, frame, _p(xyz), _p(dist), xyz.shape[0],
                             _p(ox), _p(od))
    return ox, od


def noise_angular_ray(look_at, mean, st_dev, axis, seed, frame, rays):
    rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 12)
    out = np.zeros_like(rays)
    lib().orc_noise_angular_ray(_p(_frame64(look_at)), mean, st_dev, axis, seed, frame, _p(rays), rays.shape[0], _p(out))
    return out.reshape(-1, 3, 4)


def compact(flags, field):
    flags = np.ascontiguousarray(flags, np.int32)
    src = np.ascontiguousarray(field)
    es = src.itemsize * (int(np.prod(src.shape[1:])) if src.ndim > 1 else 1)
    dst = np.zeros_like(src)
    k = lib().orc_compact(_p(flags), flags.shape[0], _p(src), es, _p(dst))
    return dst[:k]


def format_points(fields, sizes, n):
    """fields: list of arrays (or None for padding), sizes: bytes per field."""
    arrs = [None if f is None else np.ascontiguousarray(f) for f in fields]
    ptrs = (C.c_void_p * len(arrs))(*[None if a is None else a.ctypes.data for a in arrs])
    sz = np.asarray(sizes, np.int32)
    out = np.zeros(n * int(sz.sum()), np.uint8)
    lib().orc_format(n, len(arrs), ptrs, _p(sz), _p(out))
    return out


# ---------------------------------------------------------------- frame helpers (FP64)

def mat4(m34):
    m = np.eye(4)
    m[:3, :] = np.asarray(m34, dtype=np.float64).reshape(3, 4)
    return m


def inv34(m34):
    return np.linalg.inv(mat4(m34))[:3, :]


def mul34(a, b):
    return (mat4(a) @ mat4(b))[:3, :]


# ---------------------------------------------------------------- fields every return of a beam shares

def beam_shared_fields(rays_world, sensor_to_world, return_count=1, ring_ids=None):
    """Azimuth, elevation and ring id per return point (reference src/gpu/optixPrograms.cu:288-326,
    src/math/Mat3x4f.hpp:146-175), in FP64: the sensor-frame pose is inverse(sensor_to_world) @ ray;
    elevation = asin(m[1][2]) (clamped to +-pi/2 outside (-1, 1)), azimuth = atan2(-m[2][0], m[2][2])
    (0 outside (-1, 1) of m[2][1]); beam b's ring id is ring_ids[b % len(ring_ids)] as uint16."""
    rays = np.asarray(rays_world, dtype=np.float64).reshape(-1, 3, 4)
    inv = inv34(sensor_to_world)
    local = np.einsum("ij,njk->nik", inv[:, :3], rays[:, :, :3])
    m12, m21 = local[:, 1, 2], local[:, 2, 1]
    elev = np.where(m12 < 1.0, np.where(m12 > -1.0, np.arcsin(np.clip(m12, -1.0, 1.0)), -np.pi / 2), np.pi / 2)
    az = np.where((m21 < 1.0) & (m21 > -1.0), np.arctan2(-local[:, 2, 0], local[:, 2, 2]), 0.0)
    out = {"azimuth": np.repeat(az, return_count), "elevation": np.repeat(elev, return_count)}
    if ring_ids is not None:
        ids = np.asarray(ring_ids, dtype=np.int64)
        out["ring_id"] = np.repeat(ids[np.arange(rays.shape[0]) % len(ids)].astype(np.uint16), return_count)
    return out
