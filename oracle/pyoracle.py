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
                                   C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                   C.c_void_p, C.c_void_p, C.c_void_p]
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
        normal = np.zeros((npts, 3), np.float32)
        incident = np.zeros(npts, np.float32)
        tri_tie = np.zeros(npts, np.uint8)
        tf = None if ray_transform is None else np.ascontiguousarray(ray_transform, dtype=np.float32).reshape(12)
        rg = None if ranges is None else np.ascontiguousarray(ranges, dtype=np.float32).reshape(-1, 2)
        threads = threads or os.cpu_count() or 1
        ns = self._l.orc_raytrace(self.h, _p(rays), n, _p(tf), _p(rg), 0 if rg is None else rg.shape[0],
                                  int(np.int32(np.uint32(return_mode & 0xFFFFFFFF))), h_div, v_div, layers, vertices,
                                  near, far, default_intensity, threads, _p(xyz), _p(dist), _p(ent), _p(hit),
                                  _p(rtype), _p(inten), _p(amb), _p(normal), _p(incident), _p(tri_tie))
        return {"xyz": xyz, "distance": dist, "entity_id": ent, "is_hit": hit, "return_type": rtype,
                "intensity": inten, "ambiguous": amb, "normal": normal, "incident_angle": incident,
                "triangle_tie": tri_tie, "samples": ns}


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


# ---------------------------------------------------------------- velocities and velocity distortion (FP64)

def hit_velocities(hit_world, entity_now, entity_prev, dt, sensor_to_world, lin_vel, ang_vel):
    """Velocities of hit points (reference src/gpu/optixPrograms.cu:169-212): the point fixed in its
    entity moves from entity_prev @ p_obj to entity_now @ p_obj over dt (entity_prev None: no known
    previous pose, zero displacement); relative velocity = that velocity in the sensor frame minus the
    sensor's linear velocity minus angular x (hit in the sensor frame); radial speed = its component
    along the sensor-to-hit direction. Per point arrays: entity_now / entity_prev are (n, 3, 4)."""
    n = len(hit_world)
    absv = np.zeros((n, 3))
    for i in range(n):
        now = mat4(entity_now[i])
        p_obj = np.linalg.solve(now, np.append(np.asarray(hit_world[i], np.float64), 1.0))
        if entity_prev[i] is not None:
            absv[i] = (now @ p_obj - mat4(entity_prev[i]) @ p_obj)[:3] / dt
    s2w = mat4(sensor_to_world)
    rot_inv = np.linalg.inv(s2w[:3, :3])
    hit_s = (np.linalg.inv(s2w) @ np.c_[np.asarray(hit_world, np.float64), np.ones(n)].T).T[:, :3]
    rel = (rot_inv @ absv.T).T - np.asarray(lin_vel, np.float64) - np.cross(np.asarray(ang_vel, np.float64), hit_s)
    radial = np.einsum("ij,ij->i", hit_s / np.linalg.norm(hit_s, axis=1, keepdims=True), rel)
    return absv, rel, radial


def distort_rays(rays_world, sensor_to_world, offsets_ms, lin_vel, ang_vel):
    """Ray poses under velocity distortion (reference src/gpu/optixPrograms.cu:60-70): in the sensor
    frame each ray is moved by translation offset*lin/1000 and rotation Rz Ry Rx of offset*ang/1000
    rad, then returned to the world frame."""
    s2w = mat4(sensor_to_world)
    w2s = np.linalg.inv(s2w)
    out = np.zeros((len(rays_world), 3, 4))
    for i, r in enumerate(np.asarray(rays_world, np.float64).reshape(-1, 3, 4)):
        t = offsets_ms[i] * np.asarray(lin_vel, np.float64) * 1e-3
        rx, ry, rz = offsets_ms[i] * np.asarray(ang_vel, np.float64) * 1e-3
        cx, sx, cy, sy, cz, sz = np.cos(rx), np.sin(rx), np.cos(ry), np.sin(ry), np.cos(rz), np.sin(rz)
        R = (np.array([[cz, -sz, 0], [sz, cz, 0], [0, 0, 1]]) @ np.array([[cy, 0, sy], [0, 1, 0], [-sy, 0, cy]])
             @ np.array([[1, 0, 0], [0, cx, -sx], [0, sx, cx]]))
        m = np.eye(4)
        m[:3, :3] = R
        m[:3, 3] = t
        out[i] = (s2w @ m @ w2s @ mat4(r))[:3, :]
    return out.astype(np.float32)


# ---------------------------------------------------------------- mesh animation (FP64)

def skinned_vertices(rest, weights, bones, pose, restposes):
    """Linear blend skinning (reference src/gpu/sceneKernels.cu:17-38): vertex i moves to
    sum_k weights[i, k] * (pose[b] @ restposes[b]) @ rest[i] with b = bones[i, k]."""
    rest = np.asarray(rest, np.float64)
    mats = [mat4(p) @ mat4(r) for p, r in zip(pose, restposes)]
    out = np.zeros_like(rest)
    for i, v in enumerate(rest):
        for k in range(4):
            if weights[i][k] != 0.0:
                out[i] += weights[i][k] * (mats[bones[i][k]] @ np.append(v, 1.0))[:3]
    return out.astype(np.float32)


def animation_velocity(hit_world, entity_tf, tri_vertices, tri_displacements, dt):
    """Velocity of a hit on an animated mesh whose pose did not change (reference
    src/gpu/optixPrograms.cu:185-195): the triangle's vertex displacements since the previous step,
    rotated into the world and interpolated at the hit's barycentric coordinates, over dt."""
    m = mat4(entity_tf)
    p = (np.linalg.inv(m) @ np.append(np.asarray(hit_world, np.float64), 1.0))[:3]
    a, b, c = (np.asarray(x, np.float64) for x in tri_vertices)
    n = np.cross(b - a, c - a)
    u = np.dot(np.cross(p - a, c - a), n) / np.dot(n, n)
    w = np.dot(np.cross(b - a, p - a), n) / np.dot(n, n)
    da, db, dc = (m[:3, :3] @ np.asarray(x, np.float64) for x in tri_displacements)
    return ((1 - u - w) * da + u * db + w * dc) / dt
