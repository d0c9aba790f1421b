"""Python mirror of the RGL C API exported by libRobotecGPULidar.so (this project's build).

Function names, argument meaning, enum values and status codes are those of RobotecGPULidar's
include/rgl/api/core.h; every call goes through the C ABI with ctypes, so tests written with this
module exercise exactly what an engine plugin links against.  ``check()`` turns a non-success status
into ``RGLError`` carrying the library's last error string.

The library is loaded lazily from ``robotecgpulidar_gb300/_build`` (built by ``build.build()``); a
missing library raises instead of falling back to anything else.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

# ---- status codes
RGL_SUCCESS = 0
RGL_INVALID_ARGUMENT = 1
RGL_INVALID_STATE = 2
RGL_LOGGING_ERROR = 3
RGL_INVALID_API_OBJECT = 4
RGL_INVALID_FILE_PATH = 5
RGL_TAPE_ERROR = 6
RGL_UDP_ERROR = 7
RGL_ROS2_ERROR = 8
RGL_INVALID_PIPELINE = 9
RGL_INITIALIZATION_ERROR = 10
RGL_NOT_IMPLEMENTED = 404
RGL_INTERNAL_EXCEPTION = 500

# ---- fields
RGL_FIELD_XYZ_VEC3_F32 = 1
RGL_FIELD_INTENSITY_F32 = 2
RGL_FIELD_INTENSITY_U8 = 3
RGL_FIELD_IS_HIT_I32 = 4
RGL_FIELD_IS_GROUND_I32 = 5
RGL_FIELD_RAY_IDX_U32 = 6
RGL_FIELD_ENTITY_ID_I32 = 7
RGL_FIELD_DISTANCE_F32 = 8
RGL_FIELD_AZIMUTH_F32 = 9
RGL_FIELD_ELEVATION_F32 = 10
RGL_FIELD_RING_ID_U16 = 11
RGL_FIELD_RETURN_TYPE_U8 = 12
RGL_FIELD_TIME_STAMP_F64 = 13
RGL_FIELD_TIME_STAMP_U32 = 14
RGL_FIELD_ABSOLUTE_VELOCITY_VEC3_F32 = 15
RGL_FIELD_RELATIVE_VELOCITY_VEC3_F32 = 16
RGL_FIELD_RADIAL_SPEED_F32 = 17
RGL_FIELD_POWER_F32 = 18
RGL_FIELD_RCS_F32 = 19
RGL_FIELD_NOISE_F32 = 20
RGL_FIELD_SNR_F32 = 21
RGL_FIELD_NORMAL_VEC3_F32 = 22
RGL_FIELD_INCIDENT_ANGLE_F32 = 23
RGL_FIELD_RAY_POSE_MAT3x4_F32 = 24
RGL_FIELD_LASER_RETRO_F32 = 25
RGL_FIELD_PADDING_8 = 1024
RGL_FIELD_PADDING_16 = 1025
RGL_FIELD_PADDING_32 = 1026
RGL_FIELD_DYNAMIC_FORMAT = 13842

FIELD_SIZE = {
    RGL_FIELD_XYZ_VEC3_F32: 12, RGL_FIELD_INTENSITY_F32: 4, RGL_FIELD_INTENSITY_U8: 1, RGL_FIELD_IS_HIT_I32: 4,
    RGL_FIELD_IS_GROUND_I32: 4, RGL_FIELD_RAY_IDX_U32: 4, RGL_FIELD_ENTITY_ID_I32: 4, RGL_FIELD_DISTANCE_F32: 4,
    RGL_FIELD_AZIMUTH_F32: 4, RGL_FIELD_ELEVATION_F32: 4, RGL_FIELD_RING_ID_U16: 2, RGL_FIELD_RETURN_TYPE_U8: 1,
    RGL_FIELD_TIME_STAMP_F64: 8, RGL_FIELD_TIME_STAMP_U32: 4, RGL_FIELD_ABSOLUTE_VELOCITY_VEC3_F32: 12,
    RGL_FIELD_RELATIVE_VELOCITY_VEC3_F32: 12, RGL_FIELD_RADIAL_SPEED_F32: 4, RGL_FIELD_POWER_F32: 4,
    RGL_FIELD_RCS_F32: 4, RGL_FIELD_NOISE_F32: 4, RGL_FIELD_SNR_F32: 4, RGL_FIELD_NORMAL_VEC3_F32: 12,
    RGL_FIELD_INCIDENT_ANGLE_F32: 4, RGL_FIELD_RAY_POSE_MAT3x4_F32: 48, RGL_FIELD_LASER_RETRO_F32: 4,
    RGL_FIELD_PADDING_8: 1, RGL_FIELD_PADDING_16: 2, RGL_FIELD_PADDING_32: 4,
}

FIELD_DTYPE = {
    RGL_FIELD_XYZ_VEC3_F32: (np.float32, 3), RGL_FIELD_INTENSITY_F32: (np.float32, 1),
    RGL_FIELD_INTENSITY_U8: (np.uint8, 1), RGL_FIELD_IS_HIT_I32: (np.int32, 1), RGL_FIELD_IS_GROUND_I32: (np.int32, 1),
    RGL_FIELD_RAY_IDX_U32: (np.uint32, 1), RGL_FIELD_ENTITY_ID_I32: (np.int32, 1),
    RGL_FIELD_DISTANCE_F32: (np.float32, 1), RGL_FIELD_RETURN_TYPE_U8: (np.uint8, 1),
    RGL_FIELD_NORMAL_VEC3_F32: (np.float32, 3), RGL_FIELD_INCIDENT_ANGLE_F32: (np.float32, 1),
    RGL_FIELD_LASER_RETRO_F32: (np.float32, 1), RGL_FIELD_RING_ID_U16: (np.uint16, 1),
    RGL_FIELD_TIME_STAMP_F64: (np.float64, 1), RGL_FIELD_TIME_STAMP_U32: (np.uint32, 1),
    RGL_FIELD_AZIMUTH_F32: (np.float32, 1), RGL_FIELD_ELEVATION_F32: (np.float32, 1),
    RGL_FIELD_RAY_POSE_MAT3x4_F32: (np.float32, 12),
    RGL_FIELD_ABSOLUTE_VELOCITY_VEC3_F32: (np.float32, 3), RGL_FIELD_RELATIVE_VELOCITY_VEC3_F32: (np.float32, 3),
    RGL_FIELD_RADIAL_SPEED_F32: (np.float32, 1),
}

# ---- return modes
RGL_RETURN_TYPE_UNKNOWN = 0
RGL_RETURN_TYPE_STRONGEST = 1
RGL_RETURN_TYPE_LAST = 2
RGL_RETURN_TYPE_SECOND = 3
RGL_RETURN_TYPE_FIRST = 4
RGL_RETURN_TYPE_SECOND_STRONGEST = 5
_S = 1 << 24
_D = 2 << 24
RGL_RETURN_UNKNOWN = 0
RGL_RETURN_FIRST = _S | RGL_RETURN_TYPE_FIRST
RGL_RETURN_SECOND = _S | RGL_RETURN_TYPE_SECOND
RGL_RETURN_LAST = _S | RGL_RETURN_TYPE_LAST
RGL_RETURN_STRONGEST = _S | RGL_RETURN_TYPE_STRONGEST
RGL_RETURN_LAST_STRONGEST = _D | RGL_RETURN_TYPE_LAST | (RGL_RETURN_TYPE_STRONGEST << 8)
RGL_RETURN_FIRST_LAST = _D | RGL_RETURN_TYPE_FIRST | (RGL_RETURN_TYPE_LAST << 8)
RGL_RETURN_FIRST_STRONGEST = _D | RGL_RETURN_TYPE_FIRST | (RGL_RETURN_TYPE_STRONGEST << 8)
RGL_RETURN_STRONGEST_SECOND_STRONGEST = _D | RGL_RETURN_TYPE_STRONGEST | (RGL_RETURN_TYPE_SECOND_STRONGEST << 8)
RGL_RETURN_FIRST_SECOND = _D | RGL_RETURN_TYPE_FIRST | (RGL_RETURN_TYPE_SECOND << 8)

RGL_AXIS_X, RGL_AXIS_Y, RGL_AXIS_Z = 1, 2, 3
RGL_ENTITY_INVALID_ID = 0
RGL_DEFAULT_ENTITY_ID = 268435455
RGL_LOG_LEVEL_OFF = 6

LIB_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_build")
LIB_PATH = os.path.join(LIB_DIR, "libRobotecGPULidar.so")

_lib = None


class RGLError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"RGL status {status}: {message}")
        self.status = status
        self.message = message


def _proto(l):
    vp, i32, f, u64 = C.c_void_p, C.c_int32, C.c_float, C.c_uint64
    P = C.POINTER
    sigs = {
        "rgl_get_version_info": [P(i32), P(i32), P(i32)],
        "rgl_get_extension_info": [i32, P(i32)],
        "rgl_configure_logging": [i32, C.c_char_p, C.c_bool],
        "rgl_cleanup": [],
        "rgl_mesh_create": [P(vp), vp, i32, vp, i32],
        "rgl_mesh_destroy": [vp],
        "rgl_mesh_is_alive": [vp, P(C.c_bool)],
        "rgl_mesh_set_texture_coords": [vp, vp, i32],
        "rgl_entity_create": [P(vp), vp, vp],
        "rgl_entity_destroy": [vp],
        "rgl_entity_set_transform": [vp, vp],
        "rgl_entity_set_id": [vp, i32],
        "rgl_entity_set_laser_retro": [vp, f],
        "rgl_entity_is_alive": [vp, P(C.c_bool)],
        "rgl_scene_set_time": [vp, u64],
        "rgl_node_rays_from_mat3x4f": [P(vp), vp, i32],
        "rgl_node_rays_set_range": [P(vp), vp, i32],
        "rgl_node_rays_set_ring_ids": [P(vp), vp, i32],
        "rgl_node_rays_set_time_offsets": [P(vp), vp, i32],
        "rgl_node_rays_transform": [P(vp), vp],
        "rgl_node_points_transform": [P(vp), vp],
        "rgl_node_raytrace": [P(vp), vp],
        "rgl_node_raytrace_configure_velocity": [vp, vp, vp],
        "rgl_node_raytrace_configure_distortion": [vp, C.c_bool],
        "rgl_node_raytrace_configure_non_hits": [vp, f, f],
        "rgl_node_raytrace_configure_mask": [vp, vp, i32],
        "rgl_node_raytrace_configure_beam_divergence": [vp, f, f],
        "rgl_node_raytrace_configure_default_intensity": [vp, f],
        "rgl_node_raytrace_configure_return_mode": [vp, i32],
        "rgl_node_points_format": [P(vp), vp, i32],
        "rgl_node_points_yield": [P(vp), vp, i32],
        "rgl_node_points_compact_by_field": [P(vp), i32],
        "rgl_tape_record_begin": [C.c_char_p],
        "rgl_tape_record_end": [],
        "rgl_tape_record_is_active": [P(C.c_bool)],
        "rgl_tape_play": [C.c_char_p],
        "rgl_node_points_spatial_merge": [P(vp), vp, i32],
        "rgl_node_points_temporal_merge": [P(vp), vp, i32],
        "rgl_node_points_from_array": [P(vp), vp, i32, vp, i32],
        "rgl_node_points_filter_ground": [P(vp), vp, f],
        "rgl_node_gaussian_noise_angular_ray": [P(vp), f, f, i32],
        "rgl_node_gaussian_noise_angular_hitpoint": [P(vp), f, f, i32],
        "rgl_node_gaussian_noise_distance": [P(vp), f, f, f],
        "rgl_node_is_alive": [vp, P(C.c_bool)],
        "rgl_graph_run": [vp],
        "rgl_graph_destroy": [vp],
        "rgl_graph_get_result_size": [vp, i32, P(i32), P(i32)],
        "rgl_graph_get_result_data": [vp, i32, vp],
        "rgl_graph_node_add_child": [vp, vp],
        "rgl_graph_node_remove_child": [vp, vp],
        "rgl_graph_node_set_priority": [vp, i32],
        "rgl_graph_node_get_priority": [vp, P(i32)],
        # GB300 extensions (include/rgl/api/extensions/gb300.h)
        "rgl_gb300_node_gaussian_noise_set_seed": [vp, u64, u64],
        "rgl_gb300_node_raytrace_configure_beam_samples": [vp, i32, i32],
        "rgl_gb300_configure_timing": [C.c_bool],
        "rgl_gb300_graph_get_timing": [vp, P(f), P(f)],
        "rgl_gb300_get_kernel_launch_count": [P(u64)],
        "rgl_gb300_graph_sync": [vp],
        "rgl_gb300_device_info": [P(i32), P(i32)],
        "rgl_gb300_scene_get_stats": [P(C.c_int64), P(C.c_int64), P(i32)],
        "rgl_gb300_configure_blas_builder": [i32],
        "rgl_gb300_get_blas_build_stats": [P(C.c_int64), P(C.c_double)],
        "rgl_gb300_compact_by_flags_noalloc": [vp, vp, i32, i32, vp, P(i32), vp],
        "rgl_gb300_configure_cuda_graphs": [C.c_bool],
        "rgl_gb300_graph_get_capture_stats": [vp, P(C.c_int64), P(C.c_int64)],
        "rgl_gb300_batch_create": [P(vp), P(vp), i32],
        "rgl_gb300_batch_run": [vp],
        "rgl_gb300_batch_destroy": [vp],
        "rgl_gb300_batch_configure_schedule": [vp, C.c_bool, i32, i32, i32, i32, i32],
        "rgl_gb300_batch_get_schedule": [vp, P(i32), P(i32), P(i32), P(i32), P(i32)],
        "rgl_gb300_batch_get_stats": [vp, P(f), P(f), P(C.c_int64), P(C.c_int64), P(C.c_int64), P(C.c_int64), P(C.c_int64)],
        "rgl_gb300_batch_get_tuning": [vp, i32, P(i32), P(f), P(i32)],
        "rgl_gb300_batch_configure_waves": [vp, i32],
        "rgl_gb300_batch_get_waves": [vp, P(i32)],
        "rgl_gb300_configure_trace_schedule": [i32, i32, i32, i32],
        "rgl_gb300_configure_trace_order": [i32],
        "rgl_gb300_scene_create": [P(vp)],
        "rgl_gb300_scene_destroy": [vp],
        "rgl_gb300_scene_get_stats_of": [vp, P(C.c_int64), P(C.c_int64), P(i32)],
        "rgl_gb300_server_create": [P(vp), C.c_int64, i32],
        "rgl_gb300_server_destroy": [vp],
        "rgl_gb300_server_add_pattern": [vp, vp, i32, P(i32)],
        "rgl_gb300_server_submit": [vp, vp, i32, vp, i32, f, f, P(C.c_int64)],
        "rgl_gb300_server_wait": [vp, C.c_int64, f, P(C.c_bool)],
        "rgl_gb300_server_take_completed": [vp, P(C.c_int64), i32, P(i32)],
        "rgl_gb300_server_wait_completed": [vp, f, P(C.c_int64), i32, P(i32)],
        "rgl_gb300_server_get_result_size": [vp, C.c_int64, i32, P(i32), P(i32)],
        "rgl_gb300_server_get_result_data": [vp, C.c_int64, i32, vp],
        "rgl_gb300_server_get_request_timing": [vp, C.c_int64, P(C.c_double), P(C.c_double)],
        "rgl_gb300_server_get_result_host": [vp, C.c_int64, i32, P(vp), P(i32)],
        "rgl_gb300_server_release": [vp, C.c_int64],
        "rgl_gb300_server_drain": [vp],
        "rgl_gb300_server_configure_schedule": [vp, i32, i32, i32, i32, C.c_int64],
        "rgl_gb300_server_get_batch_times": [vp, C.c_bool, P(f), P(C.c_int64), P(C.c_int64)],
        "rgl_gb300_server_get_stats": [vp] + [P(C.c_int64)] * 7,
    }
    for name, args in sigs.items():
        fn = getattr(l, name)
        fn.argtypes = args
        fn.restype = C.c_int32
    l.rgl_get_last_error_string.argtypes = [C.POINTER(C.c_char_p)]
    l.rgl_get_last_error_string.restype = None


def lib():
    """Load libRobotecGPULidar.so; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"libRobotecGPULidar.so not built ({LIB_PATH}); run __graft_entry__.build()")
        l = C.CDLL(LIB_PATH)
        _proto(l)
        _lib = l
    return _lib


def last_error() -> str:
    s = C.c_char_p()
    lib().rgl_get_last_error_string(C.byref(s))
    return (s.value or b"").decode()


def check(status: int):
    if status != RGL_SUCCESS:
        raise RGLError(status, last_error())
    return status


def call(name: str, *args) -> int:
    """Call an API function by name; returns the raw status (no check)."""
    return getattr(lib(), name)(*args)


def node() -> C.c_void_p:
    return C.c_void_p(None)


def ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def mat(m) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(m, dtype=np.float32).reshape(3, 4))


# ---------------------------------------------------------------- convenience wrappers

def mesh_create(vertices, indices) -> C.c_void_p:
    v = np.ascontiguousarray(vertices, dtype=np.float32)
    i = np.ascontiguousarray(indices, dtype=np.int32)
    h = C.c_void_p()
    check(lib().rgl_mesh_create(C.byref(h), ptr(v), v.shape[0], ptr(i), i.shape[0]))
    return h


def entity_create(mesh) -> C.c_void_p:
    h = C.c_void_p()
    check(lib().rgl_entity_create(C.byref(h), None, mesh))
    return h


def entity_set_transform(entity, tf):
    m = mat(tf)
    check(lib().rgl_entity_set_transform(entity, ptr(m)))


def entity_set_id(entity, eid: int):
    check(lib().rgl_entity_set_id(entity, int(eid)))


def spawn_scene(scene):
    """Creates meshes and entities of a scenes.Scene; returns (meshes, entities)."""
    meshes = [mesh_create(m.vertices, m.indices) for m in scene.meshes]
    ents = []
    for e in scene.entities:
        h = entity_create(meshes[e.mesh])
        entity_set_transform(h, e.transform)
        entity_set_id(h, e.entity_id)
        ents.append(h)
    return meshes, ents


def rays_from_mat3x4f(node_ref, rays):
    r = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 12)
    check(lib().rgl_node_rays_from_mat3x4f(C.byref(node_ref), ptr(r), r.shape[0]))
    return node_ref


def rays_set_range(node_ref, ranges):
    r = np.ascontiguousarray(ranges, dtype=np.float32).reshape(-1, 2)
    check(lib().rgl_node_rays_set_range(C.byref(node_ref), ptr(r), r.shape[0]))
    return node_ref


def rays_transform(node_ref, tf):
    m = mat(tf)
    check(lib().rgl_node_rays_transform(C.byref(node_ref), ptr(m)))
    return node_ref


def points_transform(node_ref, tf):
    m = mat(tf)
    check(lib().rgl_node_points_transform(C.byref(node_ref), ptr(m)))
    return node_ref


def raytrace(node_ref):
    check(lib().rgl_node_raytrace(C.byref(node_ref), None))
    return node_ref


def _fields(fields):
    return np.ascontiguousarray(np.asarray(fields, dtype=np.int32))


def points_yield(node_ref, fields):
    f = _fields(fields)
    check(lib().rgl_node_points_yield(C.byref(node_ref), ptr(f), f.shape[0]))
    return node_ref


def points_format(node_ref, fields):
    f = _fields(fields)
    check(lib().rgl_node_points_format(C.byref(node_ref), ptr(f), f.shape[0]))
    return node_ref


def points_compact_by_field(node_ref, field=RGL_FIELD_IS_HIT_I32):
    check(lib().rgl_node_points_compact_by_field(C.byref(node_ref), field))
    return node_ref


def points_from_array(node_ref, data: np.ndarray, count: int, fields):
    f = _fields(fields)
    d = np.ascontiguousarray(data)
    check(lib().rgl_node_points_from_array(C.byref(node_ref), ptr(d), count, ptr(f), f.shape[0]))
    return node_ref


def points_spatial_merge(node_ref, fields):
    f = _fields(fields)
    check(lib().rgl_node_points_spatial_merge(C.byref(node_ref), ptr(f), f.shape[0]))
    return node_ref


def points_temporal_merge(node_ref, fields):
    f = _fields(fields)
    check(lib().rgl_node_points_temporal_merge(C.byref(node_ref), ptr(f), f.shape[0]))
    return node_ref


def add_child(parent, child):
    check(lib().rgl_graph_node_add_child(parent, child))


def chain(*nodes):
    for a, b in zip(nodes[:-1], nodes[1:]):
        add_child(a, b)


def graph_run(n):
    check(lib().rgl_graph_run(n))


def result_size(n, field):
    cnt, sz = C.c_int32(), C.c_int32()
    check(lib().rgl_graph_get_result_size(n, field, C.byref(cnt), C.byref(sz)))
    return cnt.value, sz.value


def result(n, field) -> np.ndarray:
    cnt, sz = result_size(n, field)
    if field in FIELD_DTYPE:
        dt, k = FIELD_DTYPE[field]
        out = np.zeros((cnt, k) if k > 1 else cnt, dtype=dt)
    else:
        out = np.zeros(cnt * sz, dtype=np.uint8)
    if cnt > 0:
        check(lib().rgl_graph_get_result_data(n, field, ptr(out)))
    return out


def result_bytes(n, field) -> np.ndarray:
    cnt, sz = result_size(n, field)
    out = np.zeros(cnt * sz, dtype=np.uint8)
    if cnt > 0:
        check(lib().rgl_graph_get_result_data(n, field, ptr(out)))
    return out


def cleanup():
    check(lib().rgl_cleanup())


def set_noise_seed(n, seed: int, frame: int = 0):
    check(lib().rgl_gb300_node_gaussian_noise_set_seed(n, seed, frame))


def configure_beam_samples(n, layers: int, vertices: int):
    check(lib().rgl_gb300_node_raytrace_configure_beam_samples(n, layers, vertices))


def kernel_launch_count() -> int:
    v = C.c_uint64()
    check(lib().rgl_gb300_get_kernel_launch_count(C.byref(v)))
    return v.value


# ---------------------------------------------------------------- batched multi-sensor frames

PACK_LANE_GROUP, PACK_SERIAL = 0, 1
ORDER_NATURAL, ORDER_OCTAHEDRAL, ORDER_MORTON, ORDER_ELEVATION = 0, 1, 2, 3


def batch_create(nodes) -> C.c_void_p:
    """One batch over the graphs of `nodes` (any node of each graph)."""
    arr = (C.c_void_p * len(nodes))(*[n.value if isinstance(n, C.c_void_p) else n for n in nodes])
    b = C.c_void_p()
    check(lib().rgl_gb300_batch_create(C.byref(b), arr, len(nodes)))
    return b


def batch_run(b):
    check(lib().rgl_gb300_batch_run(b))


def batch_destroy(b):
    check(lib().rgl_gb300_batch_destroy(b))


def batch_configure_schedule(b, autotune=True, block=128, packing=PACK_LANE_GROUP, order=ORDER_NATURAL, chunk=2, regs=96):
    check(lib().rgl_gb300_batch_configure_schedule(b, autotune, block, packing, order, chunk, regs))


def batch_schedule(b) -> dict:
    v = [C.c_int32() for _ in range(5)]
    check(lib().rgl_gb300_batch_get_schedule(b, *[C.byref(x) for x in v]))
    return dict(zip(["block", "packing", "order", "chunk", "regs"], [x.value for x in v]))


def batch_tuning(b) -> list:
    """The last tuning's candidates: [(schedule dict, ms), ...] in the order tried."""
    n = C.c_int32()
    check(lib().rgl_gb300_batch_get_tuning(b, 0, None, None, C.byref(n)))
    sch = (C.c_int32 * (5 * max(1, n.value)))()
    ms = (C.c_float * max(1, n.value))()
    check(lib().rgl_gb300_batch_get_tuning(b, n.value, sch, ms, C.byref(n)))
    keys = ["block", "packing", "order", "chunk", "regs"]
    return [(dict(zip(keys, sch[5 * i:5 * i + 5])), ms[i]) for i in range(n.value)]


def batch_configure_waves(b, waves: int = 0):
    """Waves per frame (0: automatic)."""
    check(lib().rgl_gb300_batch_configure_waves(b, waves))


def batch_waves(b) -> int:
    """Waves of the last frame (0 before the first)."""
    n = C.c_int32()
    check(lib().rgl_gb300_batch_get_waves(b, C.byref(n)))
    return n.value


def batch_stats(b) -> dict:
    fm, tm = C.c_float(), C.c_float()
    ints = [C.c_int64() for _ in range(5)]
    check(lib().rgl_gb300_batch_get_stats(b, C.byref(fm), C.byref(tm), *[C.byref(x) for x in ints]))
    out = {"frame_ms": fm.value, "trace_ms": tm.value}
    out.update(zip(["beams", "rays", "captures", "replays", "tunings"], [x.value for x in ints]))
    return out


# ---------------------------------------------------------------- resident scenes and serving


def scene_create() -> C.c_void_p:
    sc = C.c_void_p()
    check(lib().rgl_gb300_scene_create(C.byref(sc)))
    return sc


def scene_destroy(sc):
    check(lib().rgl_gb300_scene_destroy(sc))


def entity_create_in(scene, mesh) -> C.c_void_p:
    e = C.c_void_p()
    check(lib().rgl_entity_create(C.byref(e), scene, mesh))
    return e


def spawn_scene_in(scene_handle, scene, meshes=None):
    """Creates a scenes.Scene's entities in a resident scene (meshes created unless given)."""
    meshes = meshes or [mesh_create(m.vertices, m.indices) for m in scene.meshes]
    ents = []
    for e in scene.entities:
        h = entity_create_in(scene_handle, meshes[e.mesh])
        entity_set_transform(h, e.transform)
        entity_set_id(h, e.entity_id)
        ents.append(h)
    return meshes, ents


def raytrace_in(node_ref, scene):
    check(lib().rgl_node_raytrace(C.byref(node_ref), scene))
    return node_ref


class Server:
    """ctypes wrapper of rgl_gb300_server_*."""

    def __init__(self, budget_bytes: int, max_in_flight: int = 2):
        self.h = C.c_void_p()
        check(lib().rgl_gb300_server_create(C.byref(self.h), int(budget_bytes), int(max_in_flight)))

    def destroy(self):
        if self.h:
            check(lib().rgl_gb300_server_destroy(self.h))
            self.h = C.c_void_p()

    def add_pattern(self, rays) -> int:
        r = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 12)
        out = C.c_int32()
        check(lib().rgl_gb300_server_add_pattern(self.h, ptr(r), r.shape[0], C.byref(out)))
        return out.value

    def submit(self, scene, pattern: int, pose, mode: int, min_range: float = 0.0, max_range: float = float("inf")) -> int:
        m = mat(pose)
        out = C.c_int64()
        check(lib().rgl_gb300_server_submit(self.h, scene, int(pattern), ptr(m), int(np.int32(np.uint32(mode))), min_range, max_range,
                                            C.byref(out)))
        return out.value

    def wait(self, req: int, timeout_ms: float = -1.0) -> bool:
        done = C.c_bool()
        check(lib().rgl_gb300_server_wait(self.h, req, timeout_ms, C.byref(done)))
        return done.value

    def take_completed(self, capacity: int = 4096) -> list:
        buf = (C.c_int64 * capacity)()
        n = C.c_int32()
        check(lib().rgl_gb300_server_take_completed(self.h, buf, capacity, C.byref(n)))
        return list(buf[: n.value])

    def wait_completed(self, timeout_ms: float, capacity: int = 4096) -> list:
        buf = (C.c_int64 * capacity)()
        n = C.c_int32()
        check(lib().rgl_gb300_server_wait_completed(self.h, timeout_ms, buf, capacity, C.byref(n)))
        return list(buf[: n.value])

    def result(self, req: int, field: int) -> np.ndarray:
        cnt, sz = C.c_int32(), C.c_int32()
        check(lib().rgl_gb300_server_get_result_size(self.h, req, field, C.byref(cnt), C.byref(sz)))
        dt, k = FIELD_DTYPE[field]
        out = np.zeros((cnt.value, k) if k > 1 else cnt.value, dtype=dt)
        if cnt.value > 0:
            check(lib().rgl_gb300_server_get_result_data(self.h, req, field, ptr(out)))
        return out

    def timing(self, req: int):
        q, t = C.c_double(), C.c_double()
        check(lib().rgl_gb300_server_get_request_timing(self.h, req, C.byref(q), C.byref(t)))
        return q.value, t.value

    def release(self, req: int):
        check(lib().rgl_gb300_server_release(self.h, req))

    def drain(self):
        check(lib().rgl_gb300_server_drain(self.h))

    def configure_schedule(self, block=256, order=3, chunk=1, regs=128, max_batch_beams=4 << 20):
        check(lib().rgl_gb300_server_configure_schedule(self.h, block, order, chunk, regs, max_batch_beams))

    def batch_times(self, reset=True) -> dict:
        """Longest phase times (ms) and batches above 5 ms per phase since the last reset: traversal and
        compaction, the server's reaction to the counts, the result copies."""
        mx = (C.c_float * 3)()
        over = (C.c_int64 * 3)()
        n = C.c_int64()
        check(lib().rgl_gb300_server_get_batch_times(self.h, reset, mx, over, C.byref(n)))
        names = ("trace", "reaction", "copies")
        return {"batches": n.value, "max_ms": dict(zip(names, [round(x, 3) for x in mx])), "over_5ms": dict(zip(names, list(over)))}

    def stats(self) -> dict:
        v = [C.c_int64() for _ in range(7)]
        check(lib().rgl_gb300_server_get_stats(self.h, *[C.byref(x) for x in v]))
        return dict(zip(["submitted", "completed", "failed", "batches", "requests_in_batches", "peak_reserved_bytes", "device_us"],
                        [x.value for x in v]))
