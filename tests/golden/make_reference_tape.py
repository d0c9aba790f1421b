"""Writes tests/golden/reference_tape.{yaml,bin} (+ reference_tape.json): a tape in the exact form the
reference library's recorder writes, for a plugin-like session, used to check that rgl_tape_play
plays tapes recorded by the reference.

The form follows the reference recorder (src/tape/TapeRecorder.hpp:54-151, TapeRecorder.cpp:24-66)
and its hooks (src/api/apiCore.cpp, one TAPE_HOOK per call, after the call):
  * the YAML file is one block sequence; each item is `- <function>: {t: <ns>, a: [<args>]}` as
    yaml-cpp's emitter writes a flow map under a block key; the first item is
    rgl_get_version_info with the library version (0, 19, 0);
  * handles (and out-handles, dereferenced) are the recording process's addresses as unsigned
    integers; enums are their integer values; floats are written with 9 significant digits in %g
    form (yaml-cpp's float precision), infinities as .inf; booleans as true/false;
  * arrays (TAPE_ARRAY) and single vectors and matrices are appended to the binary file, each padded
    to a 16-byte multiple, and the YAML holds the byte offset where each starts;
  * int32_t* out-arguments (rgl_graph_get_result_size's count and size) hold the value written.
The expected result count comes from the FP64 oracle on the same scene and rays (no ambiguous ray).

Usage: python tests/golden/make_reference_tape.py [output directory]   (default: next to this script)
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from robotecgpulidar_gb300 import scenes  # noqa: E402

# Enum values of include/rgl/api/core.h (the reference's).
FIELD_XYZ, FIELD_IS_HIT, FIELD_ENTITY_ID, FIELD_DISTANCE = 1, 4, 7, 8
RETURN_FIRST = (1 << 24) | 4
AXIS_Z = 3


class Tape:
    def __init__(self):
        self.lines = []
        self.bin = bytearray()
        self.t = 48_213  # ns since the recording began

    def array(self, a: np.ndarray) -> int:
        off = len(self.bin)
        raw = np.ascontiguousarray(a).tobytes()
        self.bin += raw + b"\0" * ((16 - len(raw) % 16) % 16)
        return off

    def call(self, fn: str, *args):
        out = []
        for v in args:
            if isinstance(v, bool):
                out.append("true" if v else "false")
            elif isinstance(v, np.float32):
                out.append(".inf" if np.isinf(v) and v > 0 else "-.inf" if np.isinf(v) else "%.9g" % float(v))
            else:
                out.append(str(int(v)))
        self.lines.append("- %s: {t: %d, a: [%s]}" % (fn, self.t, ", ".join(out)))
        self.t += 7_000 + 131 * len(self.lines)


def f32(x) -> np.float32:
    return np.float32(x)


def session():
    """The scene and sensor of the recorded session: a ground quad and two cubes, a 16 x 128 lidar at
    1.2 m with range [0.1, 60] m, first return, distance noise, compaction by is-hit."""
    ground = scenes.Mesh(np.array([[-40, -40, -1.5], [40, -40, -1.5], [40, 40, -1.5], [-40, 40, -1.5]], np.float32),
                         np.array([[0, 1, 2], [0, 2, 3]], np.int32))
    cube = scenes.cube_mesh(1.0)
    poses = {"c1": scenes.translation(0, 0, 5), "c2": scenes.translation(0, 6, 0), "g": scenes.translation(0, 0, 0)}
    sc = scenes.Scene([ground, cube], [scenes.Entity(1, poses["c1"], 11), scenes.Entity(1, poses["c2"], 22),
                                       scenes.Entity(0, poses["g"], 33)])
    rays = scenes.lidar_rays(16, 128)
    sensor = scenes.translation(0.25, -0.5, 1.2)
    return sc, rays, sensor, poses


def main(out_dir: str = HERE):
    sc, rays, sensor, poses = session()
    tape = Tape()
    tape.call("rgl_get_version_info", 0, 19, 0)
    mesh_ground, mesh_cube = 94_371_823_942_672, 94_371_823_947_328
    ents = {"c1": 94_371_824_011_904, "c2": 94_371_824_012_256, "g": 94_371_824_013_120}
    nodes = {k: 94_371_824_100_000 + 784 * i for i, k in enumerate(("rays", "pose", "range", "trace", "noise", "cmp", "out"))}
    g, c = sc.meshes
    tape.call("rgl_mesh_create", mesh_ground, tape.array(g.vertices), len(g.vertices), tape.array(g.indices), len(g.indices))
    tape.call("rgl_mesh_create", mesh_cube, tape.array(c.vertices), len(c.vertices), tape.array(c.indices), len(c.indices))
    for key, mesh, eid, retro in (("c1", mesh_cube, 11, None), ("c2", mesh_cube, 22, 0.5), ("g", mesh_ground, 33, None)):
        tape.call("rgl_entity_create", ents[key], 0, mesh)
        tape.call("rgl_entity_set_transform", ents[key], tape.array(poses[key]))
        tape.call("rgl_entity_set_id", ents[key], eid)
        if retro is not None:
            tape.call("rgl_entity_set_laser_retro", ents[key], f32(retro))
    tape.call("rgl_scene_set_time", 0, 1_000_000)
    tape.call("rgl_node_rays_from_mat3x4f", nodes["rays"], tape.array(rays), len(rays))
    tape.call("rgl_node_rays_transform", nodes["pose"], tape.array(sensor))
    tape.call("rgl_node_rays_set_range", nodes["range"], tape.array(np.array([[0.1, 60.0]], np.float32)), 1)
    tape.call("rgl_node_raytrace", nodes["trace"], 0)
    tape.call("rgl_node_raytrace_configure_non_hits", nodes["trace"], f32(0.0), f32(np.inf))
    tape.call("rgl_node_raytrace_configure_return_mode", nodes["trace"], RETURN_FIRST)
    tape.call("rgl_node_gaussian_noise_distance", nodes["noise"], f32(0.0), f32(0.02), f32(0.001))
    tape.call("rgl_node_points_compact_by_field", nodes["cmp"], FIELD_IS_HIT)
    fields = np.array([FIELD_XYZ, FIELD_ENTITY_ID, FIELD_DISTANCE], np.int32)
    tape.call("rgl_node_points_yield", nodes["out"], tape.array(fields), len(fields))
    chain = ("rays", "pose", "range", "trace", "noise", "cmp", "out")
    for a, b in zip(chain, chain[1:]):
        tape.call("rgl_graph_node_add_child", nodes[a], nodes[b])
    tape.call("rgl_graph_run", nodes["rays"])

    import pyoracle

    o = pyoracle.OracleScene(sc).raytrace(rays, ray_transform=sensor, ranges=[[0.1, 60.0]])
    assert int(o["ambiguous"].sum()) == 0, "pick a pose without ambiguous rays"
    count = int(o["is_hit"].sum())
    for f, size in ((FIELD_XYZ, 12), (FIELD_ENTITY_ID, 4), (FIELD_DISTANCE, 4)):
        tape.call("rgl_graph_get_result_size", nodes["out"], f, count, size)
        tape.call("rgl_graph_get_result_data", nodes["out"], f, 281_473_391_214_592 + 65_536 * f)

    with open(os.path.join(out_dir, "reference_tape.yaml"), "w") as fh:
        fh.write("\n".join(tape.lines))
    with open(os.path.join(out_dir, "reference_tape.bin"), "wb") as fh:
        fh.write(bytes(tape.bin))
    ents_hit = {int(e): int((o["entity_id"][o["is_hit"] == 1] == e).sum()) for e in (11, 22, 33)}
    with open(os.path.join(out_dir, "reference_tape.json"), "w") as fh:
        json.dump({"hit_points": count, "hits_per_entity": ents_hit}, fh, indent=1)
        fh.write("\n")
    print("reference tape:", len(tape.lines), "calls,", len(tape.bin), "binary bytes,", count, "hit points", ents_hit)


if __name__ == "__main__":
    main(*sys.argv[1:2])
