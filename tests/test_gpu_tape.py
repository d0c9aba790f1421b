"""Tape recording and playback (reference src/tape/*, include/rgl/api/extensions/tape.h; format and
error cases of test/src/TapeTest.cpp:55-163): calls go to <path>.yaml (one `- fn: {t: ns, a: [...]}`
item per call, the library version first) and <path>.bin (arrays at 16-byte aligned offsets), and
playing the tape back rebuilds the recorded scene."""
import ctypes as C
import json
import os
import re
import sys

import numpy as np
import pytest

from robotecgpulidar_gb300 import scenes

pytestmark = pytest.mark.gpu

RGL_LOG_LEVEL_WARN = 3


def write(path, text):
    with open(path, "w") as f:
        f.write(text)


def play_error(rgl, base):
    st = rgl.lib().rgl_tape_play(str(base).encode())
    return st, rgl.last_error()


def test_tape_format_errors(rgl, tmp_path):
    base = tmp_path / "empty"
    write(str(base) + ".yaml", "")
    write(str(base) + ".bin", "")
    st, msg = play_error(rgl, base)
    assert st == rgl.RGL_TAPE_ERROR and "Invalid Tape: Empty YAML file detected" in msg

    base = tmp_path / "noversion"
    write(str(base) + ".yaml", "- rgl_mesh_create: {t: 0, a: [0]}\n")
    write(str(base) + ".bin", "")
    st, msg = play_error(rgl, base)
    assert st == rgl.RGL_TAPE_ERROR and "Unsupported Tape format: Missing version record in the Tape" in msg

    base = tmp_path / "old"
    write(str(base) + ".yaml", "- rgl_get_version_info: {t: 0, a: [0, 16, 2]}\n")
    write(str(base) + ".bin", "")
    st, msg = play_error(rgl, base)
    assert st == rgl.RGL_TAPE_ERROR and "Tape version is too old. Required version: 0.16.3." in msg

    base = tmp_path / "outdated"
    write(str(base) + ".yaml", "rgl_version:\n  major: 0\n  minor: 16\n  patch: 2\n")
    write(str(base) + ".bin", "")
    st, msg = play_error(rgl, base)
    assert st == rgl.RGL_TAPE_ERROR and "Unsupported Tape format: Detected outdated format" in msg

    st, msg = play_error(rgl, tmp_path / "missing")
    assert st == rgl.RGL_INVALID_FILE_PATH


def test_recording_state_errors(rgl, tmp_path):
    lib = rgl.lib()
    assert lib.rgl_tape_record_end() == rgl.RGL_TAPE_ERROR and "no recording active" in rgl.last_error()
    rgl.check(lib.rgl_tape_record_begin(str(tmp_path / "t").encode()))
    active = C.c_bool(False)
    rgl.check(lib.rgl_tape_record_is_active(C.byref(active)))
    assert active.value
    assert lib.rgl_tape_record_begin(str(tmp_path / "u").encode()) == rgl.RGL_TAPE_ERROR
    assert "recording already active" in rgl.last_error()
    assert lib.rgl_tape_play(str(tmp_path / "t").encode()) == rgl.RGL_TAPE_ERROR and "recording active" in rgl.last_error()
    rgl.check(lib.rgl_tape_record_end())
    rgl.check(lib.rgl_tape_record_is_active(C.byref(active)))
    assert not active.value


def record_session(rgl, base, log_path):
    """A plugin-like session: logging, a mesh placed twice, a sensor graph with ring ids, run, results."""
    lib = rgl.lib()
    rgl.check(lib.rgl_tape_record_begin(str(base).encode()))
    rgl.check(lib.rgl_configure_logging(rgl.RGL_LOG_LEVEL_OFF, str(log_path).encode(), False))
    cube = scenes.cube_mesh(1.0)
    m = rgl.mesh_create(cube.vertices, cube.indices)
    e1, e2 = rgl.entity_create(m), rgl.entity_create(m)
    rgl.entity_set_transform(e1, scenes.translation(0, 0, 5))
    rgl.entity_set_id(e1, 11)
    rgl.entity_set_transform(e2, scenes.translation(0, 6, 0))
    rgl.entity_set_id(e2, 22)
    rgl.check(lib.rgl_entity_set_laser_retro(e2, 0.5))
    n = {k: rgl.node() for k in ("rays", "ring", "range", "trace", "cmp", "out")}
    rays = scenes.lidar_rays(8, 64)
    rgl.rays_from_mat3x4f(n["rays"], rays)
    ids = np.arange(8, dtype=np.int32)
    rgl.check(lib.rgl_node_rays_set_ring_ids(C.byref(n["ring"]), rgl.ptr(ids), 8))
    rgl.rays_set_range(n["range"], [[0.1, 50.0]])
    rgl.raytrace(n["trace"])
    rgl.check(lib.rgl_node_raytrace_configure_return_mode(n["trace"], rgl.RGL_RETURN_FIRST))
    rgl.points_compact_by_field(n["cmp"])
    rgl.points_yield(n["out"], [rgl.RGL_FIELD_XYZ_VEC3_F32, rgl.RGL_FIELD_ENTITY_ID_I32, rgl.RGL_FIELD_RING_ID_U16])
    rgl.chain(n["rays"], n["ring"], n["range"], n["trace"], n["cmp"], n["out"])
    rgl.graph_run(n["rays"])
    ent = rgl.result(n["out"], rgl.RGL_FIELD_ENTITY_ID_I32)
    rgl.check(lib.rgl_tape_record_end())
    return ent


def probe_hits(rgl):
    """Entity ids and distances seen by two probe rays (up the +Z and +Y axes from the origin)."""
    n = {k: rgl.node() for k in ("rays", "trace", "out")}
    rgl.rays_from_mat3x4f(n["rays"], [scenes.translation(0, 0, 0), scenes.rotation_xyz(-np.pi / 2, 0, 0)])
    rgl.raytrace(n["trace"])
    rgl.points_yield(n["out"], [rgl.RGL_FIELD_ENTITY_ID_I32, rgl.RGL_FIELD_DISTANCE_F32, rgl.RGL_FIELD_LASER_RETRO_F32])
    rgl.chain(n["rays"], n["trace"], n["out"])
    rgl.graph_run(n["rays"])
    out = (rgl.result(n["out"], rgl.RGL_FIELD_ENTITY_ID_I32).tolist(), rgl.result(n["out"], rgl.RGL_FIELD_DISTANCE_F32).tolist(),
           rgl.result(n["out"], rgl.RGL_FIELD_LASER_RETRO_F32).tolist())
    rgl.check(rgl.lib().rgl_graph_destroy(n["rays"]))
    return out


def test_record_and_play_back(rgl, tmp_path):
    base = tmp_path / "session"
    ent = record_session(rgl, base, tmp_path / "rgl.log")
    assert set(ent.tolist()) <= {11, 22} and len(ent) > 0
    before = probe_hits(rgl)
    assert before[0] == [11, 22] and before[1] == [4.0, 5.0] and before[2] == [0.0, 0.5]

    lines = open(str(base) + ".yaml").read().splitlines()
    item = re.compile(r"^- (rgl_\w+): \{t: (\d+), a: \[(.*)\]\}$")
    calls = [item.match(l) for l in lines]
    assert all(calls), [l for l, c in zip(lines, calls) if not c]
    assert calls[0].group(1) == "rgl_get_version_info" and calls[0].group(3) == "0, 19, 0"
    names = [c.group(1) for c in calls]
    assert names.count("rgl_entity_create") == 2 and "rgl_graph_run" in names and "rgl_graph_get_result_data" in names
    ts = [int(c.group(2)) for c in calls]
    assert ts == sorted(ts)
    binsize = len(open(str(base) + ".bin", "rb").read())
    assert binsize % 16 == 0 and binsize > 0
    # The first entity transform stored in the binary file is the recorded matrix.
    tf_call = next(c for c in calls if c.group(1) == "rgl_entity_set_transform")
    off = int(tf_call.group(3).split(",")[1])
    data = np.frombuffer(open(str(base) + ".bin", "rb").read()[off:off + 48], np.float32).reshape(3, 4)
    assert np.array_equal(data, scenes.translation(0, 0, 5).astype(np.float32))

    rgl.check(rgl.lib().rgl_cleanup())
    assert probe_hits(rgl)[0] == [0, 0]  # empty scene after cleanup
    rgl.check(rgl.lib().rgl_tape_play(str(base).encode()))
    assert probe_hits(rgl) == before


GOLDEN_TAPE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_tape")


def test_plays_tape_in_the_reference_recorders_form(rgl, tmp_path):
    """A tape written in the reference recorder's exact form (tests/golden/make_reference_tape.py:
    yaml-cpp's block sequence of flow maps, recorded addresses as handles, enums as integers, floats
    with 9 digits and .inf, arrays at 16-byte aligned offsets of the binary file) plays back: every
    call succeeds (nothing logged at warning level or above, so the three recorded result sizes equal
    the played graph's), the scene is rebuilt with the recorded poses, ids and laser retro, and the
    same graph built by direct calls yields the recorded hit count (the oracle's) and entity mix."""
    exp = json.load(open(GOLDEN_TAPE + ".json"))
    lib = rgl.lib()
    log = tmp_path / "play.log"
    rgl.check(lib.rgl_cleanup())
    rgl.check(lib.rgl_configure_logging(RGL_LOG_LEVEL_WARN, str(log).encode(), False))
    try:
        rgl.check(lib.rgl_tape_play(GOLDEN_TAPE.encode()))
        assert probe_hits(rgl) == ([11, 22], [4.0, 5.0], [0.0, 0.5])
    finally:
        rgl.check(lib.rgl_configure_logging(rgl.RGL_LOG_LEVEL_OFF, None, False))
    text = open(log).read() if log.exists() else ""
    assert text.strip() == "", text

    sys.path.insert(0, os.path.dirname(GOLDEN_TAPE))
    import make_reference_tape as mk

    _, rays, sensor, _ = mk.session()
    n = {k: rgl.node() for k in ("rays", "pose", "range", "trace", "noise", "cmp", "out")}
    rgl.rays_from_mat3x4f(n["rays"], rays)
    rgl.rays_transform(n["pose"], sensor)
    rgl.rays_set_range(n["range"], [[0.1, 60.0]])
    rgl.raytrace(n["trace"])
    rgl.check(lib.rgl_node_raytrace_configure_return_mode(n["trace"], rgl.RGL_RETURN_FIRST))
    rgl.check(lib.rgl_node_gaussian_noise_distance(C.byref(n["noise"]), 0.0, 0.02, 0.001))
    rgl.points_compact_by_field(n["cmp"])
    rgl.points_yield(n["out"], [rgl.RGL_FIELD_XYZ_VEC3_F32, rgl.RGL_FIELD_ENTITY_ID_I32, rgl.RGL_FIELD_DISTANCE_F32])
    rgl.chain(*n.values())
    rgl.graph_run(n["rays"])
    ent = rgl.result(n["out"], rgl.RGL_FIELD_ENTITY_ID_I32)
    assert len(ent) == exp["hit_points"]
    assert {int(k): v for k, v in exp["hits_per_entity"].items()} == {e: int((ent == e).sum()) for e in (11, 22, 33)}
