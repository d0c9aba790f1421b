"""The committed reference-form tape (tests/golden/make_reference_tape.py) is what the generator
writes today, and has the reference recorder's shape: one `- fn: {t: ns, a: [...]}` item per line,
rgl_get_version_info first, increasing timestamps, and every binary offset 16-byte aligned and inside
the binary file (reference src/tape/TapeRecorder.hpp:54-151). Runs on the CPU."""
import os
import re
import subprocess
import sys

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_generator_reproduces_the_committed_tape(tmp_path):
    subprocess.run([sys.executable, os.path.join(GOLDEN, "make_reference_tape.py"), str(tmp_path)], check=True, capture_output=True)
    for ext in (".yaml", ".bin", ".json"):
        assert open(tmp_path / ("reference_tape" + ext), "rb").read() == open(os.path.join(GOLDEN, "reference_tape" + ext), "rb").read()


def test_tape_has_the_reference_shape():
    lines = open(os.path.join(GOLDEN, "reference_tape.yaml")).read().splitlines()
    binsize = os.path.getsize(os.path.join(GOLDEN, "reference_tape.bin"))
    item = re.compile(r"^- (rgl_\w+): \{t: (\d+), a: \[(.*)\]\}$")
    calls = [item.match(l) for l in lines]
    assert all(calls)
    assert calls[0].group(1) == "rgl_get_version_info" and calls[0].group(3) == "0, 19, 0"
    ts = [int(c.group(2)) for c in calls]
    assert ts == sorted(ts)
    # binary-offset arguments of the calls used, by position
    offsets = {"rgl_mesh_create": (1, 3), "rgl_entity_set_transform": (1,), "rgl_node_rays_from_mat3x4f": (1,),
               "rgl_node_rays_transform": (1,), "rgl_node_rays_set_range": (1,), "rgl_node_points_yield": (1,)}
    seen = 0
    for c in calls:
        args = [a.strip() for a in c.group(3).split(",")]
        for k in offsets.get(c.group(1), ()):
            off = int(args[k])
            assert off % 16 == 0 and off < binsize
            seen += 1
    assert seen == 11 and binsize % 16 == 0
    assert any(".inf" in c.group(3) for c in calls if c.group(1) == "rgl_node_raytrace_configure_non_hits")
    # the recorded rays are the generator's pattern, at the offset the YAML names
    rays_call = next(c for c in calls if c.group(1) == "rgl_node_rays_from_mat3x4f")
    off, n = (int(a) for a in rays_call.group(3).split(",")[1:3])
    data = np.fromfile(os.path.join(GOLDEN, "reference_tape.bin"), np.uint8)[off:off + 48 * n].view(np.float32).reshape(n, 3, 4)
    sys.path.insert(0, GOLDEN)
    import make_reference_tape as mk

    assert np.array_equal(data, mk.session()[1])
