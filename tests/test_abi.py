"""CPU tests of the drop-in boundary: libRobotecGPULidar.so loads and exports exactly the C functions
the public headers declare (reference include/rgl/api/core.h:526-1198 plus this build's extension
header). No API function is called, so no GPU is needed."""
import ctypes
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADERS = [os.path.join(ROOT, "include", "rgl", "api", "core.h"),
           os.path.join(ROOT, "include", "rgl", "api", "extensions", "tape.h"),
           os.path.join(ROOT, "include", "rgl", "api", "extensions", "gb300.h")]
REFERENCE_CORE_FUNCTION_COUNT = 60  # functions declared by the reference core.h


def declared():
    names = []
    for h in HEADERS:
        names += re.findall(r"RGL_API\s+[\w]+\s*\**\s*(rgl_\w+)\s*\(", open(h).read())
    return sorted(set(names))


@pytest.fixture(scope="module")
def library():
    from robotecgpulidar_gb300 import build, rgl

    if not os.path.exists(rgl.LIB_PATH):
        build.build()
    return rgl.LIB_PATH


def test_headers_declare_reference_api():
    core = re.findall(r"RGL_API\s+[\w]+\s*\**\s*(rgl_\w+)\s*\(", open(HEADERS[0]).read())
    assert len(core) == REFERENCE_CORE_FUNCTION_COUNT
    for must in ["rgl_mesh_create", "rgl_entity_create", "rgl_entity_set_transform", "rgl_node_rays_from_mat3x4f",
                 "rgl_node_raytrace", "rgl_node_gaussian_noise_distance", "rgl_node_points_compact_by_field",
                 "rgl_node_points_transform", "rgl_node_points_format", "rgl_graph_run", "rgl_graph_get_result_data"]:
        assert must in core


def test_library_exports_every_declared_symbol(library):
    lib = ctypes.CDLL(library)
    missing = [n for n in declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_library_exports_nothing_else(library):
    out = subprocess.run(["nm", "-D", "--defined-only", library], capture_output=True, text=True, check=True).stdout
    exported = sorted({l.split()[-1] for l in out.splitlines() if l.split() and l.split()[-1].startswith("rgl_")})
    assert exported == declared()
    others = [l.split()[-1] for l in out.splitlines() if l.split() and not l.split()[-1].startswith(("rgl_", "_"))]
    assert not [o for o in others if "rgl" in o.lower()], others


def test_enum_values_match_reference_layout():
    from robotecgpulidar_gb300 import rgl

    assert rgl.RGL_FIELD_PADDING_8 == 1024 and rgl.RGL_FIELD_DYNAMIC_FORMAT == 13842
    assert rgl.RGL_RETURN_FIRST_LAST == (2 << 24) | 4 | (2 << 8)
    assert rgl.RGL_NOT_IMPLEMENTED == 404 and rgl.RGL_INTERNAL_EXCEPTION == 500
    text = open(HEADERS[0]).read()
    assert "RGL_DEFAULT_ENTITY_ID 268435455" in text and "RGL_VERSION_MINOR 19" in text
