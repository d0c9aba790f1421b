"""The allocation-free compaction entry point, checked against the graph API's compaction.

rgl_gb300_compact_by_flags_noalloc is for callers that cannot allocate device memory while they run:
engines that hand the library only buffers from their own pre-allocated pool, and real-time loops that
must not enter the CUDA allocator. Its look-back scratch is a fixed array inside the library. This
test calls it through the C ABI on device buffers owned by the caller, twice in a row with different
sizes (a smaller second call would expose scratch left over from the first), and checks each result bit
for bit against the same compaction done by the existing entry points (rgl_node_points_from_array ->
rgl_node_points_compact_by_field -> rgl_graph_get_result_data). Compaction is integer work, so the
comparison is exact, as in the other compaction tests.

The file name sorts last so that a run stopping at the first failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_COUNT = 1 << 24


def graph_compaction(rgl, hits, xyz):
    dt = np.dtype([("xyz", np.float32, 3), ("hit", np.int32)])
    a = np.zeros(len(hits), dt)
    a["xyz"] = xyz
    a["hit"] = hits
    src, cmp = rgl.node(), rgl.node()
    rgl.points_from_array(src, a, len(hits), [rgl.RGL_FIELD_XYZ_VEC3_F32, rgl.RGL_FIELD_IS_HIT_I32])
    rgl.points_compact_by_field(cmp)
    rgl.add_child(src, cmp)
    rgl.graph_run(src)
    out = rgl.result(cmp, rgl.RGL_FIELD_XYZ_VEC3_F32)
    rgl.check(rgl.lib().rgl_graph_destroy(src))
    return out


def test_noalloc_compaction_matches_graph_compaction(rgl):
    torch = pytest.importorskip("torch")
    lib = rgl.lib()
    rng = np.random.default_rng(2024)
    for n in (300_000, 70_001):
        hits = rng.integers(0, 2, n).astype(np.int32)
        xyz = rng.normal(size=(n, 3)).astype(np.float32)
        d_flags = torch.from_numpy(hits).cuda()
        d_src = torch.from_numpy(xyz).cuda()
        d_dst = torch.zeros_like(d_src)
        torch.cuda.synchronize()
        kept = C.c_int32(-1)
        rgl.check(lib.rgl_gb300_compact_by_flags_noalloc(C.c_void_p(d_flags.data_ptr()), C.c_void_p(d_src.data_ptr()), n, 12,
                                                         C.c_void_p(d_dst.data_ptr()), C.byref(kept), None))
        got = d_dst[: kept.value].cpu().numpy()
        ref = graph_compaction(rgl, hits, xyz)
        assert kept.value == int(hits.sum()) == ref.shape[0]
        assert np.array_equal(got, ref)


def test_noalloc_rejects_counts_beyond_its_scratch(rgl):
    kept = C.c_int32()
    status = rgl.lib().rgl_gb300_compact_by_flags_noalloc(None, None, MAX_COUNT + 1, 4, None, C.byref(kept), None)
    assert status == rgl.RGL_INVALID_ARGUMENT
    assert str(MAX_COUNT) in rgl.last_error()
