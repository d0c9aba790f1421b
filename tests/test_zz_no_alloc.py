"""The allocation-free compaction entry point, checked against the graph API's compaction.

rgl_gb300_compact_by_flags_noalloc is for callers that cannot allocate device memory while they run:
engines that hand the library only buffers from their own pre-allocated pool, and real-time loops that
must not enter the CUDA allocator. Its look-back scratch is a fixed array inside the library. This
test calls it through the C ABI on device buffers owned by the caller, twice in a row with different
sizes (a smaller second call would expose scratch left over from the first), and checks each result bit
for bit against the same compaction done by the existing entry points (rgl_node_points_from_array ->
rgl_node_points_compact_by_field -> rgl_graph_get_result_data). Compaction is integer work, so the
comparison is exact, as in the other compaction tests. Further cases compare it bit for bit with a
NumPy boolean-mask compaction: 1- and 3-byte elements and buffers offset by one byte (the byte-wise
copy path), all flags clear, all flags set, a single element and an empty call.

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
    import torch

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


def noalloc_bytes(rgl, flags, data, elem, offset):
    """Runs the entry point on device copies of `flags` and `data` (count x elem bytes) placed
    `offset` bytes into caller-owned buffers; returns the kept count and the kept bytes."""
    import torch

    n = len(flags)
    d_flags = torch.from_numpy(np.ascontiguousarray(flags, np.int32)).cuda()
    d_src = torch.zeros(n * elem + offset + 16, dtype=torch.uint8, device="cuda")
    d_dst = torch.full((n * elem + offset + 16,), 0xAB, dtype=torch.uint8, device="cuda")
    if n:
        d_src[offset:offset + n * elem] = torch.from_numpy(np.ascontiguousarray(data, np.uint8).reshape(-1)).cuda()
    torch.cuda.synchronize()
    kept = C.c_int32(-1)
    rgl.check(rgl.lib().rgl_gb300_compact_by_flags_noalloc(C.c_void_p(d_flags.data_ptr()), C.c_void_p(d_src.data_ptr() + offset), n,
                                                           elem, C.c_void_p(d_dst.data_ptr() + offset), C.byref(kept), None))
    out = d_dst.cpu().numpy()
    # Nothing outside the kept elements' bytes is written.
    assert (out[:offset] == 0xAB).all() and (out[offset + kept.value * elem:] == 0xAB).all()
    return kept.value, out[offset:offset + kept.value * elem]


@pytest.mark.parametrize("n,elem,offset,kind", [(4099, 1, 0, "random"), (100_000, 3, 0, "random"), (5000, 12, 1, "random"),
                                                (33_000, 8, 0, "none"), (33_000, 4, 0, "all"), (1, 12, 0, "all"),
                                                (1, 5, 1, "none"), (0, 12, 0, "random")])
def test_noalloc_compaction_matches_boolean_mask(rgl, n, elem, offset, kind):
    rng = np.random.default_rng(n + elem + offset)
    flags = {"random": rng.integers(0, 2, n), "none": np.zeros(n), "all": rng.integers(1, 1 << 30, n)}[kind].astype(np.int32)
    data = rng.integers(0, 256, (n, elem), dtype=np.uint8)
    for _ in range(2):
        kept, got = noalloc_bytes(rgl, flags, data, elem, offset)
        want = data[flags != 0].reshape(-1)
        assert kept == int((flags != 0).sum())
        assert np.array_equal(got, want)


def test_noalloc_rejects_counts_beyond_its_scratch(rgl):
    kept = C.c_int32()
    status = rgl.lib().rgl_gb300_compact_by_flags_noalloc(None, None, MAX_COUNT + 1, 4, None, C.byref(kept), None)
    assert status == rgl.RGL_INVALID_ARGUMENT
    assert str(MAX_COUNT) in rgl.last_error()
