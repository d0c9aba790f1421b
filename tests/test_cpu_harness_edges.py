"""Traversal completeness where the conservative child boxes are tightest, against a brute-force FP64
caster, on the CPU (tests/cpp/bvh_harness.cpp runs the library's build, quantisation and traversal).

The quantised child boxes are not widened beyond outward rounding to whole grid steps; the traversal
covers its own plane-evaluation error with a small slack. These scenes aim at the cases that bound:
  * axis-aligned ground, walls and boxes, whose triangles lie exactly on child box planes (flat
    slabs), including boxes 1 cm thick;
  * every coordinate offset by about 1e4 m, so node origins are far larger than child extents, both
    baked into identity instances and carried by instance transforms (a translation, and a
    translation with an exact quarter turn);
  * grazing rays (0.02 to 3 degrees over the ground) and rays within 1e-6 rad of an axis, cast from
    next to the geometry and from 300 m away.
A ray counts as clear when the FP64 hit point lies inside its triangle by more than the FP32 path's
resolution at that distance and angle (20 u of the distances involved, divided by the grazing sine),
with no second surface at the same depth; a clear miss passes no triangle within that margin. Clear
rays must agree exactly (hit or miss, instance, triangle) and clear hits within 1e-5 relative
distance. No ambiguity band around box boundaries is granted: a box-culling loss on a clear ray is a
failure."""
import ctypes as C

import numpy as np
import pytest

from robotecgpulidar_gb300 import scenes

import test_cpu_harness as H

U = 2.0 ** -24
OFFSET = np.array([10000.0, -10000.0, 2000.0])


def quad_grid(x0, y0, z, n, cell):
    """Axis-aligned n x n grid of cell-sized quads at height z (two triangles each)."""
    xs = x0 + cell * np.arange(n + 1)
    ys = y0 + cell * np.arange(n + 1)
    v = np.array([(x, y, z) for y in ys for x in xs], np.float64)
    idx = []
    for j in range(n):
        for i in range(n):
            a = j * (n + 1) + i
            idx += [(a, a + 1, a + n + 2), (a, a + n + 2, a + n + 1)]
    return v, np.array(idx, np.int32)


def box(lo, hi):
    """Axis-aligned box [lo, hi] as 12 triangles."""
    (x0, y0, z0), (x1, y1, z1) = lo, hi
    v = np.array([(x0, y0, z0), (x1, y0, z0), (x1, y1, z0), (x0, y1, z0), (x0, y0, z1), (x1, y0, z1), (x1, y1, z1), (x0, y1, z1)])
    i = np.array([[0, 3, 1], [3, 2, 1], [4, 5, 7], [5, 6, 7], [0, 1, 4], [1, 5, 4], [2, 3, 6], [3, 7, 6], [0, 4, 3], [4, 7, 3],
                  [1, 2, 5], [2, 6, 5]], np.int32)
    return v, i


def merge(parts):
    vs, ids, base = [], [], 0
    for v, i in parts:
        vs.append(v)
        ids.append(i + base)
        base += len(v)
    return np.concatenate(vs), np.concatenate(ids)


def local_geometry(rng):
    """Ground (200 x 200 m, 10 m cells), four walls and 40 boxes, around the local origin."""
    parts = [quad_grid(-100.0, -100.0, 0.0, 20, 10.0)]
    quad = np.array([[0, 1, 2], [0, 2, 3]], np.int32)
    for c in (-60.0, 45.0):  # walls in x = const and y = const planes, 20 m long, 6 m high
        parts.append((np.array([(c, -10.0, 0.0), (c, 10.0, 0.0), (c, 10.0, 6.0), (c, -10.0, 6.0)]), quad))
        parts.append((np.array([(-10.0, c, 0.0), (10.0, c, 0.0), (10.0, c, 6.0), (-10.0, c, 6.0)]), quad))
    for k in range(40):
        c = rng.uniform(-90.0, 90.0, 2)
        size = rng.choice([0.01, 0.5, 2.0, 5.0], 3)
        lo = (np.round(c[0], 2), np.round(c[1], 2), 0.0)
        parts.append(box(lo, (lo[0] + size[0], lo[1] + size[1], size[2])))
    return merge(parts)


def make_scene(kind, rng):
    v, i = local_geometry(rng)
    if kind == "baked":
        mesh = scenes.Mesh((v + OFFSET).astype(np.float32), i)
        tf = scenes.translation(0.0, 0.0, 0.0)
    else:
        mesh = scenes.Mesh(v.astype(np.float32), i)
        tf = scenes.translation(*OFFSET)
        if kind == "quarter_turn":
            tf[:, :3] = np.array([[0, -1, 0], [1, 0, 0], [0, 0, 1]], np.float32)
    sc = scenes.Scene([mesh], [scenes.Entity(0, tf, 5)])
    return sc


def world_triangles(sc):
    e = sc.entities[0]
    m = sc.meshes[e.mesh]
    tf = e.transform.astype(np.float64)
    w = m.vertices.astype(np.float64) @ tf[:, :3].T + tf[:, 3]
    return w[m.indices]  # (T, 3, 3)


def make_rays(rng, n):
    """Origins 1.5 m over the ground near its middle, and 300 m away at 50 m height; grazing and
    nearly axis-parallel directions (FP32 values, as the harness receives them)."""
    near = OFFSET + np.column_stack([rng.uniform(-30, 30, n), rng.uniform(-30, 30, n), np.full(n, 1.5)])
    far = OFFSET + np.column_stack([np.full(n, -300.0), rng.uniform(-50, 50, n), np.full(n, 50.0)])
    o = np.concatenate([near, far])
    az = rng.uniform(-np.pi, np.pi, 2 * n)
    axis = rng.random(2 * n) < 0.4
    az[axis] = rng.integers(0, 4, axis.sum()) * (np.pi / 2) + rng.choice([0.0, 1e-6, -1e-6, 3e-7], axis.sum())
    el = -np.radians(np.exp(rng.uniform(np.log(0.02), np.log(3.0), 2 * n)))
    el[n:] = -np.radians(rng.uniform(0.02, 12.0, n))  # from 50 m height, reaching the scene 240-400 m away
    az[n:] = rng.uniform(-0.3, 0.3, n)
    d = np.column_stack([np.cos(el) * np.cos(az), np.cos(el) * np.sin(az), np.sin(el)])
    return o.astype(np.float32), d.astype(np.float32)


def brute_force(tris, o, d, tmax):
    """FP64 closest hit per ray over all triangles, with the clearance classification described above.
    Returns (t, triangle index or -1, clear flag)."""
    o, d = o.astype(np.float64), d.astype(np.float64)
    a, b, c = tris[:, 0], tris[:, 1], tris[:, 2]
    e1, e2 = b - a, c - a
    n = np.cross(e1, e2)
    area2 = np.linalg.norm(n, axis=1)
    el = [np.linalg.norm(c - b, axis=1), np.linalg.norm(a - c, axis=1), np.linalg.norm(b - a, axis=1)]
    T = np.full(len(o), np.inf)
    tri = np.full(len(o), -1)
    clear = np.zeros(len(o), bool)
    for k in range(len(o)):
        dk, ok = d[k], o[k]
        dl = np.linalg.norm(dk)
        den = n @ dk
        with np.errstate(divide="ignore", invalid="ignore"):
            t = (n * (a - ok)).sum(1) / den
            p = ok + t[:, None] * dk
            w0 = (np.cross(b - p, c - p) * n).sum(1) / area2  # signed twice-areas over |n|
            w1 = (np.cross(c - p, a - p) * n).sum(1) / area2
            w2 = (np.cross(a - p, b - p) * n).sum(1) / area2
            # in-plane distance of p inside (>0) or outside (<0) each edge
            dist_in = np.minimum(np.minimum(w0 / el[0], w1 / el[1]), w2 / el[2])
            sine = np.abs(den) / (area2 * dl)
        scale = 20.0 * U * (np.abs(t) * dl + np.linalg.norm(ok - OFFSET) + np.linalg.norm(OFFSET) * 1e-3 + 1.0)
        tol = scale / np.maximum(sine, 1e-4)
        valid = np.isfinite(t) & (t > 0) & (t <= tmax) & (area2 > 0)
        inside = valid & (dist_in > tol)
        near = valid & (dist_in > -tol)
        if not near.any():
            clear[k] = True  # a clear miss
            continue
        hit = valid & (dist_in >= 0)
        if not hit.any():
            continue  # passes close to a triangle without a clear hit
        j = int(np.argmin(np.where(hit, t, np.inf)))
        T[k], tri[k] = t[j], j
        others = near.copy()
        others[j] = False
        clear[k] = inside[j] and not (others & (t <= t[j] * (1 + 1e-5) + tol[j] / dl)).any()
    return T, tri, clear


@pytest.mark.parametrize("kind", ["baked", "translated", "quarter_turn"])
def test_tight_boxes_lose_no_clear_hit(kind):
    h = H.load_harness()
    rng = np.random.default_rng({"baked": 1, "translated": 2, "quarter_turn": 3}[kind])
    sc = make_scene(kind, rng)
    o, d = make_rays(rng, 1500)
    tmax = 2000.0
    t, inst, prim = H.cast_world(h, sc, o, d, tmax)
    T, tri, clear = brute_force(world_triangles(sc), o, d, tmax)
    assert clear.mean() > 0.8
    hits = clear & (tri >= 0)
    assert hits.sum() > 1000 and (clear & (tri < 0)).sum() > 200
    got_hit = inst >= 0
    assert np.array_equal(got_hit[clear], tri[clear] >= 0)
    assert np.array_equal(prim[hits], tri[hits])
    rel = np.abs(t[hits].astype(np.float64) - T[hits]) / T[hits]
    assert rel.max() <= 1e-5
