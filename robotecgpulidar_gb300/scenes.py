"""Deterministic synthetic scenes and lidar ray patterns for the lidar ray-casting workloads.

Every generator is seeded, so the GPU path, the CPU oracle and the benchmarks see identical inputs.
The shapes follow the workloads this engine is measured on:

* ``plain_scene``: one entity = a 100x100-cell terrain heightfield (20,000 triangles) spanning
  200x200 m with heights U[0, 0.5] m, plus 64 axis-aligned boxes (12 triangles each, sides
  U[1, 4] m, centres uniform over the terrain, resting on z = 0) -> 20,768 triangles.
* ``million_scene``: a 512x512-cell heightfield (524,288 triangles, 4-octave value noise of
  amplitude 3 m over 512x512 m), 8 subdivision-4 icospheres (5,120 triangles each, vertices jittered
  radially by U[-10%, 10%]) and 93 entities of those meshes with random rigid poses and uniform scale
  U[0.5, 5] -> 1,000,448 triangles.
* ``lidar_rays``: channels x azimuth steps ray poses; a ray pose maps local +Z to
  (cos e cos a, cos e sin a, sin e) in a Z-up world.
* ``solid_state_rays``: a rows x columns grid of directions over +-60 deg azimuth x +-12.5 deg
  elevation (a solid-state lidar).
* ``sensor_rig``: sensors with patterns drawn uniformly from 16x1800, 32x1024, 64x2048, 128x2048
  and the 120x640 solid-state grid, posed uniformly over the terrain at 1-3 m above the ground.
* ``repose``: new random poses for a fraction of a scene's posed entities (one animation frame).
* ``serving_scene``: a scene built like ``million_scene`` scaled to a triangle budget: half of it a
  value-noise heightfield, half icosphere instances, extent growing with the square root of the size.
* ``robot_fleet``: robots with a lidar pattern each (ray count log-uniform in [10k, 1M]), a home
  scene and a home pose.

Ray poses and transforms are fp32 3x4 row-major matrices (``rgl_mat3x4f``).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

__all__ = [
    "Mesh",
    "Entity",
    "Scene",
    "cube_mesh",
    "box_mesh",
    "terrain_mesh",
    "icosphere_mesh",
    "translation",
    "rotation_xyz",
    "trs",
    "lidar_rays",
    "solid_state_rays",
    "grid_rays",
    "SENSOR_PATTERNS",
    "Sensor",
    "sensor_rig",
    "repose",
    "serving_scene",
    "robot_fleet",
    "plain_scene",
    "million_scene",
]


@dataclass
class Mesh:
    vertices: np.ndarray  # (V, 3) float32
    indices: np.ndarray  # (T, 3) int32

    @property
    def triangle_count(self) -> int:
        return int(self.indices.shape[0])


@dataclass
class Entity:
    mesh: int
    transform: np.ndarray  # (3, 4) float32
    entity_id: int


@dataclass
class Scene:
    meshes: list = field(default_factory=list)
    entities: list = field(default_factory=list)
    # Heightfield of the terrain, when the scene has one: (heights (n+1, n+1), extent in metres).
    heightfield: tuple = None

    def ground_height(self, x: float, y: float) -> float:
        """Bilinear height of the terrain heightfield at (x, y) (0 without a heightfield)."""
        if self.heightfield is None:
            return 0.0
        h, extent = self.heightfield
        n = h.shape[0] - 1
        u = min(max((x / extent + 0.5) * n, 0.0), n - 1e-6)
        v = min(max((y / extent + 0.5) * n, 0.0), n - 1e-6)
        i, j = int(u), int(v)
        fu, fv = u - i, v - j
        return float((h[j, i] * (1 - fu) + h[j, i + 1] * fu) * (1 - fv) + (h[j + 1, i] * (1 - fu) + h[j + 1, i + 1] * fu) * fv)

    @property
    def triangle_count(self) -> int:
        return sum(self.meshes[e.mesh].triangle_count for e in self.entities)


def translation(x: float, y: float, z: float) -> np.ndarray:
    m = np.zeros((3, 4), dtype=np.float32)
    m[0, 0] = m[1, 1] = m[2, 2] = 1.0
    m[:, 3] = (x, y, z)
    return m


def rotation_xyz(rx: float, ry: float, rz: float) -> np.ndarray:
    """Rz(rz) @ Ry(ry) @ Rx(rx) (radians), computed in float64 and rounded to float32."""
    cx, sx, cy, sy, cz, sz = math.cos(rx), math.sin(rx), math.cos(ry), math.sin(ry), math.cos(rz), math.sin(rz)
    rxm = np.array([[1, 0, 0], [0, cx, -sx], [0, sx, cx]])
    rym = np.array([[cy, 0, sy], [0, 1, 0], [-sy, 0, cy]])
    rzm = np.array([[cz, -sz, 0], [sz, cz, 0], [0, 0, 1]])
    m = np.zeros((3, 4), dtype=np.float64)
    m[:, :3] = rzm @ rym @ rxm
    return m.astype(np.float32)


def trs(t=(0.0, 0.0, 0.0), r=(0.0, 0.0, 0.0), s=(1.0, 1.0, 1.0)) -> np.ndarray:
    """Translation @ rotation (radians, Rz Ry Rx) @ scale, float32."""
    m = rotation_xyz(*r).astype(np.float64)
    m[:, :3] = m[:, :3] @ np.diag(s)
    m[:, 3] = t
    return m.astype(np.float32)


def cube_mesh(half: float = 1.0) -> Mesh:
    """Axis-aligned cube [-half, half]^3, 8 vertices and 12 triangles wound outward."""
    h = half
    v = np.array(
        [[-h, -h, -h], [h, -h, -h], [h, h, -h], [-h, h, -h], [-h, -h, h], [h, -h, h], [h, h, h], [-h, h, h]],
        dtype=np.float32,
    )
    i = np.array(
        [
            [0, 3, 1], [3, 2, 1],  # z-
            [1, 2, 5], [2, 6, 5],  # x+
            [5, 6, 4], [6, 7, 4],  # z+
            [4, 7, 0], [7, 3, 0],  # x-
            [3, 7, 2], [7, 6, 2],  # y+
            [4, 0, 5], [0, 1, 5],  # y-
        ],
        dtype=np.int32,
    )
    return Mesh(v, i)


def box_mesh(center, size) -> Mesh:
    c = cube_mesh(0.5)
    v = c.vertices.astype(np.float64) * np.asarray(size, dtype=np.float64) + np.asarray(center, dtype=np.float64)
    return Mesh(v.astype(np.float32), c.indices.copy())


def terrain_mesh(cells_x: int, cells_y: int, extent_x: float, extent_y: float, heights: np.ndarray) -> Mesh:
    """Heightfield centred on the origin; heights has shape (cells_y+1, cells_x+1)."""
    xs = np.linspace(-extent_x / 2, extent_x / 2, cells_x + 1)
    ys = np.linspace(-extent_y / 2, extent_y / 2, cells_y + 1)
    gx, gy = np.meshgrid(xs, ys)
    v = np.stack([gx.ravel(), gy.ravel(), heights.ravel()], axis=1).astype(np.float32)
    r = np.arange(cells_y)[:, None]
    c = np.arange(cells_x)[None, :]
    v00 = (r * (cells_x + 1) + c).ravel()
    v10 = v00 + 1
    v01 = v00 + (cells_x + 1)
    v11 = v01 + 1
    t0 = np.stack([v00, v10, v11], axis=1)
    t1 = np.stack([v00, v11, v01], axis=1)
    idx = np.empty((2 * t0.shape[0], 3), dtype=np.int32)
    idx[0::2] = t0
    idx[1::2] = t1
    return Mesh(v, idx)


def _value_noise(n: int, octaves: int, amplitude: float, rng: np.random.Generator) -> np.ndarray:
    """Sum of `octaves` bilinear value-noise layers on an (n+1)^2 grid, scaled to [0, amplitude]."""
    out = np.zeros((n + 1, n + 1))
    amp = 1.0
    for o in range(octaves):
        cells = 4 * (2**o)
        lattice = rng.random((cells + 1, cells + 1))
        u = np.linspace(0, cells, n + 1)
        i0 = np.minimum(np.floor(u).astype(int), cells - 1)
        f = u - i0
        f = f * f * (3 - 2 * f)
        a = lattice[np.ix_(i0, i0)]
        b = lattice[np.ix_(i0, i0 + 1)]
        c = lattice[np.ix_(i0 + 1, i0)]
        d = lattice[np.ix_(i0 + 1, i0 + 1)]
        fy = f[:, None]
        fx = f[None, :]
        out += amp * ((a * (1 - fx) + b * fx) * (1 - fy) + (c * (1 - fx) + d * fx) * fy)
        amp *= 0.5
    out -= out.min()
    out *= amplitude / max(out.max(), 1e-12)
    return out


def icosphere_mesh(subdivisions: int, jitter: float, rng: np.random.Generator) -> Mesh:
    """Unit icosphere subdivided `subdivisions` times (20 * 4^s triangles), radially jittered."""
    t = (1.0 + 5.0**0.5) / 2.0
    verts = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
             (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    verts = [np.array(v, dtype=np.float64) / np.linalg.norm(v) for v in verts]
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2), (10, 7, 6),
             (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10),
             (8, 6, 7), (9, 8, 1)]
    for _ in range(subdivisions):
        cache = {}

        def mid(a, b):
            key = (min(a, b), max(a, b))
            if key not in cache:
                m = verts[a] + verts[b]
                verts.append(m / np.linalg.norm(m))
                cache[key] = len(verts) - 1
            return cache[key]

        nf = []
        for a, b, c in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = nf
    v = np.array(verts)
    v *= (1.0 + rng.uniform(-jitter, jitter, size=(len(v), 1)))
    return Mesh(v.astype(np.float32), np.array(faces, dtype=np.int32))


def lidar_rays(channels: int, azimuths: int, elev_min_deg: float = -25.0, elev_max_deg: float = 15.0) -> np.ndarray:
    """(channels*azimuths, 3, 4) float32 ray poses, azimuth-major (all channels of one azimuth step
    are consecutive). Local +Z maps to (cos e cos a, cos e sin a, sin e)."""
    e = np.deg2rad(np.linspace(elev_min_deg, elev_max_deg, channels)) if channels > 1 else np.array([np.deg2rad(elev_min_deg)])
    a = np.deg2rad(np.arange(azimuths) * (360.0 / azimuths))
    A, E = np.meshgrid(a, e, indexing="ij")
    A = A.ravel()
    E = E.ravel()
    # R = Rz(a) @ Ry(pi/2 - e)
    th = np.pi / 2 - E
    ct, st, ca, sa = np.cos(th), np.sin(th), np.cos(A), np.sin(A)
    m = np.zeros((A.size, 3, 4))
    m[:, 0, 0] = ca * ct
    m[:, 0, 1] = -sa
    m[:, 0, 2] = ca * st
    m[:, 1, 0] = sa * ct
    m[:, 1, 1] = ca
    m[:, 1, 2] = sa * st
    m[:, 2, 0] = -st
    m[:, 2, 1] = 0.0
    m[:, 2, 2] = ct
    return m.astype(np.float32)


def _direction_poses(A: np.ndarray, E: np.ndarray) -> np.ndarray:
    """Ray poses R = Rz(a) @ Ry(pi/2 - e): local +Z -> (cos e cos a, cos e sin a, sin e)."""
    th = np.pi / 2 - E
    ct, st, ca, sa = np.cos(th), np.sin(th), np.cos(A), np.sin(A)
    m = np.zeros((A.size, 3, 4))
    m[:, 0, 0] = ca * ct
    m[:, 0, 1] = -sa
    m[:, 0, 2] = ca * st
    m[:, 1, 0] = sa * ct
    m[:, 1, 1] = ca
    m[:, 1, 2] = sa * st
    m[:, 2, 0] = -st
    m[:, 2, 2] = ct
    return m.astype(np.float32)


def solid_state_rays(rows: int = 120, cols: int = 640, h_fov_deg: float = 120.0, v_fov_deg: float = 25.0) -> np.ndarray:
    """(rows*cols, 3, 4) ray poses on a grid over +-h_fov/2 azimuth x +-v_fov/2 elevation, row-major
    (all columns of one elevation row are consecutive)."""
    e = np.deg2rad(np.linspace(-v_fov_deg / 2, v_fov_deg / 2, rows))
    a = np.deg2rad(np.linspace(-h_fov_deg / 2, h_fov_deg / 2, cols))
    E, A = np.meshgrid(e, a, indexing="ij")
    return _direction_poses(A.ravel(), E.ravel())


# Sensor patterns of the multi-sensor workload: (channels, azimuth steps) of a spinning lidar, or
# ("grid", rows, columns) of a solid-state one.
SENSOR_PATTERNS = [(16, 1800), (32, 1024), (64, 2048), (128, 2048), ("grid", 120, 640)]


@dataclass
class Sensor:
    pattern: tuple
    pose: np.ndarray  # (3, 4) float32 sensor-to-world

    def rays(self) -> np.ndarray:
        if self.pattern[0] == "grid":
            return solid_state_rays(self.pattern[1], self.pattern[2])
        return lidar_rays(self.pattern[0], self.pattern[1])

    @property
    def beam_count(self) -> int:
        return self.pattern[1] * self.pattern[2] if self.pattern[0] == "grid" else self.pattern[0] * self.pattern[1]


def sensor_rig(scene: Scene, count: int = 64, seed: int = 4, margin: float = 0.45) -> list:
    """`count` sensors, pattern uniform over SENSOR_PATTERNS, position uniform over the middle
    (2*margin)^2 of the terrain at 1-3 m above the ground, yaw uniform."""
    rng = np.random.default_rng(seed)
    extent = scene.heightfield[1] if scene.heightfield is not None else 200.0
    out = []
    for _ in range(count):
        pattern = SENSOR_PATTERNS[int(rng.integers(0, len(SENSOR_PATTERNS)))]
        x, y = rng.uniform(-margin * extent, margin * extent, size=2)
        z = scene.ground_height(x, y) + rng.uniform(1.0, 3.0)
        yaw = rng.uniform(-np.pi, np.pi)
        out.append(Sensor(pattern, trs((x, y, z), (0.0, 0.0, yaw))))
    return out


def repose(scene: Scene, fraction: float, rng: np.random.Generator, extent: float = None) -> list:
    """New random rigid poses (scale kept) for `fraction` of the scene's entities other than entity 0
    (the terrain); returns [(entity index, new transform)] and updates scene.entities."""
    if extent is None:
        extent = scene.heightfield[1] if scene.heightfield is not None else 200.0
    movable = list(range(1, len(scene.entities)))
    k = int(round(fraction * len(movable)))
    picked = rng.choice(movable, size=k, replace=False) if k > 0 else []
    out = []
    for i in picked:
        e = scene.entities[int(i)]
        scale = float(np.linalg.norm(e.transform[:, 0].astype(np.float64)))
        x, y = rng.uniform(-0.4 * extent, 0.4 * extent, size=2)
        rot = rng.uniform(-np.pi, np.pi, size=3)
        tf = trs((x, y, scale + 1.0), rot, (scale, scale, scale))
        scene.entities[int(i)] = Entity(e.mesh, tf, e.entity_id)
        out.append((int(i), tf))
    return out


def grid_rays(min_xy, max_xy, count_xy) -> np.ndarray:
    """Grid of parallel rays along +Z (translations only)."""
    sx = (max_xy[0] - min_xy[0]) / (count_xy[0] + 1)
    sy = (max_xy[1] - min_xy[1]) / (count_xy[1] + 1)
    out = []
    for y in range(1, count_xy[1] + 1):
        for x in range(1, count_xy[0] + 1):
            out.append(translation(min_xy[0] + sx * x, min_xy[1] + sy * y, 0.0))
    return np.stack(out).astype(np.float32)


def _merge(meshes) -> Mesh:
    vs, ids, off = [], [], 0
    for m in meshes:
        vs.append(m.vertices)
        ids.append(m.indices + off)
        off += m.vertices.shape[0]
    return Mesh(np.concatenate(vs).astype(np.float32), np.concatenate(ids).astype(np.int32))


def plain_scene(seed: int = 0, entity_id: int = 1) -> Scene:
    """Terrain (100x100 cells, 200x200 m, heights U[0,0.5]) + 64 boxes merged into one entity."""
    rng = np.random.default_rng(seed)
    heights = rng.uniform(0.0, 0.5, size=(101, 101))
    terrain = terrain_mesh(100, 100, 200.0, 200.0, heights)
    boxes = []
    for _ in range(64):
        size = rng.uniform(1.0, 4.0, size=3)
        cx, cy = rng.uniform(-100.0, 100.0, size=2)
        boxes.append(box_mesh((cx, cy, size[2] / 2.0), size))
    mesh = _merge([terrain] + boxes)
    s = Scene()
    s.meshes.append(mesh)
    s.entities.append(Entity(0, translation(0, 0, 0), entity_id))
    return s


def million_scene(seed: int = 2, instances: int = 93, spheres: int = 8, cells: int = 512, extent: float = 512.0) -> Scene:
    """1,000,448-triangle scene: value-noise terrain + `instances` posed icospheres (entity ids:
    terrain 1, instances 2..instances+1)."""
    rng = np.random.default_rng(seed)
    heights = _value_noise(cells, 4, 3.0, rng)
    s = Scene()
    s.heightfield = (heights, extent)
    s.meshes.append(terrain_mesh(cells, cells, extent, extent, heights))
    srng = np.random.default_rng(seed + 1)
    for _ in range(spheres):
        s.meshes.append(icosphere_mesh(4, 0.10, srng))
    s.entities.append(Entity(0, translation(0, 0, 0), 1))
    prng = np.random.default_rng(seed + 2)
    for k in range(instances):
        mesh = 1 + int(prng.integers(0, spheres))
        scale = float(prng.uniform(0.5, 5.0))
        x, y = prng.uniform(-0.4 * extent, 0.4 * extent, size=2)
        rot = prng.uniform(-np.pi, np.pi, size=3)
        s.entities.append(Entity(mesh, trs((x, y, scale + 1.0), rot, (scale, scale, scale)), 2 + k))
    return s


def serving_scene(triangles: int, seed: int) -> Scene:
    """About `triangles` triangles: a square heightfield of triangles/2 and triangles/2 / 5,120
    icosphere instances over 8 meshes; extent 512 m x sqrt(triangles / 1M)."""
    cells = max(16, int(round(math.sqrt(triangles / 4.0))))
    instances = max(1, int(round(triangles / 2.0 / 5120.0)))
    extent = 512.0 * math.sqrt(triangles / 1.0e6)
    return million_scene(seed=seed, instances=instances, spheres=8, cells=cells, extent=extent)


@dataclass
class Robot:
    pattern: tuple  # (channels, azimuth steps)
    scene: int
    pose: np.ndarray

    @property
    def rays(self) -> int:
        return self.pattern[0] * self.pattern[1]


def robot_fleet(scene_list, count: int = 256, seed: int = 5, min_rays: int = 10_000, max_rays: int = 1_000_000) -> list:
    """`count` robots: ray count log-uniform in [min_rays, max_rays] as channels x azimuth steps
    (16, 32, 64 or 128 channels by size), a uniformly drawn home scene and a pose 1-3 m above its
    ground."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        n = math.exp(rng.uniform(math.log(min_rays), math.log(max_rays)))
        ch = 16 if n < 40_000 else 32 if n < 150_000 else 64 if n < 500_000 else 128
        az = max(1, int(round(n / ch)))
        k = int(rng.integers(0, len(scene_list)))
        sc = scene_list[k]
        extent = sc.heightfield[1]
        x, y = rng.uniform(-0.4 * extent, 0.4 * extent, size=2)
        z = sc.ground_height(x, y) + rng.uniform(1.0, 3.0)
        out.append(Robot((ch, az), k, trs((x, y, z), (0.0, 0.0, rng.uniform(-np.pi, np.pi)))))
    return out
