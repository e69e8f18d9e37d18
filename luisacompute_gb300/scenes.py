"""Seeded synthetic scenes and ray sets for the Mesh/Accel path.

Record layouts are byte-compatible with LuisaCompute:
  * ``RAY_DTYPE``  — ``Ray`` (include/luisa/runtime/rtx/ray.h:10-16), 32 B;
  * ``HIT_DTYPE``  — ``TriangleHit``/``SurfaceHit`` (include/luisa/runtime/rtx/hit.h:30-46), 24 B;
  * ``MOD_DTYPE``  — ``AccelBuildCommand::Modification`` (include/luisa/runtime/rhi/command.h:534-592), 80 B;
  * vertices are ``float3`` padded to 16 B (include/luisa/core/basic_types.h:14-18), triangles
    ``Triangle`` = 3 x uint32 (include/luisa/runtime/rtx/triangle.h:7-11).

No public dataset is involved: every workload is generated here from a seed.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

RAY_DTYPE = np.dtype([("o", "<f4", (3,)), ("tmin", "<f4"), ("d", "<f4", (3,)), ("tmax", "<f4")])
HIT_DTYPE = np.dtype([("inst", "<u4"), ("prim", "<u4"), ("bary", "<f4", (2,)), ("t", "<f4"), ("pad", "<u4")])
MOD_DTYPE = np.dtype([("index", "<u4"), ("user_id", "<u4"), ("flags", "<u4"), ("vis_mask", "<u4"),
                      ("affine", "<f4", (12,)), ("primitive", "<u8"), ("_pad", "<u8")])
assert RAY_DTYPE.itemsize == 32 and HIT_DTYPE.itemsize == 24 and MOD_DTYPE.itemsize == 80

MISS = 0xFFFFFFFF
IDENTITY = np.array([1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0], np.float32)


@dataclass
class MeshData:
    vertices: np.ndarray  # (V, 4) float32, xyz + pad (stride 16 B)
    triangles: np.ndarray  # (T, 3) uint32

    @property
    def tri_count(self) -> int:
        return int(self.triangles.shape[0])


@dataclass
class Scene:
    meshes: list
    inst_mesh: np.ndarray  # (N,) int: mesh index per instance
    inst_affine: np.ndarray  # (N, 12) float32 row-major object-to-world
    inst_mask: np.ndarray  # (N,) uint32 visibility masks
    name: str = ""
    extra: dict = field(default_factory=dict)

    @property
    def instance_count(self) -> int:
        return int(self.inst_mesh.shape[0])

    def instanced_triangles(self) -> int:
        return int(sum(self.meshes[m].tri_count for m in self.inst_mesh))

    def bounds(self):
        lo = np.full(3, np.inf)
        hi = np.full(3, -np.inf)
        for i in range(self.instance_count):
            m = self.meshes[self.inst_mesh[i]]
            if m.tri_count == 0:
                continue
            v = m.vertices[:, :3].astype(np.float64)
            a = self.inst_affine[i].astype(np.float64).reshape(3, 4)
            w = v @ a[:, :3].T + a[:, 3]
            lo = np.minimum(lo, w.min(0))
            hi = np.maximum(hi, w.max(0))
        return lo, hi


def _pad_vertices(v3: np.ndarray) -> np.ndarray:
    v = np.zeros((v3.shape[0], 4), np.float32)
    v[:, :3] = v3
    return v


_ICO_CACHE: dict = {}


def icosphere(subdiv: int, radius: float = 1.0) -> MeshData:
    """Icosahedron subdivided ``subdiv`` times: 20*4^s triangles, 10*4^s+2 vertices."""
    if radius == 1.0 and subdiv in _ICO_CACHE:
        v, f = _ICO_CACHE[subdiv]
        return MeshData(v.copy(), f.copy())
    m = _icosphere(subdiv, radius)
    if radius == 1.0:
        _ICO_CACHE[subdiv] = (m.vertices.copy(), m.triangles.copy())
    return m


def _icosphere(subdiv: int, radius: float) -> MeshData:
    t = (1.0 + 5.0 ** 0.5) / 2.0
    v = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
                  [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], np.float64)
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4], [11, 10, 2],
                  [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9], [4, 9, 5],
                  [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], np.int64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    for _ in range(subdiv):
        nv = v.shape[0]
        e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]])
        key = np.minimum(e[:, 0], e[:, 1]) * nv + np.maximum(e[:, 0], e[:, 1])
        uniq, inv = np.unique(key, return_inverse=True)
        a, b = uniq // nv, uniq % nv
        mid = v[a] + v[b]
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        v = np.concatenate([v, mid])
        m = (inv + nv).reshape(3, -1).T  # midpoints of edges (01, 12, 20) per face
        ab, bc, ca = m[:, 0], m[:, 1], m[:, 2]
        f = np.concatenate([np.stack([f[:, 0], ab, ca], 1), np.stack([f[:, 1], bc, ab], 1),
                            np.stack([f[:, 2], ca, bc], 1), np.stack([ab, bc, ca], 1)])
    return MeshData(_pad_vertices((v * radius).astype(np.float32)), f.astype(np.uint32))


def _value_noise_fbm(n: int, octaves: int, rng: np.random.Generator) -> np.ndarray:
    """fBm of bilinear value noise (smoothstep weights) on an n x n grid in [0,1]^2, result in [0,1]."""
    x = np.linspace(0.0, 1.0, n)
    out = np.zeros((n, n))
    amp, total = 1.0, 0.0
    for o in range(octaves):
        res = 4 * (2 ** o)
        lat = rng.random((res + 1, res + 1))
        g = x * res
        i0 = np.minimum(g.astype(np.int64), res - 1)
        fr = g - i0
        w = fr * fr * (3.0 - 2.0 * fr)
        a = lat[i0][:, i0]
        b = lat[i0][:, i0 + 1]
        c = lat[i0 + 1][:, i0]
        d = lat[i0 + 1][:, i0 + 1]
        wy, wx = w[:, None], w[None, :]
        out += amp * ((a * (1 - wx) + b * wx) * (1 - wy) + (c * (1 - wx) + d * wx) * wy)
        total += amp
        amp *= 0.5
    return out / total


def heightfield(n: int = 1024, octaves: int = 6, amplitude: float = 0.1, seed: int = 2) -> MeshData:
    """n x n vertex grid over [-1,1]^2 (x, z), y = fBm height; 2(n-1)^2 triangles.
    Height amplitude is ``amplitude`` times the extent (2)."""
    rng = np.random.default_rng(seed)
    h = (_value_noise_fbm(n, octaves, rng) - 0.5) * (2.0 * amplitude * 2.0)
    xs = np.linspace(-1.0, 1.0, n)
    X, Z = np.meshgrid(xs, xs, indexing="xy")
    v3 = np.stack([X.ravel(), h.ravel(), Z.ravel()], 1).astype(np.float32)
    idx = np.arange(n * n, dtype=np.int64).reshape(n, n)
    a, b, c, d = idx[:-1, :-1].ravel(), idx[:-1, 1:].ravel(), idx[1:, :-1].ravel(), idx[1:, 1:].ravel()
    tris = np.empty((2 * a.size, 3), np.int64)
    tris[0::2] = np.stack([a, c, b], 1)
    tris[1::2] = np.stack([b, c, d], 1)
    return MeshData(_pad_vertices(v3), tris.astype(np.uint32))


def grid_mesh(nx: int, ny: int) -> MeshData:
    """Flat nx x ny vertex grid over [-1,1]^2 in the xz plane: 2(nx-1)(ny-1) triangles."""
    xs, zs = np.linspace(-1.0, 1.0, nx), np.linspace(-1.0, 1.0, ny)
    X, Z = np.meshgrid(xs, zs, indexing="xy")
    v3 = np.stack([X.ravel(), np.zeros(X.size), Z.ravel()], 1).astype(np.float32)
    idx = np.arange(nx * ny, dtype=np.int64).reshape(ny, nx)
    a, b, c, d = idx[:-1, :-1].ravel(), idx[:-1, 1:].ravel(), idx[1:, :-1].ravel(), idx[1:, 1:].ravel()
    tris = np.empty((2 * a.size, 3), np.int64)
    tris[0::2] = np.stack([a, c, b], 1)
    tris[1::2] = np.stack([b, c, d], 1)
    return MeshData(_pad_vertices(v3), tris.astype(np.uint32))


def random_rotations(n: int, rng: np.random.Generator) -> np.ndarray:
    """Uniform random rotation matrices (Shoemake's quaternion method), (n, 3, 3)."""
    u1, u2, u3 = rng.random(n), rng.random(n), rng.random(n)
    q = np.stack([np.sqrt(1 - u1) * np.sin(2 * np.pi * u2), np.sqrt(1 - u1) * np.cos(2 * np.pi * u2),
                  np.sqrt(u1) * np.sin(2 * np.pi * u3), np.sqrt(u1) * np.cos(2 * np.pi * u3)], 1)
    x, y, z, w = q.T
    return np.stack([
        np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)], 1),
        np.stack([2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)], 1),
        np.stack([2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)], 1)], 1)


def affine_rows(rot: np.ndarray, scale: np.ndarray, trans: np.ndarray) -> np.ndarray:
    """Row-major 3x4 object-to-world matrices ``[s R | t]`` as (n, 12) float32."""
    m = np.zeros((rot.shape[0], 3, 4))
    m[:, :, :3] = rot * scale.reshape(-1, 1, 1)
    m[:, :, 3] = trans
    return m.reshape(-1, 12).astype(np.float32)


def camera_rays(width: int, height: int, eye=(0.0, 0.0, 3.0), target=(0.0, 0.0, 0.0), fov_deg: float = 45.0,
                seed: int = 1) -> np.ndarray:
    """Pinhole primary rays, one per pixel with uniform jitter inside the pixel; t in [0, 1e30]."""
    rng = np.random.default_rng(seed)
    eye = np.asarray(eye, np.float64)
    fwd = np.asarray(target, np.float64) - eye
    fwd /= np.linalg.norm(fwd)
    up0 = np.array([0.0, 1.0, 0.0])
    right = np.cross(fwd, up0)
    right /= np.linalg.norm(right)
    up = np.cross(right, fwd)
    th = math.tan(math.radians(fov_deg) * 0.5)
    aspect = width / height
    py, px = np.meshgrid(np.arange(height), np.arange(width), indexing="ij")
    jit = rng.random((height, width, 2))
    sx = ((px + jit[..., 0]) / width * 2.0 - 1.0) * th * aspect
    sy = (1.0 - (py + jit[..., 1]) / height * 2.0) * th
    d = fwd + sx[..., None] * right + sy[..., None] * up
    d /= np.linalg.norm(d, axis=-1, keepdims=True)
    rays = np.zeros(width * height, RAY_DTYPE)
    rays["o"] = eye.astype(np.float32)
    rays["d"] = d.reshape(-1, 3).astype(np.float32)
    rays["tmin"] = 0.0
    rays["tmax"] = 1e30
    return rays


def sphere_rays(n: int, lo, hi, seed: int) -> np.ndarray:
    """Incoherent rays: origins uniform in the box [lo, hi], directions uniform on S^2."""
    rng = np.random.default_rng(seed)
    lo, hi = np.asarray(lo, np.float64), np.asarray(hi, np.float64)
    o = lo + rng.random((n, 3)) * (hi - lo)
    d = rng.standard_normal((n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = np.zeros(n, RAY_DTYPE)
    rays["o"] = o.astype(np.float32)
    rays["d"] = d.astype(np.float32)
    rays["tmin"] = 0.0
    rays["tmax"] = 1e30
    return rays


def shadow_rays(n: int, lo, hi, light, seed: int) -> np.ndarray:
    """Rays from origins uniform in [lo, hi] toward a point light; t_max = light distance."""
    rng = np.random.default_rng(seed)
    lo, hi = np.asarray(lo, np.float64), np.asarray(hi, np.float64)
    o = lo + rng.random((n, 3)) * (hi - lo)
    v = np.asarray(light, np.float64) - o
    dist = np.linalg.norm(v, axis=1)
    rays = np.zeros(n, RAY_DTYPE)
    rays["o"] = o.astype(np.float32)
    rays["d"] = (v / dist[:, None]).astype(np.float32)
    rays["tmin"] = 0.0
    rays["tmax"] = dist.astype(np.float32)
    return rays


# ------------------------------------------------------------------ workloads
def icosphere_scene(subdiv: int = 6) -> Scene:
    """One icosphere (81,920 triangles at subdiv 6), one identity instance."""
    return Scene([icosphere(subdiv)], np.zeros(1, np.int64), IDENTITY[None, :].copy(),
                 np.full(1, 0xFF, np.uint32), name=f"icosphere{subdiv}")


def primary_rays_icosphere(width: int = 1024, height: int = 1024, seed: int = 1) -> np.ndarray:
    """1024x1024 pinhole rays from (0,0,3) toward the origin, 45 degree FOV."""
    return camera_rays(width, height, seed=seed)


def terrain_scene(n: int = 1024, sphere_count: int = 256, sphere_subdiv: int = 5, seed_terrain: int = 2,
                  seed_inst: int = 3) -> Scene:
    """Heightfield (2,093,058 triangles at n=1024) plus ``sphere_count`` instances of an
    icosphere (20,480 triangles at subdiv 5) with uniform rotation, log-uniform scale in
    [0.01, 0.1] and translation uniform over the terrain."""
    terrain = heightfield(n, seed=seed_terrain)
    sphere = icosphere(sphere_subdiv)
    rng = np.random.default_rng(seed_inst)
    rot = random_rotations(sphere_count, rng)
    scale = np.exp(rng.uniform(np.log(0.01), np.log(0.1), sphere_count))
    hy = terrain.vertices[:, 1]
    trans = np.stack([rng.uniform(-1, 1, sphere_count), rng.uniform(float(hy.min()), float(hy.max()) + 0.1,
                                                                      sphere_count),
                      rng.uniform(-1, 1, sphere_count)], 1)
    aff = np.concatenate([IDENTITY[None, :], affine_rows(rot, scale, trans)])
    inst_mesh = np.concatenate([[0], np.ones(sphere_count, np.int64)])
    return Scene([terrain, sphere], inst_mesh, aff, np.full(sphere_count + 1, 0xFF, np.uint32), name="terrain")


def terrain_rays(scene: Scene, n: int, seed: int = 4) -> np.ndarray:
    lo, hi = scene.bounds()
    return sphere_rays(n, lo, hi, seed)


def terrain_shadow_rays(scene: Scene, n: int, seed: int = 5, light=(0.25, 1.0, -0.25)) -> np.ndarray:
    lo, hi = scene.bounds()
    return shadow_rays(n, lo, hi, light, seed)


def displaced_mesh(tri_target: int, rng: np.random.Generator) -> MeshData:
    """An icosphere or a grid with about ``tri_target`` triangles and Gaussian vertex
    displacement (sigma = 1% of the extent)."""
    if rng.random() < 0.5:
        s = int(round(math.log(max(tri_target, 20) / 20.0, 4)))
        m = icosphere(max(0, min(s, 8)))
        extent = 2.0
    else:
        cells = max(1, tri_target // 2)
        nx = max(2, int(round(math.sqrt(cells))) + 1)
        ny = max(2, int(round(cells / (nx - 1))) + 1)
        m = grid_mesh(nx, ny)
        extent = 2.0
    v = m.vertices
    v[:, :3] += (rng.standard_normal((v.shape[0], 3), dtype=np.float32) * np.float32(0.01 * extent))
    return MeshData(v, m.triangles)


def batch_meshes(count: int = 4096, lo: int = 64, hi: int = 262144, seed: int = 6):
    """``count`` meshes with triangle counts log-uniform in [lo, hi]."""
    rng = np.random.default_rng(seed)
    targets = np.exp(rng.uniform(np.log(lo), np.log(hi), count)).astype(np.int64)
    return [displaced_mesh(int(t), rng) for t in targets]


# ---------------------------------------------------------------- curves
CURVE_STEP = {0: 1, 1: 1, 2: 1, 3: 3}  # control points between segment starts, per basis
CURVE_POINTS = {0: 2, 1: 4, 2: 4, 3: 4}  # control points per segment


def curve_segments(n_curves: int, n_cp: int, basis: int) -> np.ndarray:
    """Segment starts of ``n_curves`` curves of ``n_cp`` consecutive control points each: every
    segment a basis allows along each curve (Bezier segments share their end points)."""
    step, need = CURVE_STEP[basis], CURVE_POINTS[basis]
    per = (n_cp - need) // step + 1
    starts = np.arange(per, dtype=np.uint32) * step
    return (np.arange(n_curves, dtype=np.uint32)[:, None] * n_cp + starts[None, :]).reshape(-1)


def hair_curves(n_curves: int, n_cp: int, rng: np.random.Generator, step: float = 0.12,
                radius=(0.03, 0.004), lo=(-1.0, -1.0, -1.0), hi=(1.0, 1.0, 1.0)) -> np.ndarray:
    """Control points (n_curves * n_cp, 4) of random smooth strands: roots uniform in [lo, hi], a
    direction that wanders a little per step, radius tapering from ``radius[0]`` to ``radius[1]``."""
    lo, hi = np.asarray(lo, np.float64), np.asarray(hi, np.float64)
    p = lo + rng.random((n_curves, 3)) * (hi - lo)
    d = rng.standard_normal((n_curves, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    out = np.zeros((n_curves, n_cp, 4), np.float32)
    taper = np.linspace(radius[0], radius[1], n_cp)
    for k in range(n_cp):
        out[:, k, :3] = p
        out[:, k, 3] = taper[k]
        d = d + 0.35 * rng.standard_normal((n_curves, 3))
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        p = p + step * d
    return out.reshape(-1, 4)
