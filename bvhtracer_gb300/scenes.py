"""Seeded synthetic workloads (no datasets are involved anywhere).

Every random number comes from a counter-based SplitMix64 stream, so a workload is a
pure function of (seed, sizes) and is reproducible on any machine.  Geometry is
computed in float64 and rounded once to float32; the rounded arrays are what both
the GPU library and the CPU checker consume.

Workloads:
  soup(n, seed)                 random triangle soup: v0 = 9 U^3 - 5, v1 = v0 + U^3, v2 = v0 + U^3
  icosphere(level)              unit icosphere (20 * 4^level triangles, shared-vertex index map)
  displaced_icosphere(level)    radius 1 + 0.15 sum_k a_k sin(f_k (d . w_k) + phi_k), k = 1..8
  pinhole_rays(...)             one ray per pixel centre, in the reference renderer's 8x8 tile order
"""
from __future__ import annotations

import math

import numpy as np

# The ray record of the C ABI (bvhgpu_ray, 32 bytes).  Defined here rather than imported so that
# this module has no dependency on the rest of the package: it can be loaded on its own (by file
# path) by code that must not touch the CUDA library, such as a CPU-only timing of the same inputs.
RAY = np.dtype([("origin", "<f4", 3), ("t", "<f4"), ("direction", "<f4", 3), ("reserved", "<u4")])
FLT_MAX = np.float32(np.finfo(np.float32).max)

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def _splitmix64(x: np.ndarray) -> np.ndarray:
    with np.errstate(over="ignore"):
        z = x + np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


def uniform(seed: int, stream: int, n: int) -> np.ndarray:
    """n float64 samples in [0, 1) (53-bit) from the (seed, stream) counter stream."""
    base = _splitmix64(np.array([(seed * 0x632BE59BD9B4E019 + stream * 0x9E3779B97F4A7C15) & 0xFFFFFFFFFFFFFFFF],
                                np.uint64))[0]
    with np.errstate(over="ignore"):
        ctr = base + np.arange(n, dtype=np.uint64) * np.uint64(0xD1B54A32D192ED03)
    return (_splitmix64(ctr) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def normal(seed: int, stream: int, n: int) -> np.ndarray:
    """Standard normal samples (Box-Muller on the counter stream)."""
    u1 = uniform(seed, 2 * stream + 1, n)
    u2 = uniform(seed, 2 * stream + 2, n)
    return np.sqrt(-2.0 * np.log1p(-u1)) * np.cos(2.0 * np.pi * u2)


# ---- geometry ---------------------------------------------------------------------------------

def soup(n: int, seed: int, scale: float = 1.0) -> np.ndarray:
    """Random triangle soup [n, 9] float32: v0 = 9 U^3 - 5, v1 = v0 + U^3, v2 = v0 + U^3.

    ``scale`` > 1 grows the box (not the triangles) so that larger soups keep the density
    of the 4096-triangle case.
    """
    u = uniform(seed, 1, 9 * n).reshape(n, 3, 3)
    v0 = (9.0 * u[:, 0] - 5.0) * scale
    v1 = v0 + u[:, 1]
    v2 = v0 + u[:, 2]
    return np.ascontiguousarray(np.concatenate([v0, v1, v2], axis=1).astype(np.float32))


def icosphere(level: int):
    """Unit icosphere: (vertices [V, 3] float64 unit directions, faces [F, 3] int64)."""
    t = (1.0 + math.sqrt(5.0)) / 2.0
    verts = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0],
                      [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
                      [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], np.float64)
    verts /= np.linalg.norm(verts, axis=1, keepdims=True)
    faces = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11],
                      [1, 5, 9], [5, 11, 4], [11, 10, 2], [10, 7, 6], [7, 1, 8],
                      [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9],
                      [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], np.int64)
    for _ in range(level):
        e = np.concatenate([faces[:, [0, 1]], faces[:, [1, 2]], faces[:, [2, 0]]])
        e.sort(axis=1)
        uniq, inv = np.unique(e, axis=0, return_inverse=True)
        inv = inv.reshape(-1)
        mids = verts[uniq[:, 0]] + verts[uniq[:, 1]]
        mids /= np.linalg.norm(mids, axis=1, keepdims=True)
        base = len(verts)
        verts = np.concatenate([verts, mids])
        f = len(faces)
        a, b, c = faces[:, 0], faces[:, 1], faces[:, 2]
        ab, bc, ca = base + inv[:f], base + inv[f:2 * f], base + inv[2 * f:]
        faces = np.concatenate([np.stack([a, ab, ca], 1), np.stack([b, bc, ab], 1),
                                np.stack([c, ca, bc], 1), np.stack([ab, bc, ca], 1)])
    return verts, faces


def displacement_params(seed: int):
    w = normal(seed, 10, 24).reshape(8, 3)
    w /= np.linalg.norm(w, axis=1, keepdims=True)
    a = uniform(seed, 11, 8) / 8.0
    f = 2.0 + 10.0 * uniform(seed, 12, 8)
    phi = 2.0 * np.pi * uniform(seed, 13, 8)
    return w, a, f, phi


def displaced_radius(dirs: np.ndarray, seed: int) -> np.ndarray:
    """1 + 0.15 * sum_k a_k sin(f_k (d . w_k) + phi_k) for unit directions d."""
    w, a, f, phi = displacement_params(seed)
    arg = (dirs @ w.T) * f[None, :] + phi[None, :]
    return 1.0 + 0.15 * (np.sin(arg) * a[None, :]).sum(axis=1)


class Mesh:
    """Indexed mesh: unique vertices (float64 directions + radii) and faces."""

    def __init__(self, dirs, radius, faces):
        self.dirs = dirs
        self.radius = radius
        self.faces = faces

    @property
    def vertices(self) -> np.ndarray:
        return (self.dirs * self.radius[:, None]).astype(np.float32)

    def triangles(self, vertices: np.ndarray | None = None) -> np.ndarray:
        v = self.vertices if vertices is None else vertices
        return np.ascontiguousarray(v[self.faces].reshape(-1, 9).astype(np.float32))


def displaced_icosphere(level: int, seed: int) -> Mesh:
    dirs, faces = icosphere(level)
    return Mesh(dirs, displaced_radius(dirs, seed), faces)


# ---- rays ---------------------------------------------------------------------------------------

def tile_order(width: int, height: int):
    """Pixel (x, y) of ray i in the reference renderer's order: 8x8 tiles, row by row inside
    a tile (renderer.rs:353-368), tiles row-major."""
    tx, ty = (width + 7) // 8, (height + 7) // 8
    i = np.arange(tx * ty * 64)
    tile, within = i // 64, i % 64
    x = (tile % tx) * 8 + within % 8
    y = (tile // tx) * 8 + within // 8
    keep = (x < width) & (y < height)
    return x[keep], y[keep]


def make_rays(origins: np.ndarray, dirs: np.ndarray) -> np.ndarray:
    r = np.zeros(len(dirs), RAY)
    r["origin"] = np.asarray(origins, np.float32)
    r["direction"] = np.asarray(dirs, np.float32)
    r["t"] = FLT_MAX
    return r


def plane_rays(width: int, height: int, eye, plane_z: float, half_w: float, half_h: float) -> np.ndarray:
    """Rays from `eye` through pixel centres of the plane z = plane_z spanning
    [-half_w, half_w] x [-half_h, half_h] (top row first), in tile order."""
    x, y = tile_order(width, height)
    px = -half_w + (x + 0.5) * (2.0 * half_w / width)
    py = half_h - (y + 0.5) * (2.0 * half_h / height)
    eye = np.asarray(eye, np.float64)
    d = np.stack([px - eye[0], py - eye[1], np.full_like(px, plane_z - eye[2])], axis=1)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return make_rays(np.broadcast_to(eye, d.shape), d)


def look_at_rays(width: int, height: int, eye, target, fovy_deg: float) -> np.ndarray:
    """Pinhole primaries through pixel centres (tile order) for a camera at `eye` looking at
    `target` (world up +y), vertical field of view fovy_deg."""
    eye = np.asarray(eye, np.float64)
    fwd = np.asarray(target, np.float64) - eye
    fwd /= np.linalg.norm(fwd)
    up0 = np.array([0.0, 1.0, 0.0])
    right = np.cross(up0, fwd)
    if np.linalg.norm(right) < 1e-9:
        right = np.array([1.0, 0.0, 0.0])
    right /= np.linalg.norm(right)
    up = np.cross(fwd, right)
    x, y = tile_order(width, height)
    th = math.tan(math.radians(fovy_deg) / 2.0)
    tw = th * width / height
    sx = (2.0 * (x + 0.5) / width - 1.0) * tw
    sy = (1.0 - 2.0 * (y + 0.5) / height) * th
    d = fwd[None, :] + sx[:, None] * right[None, :] + sy[:, None] * up[None, :]
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return make_rays(np.broadcast_to(eye, d.shape), d)


def sphere_rays(n: int, seed: int, box: float = 10.0) -> np.ndarray:
    """Origins U[-box, box]^3, directions uniform on the unit sphere."""
    o = (2.0 * uniform(seed, 20, 3 * n).reshape(n, 3) - 1.0) * box
    z = 2.0 * uniform(seed, 21, n) - 1.0
    phi = 2.0 * np.pi * uniform(seed, 22, n)
    r = np.sqrt(np.maximum(0.0, 1.0 - z * z))
    d = np.stack([r * np.cos(phi), r * np.sin(phi), z], axis=1)
    return make_rays(o, d)


# ---- the benchmark workloads ---------------------------------------------------------------------

def soup_frame(seed: int = 0):
    """4096-triangle soup, camera (0,0,-18) through the plane z = -15 spanning [-1,1]^2,
    640 x 640 pixel-centre rays."""
    tris = soup(4096, seed)
    rays = plane_rays(640, 640, (0.0, 0.0, -18.0), -15.0, 1.0, 1.0)
    return tris, rays


def icosphere_frame(seed: int = 0, width: int = 1920, height: int = 1080):
    """Displaced icosphere, 6 subdivisions (81,920 triangles), camera at distance 3,
    1920 x 1080 primaries (a cosine bounce per hit pixel is generated on the GPU)."""
    mesh = displaced_icosphere(6, seed)
    tris = mesh.triangles()
    rays = look_at_rays(width, height, (0.0, 0.0, -3.0), (0.0, 0.0, 0.0), 45.0)
    return tris, rays, mesh


def batch_specs(seed: int = 0, nscenes: int = 64, tri_range=(1_000, 2_000_000), ray_range=(65_536, 4_194_304)):
    """Sizes of the uneven batch: triangle and ray counts log-uniform in the given ranges."""
    u_t = uniform(seed, 30, nscenes)
    u_r = uniform(seed, 31, nscenes)
    lt = np.log(tri_range[0]) + u_t * (np.log(tri_range[1]) - np.log(tri_range[0]))
    lr = np.log(ray_range[0]) + u_r * (np.log(ray_range[1]) - np.log(ray_range[0]))
    return np.round(np.exp(lt)).astype(np.int64), np.round(np.exp(lr)).astype(np.int64)


def batch_scene(i: int, ntris: int, nrays: int, seed: int = 0):
    """Scene i of the uneven batch: even i a soup (the soup_frame formula) grown to `ntris` triangles
    (box scaled by (ntris/4096)^(1/3)), odd i a displaced icosphere at the subdivision level
    nearest to `ntris`; rays: half pinhole primaries (tile order), half origins
    U[-10, 10]^3 (times the scene scale) with uniform-sphere directions."""
    sseed = seed * 1000 + i
    if i % 2 == 0:
        scale = (ntris / 4096.0) ** (1.0 / 3.0)
        tris = soup(int(ntris), sseed, scale=scale)
        n_prim = nrays // 2
        side = int(np.ceil(np.sqrt(n_prim) / 8.0) * 8)
        prim = plane_rays(side, side, (0.0, 0.0, -18.0 * scale), -15.0 * scale, scale, scale)[:n_prim]
        box = 10.0 * scale
    else:
        level = int(np.clip(np.round(np.log(ntris / 20.0) / np.log(4.0)), 1, 8))
        tris = displaced_icosphere(level, sseed).triangles()
        n_prim = nrays // 2
        side = int(np.ceil(np.sqrt(n_prim) / 8.0) * 8)
        prim = look_at_rays(side, side, (0.0, 0.0, -3.0), (0.0, 0.0, 0.0), 45.0)[:n_prim]
        box = 10.0
    rnd = sphere_rays(int(nrays - n_prim), sseed + 7, box=box)
    return tris, np.concatenate([prim, rnd])


def lambert_scene(seed: int = 0, level: int = 7, width: int = 512, height: int = 512, sigma: float = 0.01,
            scale: float = 10.0):
    """Differentiable-render workload: displaced icosphere (icosphere_frame's displacement) with `level`
    subdivisions, its radial unit directions as fixed vertex normals, a target mesh whose vertices
    are moved radially by N(0, sigma^2), a point light at (2, 2, -3), and width x height
    pixel-centre primaries from distance 3 (tile order) -- all lengths multiplied by `scale`.

    The scale exists because the reference's Moeller-Trumbore test rejects |e1 . (d x e2)| < 1e-4
    (triangle.rs:47-51), an absolute threshold on a quantity proportional to the triangle's area:
    at unit radius the 7-subdivision sphere's triangles (edges ~0.01) are all rejected.  A uniform
    scale leaves the Lambertian image unchanged up to rounding."""
    mesh = displaced_icosphere(level, seed)
    verts = (mesh.dirs * (scale * mesh.radius)[:, None]).astype(np.float32)
    vnormals = mesh.dirs.astype(np.float32)
    target_r = scale * (mesh.radius + sigma * normal(seed, 40, len(mesh.radius)))
    target_verts = (mesh.dirs * target_r[:, None]).astype(np.float32)
    rays = look_at_rays(width, height, (0.0, 0.0, -3.0 * scale), (0.0, 0.0, 0.0), 45.0)
    light = np.array([2.0 * scale, 2.0 * scale, -3.0 * scale], np.float32)
    return verts, mesh.faces.astype(np.uint32), vnormals, target_verts, rays, light


def instanced_animation(seed: int = 0, ninstances: int = 256, width: int = 1280, height: int = 720, levels=(4, 5, 6)):
    """Instanced animated scene: three displaced icospheres (icosphere_frame's displacement) at the given
    subdivision levels, `ninstances` instances (instance i uses mesh i % 3) with a seeded random
    rotation, uniform scale U[0.5, 2] and translation in a 40^3 box; per frame (dt = 1/30 s) each
    instance turns about a seeded axis at U[-1, 1] rad/s and every vertex wobbles radially by
    0.02 sin(3 t + phase_v).  Camera: width x height pixel-centre primaries from (0, 0, -60),
    60 degree field of view, tile order."""
    meshes = []
    for k, lvl in enumerate(levels):
        m = displaced_icosphere(lvl, seed * 100 + k)
        phase = 2.0 * np.pi * uniform(seed * 100 + k, 50, len(m.radius))
        meshes.append({"verts": m.vertices, "faces": m.faces.astype(np.uint32),
                       "dirs": m.dirs.astype(np.float32), "r0": m.radius.astype(np.float32),
                       "phase": phase.astype(np.float32)})
    n = ninstances
    q = normal(seed, 60, 4 * n).reshape(n, 4)
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    w, x, y, z = q.T
    rot0 = np.stack([np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)], -1),
                     np.stack([2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)], -1),
                     np.stack([2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)], -1)], 1)
    axis = normal(seed, 61, 3 * n).reshape(n, 3)
    axis /= np.linalg.norm(axis, axis=1, keepdims=True)
    inst = {"blas_of": (np.arange(n) % len(levels)).astype(np.uint32),
            "rot0": np.ascontiguousarray(rot0.astype(np.float32)),
            "axis": np.ascontiguousarray(axis.astype(np.float32)),
            "omega": (2.0 * uniform(seed, 62, n) - 1.0).astype(np.float32),
            "scale": (0.5 + 1.5 * uniform(seed, 63, n)).astype(np.float32),
            "trans": ((2.0 * uniform(seed, 64, 3 * n) - 1.0) * 20.0).reshape(n, 3).astype(np.float32)}
    rays = look_at_rays(width, height, (0.0, 0.0, -60.0), (0.0, 0.0, 0.0), 60.0)
    return {"meshes": meshes, "instances": inst, "rays": rays, "dt": 1.0 / 30.0, "amp": 0.02, "freq": 3.0}
