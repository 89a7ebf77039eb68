"""ctypes wrapper around the CPU oracle (``oracle/bvh_oracle.cpp``).

TEST INFRASTRUCTURE ONLY.  The oracle is a restatement of the reference's CPU
ray-BVH path (lambdaxymox/bvhtracer, Rust).  Only the tests, the smoke check
and the CPU-baseline leg of ``bench.py`` use it, always as the checker or as
the timed CPU baseline; the product library (``bvhtracer_gb300``) never
imports it.

Parity pin: the reference cannot be compiled here (Rust, no cargo), so the
restatement is pinned against the known answers of the reference's own tests
(``tests/test_oracle_known_answers.py``).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liborc.so")

NODE = np.dtype([("bounds_min", "<f4", 3), ("bounds_max", "<f4", 3),
                 ("primitive_count", "<u4"), ("left_first", "<u4")])
RAY = np.dtype([("origin", "<f4", 3), ("t", "<f4"), ("direction", "<f4", 3), ("reserved", "<u4")])
HIT = np.dtype([("t", "<f4"), ("u", "<f4"), ("v", "<f4"), ("prim", "<u4"), ("inst", "<u4")])
TLAS_NODE = np.dtype([("bounds_min", "<f4", 3), ("bounds_max", "<f4", 3),
                      ("left_right", "<u4"), ("blas", "<u4")])
COUNTERS = np.dtype([("interior", "<u4"), ("leaves", "<u4"), ("tris", "<u4"),
                     ("tlas_interior", "<u4"), ("blas_entries", "<u4")])
assert NODE.itemsize == 32 and RAY.itemsize == 32 and HIT.itemsize == 20 and TLAS_NODE.itemsize == 32

MISS = 0xFFFFFFFF
FLT_MAX = np.float32(np.finfo(np.float32).max)

# accumulator / shader kinds (same values as the product ABI)
ACC_INTERSECTION, ACC_DEPTH, ACC_UV, ACC_NORMAL = 0, 1, 2, 3
SH_RADIANCE, SH_INTERSECTION, SH_DEPTH = 0, 1, 2

CXXFLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math"]


def build(force: bool = False) -> str:
    """Compile the oracle shared library with g++ (no fused multiply-add)."""
    src = os.path.join(HERE, "bvh_oracle.cpp")
    hdr = os.path.join(HERE, "bvh_oracle.h")
    if (not force and os.path.exists(LIB_PATH)
            and os.path.getmtime(LIB_PATH) >= max(os.path.getmtime(src), os.path.getmtime(hdr))):
        return LIB_PATH
    os.makedirs(os.path.dirname(LIB_PATH), exist_ok=True)
    tmp = LIB_PATH + f".tmp{os.getpid()}"
    subprocess.check_call(["g++", *CXXFLAGS, "-shared", "-o", tmp, src, "-lpthread"])
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.c_void_p
        u32 = ctypes.c_uint32
        i32 = ctypes.c_int
        f32 = ctypes.c_float
        L.orc_triangle_intersect.argtypes = [P, P, P, P, P]
        L.orc_aabb_intersect.argtypes = [P, P, P, P]
        L.orc_normalize.argtypes = [P, P]
        L.orc_normalize.restype = None
        L.orc_triangle_centroid.argtypes = [P, P]
        L.orc_triangle_centroid.restype = None
        L.orc_bvh_build.argtypes = [P, u32, P, P]
        L.orc_bvh_intersect.argtypes = [P, u32, P, u32, P, u32, P, P]
        L.orc_bvh_intersect_mt.argtypes = [P, u32, P, u32, P, u32, P, i32]
        L.orc_two_nearest_mt.argtypes = [P, P, P, u32, P, P, i32]
        L.orc_triangles_intersect.argtypes = [P, u32, P, u32, i32, P]
        L.orc_world_start_frame.argtypes = [P, u32]
        L.orc_world_step.argtypes = [P, u32, P, u32, ctypes.c_float]
        L.orc_object_transforms.argtypes = [P, P, P, u32, P, P]
        L.orc_bvh_refit.argtypes = [P, u32, P, u32]
        L.orc_bvh_depth.argtypes = [P, u32]
        L.orc_bvh_depth.restype = u32
        L.orc_object_bounds.argtypes = [P, P, P, P, P]
        L.orc_object_bounds.restype = None
        L.orc_tlas_build.argtypes = [P, P, u32, P, P]
        L.orc_scene_intersect.argtypes = [P, u32, P, P, u32, P, P, P, P, P, u32, P, P, i32]
        L.orc_scene_intersect_mt.argtypes = [P, u32, P, P, u32, P, P, P, P, P, u32, P, i32]
        L.orc_camera_ray.argtypes = [P, P, f32, f32, P]
        L.orc_camera_ray.restype = None
        L.orc_render.argtypes = [P, P, i32, i32, i32, P, i32, P, P, u32, P, u32, P, P, P]
        L.orc_render_textured.argtypes = [P, P, i32, i32, i32, P, i32, P, P, u32, P, u32, P, P, P, u32, u32, P, P]
        L.orc_render_scene.argtypes = [P, P, i32, i32, i32, P, i32, P, P, P, P, P, u32, P, P, P, P, P, P, P, P, P,
                                       P, P, i32, P, P]
        L.orc_bounce_ray.argtypes = [P, P, P, u32, u32, P]
        L.orc_bounce_rays.argtypes = [P, P, u32, P, u32, P, P]
        L.orc_scene_bounce_rays.argtypes = [P, P, P, P, P, P, u32, u32, P, P]
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def _c(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype)


# --- primitives ---------------------------------------------------------------

def make_rays(origins, directions, t=None) -> np.ndarray:
    origins = np.asarray(origins, np.float32).reshape(-1, 3)
    directions = np.asarray(directions, np.float32).reshape(-1, 3)
    r = np.zeros(len(origins), RAY)
    r["origin"] = origins
    r["direction"] = directions
    r["t"] = FLT_MAX if t is None else np.asarray(t, np.float32)
    return r


def normalize(v):
    v = np.ascontiguousarray(v, np.float32)
    out = np.zeros(3, np.float32)
    lib().orc_normalize(_p(v), _p(out))
    return out


def triangle_intersect(tri, ray):
    """Triangle::intersect (triangle.rs:42-72).  Returns (t, u, v) or None."""
    tri = _c(tri, np.float32).reshape(9)
    ray = _c(ray, RAY).reshape(1)
    t, u, v = (np.zeros(1, np.float32) for _ in range(3))
    hit = lib().orc_triangle_intersect(_p(tri), _p(ray), _p(t), _p(u), _p(v))
    return (t[0], u[0], v[0]) if hit else None


def aabb_intersect(bmin, bmax, ray):
    """Aabb::intersect (aabb.rs:65-84).  Returns tmin or None."""
    bmin = _c(bmin, np.float32)
    bmax = _c(bmax, np.float32)
    ray = _c(ray, RAY).reshape(1)
    t = np.zeros(1, np.float32)
    return t[0] if lib().orc_aabb_intersect(_p(bmin), _p(bmax), _p(ray), _p(t)) else None


def centroid(tri):
    tri = _c(tri, np.float32).reshape(9)
    out = np.zeros(3, np.float32)
    lib().orc_triangle_centroid(_p(tri), _p(out))
    return out


# --- BLAS ---------------------------------------------------------------------

def bvh_build(tris):
    """BvhBuilder::build_for.  Returns (reordered tris [n,9], nodes [2n], nodes_used)."""
    tris = np.array(tris, np.float32, copy=True).reshape(-1, 9)
    n = len(tris)
    nodes = np.zeros(max(2 * n, 1), NODE)
    used = np.zeros(1, np.uint32)
    rc = lib().orc_bvh_build(_p(tris), n, _p(nodes), _p(used))
    if rc != 0:
        raise RuntimeError(f"oracle bvh_build failed ({rc}): the reference would panic on this mesh")
    return tris, nodes, int(used[0])


def bvh_intersect(nodes, nodes_used, tris, rays, counters=False, threads=1):
    nodes = _c(nodes, NODE)
    tris = _c(tris, np.float32).reshape(-1, 9)
    rays = _c(rays, RAY)
    hits = np.zeros(len(rays), HIT)
    if threads > 1:
        rc = lib().orc_bvh_intersect_mt(_p(nodes), nodes_used, _p(tris), len(tris), _p(rays), len(rays),
                                        _p(hits), threads)
        assert rc == 0
        return hits
    cnt = np.zeros(len(rays), COUNTERS) if counters else None
    rc = lib().orc_bvh_intersect(_p(nodes), nodes_used, _p(tris), len(tris), _p(rays), len(rays), _p(hits),
                                 _p(cnt))
    assert rc == 0
    return (hits, cnt) if counters else hits


def triangles_intersect(tris, rays, mode=0):
    """Triangle::intersect (mode 0, first smallest t) or Triangle::intersect_mut (mode 1) of every
    ray against the triangle list in order."""
    tris = _c(tris, np.float32).reshape(-1, 9)
    rays = _c(rays, RAY)
    hits = np.zeros(len(rays), HIT)
    assert lib().orc_triangles_intersect(_p(tris), len(tris), _p(rays), len(rays), mode, _p(hits)) == 0
    return hits


def world_start_frame(bodies):
    """World::start_frame on a structured array of rigid bodies (modified in place)."""
    assert lib().orc_world_start_frame(_p(bodies), len(bodies)) == 0


def world_step(bodies, gens, dt):
    """World::run_physics(dt) in place: the registry's forces in order, then integrate."""
    g = np.ascontiguousarray(gens)
    assert lib().orc_world_step(_p(bodies), len(bodies), _p(g) if len(g) else None, len(g), float(dt)) == 0


def object_transforms(bodies, body_of, init):
    """SceneObject::update_transform: (xf, inv) [nobj, 16], body transform * initial transform."""
    body_of = _c(body_of, np.uint32)
    init = _c(init, np.float32).reshape(-1, 16)
    xf = init.copy()
    inv = np.zeros_like(init)
    assert lib().orc_object_transforms(_p(bodies), _p(body_of), _p(init), len(body_of), _p(xf), _p(inv)) == 0
    return xf, inv


def two_nearest(nodes, tris, rays, threads=8):
    """The two smallest hit distances of every ray over the whole BVH (FLT_MAX: none)."""
    nodes = _c(nodes, NODE)
    tris = _c(tris, np.float32).reshape(-1, 9)
    rays = _c(rays, RAY)
    t1 = np.zeros(len(rays), np.float32)
    t2 = np.zeros(len(rays), np.float32)
    assert lib().orc_two_nearest_mt(_p(nodes), _p(tris), _p(rays), len(rays), _p(t1), _p(t2), threads) == 0
    return t1, t2


def near_ties(nodes, tris, rays, rel=1e-5, threads=8):
    """Mask of the rays whose two nearest hits lie within `rel` relative in t (the parity rule
    counts them apart: a 1-ulp difference in t could swap which triangle is closest)."""
    t1, t2 = two_nearest(nodes, tris, rays, threads)
    fmax = np.finfo(np.float32).max
    both = (t1 < fmax) & (t2 < fmax)
    return both & ((t2.astype(np.float64) - t1) <= rel * np.abs(t1.astype(np.float64)))


def bvh_refit(nodes, nodes_used, tris):
    nodes = np.array(nodes, NODE, copy=True)
    tris = _c(tris, np.float32).reshape(-1, 9)
    rc = lib().orc_bvh_refit(_p(nodes), nodes_used, _p(tris), len(tris))
    assert rc == 0
    return nodes


def bvh_depth(nodes, nodes_used):
    nodes = _c(nodes, NODE)
    return int(lib().orc_bvh_depth(_p(nodes), nodes_used))


# --- TLAS / scene --------------------------------------------------------------

def object_bounds(model_min, model_max, xf):
    mn = _c(model_min, np.float32)
    mx = _c(model_max, np.float32)
    xf = _c(xf, np.float32).reshape(16)
    omn = np.zeros(3, np.float32)
    omx = np.zeros(3, np.float32)
    lib().orc_object_bounds(_p(mn), _p(mx), _p(xf), _p(omn), _p(omx))
    return omn, omx


def tlas_build(obj_min, obj_max):
    obj_min = _c(obj_min, np.float32).reshape(-1, 3)
    obj_max = _c(obj_max, np.float32).reshape(-1, 3)
    n = len(obj_min)
    nodes = np.zeros(max(2 * n, 1), TLAS_NODE)
    used = np.zeros(1, np.uint32)
    rc = lib().orc_tlas_build(_p(obj_min), _p(obj_max), n, _p(nodes), _p(used))
    if rc != 0:
        raise RuntimeError(f"oracle tlas_build failed ({rc})")
    return nodes, int(used[0])


class SceneArrays:
    """Concatenated BLAS arrays + per-object data for the scene oracle."""

    def __init__(self, blases, blas_of, inv):
        # blases: list of (nodes, nodes_used, tris)
        self.node_off = np.zeros(len(blases), np.uint32)
        self.tri_off = np.zeros(len(blases), np.uint32)
        no = to = 0
        for i, (nodes, _, tris) in enumerate(blases):
            self.node_off[i] = no
            self.tri_off[i] = to
            no += len(nodes)
            to += len(tris)
        self.nodes = np.concatenate([b[0] for b in blases]).astype(NODE)
        self.tris = np.ascontiguousarray(np.concatenate([np.asarray(b[2], np.float32).reshape(-1, 9)
                                                         for b in blases]))
        self.blas_of = _c(blas_of, np.uint32)
        self.inv = _c(inv, np.float32).reshape(-1, 16)


def scene_intersect(tlas, tlas_used, sa: SceneArrays, rays, counters=False, instance_zero=False, threads=1):
    tlas = _c(tlas, TLAS_NODE)
    rays = _c(rays, RAY)
    hits = np.zeros(len(rays), HIT)
    if threads > 1:
        rc = lib().orc_scene_intersect_mt(_p(tlas), tlas_used, _p(sa.blas_of), _p(sa.inv), len(sa.blas_of),
                                          _p(sa.nodes), _p(sa.node_off), _p(sa.tris), _p(sa.tri_off),
                                          _p(rays), len(rays), _p(hits), threads)
        assert rc == 0
        return hits
    cnt = np.zeros(len(rays), COUNTERS) if counters else None
    rc = lib().orc_scene_intersect(_p(tlas), tlas_used, _p(sa.blas_of), _p(sa.inv), len(sa.blas_of),
                                   _p(sa.nodes), _p(sa.node_off), _p(sa.tris), _p(sa.tri_off),
                                   _p(rays), len(rays), _p(hits), _p(cnt), int(instance_zero))
    assert rc == 0
    return (hits, cnt) if counters else hits


# --- camera / render / bounce ---------------------------------------------------

def camera_ray(corners, view_inv, u, v):
    corners = _c(corners, np.float32).reshape(9)
    view_inv = _c(view_inv, np.float32).reshape(16)
    r = np.zeros(1, RAY)
    lib().orc_camera_ray(_p(corners), _p(view_inv), float(u), float(v), _p(r))
    return r[0]


def render(corners, view_inv, width, height, nodes, nodes_used, tris, accumulator, shader,
           acc_params=None, shader_params=None, normals=None, tex_coords=None, texels=None):
    """PathTracer::evaluate; texels ([h, w, 3] uint8) and tex_coords ([n, 6]) for accumulator 4."""
    corners = _c(corners, np.float32).reshape(9)
    view_inv = _c(view_inv, np.float32).reshape(16)
    nodes = _c(nodes, NODE)
    tris = _c(tris, np.float32).reshape(-1, 9)
    ap = None if acc_params is None else _c(acc_params, np.float32)
    sp = None if shader_params is None else _c(shader_params, np.float32)
    nrm = None if normals is None else _c(normals, np.float32).reshape(-1, 9)
    rgba = np.zeros((height, width, 4), np.uint8)
    rad = np.zeros((height, width, 3), np.float32)
    tc = None if tex_coords is None else _c(tex_coords, np.float32).reshape(-1, 6)
    tx = None if texels is None else _c(texels, np.uint8)
    th, tw = (0, 0) if tx is None else tx.shape[:2]
    rc = lib().orc_render_textured(_p(corners), _p(view_inv), width, height, accumulator, _p(ap), shader, _p(sp),
                                   _p(nodes), nodes_used, _p(tris), len(tris), _p(nrm), _p(tc), _p(tx), tw, th,
                                   _p(rgba), _p(rad))
    if rc != 0:
        raise RuntimeError(f"oracle render failed ({rc})")
    return rgba, rad


def render_scene(corners, view_inv, width, height, tlas, sa: SceneArrays, xf, accumulator, shader,
                 acc_params=None, shader_params=None, normals=None, tex_coords=None, textures=None, lookup=0):
    """PathTracer::evaluate over a scene (TLAS + instances).  normals / tex_coords: one array per BLAS
    of `sa` ([ntris, 9] / [ntris, 6]) or None; textures: one [h, w, 3] uint8 array per BLAS or None.
    lookup 0 = the reference's instance-0 lookup for the normal / texture accumulators, 1 = the hit's
    object.  Raises PanicError where the reference would panic (a primitive index outside object 0's
    mesh)."""
    corners = _c(corners, np.float32).reshape(9)
    view_inv = _c(view_inv, np.float32).reshape(16)
    tlas = _c(tlas, TLAS_NODE)
    xf = _c(xf, np.float32).reshape(-1, 16)
    nb = len(sa.node_off)
    counts = np.array([(sa.tri_off[i + 1] if i + 1 < nb else len(sa.tris)) - sa.tri_off[i] for i in range(nb)],
                      np.uint32)
    nrm = None if normals is None else _c(np.concatenate([np.asarray(a, np.float32).reshape(-1, 9)
                                                          for a in normals]), np.float32)
    tc = None if tex_coords is None else _c(np.concatenate([np.asarray(a, np.float32).reshape(-1, 6)
                                                           for a in tex_coords]), np.float32)
    tx = toff = tw = th = None
    if textures is not None:
        tx = _c(np.concatenate([np.asarray(t, np.uint8).reshape(-1) for t in textures]), np.uint8)
        sizes = [np.asarray(t).size for t in textures]
        toff = np.concatenate([[0], np.cumsum(sizes)[:-1]]).astype(np.uint64)
        tw = np.array([np.asarray(t).shape[1] for t in textures], np.uint32)
        th = np.array([np.asarray(t).shape[0] for t in textures], np.uint32)
    ap = None if acc_params is None else _c(acc_params, np.float32)
    sp = None if shader_params is None else _c(shader_params, np.float32)
    rgba = np.zeros((height, width, 4), np.uint8)
    rad = np.zeros((height, width, 3), np.float32)
    rc = lib().orc_render_scene(_p(corners), _p(view_inv), width, height, accumulator, _p(ap), shader, _p(sp),
                                _p(tlas), _p(sa.blas_of), _p(xf), _p(sa.inv), len(sa.blas_of), _p(sa.nodes),
                                _p(sa.node_off), _p(sa.tris), _p(sa.tri_off), _p(counts), _p(nrm), _p(tc), _p(tx),
                                _p(toff), _p(tw), _p(th), int(lookup), _p(rgba), _p(rad))
    if rc == 2:
        raise PanicError("the reference would panic: a hit's primitive index is outside object 0's mesh")
    if rc != 0:
        raise RuntimeError(f"oracle render_scene failed ({rc})")
    return rgba, rad


class PanicError(RuntimeError):
    """The reference would panic on this input."""


def bounce_rays(primaries, hits, tris, seed):
    primaries = _c(primaries, RAY)
    hits = _c(hits, HIT)
    tris = _c(tris, np.float32).reshape(-1, 9)
    out = np.zeros(len(primaries), RAY)
    valid = np.zeros(len(primaries), np.uint8)
    rc = lib().orc_bounce_rays(_p(primaries), _p(hits), len(primaries), _p(tris), seed, _p(out), _p(valid))
    assert rc == 0
    return out, valid.astype(bool)


def scene_bounce_rays(sa: SceneArrays, primaries, hits, seed):
    primaries = _c(primaries, RAY)
    hits = _c(hits, HIT)
    out = np.zeros(len(primaries), RAY)
    valid = np.zeros(len(primaries), np.uint8)
    rc = lib().orc_scene_bounce_rays(_p(sa.blas_of), _p(sa.inv), _p(sa.tris), _p(sa.tri_off), _p(primaries),
                                     _p(hits), len(primaries), seed, _p(out), _p(valid))
    assert rc == 0
    return out, valid.astype(bool)


def bytes_per_ray(counters) -> np.ndarray:
    """Algorithmic bytes per ray: 32*(1 + 2*I) + 36*T + 24 + 20 (+ TLAS terms)."""
    c = counters
    b = (32 * (1 + 2 * c["interior"].astype(np.int64)) + 36 * c["tris"].astype(np.int64) + 24 + 20)
    b += 32 * (2 * c["tlas_interior"].astype(np.int64)) + 48 * c["blas_entries"].astype(np.int64)
    return b
