"""Host-side mirror of the reference's ray-BVH interface over the bvhgpu C ABI.

Names follow the reference crate (lambdaxymox/bvhtracer): ``BvhBuilder.build_for``
(BT/src/model/bvh.rs:524-541), ``ModelInstance.intersect`` / ``refit``
(BT/src/model/model.rs:27-33), ``Scene.intersect`` / ``rebuild``
(BT/src/scene/scene.rs:32-38), ``Camera.get_ray_world`` (BT/src/camera/camera.rs:1004),
``Renderer.render`` with a GPU integrator (BT/src/renderer.rs:388-400).  Misses are
reported as ``t = FLT_MAX, prim = inst = MISS`` (the reference's ``Option::None``).
Errors raise :class:`BvhGpuError`; there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import _lib
from ._lib import (BATCH_ITEM, FLT_MAX, HIT, MISS, NODE, RAY, TLAS_NODE, BvhGpuError, ptr)


class Context:
    """One bvhgpu context on one CUDA device (not thread-safe, like the reference's Rc model)."""

    def __init__(self, device: int = 0):
        self.lib = _lib.load()
        h = ctypes.c_void_p()
        rc = self.lib.bvhgpu_create(ctypes.byref(h), device)
        if rc != 0:
            raise BvhGpuError(rc, "bvhgpu_create failed (is a CUDA device present?)")
        self.h = h

    def close(self):
        if self.h:
            self.lib.bvhgpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def check(self, rc: int):
        if rc != 0:
            msg = self.lib.bvhgpu_last_error(self.h)
            raise BvhGpuError(rc, msg.decode() if msg else "")

    def sync(self):
        self.check(self.lib.bvhgpu_sync(self.h))

    def set_deadline(self, ns: int):
        """Time budget of each persistent launch in nanoseconds (0: none); a launch past it stops
        and the next synchronising call raises BvhGpuError with code ERR_DEADLINE."""
        self.check(self.lib.bvhgpu_set_deadline(self.h, int(ns)))

    @property
    def stream(self):
        return self.lib.bvhgpu_get_stream(self.h)

    def launch_count(self) -> int:
        return int(self.lib.bvhgpu_launch_count())

    # -- memory ---------------------------------------------------------------------------
    def device_buffer(self, nbytes: int) -> "DeviceBuffer":
        return DeviceBuffer(self, nbytes)

    def to_device(self, arr: np.ndarray) -> "DeviceBuffer":
        arr = np.ascontiguousarray(arr)
        buf = DeviceBuffer(self, arr.nbytes)
        buf.upload(arr)
        return buf

    def pinned(self, shape, dtype) -> "PinnedArray":
        return PinnedArray(self, shape, dtype)

    def flush_l2(self, stream=None):
        self.check(self.lib.bvhgpu_flush_l2(self.h, stream))

    def event(self) -> "Event":
        return Event(self)

    def profile(self, enable: bool):
        self.check(self.lib.bvhgpu_profile_enable(self.h, int(enable)))

    def profile_read(self) -> dict:
        ms = np.zeros(len(_lib.KERNELS), np.float64)
        n = np.zeros(len(_lib.KERNELS), np.uint64)
        self.check(self.lib.bvhgpu_profile_read(self.h, ptr(ms), ptr(n)))
        return {k: (float(ms[i]), int(n[i])) for i, k in enumerate(_lib.KERNELS) if n[i]}

    # -- objects --------------------------------------------------------------------------
    def upload_blas(self, bvh: "Bvh", tris: np.ndarray) -> "Blas":
        return Blas(self, bvh, tris)

    def scene(self, blases, transforms=None, inverses=None) -> "Scene":
        return Scene(self, blases, transforms, inverses)

    # -- frame graphs -------------------------------------------------------------------
    def advance_time_async(self, d_time: "DeviceBuffer", dt: float, stream=None):
        self.check(self.lib.bvhgpu_advance_time_async(self.h, d_time.ptr, float(dt), stream))

    def graph_begin(self):
        self.check(self.lib.bvhgpu_graph_begin(self.h))

    def graph_end(self) -> int:
        gid = ctypes.c_uint32()
        self.check(self.lib.bvhgpu_graph_end(self.h, ctypes.byref(gid)))
        return gid.value

    def graph_launch(self, graph_id: int):
        self.check(self.lib.bvhgpu_graph_launch(self.h, graph_id))

    def graph_free(self, graph_id: int):
        self.check(self.lib.bvhgpu_graph_free(self.h, graph_id))

    def trace_batch(self, items, rays: np.ndarray, mode: int) -> np.ndarray:
        items = np.ascontiguousarray(items, BATCH_ITEM)
        rays = np.ascontiguousarray(rays, RAY)
        hits = np.zeros(len(rays), HIT)
        self.check(self.lib.bvhgpu_trace_batch(self.h, ptr(items), len(items), ptr(rays), len(rays), mode,
                                               ptr(hits)))
        return hits

    def trace_batch_async(self, items, d_rays: "DeviceBuffer", nrays: int, mode: int, d_hits: "DeviceBuffer",
                          stream=None):
        items = np.ascontiguousarray(items, BATCH_ITEM)
        self.check(self.lib.bvhgpu_trace_batch_async(self.h, ptr(items), len(items), d_rays.ptr, nrays, mode,
                                                     d_hits.ptr, stream))


    def build_bvh(self, mesh: np.ndarray, perm: bool = False):
        """BvhBuilder::build_for on the GPU (same result as BvhBuilder().build_for); reorders ``mesh``
        ([n, 9] float32, C-contiguous) in place.  With perm=True also returns the input index of the
        triangle at each position."""
        if mesh.dtype != np.float32 or not mesh.flags.c_contiguous or mesh.ndim != 2 or mesh.shape[1] != 9:
            raise ValueError("mesh must be a C-contiguous float32 array of shape [n, 9]")
        n = mesh.shape[0]
        nodes = np.zeros(max(2 * n, 1), NODE)
        used = ctypes.c_uint32()
        p = np.zeros(n, np.uint32) if perm else None
        self.check(self.lib.bvhgpu_build_bvh_device(self.h, ptr(mesh), n, ptr(nodes), ctypes.byref(used), ptr(p)))
        bvh = Bvh(nodes, used.value)
        return (bvh, p) if perm else bvh

    def world(self, bodies, gens=None) -> "World":
        return World(self, bodies, gens)

    def triangles_intersect(self, tris: np.ndarray, rays: np.ndarray, mode: int = _lib.LIST_CLOSEST) -> np.ndarray:
        """Triangle::intersect (mode LIST_CLOSEST) or Triangle::intersect_mut (LIST_MUT) of every ray
        against a triangle list in index order, no BVH."""
        tris = np.ascontiguousarray(tris, np.float32).reshape(-1, 9)
        rays = np.ascontiguousarray(rays, RAY)
        hits = np.zeros(len(rays), HIT)
        self.check(self.lib.bvhgpu_triangles_intersect(self.h, ptr(tris), len(tris), ptr(rays), len(rays), mode,
                                                       ptr(hits)))
        return hits

    # ---- launch configuration / autotuning (bvhgpu_tune_*, bvhgpu_autotune) ----
    def tune_get(self, kernel: int) -> dict:
        c = np.zeros(1, _lib.TUNE_CONFIG)
        self.check(self.lib.bvhgpu_tune_get(self.h, kernel, ptr(c)))
        return {k: int(c[0][k]) for k in _lib.TUNE_CONFIG.names}

    def tune_set(self, kernel: int, **cfg):
        c = np.zeros(1, _lib.TUNE_CONFIG)
        cur = self.tune_get(kernel)
        cur.update(cfg)
        for k, v in cur.items():
            c[0][k] = v
        self.check(self.lib.bvhgpu_tune_set(self.h, kernel, ptr(c)))

    @staticmethod
    def tune_space(kernel: int) -> list:
        lib = _lib.load()
        n = ctypes.c_uint32()
        rc = lib.bvhgpu_tune_space(kernel, None, 0, ctypes.byref(n))
        if rc:
            raise _lib.BvhGpuError(rc, "tune_space")
        out = np.zeros(n.value, _lib.TUNE_CONFIG)
        lib.bvhgpu_tune_space(kernel, ptr(out), n.value, ctypes.byref(n))
        return [{k: int(r[k]) for k in _lib.TUNE_CONFIG.names} for r in out]

    def autotune(self, kernel: int, d_rays: "DeviceBuffer", n: int, d_hits0: "DeviceBuffer", d_hits1=None,
                 target: int = 0, seed: int = 0, items=None, reps: int = 3):
        """Runs bvhgpu_autotune on one call of `kernel`; returns (config dict, ms per call)."""
        job = _lib.TuneJob()
        job.kernel = kernel
        job.target = target
        job.d_rays = d_rays.ptr.value if isinstance(d_rays.ptr, ctypes.c_void_p) else d_rays.ptr
        job.n = n
        job.seed = seed
        job.d_hits0 = d_hits0.ptr.value if isinstance(d_hits0.ptr, ctypes.c_void_p) else d_hits0.ptr
        if d_hits1 is not None:
            job.d_hits1 = d_hits1.ptr.value if isinstance(d_hits1.ptr, ctypes.c_void_p) else d_hits1.ptr
        keep = None
        if items is not None:
            keep = np.ascontiguousarray(items, BATCH_ITEM)
            job.items = keep.ctypes.data
            job.nitems = len(keep)
        best = np.zeros(1, _lib.TUNE_CONFIG)
        ms = ctypes.c_float()
        self.check(self.lib.bvhgpu_autotune(self.h, ctypes.byref(job), reps, ptr(best), ctypes.byref(ms)))
        return {k: int(best[0][k]) for k in _lib.TUNE_CONFIG.names}, float(ms.value)


class World:
    """World (physics/world.rs): rigid bodies and force generators on the device."""

    def __init__(self, ctx: "Context", bodies, gens=None):
        self.ctx = ctx
        self.bodies = np.ascontiguousarray(bodies, _lib.RIGID_BODY)
        g = np.ascontiguousarray(gens if gens is not None else np.zeros(0, _lib.FORCE_GENERATOR),
                                 _lib.FORCE_GENERATOR)
        wid = ctypes.c_uint32()
        ctx.check(ctx.lib.bvhgpu_world_create(ctx.h, ptr(self.bodies), len(self.bodies), ptr(g), len(g),
                                              ctypes.byref(wid)))
        self.id = wid.value

    def start_frame_async(self, stream=None):
        self.ctx.check(self.ctx.lib.bvhgpu_world_start_frame_async(self.ctx.h, self.id, stream))

    def step_async(self, dt: float, stream=None):
        self.ctx.check(self.ctx.lib.bvhgpu_world_step_async(self.ctx.h, self.id, dt, stream))

    def download(self) -> np.ndarray:
        out = np.zeros(len(self.bodies), _lib.RIGID_BODY)
        self.ctx.check(self.ctx.lib.bvhgpu_world_download(self.ctx.h, self.id, ptr(out)))
        return out

    def free(self):
        if self.id:
            self.ctx.lib.bvhgpu_world_free(self.ctx.h, self.id)
            self.id = 0


def decode_mesh(data, fmt: int = _lib.MESH_TRI):
    """Decodes a `.tri` (MESH_TRI) or `.obj` (MESH_OBJ) mesh from text / bytes: returns
    (tris [n, 9], normals [n, 9], uvs [n, 6]) float32 (bvhgpu_mesh_decode)."""
    lib = _lib.load()
    raw = data.encode() if isinstance(data, str) else bytes(data)
    n = ctypes.c_uint32()
    err = ctypes.create_string_buffer(512)
    rc = lib.bvhgpu_mesh_decode(raw, len(raw), fmt, None, None, None, 0, ctypes.byref(n), err, 512)
    if rc:
        raise BvhGpuError(rc, err.value.decode(errors="replace"))
    tris = np.zeros((n.value, 9), np.float32)
    normals = np.zeros((n.value, 9), np.float32)
    uvs = np.zeros((n.value, 6), np.float32)
    rc = lib.bvhgpu_mesh_decode(raw, len(raw), fmt, ptr(tris), ptr(normals), ptr(uvs), n.value, ctypes.byref(n),
                                err, 512)
    if rc:
        raise BvhGpuError(rc, err.value.decode(errors="replace"))
    return tris, normals, uvs


def load_mesh(path: str):
    """decode_mesh of a file; the format from its extension (.tri / .obj)."""
    fmt = _lib.MESH_OBJ if str(path).lower().endswith(".obj") else _lib.MESH_TRI
    with open(path, "rb") as f:
        return decode_mesh(f.read(), fmt)


class DeviceBuffer:
    def __init__(self, ctx: Context, nbytes: int):
        self.ctx = ctx
        self.nbytes = int(nbytes)
        p = ctypes.c_void_p()
        ctx.check(ctx.lib.bvhgpu_device_alloc(ctx.h, max(self.nbytes, 16), ctypes.byref(p)))
        self.p = p

    @property
    def ptr(self):
        return self.p

    def upload(self, arr: np.ndarray, stream=None, sync: bool = True):
        arr = np.ascontiguousarray(arr)
        assert arr.nbytes <= self.nbytes
        self.ctx.check(self.ctx.lib.bvhgpu_copy_to_device(self.ctx.h, self.p, ptr(arr), arr.nbytes, stream))
        if sync:
            self.ctx.sync()

    def download(self, out: np.ndarray, stream=None, sync: bool = True) -> np.ndarray:
        assert out.flags.c_contiguous and out.nbytes <= self.nbytes
        self.ctx.check(self.ctx.lib.bvhgpu_copy_to_host(self.ctx.h, ptr(out), self.p, out.nbytes, stream))
        if sync:
            self.ctx.sync()
        return out

    def zero(self, stream=None):
        self.ctx.check(self.ctx.lib.bvhgpu_memset_device(self.ctx.h, self.p, 0, self.nbytes, stream))

    def free(self):
        if self.p:
            self.ctx.lib.bvhgpu_device_free(self.ctx.h, self.p)
            self.p = None

    def __del__(self):
        try:
            if self.ctx.h:
                self.free()
        except Exception:
            pass


class PinnedArray:
    """A numpy view over page-locked host memory (for asynchronous copies)."""

    def __init__(self, ctx: Context, shape, dtype):
        self.ctx = ctx
        dtype = np.dtype(dtype)
        n = int(np.prod(shape)) * dtype.itemsize
        p = ctypes.c_void_p()
        ctx.check(ctx.lib.bvhgpu_host_alloc(ctx.h, max(n, 16), ctypes.byref(p)))
        self.p = p
        buf = (ctypes.c_char * max(n, 16)).from_address(p.value)
        self.array = np.frombuffer(buf, dtype=np.uint8, count=n).view(dtype).reshape(shape)

    def free(self):
        if self.p:
            self.array = None
            self.ctx.lib.bvhgpu_host_free(self.ctx.h, self.p)
            self.p = None


class Event:
    def __init__(self, ctx: Context):
        self.ctx = ctx
        p = ctypes.c_void_p()
        ctx.check(ctx.lib.bvhgpu_event_create(ctx.h, ctypes.byref(p)))
        self.p = p

    def record(self, stream=None):
        self.ctx.check(self.ctx.lib.bvhgpu_event_record(self.ctx.h, self.p, stream))

    def elapsed_ms(self, later: "Event") -> float:
        ms = ctypes.c_float()
        self.ctx.check(self.ctx.lib.bvhgpu_event_elapsed_ms(self.ctx.h, self.p, later.p, ctypes.byref(ms)))
        return float(ms.value)


# ---- BVH build (host) -----------------------------------------------------------------------

class Bvh:
    """The reference's Bvh node array (bvh.rs:227-233): nodes[2n], nodes_used."""

    def __init__(self, nodes: np.ndarray, nodes_used: int):
        self.nodes = nodes
        self.nodes_used = int(nodes_used)

    def bounds(self):
        """Bvh::bounds (bvh.rs:499-501)."""
        return self.nodes[0]["bounds_min"].copy(), self.nodes[0]["bounds_max"].copy()


class BvhBuilder:
    """BvhBuilder::build_for (bvh.rs:524-541): SAH binned build on the host (8 bins)."""

    def build_for(self, mesh: np.ndarray) -> Bvh:
        """Builds the BVH and reorders ``mesh`` ([n, 9] float32, C-contiguous) in place."""
        if mesh.dtype != np.float32 or not mesh.flags.c_contiguous or mesh.ndim != 2 or mesh.shape[1] != 9:
            raise ValueError("mesh must be a C-contiguous float32 array of shape [n, 9]")
        n = mesh.shape[0]
        nodes = np.zeros(max(2 * n, 1), NODE)
        used = ctypes.c_uint32()
        lib = _lib.load()
        rc = lib.bvhgpu_build_bvh_host(ptr(mesh), n, ptr(nodes), ctypes.byref(used))
        if rc != 0:
            raise BvhGpuError(rc, "BvhBuilder::build_for: the reference build would panic on this mesh"
                              if rc == 6 else "bad mesh")
        return Bvh(nodes, used.value)


# ---- BLAS on the GPU --------------------------------------------------------------------------

class Blas:
    """A BVH + its triangles resident on the GPU: ModelInstance's intersect / refit."""

    def __init__(self, ctx: Context, bvh: Bvh, tris: np.ndarray):
        self.ctx = ctx
        tris = np.ascontiguousarray(tris, np.float32).reshape(-1, 9)
        nodes = np.ascontiguousarray(bvh.nodes[:bvh.nodes_used])
        bid = ctypes.c_uint32()
        ctx.check(ctx.lib.bvhgpu_blas_upload(ctx.h, ptr(nodes), bvh.nodes_used, ptr(tris), len(tris),
                                             ctypes.byref(bid)))
        self.id = bid.value
        self.nodes_used = bvh.nodes_used
        self.ntris = len(tris)
        nu, nt, depth = ctypes.c_uint32(), ctypes.c_uint32(), ctypes.c_uint32()
        ctx.check(ctx.lib.bvhgpu_blas_info(ctx.h, self.id, ctypes.byref(nu), ctypes.byref(nt), ctypes.byref(depth)))
        self.depth = depth.value

    def hidden(self) -> dict:
        """Size of the hidden trees under the large leaves: nodes, pairs, depth below the leaf."""
        n, p, d = ctypes.c_uint32(), ctypes.c_uint32(), ctypes.c_uint32()
        self.ctx.check(self.ctx.lib.bvhgpu_blas_hidden(self.ctx.h, self.id, ctypes.byref(n), ctypes.byref(p),
                                                       ctypes.byref(d)))
        return {"nodes": n.value, "pairs": p.value, "depth": d.value}

    def hidden_download(self) -> dict:
        """The hidden trees' device data (bvhgpu_blas_hidden_download): node records (n x 8 float32,
        `first` / `count` as their bits), cone records (m x 8), pair slots (pairs x 2 uint32) and the
        per-triangle table ((ntris + 1) & ~1 x 2 uint32)."""
        h = self.hidden()
        nc = ctypes.c_uint32()
        self.ctx.check(self.ctx.lib.bvhgpu_blas_hidden_download(self.ctx.h, self.id, None, None, None, None,
                                                                 ctypes.byref(nc)))
        ntris = self.ntris
        nodes = np.zeros((h["nodes"], 8), np.float32)
        cones = np.zeros((nc.value, 8), np.float32)
        slots = np.zeros((h["pairs"], 2), np.uint32)
        table = np.zeros(((ntris + 1) & ~1, 2), np.uint32)
        self.ctx.check(self.ctx.lib.bvhgpu_blas_hidden_download(self.ctx.h, self.id, ptr(nodes), ptr(cones), ptr(slots),
                                                                 ptr(table), ctypes.byref(nc)))
        return {"nodes": nodes, "cones": cones, "slots": slots, "table": table}

    TRACE_COUNT_NAMES = ("ref_nodes", "hidden_boxes", "hidden_entries", "hidden_pairs", "lane_tris", "warp_tris",
                         "cone_switches")

    def trace_counts(self, d_rays: "DeviceBuffer", n: int, d_hits: "DeviceBuffer") -> dict:
        """The plain traversal with work counters summed over the rays (bvhgpu_blas_trace_counts)."""
        out = (ctypes.c_uint64 * 7)()
        self.ctx.check(self.ctx.lib.bvhgpu_blas_trace_counts(self.ctx.h, self.id, d_rays.ptr, n, d_hits.ptr, out))
        return {k: int(v) for k, v in zip(self.TRACE_COUNT_NAMES, out)}

    def intersect(self, rays: np.ndarray) -> np.ndarray:
        """Bvh::intersect for every ray (host arrays in, host hits out)."""
        rays = np.ascontiguousarray(rays, RAY)
        hits = np.zeros(len(rays), HIT)
        self.ctx.check(self.ctx.lib.bvhgpu_blas_intersect(self.ctx.h, self.id, ptr(rays), len(rays), ptr(hits)))
        return hits

    def intersect_async(self, d_rays: DeviceBuffer, n: int, d_hits: DeviceBuffer, stream=None):
        self.ctx.check(self.ctx.lib.bvhgpu_blas_intersect_async(self.ctx.h, self.id, d_rays.ptr, n, d_hits.ptr,
                                                                stream))

    def trace_bounce(self, rays: np.ndarray, seed: int, mode: int):
        rays = np.ascontiguousarray(rays, RAY)
        h0 = np.zeros(len(rays), HIT)
        h1 = np.zeros(len(rays), HIT)
        nb = ctypes.c_uint32()
        self.ctx.check(self.ctx.lib.bvhgpu_blas_trace_bounce(self.ctx.h, self.id, ptr(rays), len(rays), seed, mode,
                                                             ptr(h0), ptr(h1), ctypes.byref(nb)))
        return h0, h1, nb.value

    def trace_bounce_async(self, d_rays, n, seed, mode, d_h0, d_h1, stream=None):
        self.ctx.check(self.ctx.lib.bvhgpu_blas_trace_bounce_async(self.ctx.h, self.id, d_rays.ptr, n, seed, mode,
                                                                   d_h0.ptr, d_h1.ptr, stream))

    def bounce_rays(self, rays: np.ndarray, seed: int):
        rays = np.ascontiguousarray(rays, RAY)
        out = np.zeros(len(rays), RAY)
        valid = np.zeros(len(rays), np.uint8)
        self.ctx.check(self.ctx.lib.bvhgpu_blas_bounce_rays(self.ctx.h, self.id, ptr(rays), len(rays), seed,
                                                            ptr(out), ptr(valid)))
        return out, valid.astype(bool)

    def update_vertices(self, tris: np.ndarray):
        tris = np.ascontiguousarray(tris, np.float32).reshape(-1, 9)
        assert len(tris) == self.ntris
        self.ctx.check(self.ctx.lib.bvhgpu_blas_update_vertices(self.ctx.h, self.id, ptr(tris)))

    def update_vertices_async(self, d_tris: DeviceBuffer, stream=None):
        self.ctx.check(self.ctx.lib.bvhgpu_blas_update_vertices_async(self.ctx.h, self.id, d_tris.ptr, stream))

    def refit(self):
        """Bvh::refit (bvh.rs:469-493) on the GPU."""
        self.ctx.check(self.ctx.lib.bvhgpu_blas_refit(self.ctx.h, self.id))

    def refit_async(self, stream=None):
        self.ctx.check(self.ctx.lib.bvhgpu_blas_refit_async(self.ctx.h, self.id, stream))

    def download_nodes(self) -> np.ndarray:
        out = np.zeros(self.nodes_used, NODE)
        self.ctx.check(self.ctx.lib.bvhgpu_blas_download_nodes(self.ctx.h, self.id, ptr(out)))
        return out

    def set_shading(self, normals=None, tex_coords=None, texels=None):
        """The model's shading data for scene renders: corner normals [ntris, 9], corner texture
        coordinates [ntris, 6] (BLAS triangle order), RGB8 texture [h, w, 3]; None keeps an array."""
        nrm = None if normals is None else np.ascontiguousarray(normals, np.float32).reshape(self.ntris, 9)
        tc = None if tex_coords is None else np.ascontiguousarray(tex_coords, np.float32).reshape(self.ntris, 6)
        tx = None if texels is None else np.ascontiguousarray(texels, np.uint8)
        th, tw = (0, 0) if tx is None else tx.shape[:2]
        self.ctx.check(self.ctx.lib.bvhgpu_blas_set_shading(self.ctx.h, self.id, ptr(nrm), ptr(tc), ptr(tx), tw, th))

    def render(self, camera: "Camera", width: int, height: int, accumulator: int, shader: int,
               acc_params=None, shader_params=None, normals=None):
        """PathTracer::evaluate on this BLAS: returns (rgba [h, w, 4] uint8, rays traced)."""
        cam = camera.to_struct()
        rgba = np.zeros((height, width, 4), np.uint8)
        ap = None if acc_params is None else np.ascontiguousarray(acc_params, np.float32)
        sp = None if shader_params is None else np.ascontiguousarray(shader_params, np.float32)
        nrm = None if normals is None else np.ascontiguousarray(normals, np.float32).reshape(-1, 9)
        rays = ctypes.c_uint64()
        self.ctx.check(self.ctx.lib.bvhgpu_render(self.ctx.h, self.id, ptr(cam), width, height, accumulator,
                                                  ptr(ap), shader, ptr(sp), ptr(nrm), ptr(rgba),
                                                  ctypes.byref(rays)))
        return rgba, rays.value

    def render_textured(self, camera: "Camera", width: int, height: int, tex_coords, texels, shader: int = 0,
                        shader_params=None):
        """TextureMaterialAccumulator + shader: tex_coords [n, 6] (per-corner u, v, in this BLAS's
        triangle order), texels [h, w, 3] uint8.  Returns (rgba [h, w, 4], rays traced)."""
        cam = camera.to_struct()
        rgba = np.zeros((height, width, 4), np.uint8)
        tc = np.ascontiguousarray(tex_coords, np.float32).reshape(-1, 6)
        tx = np.ascontiguousarray(texels, np.uint8)
        sp = None if shader_params is None else np.ascontiguousarray(shader_params, np.float32)
        rays = ctypes.c_uint64()
        self.ctx.check(self.ctx.lib.bvhgpu_render_textured(self.ctx.h, self.id, ptr(cam), width, height, ptr(tc),
                                                           ptr(tx), tx.shape[1], tx.shape[0], shader, ptr(sp),
                                                           ptr(rgba), ctypes.byref(rays)))
        return rgba, rays.value

    def free(self):
        if self.id:
            self.ctx.lib.bvhgpu_blas_free(self.ctx.h, self.id)
            self.id = 0


class Scene:
    """Scene over instanced BLASes with a GPU-rebuilt TLAS (scene.rs, tlas.rs, scene_object.rs)."""

    def __init__(self, ctx: Context, blases, transforms=None, inverses=None):
        self.ctx = ctx
        ids = np.ascontiguousarray([b.id for b in blases], np.uint32)
        sid = ctypes.c_uint32()
        ctx.check(ctx.lib.bvhgpu_scene_create(ctx.h, ptr(ids), len(ids), ctypes.byref(sid)))
        self.id = sid.value
        self.nobjects = len(ids)
        if transforms is not None:
            self.set_transforms(transforms, inverses)
            self.rebuild()

    def set_transforms(self, xf, inv):
        """SceneObject::set_transform for every object: 4x4 column-major transforms + inverses."""
        xf = np.ascontiguousarray(xf, np.float32).reshape(self.nobjects, 16)
        inv = np.ascontiguousarray(inv, np.float32).reshape(self.nobjects, 16)
        self.ctx.check(self.ctx.lib.bvhgpu_scene_set_transforms(self.ctx.h, self.id, ptr(xf), ptr(inv)))

    def set_transforms_async(self, d_xf: DeviceBuffer, d_inv: DeviceBuffer, stream=None):
        self.ctx.check(self.ctx.lib.bvhgpu_scene_set_transforms_async(self.ctx.h, self.id, d_xf.ptr, d_inv.ptr,
                                                                      stream))

    def rebuild(self):
        """Scene::rebuild (TLAS rebuild on the GPU)."""
        self.ctx.check(self.ctx.lib.bvhgpu_scene_rebuild(self.ctx.h, self.id))

    def rebuild_async(self, stream=None):
        self.ctx.check(self.ctx.lib.bvhgpu_scene_rebuild_async(self.ctx.h, self.id, stream))

    def trace_bounce_async(self, d_rays: DeviceBuffer, n: int, seed: int, d_hits0: DeviceBuffer,
                           d_hits1: DeviceBuffer, stream=None):
        self.ctx.check(self.ctx.lib.bvhgpu_scene_trace_bounce_async(self.ctx.h, self.id, d_rays.ptr, n, seed,
                                                                    d_hits0.ptr, d_hits1.ptr, stream))

    def bounce_rays(self, rays: np.ndarray, seed: int):
        rays = np.ascontiguousarray(rays, RAY)
        out = np.zeros(len(rays), RAY)
        valid = np.zeros(len(rays), np.uint8)
        self.ctx.check(self.ctx.lib.bvhgpu_scene_bounce_rays(self.ctx.h, self.id, ptr(rays), len(rays), seed,
                                                             ptr(out), ptr(valid)))
        return out, valid.astype(bool)

    def download_transforms(self):
        xf = np.zeros((self.nobjects, 16), np.float32)
        inv = np.zeros((self.nobjects, 16), np.float32)
        self.ctx.check(self.ctx.lib.bvhgpu_scene_download_transforms(self.ctx.h, self.id, ptr(xf), ptr(inv)))
        return xf, inv

    def animate_async(self, d_rot0, d_axis, d_omega, d_scale, d_trans, d_time, stream=None):
        self.ctx.check(self.ctx.lib.bvhgpu_scene_animate_async(self.ctx.h, self.id, d_rot0.ptr, d_axis.ptr,
                                                               d_omega.ptr, d_scale.ptr, d_trans.ptr, d_time.ptr,
                                                               stream))

    def bind_world(self, world: "World", body_of, transform_init):
        """Object i follows body body_of[i] (0xFFFFFFFF: none) from initial transform
        transform_init[i] (16 floats, column-major)."""
        bo = np.ascontiguousarray(body_of, np.uint32)
        ti = np.ascontiguousarray(transform_init, np.float32).reshape(-1, 16)
        self.ctx.check(self.ctx.lib.bvhgpu_scene_bind_world(self.ctx.h, self.id, world.id, ptr(bo), ptr(ti)))

    def run_async(self, dt: float, stream=None):
        """Scene::run(dt): physics step, object transforms from the bodies, TLAS rebuild."""
        self.ctx.check(self.ctx.lib.bvhgpu_scene_run_async(self.ctx.h, self.id, dt, stream))

    def download_tlas(self):
        nodes = np.zeros(2 * self.nobjects, TLAS_NODE)
        used = ctypes.c_uint32()
        self.ctx.check(self.ctx.lib.bvhgpu_scene_download_tlas(self.ctx.h, self.id, ptr(nodes), ctypes.byref(used)))
        return nodes, used.value

    def intersect(self, rays: np.ndarray) -> np.ndarray:
        rays = np.ascontiguousarray(rays, RAY)
        hits = np.zeros(len(rays), HIT)
        self.ctx.check(self.ctx.lib.bvhgpu_scene_intersect(self.ctx.h, self.id, ptr(rays), len(rays), ptr(hits)))
        return hits

    def intersect_async(self, d_rays: DeviceBuffer, n: int, d_hits: DeviceBuffer, stream=None):
        self.ctx.check(self.ctx.lib.bvhgpu_scene_intersect_async(self.ctx.h, self.id, d_rays.ptr, n, d_hits.ptr,
                                                                 stream))

    def render(self, camera: "Camera", width: int, height: int, accumulator: int, shader: int,
               acc_params=None, shader_params=None, lookup: int = _lib.LOOKUP_REFERENCE):
        """PathTracer::evaluate over the whole scene (Renderer::render with a Scene): returns (rgba
        [h, w, 4] uint8, rays traced).  The normal / texture accumulators read the shading data set
        with Blas.set_shading; `lookup` picks the reference's instance-0 lookup or the hit's object."""
        cam = camera.to_struct()
        rgba = np.zeros((height, width, 4), np.uint8)
        ap = None if acc_params is None else np.ascontiguousarray(acc_params, np.float32)
        sp = None if shader_params is None else np.ascontiguousarray(shader_params, np.float32)
        rays = ctypes.c_uint64()
        self.ctx.check(self.ctx.lib.bvhgpu_render_scene(self.ctx.h, self.id, ptr(cam), width, height, accumulator,
                                                        ptr(ap), shader, ptr(sp), lookup, ptr(rgba),
                                                        ctypes.byref(rays)))
        return rgba, rays.value

    def free(self):
        if self.id:
            self.ctx.lib.bvhgpu_scene_free(self.ctx.h, self.id)
            self.id = 0


# ---- differentiable Lambertian render ------------------------------------------------------------

class DiffMesh:
    """Indexed mesh for the differentiable Lambertian render: a BLAS built by the reference's SAH
    build over the mesh's triangles, the face list permuted the way that build reordered the
    triangles, and device vertices / shading normals."""

    def __init__(self, ctx: Context, verts: np.ndarray, faces: np.ndarray, vnormals: np.ndarray):
        self.ctx = ctx
        verts = np.ascontiguousarray(verts, np.float32).reshape(-1, 3)
        faces = np.ascontiguousarray(faces, np.uint32).reshape(-1, 3)
        vnormals = np.ascontiguousarray(vnormals, np.float32).reshape(-1, 3)
        tris = np.ascontiguousarray(verts[faces].reshape(-1, 9), np.float32)
        n = len(tris)
        nodes = np.zeros(2 * n, NODE)
        perm = np.zeros(n, np.uint32)
        used = ctypes.c_uint32()
        rc = ctx.lib.bvhgpu_build_bvh_host_indexed(ptr(tris), n, ptr(nodes), ctypes.byref(used), ptr(perm))
        if rc != 0:
            raise BvhGpuError(rc, "build of the mesh's BVH failed")
        self.bvh = Bvh(nodes, used.value)
        self.tris = tris
        self.faces = np.ascontiguousarray(faces[perm], np.uint32)
        self.nverts = len(verts)
        self.blas = Blas(ctx, self.bvh, tris)
        mid = ctypes.c_uint32()
        ctx.check(ctx.lib.bvhgpu_mesh_create(ctx.h, self.blas.id, ptr(self.faces), n, ptr(verts), ptr(vnormals),
                                             self.nverts, ctypes.byref(mid)))
        self.id = mid.value

    def set_vertices(self, verts: np.ndarray):
        verts = np.ascontiguousarray(verts, np.float32).reshape(self.nverts, 3)
        self.ctx.check(self.ctx.lib.bvhgpu_mesh_set_vertices(self.ctx.h, self.id, ptr(verts)))

    def vertices(self) -> np.ndarray:
        p = ctypes.c_void_p()
        self.ctx.check(self.ctx.lib.bvhgpu_mesh_vertices(self.ctx.h, self.id, ctypes.byref(p)))
        out = np.zeros((self.nverts, 3), np.float32)
        self.ctx.sync()
        self.ctx.check(self.ctx.lib.bvhgpu_copy_to_host(self.ctx.h, ptr(out), p, out.nbytes, None))
        self.ctx.sync()
        return out

    def update_async(self, stream=None):
        self.ctx.check(self.ctx.lib.bvhgpu_mesh_update_async(self.ctx.h, self.id, stream))

    def checkpoint(self, path: str, step: int, losses=(), lr: float | None = None):
        """Saves the descent state: the device vertices, the step count and the loss history."""
        save_descent_state(path, self.vertices(), step, losses, lr)

    def resume(self, path: str) -> dict:
        """Restores the vertices of a checkpoint (and refits the BLAS); returns the checkpoint."""
        state = load_descent_state(path)
        self.set_vertices(state["verts"])
        return state

    def forward_async(self, d_rays: DeviceBuffer, n: int, light, d_image: DeviceBuffer, d_hits: DeviceBuffer,
                      stream=None):
        L = np.ascontiguousarray(light, np.float32)
        self.ctx.check(self.ctx.lib.bvhgpu_lambert_forward_async(self.ctx.h, self.id, d_rays.ptr, n, ptr(L),
                                                                 d_image.ptr, d_hits.ptr, stream))

    def adjoint_async(self, d_rays: DeviceBuffer, n: int, light, d_hits: DeviceBuffer, d_image: DeviceBuffer,
                      d_target: DeviceBuffer, d_grad: DeviceBuffer, stream=None):
        L = np.ascontiguousarray(light, np.float32)
        self.ctx.check(self.ctx.lib.bvhgpu_lambert_adjoint_async(self.ctx.h, self.id, d_rays.ptr, n, ptr(L),
                                                                 d_hits.ptr, d_image.ptr, d_target.ptr, d_grad.ptr,
                                                                 stream))

    def wobble_async(self, d_dirs: DeviceBuffer, d_r0: DeviceBuffer, d_phase: DeviceBuffer, amp: float,
                     freq: float, d_time: DeviceBuffer, stream=None):
        self.ctx.check(self.ctx.lib.bvhgpu_mesh_wobble_async(self.ctx.h, self.id, d_dirs.ptr, d_r0.ptr, d_phase.ptr,
                                                             float(amp), float(freq), d_time.ptr, stream))

    def sgd_step_async(self, d_grad: DeviceBuffer, lr: float, stream=None):
        self.ctx.check(self.ctx.lib.bvhgpu_mesh_sgd_step_async(self.ctx.h, self.id, d_grad.ptr, float(lr), stream))


def save_descent_state(path: str, verts: np.ndarray, step: int, losses=(), lr: float | None = None):
    """Checkpoint of a gradient descent on a mesh's vertices: the vertices (float32 [nverts, 3]), the
    number of steps taken, the loss history and the learning rate, written to `path` (.npz) through a
    temporary file and a rename, so an interrupted write never leaves a partial checkpoint."""
    tmp = f"{path}.tmp{os.getpid()}.npz"
    np.savez(tmp, verts=np.ascontiguousarray(verts, np.float32), step=np.int64(step),
             losses=np.asarray(list(losses), np.float64), lr=np.float64(np.nan if lr is None else lr))
    os.replace(tmp, path)


def load_descent_state(path: str) -> dict:
    """The checkpoint written by save_descent_state: {verts, step, losses, lr}."""
    with np.load(path) as d:
        lr = float(d["lr"])
        return {"verts": d["verts"].astype(np.float32), "step": int(d["step"]),
                "losses": [float(x) for x in d["losses"]], "lr": None if np.isnan(lr) else lr}


def mse_loss(ctx: Context, d_image: DeviceBuffer, d_target: DeviceBuffer, n: int) -> float:
    loss = ctypes.c_double()
    ctx.check(ctx.lib.bvhgpu_mse_loss(ctx.h, d_image.ptr, d_target.ptr, n, ctypes.byref(loss)))
    return loss.value


# ---- camera ---------------------------------------------------------------------------------

CAMERA = np.dtype([("top_left", "<f4", 3), ("top_right", "<f4", 3), ("bottom_left", "<f4", 3),
                   ("view_inv", "<f4", 16)])


class Camera:
    """Camera<f32, PerspectiveProjection> reduced to what get_ray_world needs (camera.rs:994-1010).

    ``box_spec`` = (left, right, bottom, top, near, far) as BoxSpec (camera.rs:343-368);
    attitude = position, forward, right, up (CameraAttitudeSpec, camera.rs:652-700).
    view_matrix_inv is the inverse of rotation * translation(-position) (camera.rs:809-834),
    computed in float64 and rounded to float32.
    """

    def __init__(self, box_spec, position, forward, right, up):
        left, rgt, bottom, top, near, _far = [np.float32(x) for x in box_spec]
        ext_x = rgt - left
        ext_y = top - bottom
        self.top_left = np.array([left, top, -near], np.float32)
        self.top_right = np.array([left + ext_x, top, -near], np.float32)
        self.bottom_left = np.array([left, top - ext_y, -near], np.float32)
        r = np.asarray(right, np.float64)
        u = np.asarray(up, np.float64)
        f = np.asarray(forward, np.float64)
        p = np.asarray(position, np.float64)
        rot = np.eye(4)
        rot[0, :3], rot[1, :3], rot[2, :3] = r, u, -f     # rows: right, up, -forward
        trans = np.eye(4)
        trans[:3, 3] = -p
        view = rot @ trans
        inv = np.linalg.inv(view)
        self.view_inv = np.ascontiguousarray(inv.T.astype(np.float32)).reshape(16)  # column-major

    @staticmethod
    def symmetric_fov(fovy_deg, aspect, near, far, position, forward, right, up) -> "Camera":
        """SymmetricFovSpec -> frustum (camera.rs:219-252)."""
        top = np.float32(near) * np.float32(np.tan(np.radians(fovy_deg) / 2.0))
        right_x = np.float32(aspect) * top
        return Camera((-right_x, right_x, -top, top, near, far), position, forward, right, up)

    def corners(self) -> np.ndarray:
        return np.concatenate([self.top_left, self.top_right, self.bottom_left]).astype(np.float32)

    def to_struct(self) -> np.ndarray:
        s = np.zeros(1, CAMERA)
        s["top_left"] = self.top_left
        s["top_right"] = self.top_right
        s["bottom_left"] = self.bottom_left
        s["view_inv"] = self.view_inv
        return s


__all__ = ["Context", "DeviceBuffer", "PinnedArray", "Event", "Bvh", "BvhBuilder", "Blas", "Scene", "Camera",
           "DiffMesh", "mse_loss",
           "RAY", "HIT", "NODE", "TLAS_NODE", "BATCH_ITEM", "MISS", "FLT_MAX"]
