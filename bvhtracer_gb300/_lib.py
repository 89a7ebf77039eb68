"""ctypes binding of the bvhgpu C ABI (include/bvhgpu.h).

The library is the in-tree ``bvhtracer_gb300/_build/libbvhgpu.so`` built by
``bvhtracer_gb300.build``.  There is no CPU fallback: if the library is missing
or no CUDA device is present, the calls raise.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build

NODE = np.dtype([("bounds_min", "<f4", 3), ("bounds_max", "<f4", 3),
                 ("primitive_count", "<u4"), ("left_first", "<u4")])
RAY = np.dtype([("origin", "<f4", 3), ("t", "<f4"), ("direction", "<f4", 3), ("reserved", "<u4")])
HIT = np.dtype([("t", "<f4"), ("u", "<f4"), ("v", "<f4"), ("prim", "<u4"), ("inst", "<u4")])
TLAS_NODE = np.dtype([("bounds_min", "<f4", 3), ("bounds_max", "<f4", 3),
                      ("left_right", "<u4"), ("blas", "<u4")])
BATCH_ITEM = np.dtype([("blas", "<u4"), ("ray_offset", "<u4"), ("ray_count", "<u4"), ("reserved", "<u4")])
assert NODE.itemsize == 32 and RAY.itemsize == 32 and HIT.itemsize == 20
assert TLAS_NODE.itemsize == 32 and BATCH_ITEM.itemsize == 16
TUNE_CONFIG = np.dtype([("block", "<u4"), ("min_blocks", "<u4"), ("stack", "<u4"), ("big_leaf", "<u4"),
                        ("refill", "<u4"), ("hidden", "<u4")])
BIG_LEAF_NEVER = 0xFFFFFFFF
RIGID_BODY = np.dtype([("inverse_mass", "<f4"), ("inverse_inertia", "<f4", 9), ("linear_drag", "<f4"),
                       ("angular_drag", "<f4"), ("position", "<f4", 3), ("orientation", "<f4", 4),
                       ("velocity", "<f4", 3), ("rotation", "<f4", 3), ("inverse_inertia_world", "<f4", 9),
                       ("motion", "<f4"), ("is_awake", "<u4"), ("can_sleep", "<u4"), ("transform", "<f4", 16),
                       ("force_accum", "<f4", 3), ("torque_accum", "<f4", 3), ("acceleration", "<f4", 3),
                       ("last_frame_acceleration", "<f4", 3)])
FORCE_GENERATOR = np.dtype([("kind", "<u4"), ("body", "<u4"), ("other", "<u4"), ("reserved", "<u4"),
                            ("gravity", "<f4", 3), ("spring_point", "<f4", 3), ("other_point", "<f4", 3),
                            ("spring_constant", "<f4"), ("rest_length", "<f4")])
assert RIGID_BODY.itemsize == 260 and FORCE_GENERATOR.itemsize == 60
FORCE_GRAVITY, FORCE_SPRING = 0, 1


def rigid_body_default(n=1):
    """RigidBody::default (physics/rigid_body.rs:98-122): inverse mass f32::MAX, identity inertia,
    drag 1, orientation unit_z, asleep, can sleep, identity transform."""
    b = np.zeros(n, RIGID_BODY)
    b["inverse_mass"] = np.finfo(np.float32).max
    b["inverse_inertia"] = np.eye(3, dtype=np.float32).reshape(9)
    b["inverse_inertia_world"] = np.eye(3, dtype=np.float32).reshape(9)
    b["linear_drag"] = b["angular_drag"] = 1.0
    b["orientation"] = (0.0, 0.0, 0.0, 1.0)
    b["can_sleep"] = 1
    b["transform"] = np.eye(4, dtype=np.float32).reshape(16)
    return b


class TuneJob(ctypes.Structure):
    """bvhgpu_tune_job."""
    _fields_ = [("kernel", ctypes.c_int), ("target", ctypes.c_uint32), ("d_rays", ctypes.c_void_p),
                ("n", ctypes.c_uint32), ("seed", ctypes.c_uint32), ("d_hits0", ctypes.c_void_p),
                ("d_hits1", ctypes.c_void_p), ("items", ctypes.c_void_p), ("nitems", ctypes.c_uint32)]


MISS = 0xFFFFFFFF
FLT_MAX = np.float32(np.finfo(np.float32).max)

OK = 0
ERRORS = {1: "invalid argument", 2: "out of memory", 3: "CUDA error", 4: "stack depth exceeded",
          5: "step cap exceeded", 6: "build would panic", 7: "no CUDA device",
          8: "input larger than the entry point's fixed maximum", 9: "launch stopped at the deadline"}
ERR_DEADLINE = 9

ACC_INTERSECTION, ACC_DEPTH, ACC_UV, ACC_NORMAL, ACC_TEXTURE = 0, 1, 2, 3, 4
SHADER_RADIANCE, SHADER_INTERSECTION, SHADER_DEPTH = 0, 1, 2
MODE_PLAIN, MODE_PERSISTENT = 0, 1
LOOKUP_REFERENCE, LOOKUP_HIT_OBJECT = 0, 1
LIST_CLOSEST, LIST_MUT = 0, 1
MESH_TRI, MESH_OBJ = 0, 1

KERNELS = ["trace_blas", "trace_scene", "persistent_bounce", "bounce_gen", "trace_queue", "trace_batch",
           "refit", "tlas_build", "render", "other", "lambert_forward", "lambert_adjoint", "scene_bounce"]

# Exported symbols and their ctypes signatures (kept in the order of include/bvhgpu.h).
_P = ctypes.c_void_p
_U32 = ctypes.c_uint32
_I = ctypes.c_int
_SZ = ctypes.c_size_t
SIGNATURES = {
    "bvhgpu_create": (_I, [_P, _I]),
    "bvhgpu_destroy": (_I, [_P]),
    "bvhgpu_last_error": (ctypes.c_char_p, [_P]),
    "bvhgpu_launch_count": (ctypes.c_uint64, []),
    "bvhgpu_sync": (_I, [_P]),
    "bvhgpu_get_stream": (_P, [_P]),
    "bvhgpu_device_alloc": (_I, [_P, _SZ, _P]),
    "bvhgpu_device_free": (_I, [_P, _P]),
    "bvhgpu_host_alloc": (_I, [_P, _SZ, _P]),
    "bvhgpu_host_free": (_I, [_P, _P]),
    "bvhgpu_copy_to_device": (_I, [_P, _P, _P, _SZ, _P]),
    "bvhgpu_copy_to_host": (_I, [_P, _P, _P, _SZ, _P]),
    "bvhgpu_memset_device": (_I, [_P, _P, _I, _SZ, _P]),
    "bvhgpu_flush_l2": (_I, [_P, _P]),
    "bvhgpu_event_create": (_I, [_P, _P]),
    "bvhgpu_event_destroy": (_I, [_P, _P]),
    "bvhgpu_event_record": (_I, [_P, _P, _P]),
    "bvhgpu_event_elapsed_ms": (_I, [_P, _P, _P, _P]),
    "bvhgpu_profile_enable": (_I, [_P, _I]),
    "bvhgpu_profile_read": (_I, [_P, _P, _P]),
    "bvhgpu_build_bvh_host": (_I, [_P, _U32, _P, _P]),
    "bvhgpu_build_bvh_host_indexed": (_I, [_P, _U32, _P, _P, _P]),
    "bvhgpu_blas_upload": (_I, [_P, _P, _U32, _P, _U32, _P]),
    "bvhgpu_blas_free": (_I, [_P, _U32]),
    "bvhgpu_blas_info": (_I, [_P, _U32, _P, _P, _P]),
    "bvhgpu_blas_hidden": (_I, [_P, _U32, _P, _P, _P]),
    "bvhgpu_blas_hidden_download": (_I, [_P, _U32, _P, _P, _P, _P, _P]),
    "bvhgpu_set_deadline": (_I, [_P, ctypes.c_uint64]),
    "bvhgpu_blas_trace_counts": (_I, [_P, _U32, _P, _U32, _P, _P]),
    "bvhgpu_blas_update_vertices": (_I, [_P, _U32, _P]),
    "bvhgpu_blas_update_vertices_async": (_I, [_P, _U32, _P, _P]),
    "bvhgpu_blas_refit": (_I, [_P, _U32]),
    "bvhgpu_blas_refit_async": (_I, [_P, _U32, _P]),
    "bvhgpu_blas_download_nodes": (_I, [_P, _U32, _P]),
    "bvhgpu_blas_intersect": (_I, [_P, _U32, _P, _U32, _P]),
    "bvhgpu_blas_intersect_async": (_I, [_P, _U32, _P, _U32, _P, _P]),
    "bvhgpu_blas_trace_bounce": (_I, [_P, _U32, _P, _U32, _U32, _I, _P, _P, _P]),
    "bvhgpu_blas_trace_bounce_async": (_I, [_P, _U32, _P, _U32, _U32, _I, _P, _P, _P]),
    "bvhgpu_blas_bounce_rays": (_I, [_P, _U32, _P, _U32, _U32, _P, _P]),
    "bvhgpu_trace_batch": (_I, [_P, _P, _U32, _P, _U32, _I, _P]),
    "bvhgpu_trace_batch_async": (_I, [_P, _P, _U32, _P, _U32, _I, _P, _P]),
    "bvhgpu_scene_create": (_I, [_P, _P, _U32, _P]),
    "bvhgpu_scene_free": (_I, [_P, _U32]),
    "bvhgpu_scene_set_transforms": (_I, [_P, _U32, _P, _P]),
    "bvhgpu_scene_set_transforms_async": (_I, [_P, _U32, _P, _P, _P]),
    "bvhgpu_scene_rebuild": (_I, [_P, _U32]),
    "bvhgpu_scene_rebuild_async": (_I, [_P, _U32, _P]),
    "bvhgpu_scene_download_tlas": (_I, [_P, _U32, _P, _P]),
    "bvhgpu_scene_intersect": (_I, [_P, _U32, _P, _U32, _P]),
    "bvhgpu_scene_intersect_async": (_I, [_P, _U32, _P, _U32, _P, _P]),
    "bvhgpu_scene_trace_bounce_async": (_I, [_P, _U32, _P, _U32, _U32, _P, _P, _P]),
    "bvhgpu_scene_bounce_rays": (_I, [_P, _U32, _P, _U32, _U32, _P, _P]),
    "bvhgpu_scene_download_transforms": (_I, [_P, _U32, _P, _P]),
    "bvhgpu_mesh_wobble_async": (_I, [_P, _U32, _P, _P, _P, ctypes.c_float, ctypes.c_float, _P, _P]),
    "bvhgpu_scene_animate_async": (_I, [_P, _U32, _P, _P, _P, _P, _P, _P, _P]),
    "bvhgpu_advance_time_async": (_I, [_P, _P, ctypes.c_float, _P]),
    "bvhgpu_graph_begin": (_I, [_P]),
    "bvhgpu_graph_end": (_I, [_P, _P]),
    "bvhgpu_graph_launch": (_I, [_P, _U32]),
    "bvhgpu_graph_free": (_I, [_P, _U32]),
    "bvhgpu_render": (_I, [_P, _U32, _P, _I, _I, _I, _P, _I, _P, _P, _P, _P]),
    "bvhgpu_render_textured": (_I, [_P, _U32, _P, _I, _I, _P, _P, _U32, _U32, _I, _P, _P, _P]),
    "bvhgpu_blas_set_shading": (_I, [_P, _U32, _P, _P, _P, _U32, _U32]),
    "bvhgpu_render_scene": (_I, [_P, _U32, _P, _I, _I, _I, _P, _I, _P, _I, _P, _P]),
    "bvhgpu_mesh_create": (_I, [_P, _U32, _P, _U32, _P, _P, _U32, _P]),
    "bvhgpu_mesh_free": (_I, [_P, _U32]),
    "bvhgpu_mesh_vertices": (_I, [_P, _U32, _P]),
    "bvhgpu_mesh_set_vertices": (_I, [_P, _U32, _P]),
    "bvhgpu_mesh_update_async": (_I, [_P, _U32, _P]),
    "bvhgpu_lambert_forward_async": (_I, [_P, _U32, _P, _U32, _P, _P, _P, _P]),
    "bvhgpu_mse_loss": (_I, [_P, _P, _P, _U32, _P]),
    "bvhgpu_lambert_adjoint_async": (_I, [_P, _U32, _P, _U32, _P, _P, _P, _P, _P, _P]),
    "bvhgpu_mesh_sgd_step_async": (_I, [_P, _U32, _P, ctypes.c_float, _P]),
    "bvhgpu_mesh_decode": (_I, [ctypes.c_char_p, _SZ, _I, _P, _P, _P, _U32, _P, ctypes.c_char_p, _SZ]),
    "bvhgpu_mesh_decode_file": (_I, [ctypes.c_char_p, _I, _P, _P, _P, _U32, _P, ctypes.c_char_p, _SZ]),
    "bvhgpu_build_bvh_device": (_I, [_P, _P, _U32, _P, _P, _P]),
    "bvhgpu_blas_build": (_I, [_P, _P, _U32, _P]),
    "bvhgpu_triangles_intersect": (_I, [_P, _P, _U32, _P, _U32, _I, _P]),
    "bvhgpu_triangles_intersect_async": (_I, [_P, _P, _U32, _P, _U32, _I, _P, _P]),
    "bvhgpu_tune_get": (_I, [_P, _I, _P]),
    "bvhgpu_tune_set": (_I, [_P, _I, _P]),
    "bvhgpu_tune_space": (_I, [_I, _P, _U32, _P]),
    "bvhgpu_autotune": (_I, [_P, _P, _U32, _P, _P]),
    "bvhgpu_world_create": (_I, [_P, _P, _U32, _P, _U32, _P]),
    "bvhgpu_world_free": (_I, [_P, _U32]),
    "bvhgpu_world_start_frame_async": (_I, [_P, _U32, _P]),
    "bvhgpu_world_step_async": (_I, [_P, _U32, ctypes.c_float, _P]),
    "bvhgpu_world_download": (_I, [_P, _U32, _P]),
    "bvhgpu_scene_bind_world": (_I, [_P, _U32, _U32, _P, _P]),
    "bvhgpu_scene_run_async": (_I, [_P, _U32, ctypes.c_float, _P]),
    "bvhgpu_refit_noalloc": (_I, [_P, _U32, _P, _U32, _P, _P]),
}

_lib = None


def load(build_if_missing: bool = True):
    """Load libbvhgpu.so (building it in-tree first if it is missing or stale)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if build_if_missing and not _build.up_to_date():
        _build.build()
    if not os.path.exists(path):
        raise RuntimeError(f"libbvhgpu.so not found at {path}; run bvhtracer_gb300.build.build()")
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def ptr(a):
    if a is None:
        return None
    if isinstance(a, int):
        return ctypes.c_void_p(a)
    return a.ctypes.data_as(ctypes.c_void_p)


class BvhGpuError(RuntimeError):
    def __init__(self, code, message):
        super().__init__(f"bvhgpu error {code} ({ERRORS.get(code, '?')}): {message}")
        self.code = code
