"""bvhtracer_gb300: the ray-BVH hot path of lambdaxymox/bvhtracer on one GB300 (sm_103a).

The compute path is the CUDA library ``libbvhgpu.so`` (C ABI in include/bvhgpu.h);
this package is its host-side mirror of the reference's interface (see ``api``) plus
the seeded synthetic workloads (``scenes``).
"""
from . import scenes  # noqa: F401
from .api import (BATCH_ITEM, FLT_MAX, HIT, MISS, NODE, RAY, TLAS_NODE, Blas, Bvh, BvhBuilder, Camera, Context,
                  DeviceBuffer, DiffMesh, Event, PinnedArray, Scene, World, decode_mesh, load_descent_state,
                  load_mesh, mse_loss, save_descent_state)
from ._lib import (ACC_DEPTH, ACC_INTERSECTION, ACC_NORMAL, ACC_TEXTURE, ACC_UV, BIG_LEAF_NEVER, LIST_CLOSEST, LIST_MUT,
                   LOOKUP_HIT_OBJECT, LOOKUP_REFERENCE, ERR_DEADLINE, MESH_OBJ, MESH_TRI, MODE_PERSISTENT, MODE_PLAIN, RIGID_BODY, FORCE_GENERATOR, FORCE_GRAVITY,
                   FORCE_SPRING, rigid_body_default,
                   SHADER_DEPTH, SHADER_INTERSECTION, SHADER_RADIANCE, BvhGpuError)
from ._lib import KERNELS as _KERNELS

# kernel ids (BVHGPU_K_*) of the tunable traversal kernels
K_TRACE_BLAS = _KERNELS.index("trace_blas")
K_TRACE_SCENE = _KERNELS.index("trace_scene")
K_PERSISTENT_BOUNCE = _KERNELS.index("persistent_bounce")
K_TRACE_BATCH = _KERNELS.index("trace_batch")
K_SCENE_BOUNCE = _KERNELS.index("scene_bounce")

__all__ = ["Context", "DeviceBuffer", "PinnedArray", "Event", "Bvh", "BvhBuilder", "Blas", "Scene", "Camera",
           "DiffMesh", "mse_loss", "save_descent_state", "load_descent_state",
           "RAY", "HIT", "NODE", "TLAS_NODE", "BATCH_ITEM", "MISS", "FLT_MAX", "BvhGpuError",
           "ACC_INTERSECTION", "ACC_DEPTH", "ACC_UV", "ACC_NORMAL", "ACC_TEXTURE", "SHADER_RADIANCE", "SHADER_INTERSECTION",
           "SHADER_DEPTH", "MODE_PLAIN", "MODE_PERSISTENT", "LOOKUP_REFERENCE", "LOOKUP_HIT_OBJECT", "ERR_DEADLINE", "BIG_LEAF_NEVER", "LIST_CLOSEST", "LIST_MUT", "MESH_TRI", "MESH_OBJ", "decode_mesh", "load_mesh", "World", "RIGID_BODY", "FORCE_GENERATOR", "FORCE_GRAVITY", "FORCE_SPRING",
           "rigid_body_default", "K_TRACE_BLAS", "K_TRACE_SCENE",
           "K_PERSISTENT_BOUNCE", "K_TRACE_BATCH", "K_SCENE_BOUNCE"]
