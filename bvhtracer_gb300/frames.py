"""Animated instanced frames (the per-frame pattern of the reference's demos: refit the animated
models, rebuild the TLAS, render), run on the GPU and captured as one CUDA graph.

Per frame: the time in device memory advances by dt; every mesh's vertices wobble radially and its
BLAS is regenerated and refit (ModelInstance::refit, BT/src/model/model.rs:31-33); every instance
turns about its axis (SceneObject::set_transform, BT/src/scene/scene_object.rs:60-75); the TLAS is
rebuilt (Scene::rebuild, BT/src/scene/scene.rs:36-38); then the camera's primaries and one diffuse
bounce per hit are traced in one persistent launch.  After capture() the whole frame is a single
graph launch.
"""
from __future__ import annotations

import numpy as np

from .api import HIT, Context, DiffMesh


class AnimatedScene:
    def __init__(self, ctx: Context, cfg: dict, bounce_seed: int = 12345):
        self.ctx = ctx
        self.cfg = cfg
        self.seed = bounce_seed
        self.meshes = [DiffMesh(ctx, m["verts"], m["faces"], m["dirs"]) for m in cfg["meshes"]]
        self.mesh_bufs = [(ctx.to_device(m["dirs"]), ctx.to_device(m["r0"]), ctx.to_device(m["phase"]))
                          for m in cfg["meshes"]]
        inst = cfg["instances"]
        self.blas_of = inst["blas_of"]
        self.scene = ctx.scene([self.meshes[b].blas for b in self.blas_of])
        self.inst_bufs = [ctx.to_device(np.ascontiguousarray(inst[k], np.float32))
                          for k in ("rot0", "axis", "omega", "scale", "trans")]
        self.d_time = ctx.to_device(np.zeros(1, np.float32))
        self.rays = cfg["rays"]
        self.n = len(self.rays)
        self.d_rays = ctx.to_device(self.rays)
        self.d_hits0 = ctx.device_buffer(self.n * HIT.itemsize)
        self.d_hits1 = ctx.device_buffer(self.n * HIT.itemsize)
        self.graph = None

    def set_time(self, t: float):
        self.d_time.upload(np.array([t], np.float32))

    def frame_async(self):
        ctx, cfg = self.ctx, self.cfg
        ctx.advance_time_async(self.d_time, cfg["dt"])
        for mesh, (d_dirs, d_r0, d_phase) in zip(self.meshes, self.mesh_bufs):
            mesh.wobble_async(d_dirs, d_r0, d_phase, cfg["amp"], cfg["freq"], self.d_time)
            mesh.update_async()
        self.scene.animate_async(*self.inst_bufs, self.d_time)
        self.scene.rebuild_async()
        self.scene.trace_bounce_async(self.d_rays, self.n, self.seed, self.d_hits0, self.d_hits1)

    def capture(self):
        self.ctx.graph_begin()
        self.frame_async()
        self.graph = self.ctx.graph_end()
        return self.graph

    def launch(self):
        self.ctx.graph_launch(self.graph)

    def hits(self):
        h0 = self.d_hits0.download(np.zeros(self.n, HIT))
        h1 = self.d_hits1.download(np.zeros(self.n, HIT))
        return h0, h1
