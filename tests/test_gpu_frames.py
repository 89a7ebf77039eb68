"""Animated instanced frames captured in a CUDA graph (the instanced-animation workload's pattern) against the oracle on
the frame's own state: refit nodes, TLAS, primary hits, bounce rays and bounce hits all
bit-identical."""
import numpy as np
import pytest

import bvhtracer_gb300 as bt
from bvhtracer_gb300 import scenes
from bvhtracer_gb300.frames import AnimatedScene
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


def test_animated_frames_in_a_graph_match_the_oracle():
    cfg = scenes.instanced_animation(seed=2, ninstances=48, width=256, height=144)
    with bt.Context(0) as ctx:
        sc = AnimatedScene(ctx, cfg)
        initial = [(m.bvh.nodes.copy(), m.bvh.nodes_used) for m in sc.meshes]
        sc.capture()
        for _ in range(3):
            sc.launch()
        ctx.sync()
        h0, h1 = sc.hits()
        blases = []
        for m, (nodes0, used) in zip(sc.meshes, initial):
            verts = m.vertices()
            tris = np.ascontiguousarray(verts[m.faces].reshape(-1, 9), np.float32)
            gpu_nodes = m.blas.download_nodes()
            ref_nodes = orc.bvh_refit(nodes0, used, tris)[:used]
            assert gpu_nodes.tobytes() == ref_nodes.tobytes(), "refit differs"
            blases.append((ref_nodes, used, tris))
        xf, inv = sc.scene.download_transforms()
        tlas, tused = sc.scene.download_tlas()
        n = len(sc.blas_of)
        omin = np.zeros((n, 3), np.float32)
        omax = np.zeros((n, 3), np.float32)
        for i in range(n):
            root = blases[sc.blas_of[i]][0][0]
            omin[i], omax[i] = orc.object_bounds(root["bounds_min"], root["bounds_max"], xf[i])
        ref_tlas, ref_used = orc.tlas_build(omin, omax)
        assert tused == ref_used and tlas.tobytes() == ref_tlas.tobytes(), "TLAS differs"
        sa = orc.SceneArrays(blases, sc.blas_of, inv)
        ref0 = orc.scene_intersect(ref_tlas, ref_used, sa, cfg["rays"])
        assert np.array_equal(h0["prim"], ref0["prim"]) and np.array_equal(h0["inst"], ref0["inst"])
        assert h0.tobytes() == ref0.tobytes(), "primary hits differ"
        assert (h0["prim"] != bt.MISS).sum() > 100
        # bounce rays: the GPU's (generated the same way as inside the persistent frame kernel)
        gb, gvalid = sc.scene.bounce_rays(cfg["rays"], sc.seed)
        rb, rvalid = orc.scene_bounce_rays(sa, cfg["rays"], ref0, sc.seed)
        assert np.array_equal(gvalid, rvalid)
        assert gb[rvalid].tobytes() == rb[rvalid].tobytes(), "bounce rays differ"
        ref1 = np.zeros(len(cfg["rays"]), orc.HIT)
        ref1["t"] = np.finfo(np.float32).max
        ref1["prim"] = ref1["inst"] = bt.MISS
        ref1[rvalid] = orc.scene_intersect(ref_tlas, ref_used, sa, rb[rvalid])
        assert h1.tobytes() == ref1.tobytes(), "bounce hits differ"
