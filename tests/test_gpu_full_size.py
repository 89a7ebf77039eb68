"""GPU parity at the benchmarked sizes: every timed workload's outputs against the oracle.

- the displaced-icosphere frame at 1920 x 1080 plus its bounce rays, both pipelines (persistent
  launch and plain trace / compact / trace), every ray;
- the instanced animation at 256 instances and 1280 x 720, three frames replayed from one CUDA
  graph: refit nodes, TLAS, primary hits, bounce rays and bounce hits of the last frame;
- all 64 scenes of the uneven batch, the first 4,096 rays of each, persistent and plain launches.

Bar: identical primitive / instance ids; t, u, v within 1e-5 relative and in fact bit-identical;
rays whose two nearest hits lie within 1e-5 relative in t are counted apart (none may differ
either way, since the kernels keep the reference's visit order and strict `<`).
"""
import os

import numpy as np
import pytest

import bvhtracer_gb300 as bt
from bvhtracer_gb300 import scenes
from bvhtracer_gb300.frames import AnimatedScene
from oracle import checks
from oracle import oracle as orc

pytestmark = pytest.mark.gpu
THREADS = len(os.sched_getaffinity(0))
BOUNCE_SEED = 12345


def assert_identical(result, what):
    assert result["prim_mismatch"] == 0 and result["inst_mismatch"] == 0, f"{what}: {result}"
    assert result["tuv_out_of_tolerance"] == 0, f"{what}: {result}"
    assert result["tuv_not_bit_identical"] == 0, f"{what}: {result}"


def test_icosphere_1080p_frame_with_bounces_both_pipelines():
    tris, rays, _ = scenes.icosphere_frame(seed=0)
    n = len(rays)
    assert n == 1920 * 1080
    tris = np.ascontiguousarray(tris)
    bvh = bt.BvhBuilder().build_for(tris)
    o_tris, o_nodes, o_used = orc.bvh_build(scenes.icosphere_frame(seed=0)[0])
    assert o_used == bvh.nodes_used and o_nodes[:o_used].tobytes() == bvh.nodes[:o_used].tobytes()
    assert o_tris.tobytes() == tris.tobytes()
    r0, rb, rvalid, r1 = checks.frame_with_bounce(o_nodes, o_used, o_tris, rays, BOUNCE_SEED, threads=THREADS)
    near0, near1 = checks.frame_near_ties(o_nodes, o_tris, rays, rb, rvalid, threads=THREADS)
    assert rvalid.sum() > 500_000
    with bt.Context(0) as ctx:
        blas = ctx.upload_blas(bvh, tris)
        d_rays = ctx.to_device(rays)
        d_h0 = ctx.device_buffer(n * bt.HIT.itemsize)
        d_h1 = ctx.device_buffer(n * bt.HIT.itemsize)
        for mode in (bt.MODE_PERSISTENT, bt.MODE_PLAIN):
            d_h0.zero()
            d_h1.zero()
            blas.trace_bounce_async(d_rays, n, BOUNCE_SEED, mode, d_h0, d_h1)
            ctx.sync()
            h0 = d_h0.download(np.zeros(n, bt.HIT))
            h1 = d_h1.download(np.zeros(n, bt.HIT))
            assert_identical(checks.compare_hits(h0, r0, near0), f"mode {mode} primaries")
            assert_identical(checks.compare_hits(h1, r1, near1), f"mode {mode} bounces")
        # the bounce rays the plain mode traced are the oracle's, bit for bit
        gb, gvalid = blas.bounce_rays(rays, BOUNCE_SEED)
        assert np.array_equal(gvalid, rvalid) and gb[rvalid].tobytes() == rb[rvalid].tobytes()


def test_instanced_animation_256_instances_720p_three_graph_frames():
    cfg = scenes.instanced_animation(seed=0)
    assert len(cfg["instances"]["blas_of"]) == 256 and len(cfg["rays"]) == 1280 * 720
    with bt.Context(0) as ctx:
        sc = AnimatedScene(ctx, cfg)
        initial = [(m.bvh.nodes.copy(), m.bvh.nodes_used) for m in sc.meshes]
        sc.capture()
        for _ in range(3):
            sc.launch()
        ctx.sync()
        h0, h1 = sc.hits()
        blas_states = []
        for m, (nodes0, used) in zip(sc.meshes, initial):
            verts = m.vertices()
            tris = np.ascontiguousarray(verts[m.faces].reshape(-1, 9), np.float32)
            ref_nodes = orc.bvh_refit(nodes0, used, tris)[:used]
            assert m.blas.download_nodes().tobytes() == ref_nodes.tobytes(), "refit differs"
            blas_states.append((ref_nodes, used, tris))
        xf, inv = sc.scene.download_transforms()
        tlas, tused = sc.scene.download_tlas()
        ref_tlas, ref_used, sa = checks.scene_state_reference(blas_states, sc.blas_of, xf, inv)
        assert tused == ref_used and tlas.tobytes() == ref_tlas.tobytes(), "TLAS differs"
        r0, rb, rvalid, r1 = checks.scene_frame_with_bounce(ref_tlas, ref_used, sa, cfg["rays"], sc.seed,
                                                            threads=THREADS)
        gb, gvalid = sc.scene.bounce_rays(cfg["rays"], sc.seed)
    assert (r0["prim"] != orc.MISS).sum() > 50_000
    assert_identical(checks.compare_hits(h0, r0), "primaries")
    assert np.array_equal(gvalid, rvalid) and gb[rvalid].tobytes() == rb[rvalid].tobytes(), "bounce rays differ"
    assert_identical(checks.compare_hits(h1, r1), "bounces")


def test_uneven_batch_all_64_scenes_first_4096_rays():
    from concurrent.futures import ThreadPoolExecutor
    ntris, nrays = scenes.batch_specs(0, 64)

    def make(i):
        tris, rays = scenes.batch_scene(i, int(ntris[i]), int(nrays[i]), 0)
        t, nodes, used = orc.bvh_build(tris)
        return t, nodes, used, rays[:4096]

    with ThreadPoolExecutor(max_workers=THREADS) as ex:
        built = list(ex.map(make, range(64)))
    with ThreadPoolExecutor(max_workers=THREADS) as ex:
        refs = list(ex.map(lambda b: orc.bvh_intersect(b[1], b[2], b[0], b[3]), built))
        nears = list(ex.map(lambda b: orc.near_ties(b[1], b[0], b[3], threads=1), built))
    rays = np.concatenate([b[3] for b in built])
    ref = np.concatenate(refs)
    near = np.concatenate(nears)
    with bt.Context(0) as ctx:
        items = np.zeros(64, bt.BATCH_ITEM)
        off = 0
        blases = []
        for i, (t, nodes, used, r) in enumerate(built):
            blases.append(ctx.upload_blas(bt.Bvh(nodes, used), t))
            items[i] = (blases[-1].id, off, len(r), 0)
            off += len(r)
        pers = ctx.trace_batch(items, rays, bt.MODE_PERSISTENT)
        plain = ctx.trace_batch(items, rays, bt.MODE_PLAIN)
    assert (ref["prim"] != orc.MISS).sum() > 10_000
    assert_identical(checks.compare_hits(pers, ref, near), "persistent batch")
    assert_identical(checks.compare_hits(plain, ref, near), "plain batch")
