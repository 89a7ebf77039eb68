"""Launch configurations: every compiled variant of the five traversal kernels and the Lambertian
forward pass (launch shape x stack) with both leaf layouts, hidden trees on and off and two refill sizes gives the oracle's hits
bit for bit, and the autotuner returns a config from the search space under which the results are
unchanged."""
import numpy as np
import pytest

import bvhtracer_gb300 as bt
from bvhtracer_gb300 import scenes
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = bt.Context(0)
    yield c
    c.close()


def subset(kernel):
    """All shapes x stacks; big_leaf 8 (warp-cooperative) and NEVER (per lane); refill 1 and 16;
    hidden trees never (0) and at the widest margin (1000)."""
    return [c for c in bt.Context.tune_space(kernel)
            if c["big_leaf"] in (8, bt.BIG_LEAF_NEVER) and c["refill"] in (1, 16) and c["hidden"] in (0, 1000)]


def build(tris):
    tris = np.ascontiguousarray(tris, np.float32).copy()
    return tris, bt.BvhBuilder().build_for(tris)


def bounce_refs(primaries, ref0, bounce_fn, trace_fn):
    rb, valid = bounce_fn(primaries, ref0)
    ref1 = np.zeros(len(primaries), orc.HIT)
    ref1["t"] = np.finfo(np.float32).max
    ref1["prim"] = ref1["inst"] = bt.MISS
    ref1[valid] = trace_fn(rb[valid])
    return ref1


@pytest.fixture(scope="module")
def blas_case(ctx):
    tris, cam, _ = scenes.icosphere_frame(seed=8, width=96, height=64)
    rays = np.concatenate([cam, scenes.sphere_rays(2048, 3, box=1.5)])
    tris, bvh = build(tris)
    blas = ctx.upload_blas(bvh, tris)
    seed = 77
    ref0 = orc.bvh_intersect(bvh.nodes, bvh.nodes_used, tris, rays, threads=8)
    ref1 = bounce_refs(rays, ref0, lambda p, h: orc.bounce_rays(p, h, tris, seed),
                       lambda r: orc.bvh_intersect(bvh.nodes, bvh.nodes_used, tris, r, threads=8))
    return blas, rays, seed, ref0, ref1


def test_trace_blas_every_variant(ctx, blas_case):
    blas, rays, seed, ref0, ref1 = blas_case
    default = ctx.tune_get(bt.K_TRACE_BLAS)
    try:
        for cfg in subset(bt.K_TRACE_BLAS):
            ctx.tune_set(bt.K_TRACE_BLAS, **cfg)
            h = blas.intersect(rays)
            assert h.tobytes() == ref0.tobytes(), f"trace_blas {cfg}"
            if cfg["big_leaf"] == 8:  # the plain bounce pipeline runs the same kernel twice
                h0, h1, _ = blas.trace_bounce(rays, seed, bt.MODE_PLAIN)
                assert h0.tobytes() == ref0.tobytes() and h1.tobytes() == ref1.tobytes(), f"plain bounce {cfg}"
    finally:
        ctx.tune_set(bt.K_TRACE_BLAS, **default)


def test_persistent_bounce_every_variant(ctx, blas_case):
    blas, rays, seed, ref0, ref1 = blas_case
    default = ctx.tune_get(bt.K_PERSISTENT_BOUNCE)
    try:
        for cfg in subset(bt.K_PERSISTENT_BOUNCE):
            ctx.tune_set(bt.K_PERSISTENT_BOUNCE, **cfg)
            h0, h1, _ = blas.trace_bounce(rays, seed, bt.MODE_PERSISTENT)
            assert h0.tobytes() == ref0.tobytes() and h1.tobytes() == ref1.tobytes(), f"persistent {cfg}"
    finally:
        ctx.tune_set(bt.K_PERSISTENT_BOUNCE, **default)


def random_instances(n, seed):
    rng = np.random.default_rng(seed)
    q = rng.standard_normal((n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    w, x, y, z = q.T
    R = np.stack([np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)], -1),
                  np.stack([2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)], -1),
                  np.stack([2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)], -1)], 1)
    M = np.zeros((n, 4, 4))
    M[:, :3, :3] = R * rng.uniform(0.5, 2.0, n)[:, None, None]
    M[:, :3, 3] = rng.uniform(-12, 12, (n, 3))
    M[:, 3, 3] = 1
    inv = np.linalg.inv(M)
    return (np.ascontiguousarray(M.transpose(0, 2, 1).reshape(n, 16), np.float32),
            np.ascontiguousarray(inv.transpose(0, 2, 1).reshape(n, 16), np.float32))


def test_lambert_forward_every_variant(ctx):
    """The persistent Lambertian forward pass runs under the single-ray trace kernel's config:
    every variant gives the oracle's hits and one and the same image."""
    verts, faces, vn, _, rays, light = scenes.lambert_scene(seed=4, level=5, width=64, height=64)
    n = len(rays)
    m = bt.DiffMesh(ctx, verts, faces, vn)
    d_rays = ctx.to_device(rays)
    d_img = ctx.device_buffer(4 * n)
    d_hits = ctx.device_buffer(bt.HIT.itemsize * n)
    ref = orc.bvh_intersect(m.bvh.nodes, m.bvh.nodes_used, m.tris, rays, threads=8)
    default = ctx.tune_get(bt.K_TRACE_BLAS)
    image = None
    try:
        for cfg in subset(bt.K_TRACE_BLAS):
            ctx.tune_set(bt.K_TRACE_BLAS, **cfg)
            d_img.zero()
            m.forward_async(d_rays, n, light, d_img, d_hits)
            ctx.sync()
            h = d_hits.download(np.zeros(n, bt.HIT))
            img = d_img.download(np.zeros(n, np.float32))
            assert h.tobytes() == ref.tobytes(), f"lambert forward {cfg}"
            if image is None:
                image = img
            assert img.tobytes() == image.tobytes(), f"lambert forward image {cfg}"
        assert (ref["prim"] != bt.MISS).mean() > 0.2
    finally:
        ctx.tune_set(bt.K_TRACE_BLAS, **default)


def test_scene_kernels_every_variant(ctx):
    blases, host = [], []
    for lvl, sd in ((2, 1), (3, 2), (4, 3)):
        tris, bvh = build(scenes.displaced_icosphere(lvl, sd).triangles())
        blases.append(ctx.upload_blas(bvh, tris))
        host.append((bvh.nodes[:bvh.nodes_used], bvh.nodes_used, tris))
    n = 40
    blas_of = np.arange(n) % 3
    xf, inv = random_instances(n, 11)
    sc = ctx.scene([blases[i] for i in blas_of], xf, inv)
    tlas, tused = sc.download_tlas()
    sa = orc.SceneArrays(host, blas_of, inv)
    rays = np.concatenate([scenes.look_at_rays(96, 64, (0, 0, -40), (0, 0, 0), 50.0),
                           scenes.sphere_rays(2048, 5, box=15.0)])
    seed = 5
    ref0 = orc.scene_intersect(tlas, tused, sa, rays)
    assert (ref0["prim"] != bt.MISS).sum() > 500
    ref1 = bounce_refs(rays, ref0, lambda p, h: orc.scene_bounce_rays(sa, p, h, seed),
                       lambda r: orc.scene_intersect(tlas, tused, sa, r))
    d_rays = ctx.to_device(rays)
    d_h0 = ctx.device_buffer(bt.HIT.itemsize * len(rays))
    d_h1 = ctx.device_buffer(bt.HIT.itemsize * len(rays))
    defaults = {k: ctx.tune_get(k) for k in (bt.K_TRACE_SCENE, bt.K_SCENE_BOUNCE)}
    try:
        for cfg in subset(bt.K_TRACE_SCENE):
            ctx.tune_set(bt.K_TRACE_SCENE, **cfg)
            assert sc.intersect(rays).tobytes() == ref0.tobytes(), f"trace_scene {cfg}"
        for cfg in subset(bt.K_SCENE_BOUNCE):
            ctx.tune_set(bt.K_SCENE_BOUNCE, **cfg)
            sc.trace_bounce_async(d_rays, len(rays), seed, d_h0, d_h1)
            ctx.sync()
            h0 = d_h0.download(np.zeros(len(rays), bt.HIT))
            h1 = d_h1.download(np.zeros(len(rays), bt.HIT))
            assert h0.tobytes() == ref0.tobytes() and h1.tobytes() == ref1.tobytes(), f"scene bounce {cfg}"
    finally:
        for k, v in defaults.items():
            ctx.tune_set(k, **v)


def uneven_batch(ctx):
    specs = [(scenes.soup(1000, 1), 3000), (scenes.displaced_icosphere(3, 2).triangles(), 9000),
             (scenes.soup(5000, 3, scale=1.5), 700), (scenes.displaced_icosphere(1, 4).triangles(), 64)]
    items, rays_all, refs = [], [], []
    off = 0
    for k, (t, nr) in enumerate(specs):
        tris, bvh = build(t)
        b = ctx.upload_blas(bvh, tris)
        npx = nr // 2 // 8 * 8 or 8
        rays = np.concatenate([scenes.look_at_rays(npx, 2, (0, 0, -25), (0, 0, 0), 40.0),
                               scenes.sphere_rays(nr - npx * 2, 10 + k)])
        items.append((b.id, off, len(rays), 0))
        rays_all.append(rays)
        refs.append(orc.bvh_intersect(bvh.nodes, bvh.nodes_used, tris, rays, threads=8))
        off += len(rays)
    return np.array(items, dtype=bt.BATCH_ITEM), np.concatenate(rays_all), np.concatenate(refs)


def test_batch_every_variant_and_autotune(ctx):
    items, rays, ref = uneven_batch(ctx)
    defaults = {k: ctx.tune_get(k) for k in (bt.K_TRACE_BATCH, bt.K_TRACE_BLAS)}
    try:
        for cfg in subset(bt.K_TRACE_BATCH):
            ctx.tune_set(bt.K_TRACE_BATCH, **cfg)
            assert ctx.trace_batch(items, rays, bt.MODE_PERSISTENT).tobytes() == ref.tobytes(), f"batch {cfg}"
        d_rays = ctx.to_device(rays)
        d_h = ctx.device_buffer(bt.HIT.itemsize * len(rays))
        for kernel in (bt.K_TRACE_BATCH, bt.K_TRACE_BLAS):
            cfg, ms = ctx.autotune(kernel, d_rays, len(rays), d_h, items=items, reps=2)
            assert ms > 0 and cfg == ctx.tune_get(kernel)
            assert cfg in bt.Context.tune_space(kernel) or cfg["stack"] == 0
            mode = bt.MODE_PERSISTENT if kernel == bt.K_TRACE_BATCH else bt.MODE_PLAIN
            assert ctx.trace_batch(items, rays, mode).tobytes() == ref.tobytes(), f"after autotune {cfg}"
    finally:
        for k, v in defaults.items():
            ctx.tune_set(k, **v)


def test_autotune_persistent_bounce(ctx, blas_case):
    blas, rays, seed, ref0, ref1 = blas_case
    default = ctx.tune_get(bt.K_PERSISTENT_BOUNCE)
    try:
        d_rays = ctx.to_device(rays)
        d_h0 = ctx.device_buffer(bt.HIT.itemsize * len(rays))
        d_h1 = ctx.device_buffer(bt.HIT.itemsize * len(rays))
        cfg, ms = ctx.autotune(bt.K_PERSISTENT_BOUNCE, d_rays, len(rays), d_h0, d_h1, target=blas.id, seed=seed,
                               reps=2)
        assert ms > 0 and cfg == ctx.tune_get(bt.K_PERSISTENT_BOUNCE)
        h0, h1, _ = blas.trace_bounce(rays, seed, bt.MODE_PERSISTENT)
        assert h0.tobytes() == ref0.tobytes() and h1.tobytes() == ref1.tobytes()
    finally:
        ctx.tune_set(bt.K_PERSISTENT_BOUNCE, **default)


def test_tune_set_rejects_uncompiled_variants(ctx):
    with pytest.raises(bt.BvhGpuError):
        ctx.tune_set(bt.K_TRACE_BLAS, block=96)
    with pytest.raises(bt.BvhGpuError):
        ctx.tune_set(bt.K_TRACE_BLAS, stack=12)
    with pytest.raises(bt.BvhGpuError):
        ctx.tune_set(bt.K_PERSISTENT_BOUNCE, refill=0)
