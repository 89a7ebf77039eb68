"""Launch deadline (bvhgpu_set_deadline): a persistent launch that runs past its budget stops taking
and tracing rays, raises a status flag and leaves -- no fault, no wait -- and the call reports
BVHGPU_ERR_DEADLINE.  The context stays usable: the next launch without a deadline (or with a
generous one) gives the same results as a launch that never had one, including the Lambertian
forward pass, whose per-mesh schedule ignores the flags and list of a pass that stopped early."""
import numpy as np
import pytest

import bvhtracer_gb300 as bt
from bvhtracer_gb300 import scenes

pytestmark = pytest.mark.gpu
SEED = 12345
TIGHT = 1_000        # 1 microsecond: every launch of these sizes runs past it
GENEROUS = 10 ** 10  # 10 s


def expect_deadline(fn):
    with pytest.raises(bt.BvhGpuError) as e:
        fn()
    assert e.value.code == bt.ERR_DEADLINE


def test_persistent_bounce_stops_at_the_deadline_and_recovers():
    tris, rays, _ = scenes.icosphere_frame(seed=0, width=960, height=540)
    tris = np.ascontiguousarray(tris)
    bvh = bt.BvhBuilder().build_for(tris)
    with bt.Context(0) as ctx:
        blas = ctx.upload_blas(bvh, tris)
        ref0, ref1, nb = blas.trace_bounce(rays, SEED, bt.MODE_PERSISTENT)
        assert nb > 10_000
        ctx.set_deadline(TIGHT)
        expect_deadline(lambda: blas.trace_bounce(rays, SEED, bt.MODE_PERSISTENT))
        ctx.set_deadline(GENEROUS)
        h0, h1, nb2 = blas.trace_bounce(rays, SEED, bt.MODE_PERSISTENT)
        assert nb2 == nb and h0.tobytes() == ref0.tobytes() and h1.tobytes() == ref1.tobytes()
        ctx.set_deadline(0)
        h0, h1, _ = blas.trace_bounce(rays, SEED, bt.MODE_PERSISTENT)
        assert h0.tobytes() == ref0.tobytes() and h1.tobytes() == ref1.tobytes()
        ctx.set_deadline(2 ** 64 - 1)  # "no limit" from a caller: the end time saturates, no wrap
        h0, h1, _ = blas.trace_bounce(rays, SEED, bt.MODE_PERSISTENT)
        assert h0.tobytes() == ref0.tobytes() and h1.tobytes() == ref1.tobytes()


def test_batch_stops_at_the_deadline_and_recovers():
    with bt.Context(0) as ctx:
        items = np.zeros(4, bt.BATCH_ITEM)
        blases, rays = [], []
        off = 0
        for i in range(4):
            t, r = scenes.batch_scene(i, 2000 * (i + 1), 20000, 0)
            b = ctx.upload_blas(bt.BvhBuilder().build_for(t), t)
            blases.append(b)
            items[i] = (b.id, off, len(r), 0)
            rays.append(r)
            off += len(r)
        rays = np.concatenate(rays)
        ref = ctx.trace_batch(items, rays, bt.MODE_PERSISTENT)
        ctx.set_deadline(TIGHT)
        expect_deadline(lambda: ctx.trace_batch(items, rays, bt.MODE_PERSISTENT))
        ctx.set_deadline(0)
        assert ctx.trace_batch(items, rays, bt.MODE_PERSISTENT).tobytes() == ref.tobytes()


def test_lambertian_forward_stops_and_its_schedule_recovers():
    verts, faces, vn, _, rays, light = scenes.lambert_scene(seed=6, level=7, width=256, height=256)
    n = len(rays)
    with bt.Context(0) as ctx:
        m = bt.DiffMesh(ctx, verts, faces, vn)
        d_rays = ctx.to_device(rays)
        d_img = ctx.device_buffer(4 * n)
        d_hits = ctx.device_buffer(bt.HIT.itemsize * n)

        def forward():
            d_img.zero()
            d_hits.zero()
            m.forward_async(d_rays, n, light, d_img, d_hits)
            ctx.sync()
            return d_img.download(np.zeros(n, np.float32)).tobytes(), d_hits.download(np.zeros(n, bt.HIT)).tobytes()

        ref = forward()
        assert forward() == ref  # a scheduled pass
        ctx.set_deadline(TIGHT)
        expect_deadline(forward)
        ctx.set_deadline(0)
        for _ in range(3):  # the pass after the stopped one ignores its schedule; the next ones use theirs
            assert forward() == ref
