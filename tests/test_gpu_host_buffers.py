"""bvhgpu_blas_trace_bounce with host buffers of every kind gives the same hit records: page-locked
buffers and, on a GPU that accesses ordinary memory coherently, ordinary (pageable) buffers are read
and written in place by the launch (the hit pages first touched by the CPU, fresh never-touched
allocations included); views whose ray array is not 16-byte aligned are staged instead (the kernels
read a ray as two float4).  Both modes.  A device ray array that is not 16-byte aligned is refused
with status 1 before any launch."""
import ctypes

import numpy as np
import pytest

import bvhtracer_gb300 as bt
from bvhtracer_gb300 import scenes
from bvhtracer_gb300._lib import ptr

pytestmark = pytest.mark.gpu
SEED = 777


def call(ctx, blas, rays, h0, h1, mode):
    nb = ctypes.c_uint32()
    ctx.check(ctx.lib.bvhgpu_blas_trace_bounce(ctx.h, blas.id, ptr(rays), len(rays), SEED, mode, ptr(h0), ptr(h1),
                                               ctypes.byref(nb)))
    return nb.value


@pytest.mark.parametrize("mode", [bt.MODE_PERSISTENT, bt.MODE_PLAIN])
def test_trace_bounce_with_every_kind_of_host_buffer(mode):
    tris, rays, _ = scenes.icosphere_frame(seed=3, width=640, height=360)
    tris = np.ascontiguousarray(tris)
    bvh = bt.BvhBuilder().build_for(tris)
    n = len(rays)
    with bt.Context(0) as ctx:
        blas = ctx.upload_blas(bvh, tris)
        d_rays = ctx.to_device(rays)
        d0 = ctx.device_buffer(n * bt.HIT.itemsize)
        d1 = ctx.device_buffer(n * bt.HIT.itemsize)
        blas.trace_bounce_async(d_rays, n, SEED, mode, d0, d1)
        ctx.sync()
        ref0 = d0.download(np.zeros(n, bt.HIT))
        ref1 = d1.download(np.zeros(n, bt.HIT))
        nref = int((ref0["prim"] != bt.MISS).sum())
        assert nref > 10_000

        # page-locked
        pr = ctx.pinned((n,), bt.RAY)
        pr.array[:] = rays
        p0, p1 = ctx.pinned((n,), bt.HIT), ctx.pinned((n,), bt.HIT)
        assert call(ctx, blas, pr.array, p0.array, p1.array, mode) == nref
        assert p0.array.tobytes() == ref0.tobytes() and p1.array.tobytes() == ref1.tobytes()

        # ordinary memory: fresh (never touched), then reused, then views at an odd offset
        r = np.ascontiguousarray(rays)
        for _ in range(2):
            h0, h1 = np.empty(n, bt.HIT), np.empty(n, bt.HIT)
            assert call(ctx, blas, r, h0, h1, mode) == nref
            assert h0.tobytes() == ref0.tobytes() and h1.tobytes() == ref1.tobytes()
            assert call(ctx, blas, r, h0, h1, mode) == nref
            assert h0.tobytes() == ref0.tobytes() and h1.tobytes() == ref1.tobytes()
        raw_r = np.zeros(n * bt.RAY.itemsize + 4, np.uint8)
        raw0 = np.zeros(n * bt.HIT.itemsize + 4, np.uint8)
        raw1 = np.zeros(n * bt.HIT.itemsize + 4, np.uint8)
        vr = raw_r[4:].view(bt.RAY)
        vr[:] = rays
        v0, v1 = raw0[4:].view(bt.HIT), raw1[4:].view(bt.HIT)
        assert call(ctx, blas, vr, v0, v1, mode) == nref
        assert v0.tobytes() == ref0.tobytes() and v1.tobytes() == ref1.tobytes()


class Offset:
    """A device address `off` bytes into a buffer (for the alignment check)."""

    def __init__(self, buf, off):
        self.ptr = ctypes.c_void_p(buf.ptr.value + off)


def test_misaligned_device_arrays_are_refused():
    tris, rays, _ = scenes.icosphere_frame(seed=3, width=64, height=32)
    tris = np.ascontiguousarray(tris)
    bvh = bt.BvhBuilder().build_for(tris)
    n = len(rays)
    with bt.Context(0) as ctx:
        blas = ctx.upload_blas(bvh, tris)
        d_rays = ctx.device_buffer(n * bt.RAY.itemsize + 16)
        d_hits = ctx.device_buffer(n * bt.HIT.itemsize + 16)
        for rays_off, hits_off in ((4, 0), (8, 0), (0, 2)):
            with pytest.raises(bt.BvhGpuError) as e:
                blas.intersect_async(Offset(d_rays, rays_off), n, Offset(d_hits, hits_off))
            assert e.value.code == 1
        # the context is untouched: an aligned call still works
        d_ok = ctx.to_device(rays)
        blas.intersect_async(d_ok, n, d_hits)
        ctx.sync()

