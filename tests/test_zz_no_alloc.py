"""The allocation-free refit entry point (bvhgpu_refit_noalloc) against the regular one.

Some callers cannot call cudaMalloc -- engines that reserve all device memory in their own pool
at start-up, or latency-critical threads where a driver allocation (which can synchronise the
device) is not allowed.  bvhgpu_refit_noalloc refits a caller-owned device node array using a
fixed static scratch array instead.  This file is collected last so that a run stopping at the
first failure has already run every other test; it also passes on its own in a fresh process.
"""
import ctypes

import numpy as np
import pytest

import bvhtracer_gb300 as bt
from bvhtracer_gb300 import _lib, scenes

pytestmark = pytest.mark.gpu


def animate(tris, seed):
    rng = np.random.default_rng(seed)
    k = (1 + 0.05 * rng.standard_normal((len(tris), 3, 1))).astype(np.float32)
    return np.ascontiguousarray((tris.reshape(-1, 3, 3) * k).reshape(-1, 9), np.float32)


def test_refit_noalloc_matches_regular_refit_twice():
    tris = scenes.displaced_icosphere(5, seed=21).triangles()
    bvh = bt.BvhBuilder().build_for(tris)
    nodes0 = np.ascontiguousarray(bvh.nodes[:bvh.nodes_used])
    with bt.Context(0) as ctx:
        blas = ctx.upload_blas(bvh, tris)
        d_nodes = ctx.to_device(nodes0)
        d_tris = ctx.device_buffer(tris.nbytes)
        d_status = ctx.to_device(np.zeros(1, np.uint32))
        lib = ctx.lib
        for frame in (1, 2):  # two calls in a row; the second sees the first call's scratch
            moved = animate(tris, frame)
            blas.update_vertices(moved)
            blas.refit()
            expected = blas.download_nodes()
            d_tris.upload(moved)
            # on the context's stream, so that the download below is ordered after the refit
            rc = lib.bvhgpu_refit_noalloc(d_nodes.ptr, bvh.nodes_used, d_tris.ptr, len(moved), ctx.stream,
                                          d_status.ptr)
            assert rc == 0
            ctx.sync()
            got = d_nodes.download(np.zeros(bvh.nodes_used, bt.NODE))
            # refit nodes are compared bit for bit, as for every other refit test
            assert got.tobytes() == expected.tobytes(), f"frame {frame}: refit differs"
        status = d_status.download(np.zeros(1, np.uint32))
        assert status[0] == 0


def test_refit_noalloc_rejects_oversize_and_bad_arguments():
    lib = _lib.load()
    dummy = ctypes.c_void_p(16)  # never dereferenced: the size check comes first
    too_many = 2 ** 20 + 1
    assert lib.bvhgpu_refit_noalloc(dummy, too_many, dummy, 10, None, None) == 8
    assert lib.bvhgpu_refit_noalloc(None, 10, dummy, 10, None, None) == 1
    assert lib.bvhgpu_refit_noalloc(dummy, 0, dummy, 10, None, None) == 1
