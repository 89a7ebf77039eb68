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
from oracle import oracle as orc

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
            # refit nodes are compared bit for bit, as for every other refit test: with the library's
            # other refit and with the oracle's Bvh::refit (bvh.rs:469-493)
            assert got.tobytes() == expected.tobytes(), f"frame {frame}: refit differs"
            ref = orc.bvh_refit(nodes0, bvh.nodes_used, moved)[:bvh.nodes_used]
            assert got.tobytes() == ref.tobytes(), f"frame {frame}: refit differs from the oracle"
        status = d_status.download(np.zeros(1, np.uint32))
        assert status[0] == 0


def test_refit_noalloc_rejects_oversize_and_bad_arguments():
    lib = _lib.load()
    dummy = ctypes.c_void_p(16)  # never dereferenced: the size check comes first
    too_many = 2 ** 20 + 1
    assert lib.bvhgpu_refit_noalloc(dummy, too_many, dummy, 10, None, None) == 8
    assert lib.bvhgpu_refit_noalloc(None, 10, dummy, 10, None, None) == 1
    assert lib.bvhgpu_refit_noalloc(dummy, 0, dummy, 10, None, None) == 1


def _ancestors_or_self(nodes, used, targets):
    parent = {}
    for i in range(used):
        if i != 1 and nodes[i]["primitive_count"] == 0:
            parent[int(nodes[i]["left_first"])] = i
            parent[int(nodes[i]["left_first"]) + 1] = i
    out = set()
    for t in targets:
        while t is not None:
            out.add(t)
            t = parent.get(t)
    return out


def test_refit_noalloc_reports_malformed_nodes_and_refits_the_rest():
    """Corrupt one branch's child index (status value 1), one leaf's triangle count (2) and make a
    branch claim another branch's children (4): those nodes are skipped without any out-of-range
    access, the status word carries 1 | 2 | 4, every node outside the corrupted nodes' ancestor
    chains equals the oracle's refit, and the bad branch's and bad leaf's chains keep their input."""
    tris = scenes.soup(6000, seed=8)
    bvh = bt.BvhBuilder().build_for(tris)
    used = bvh.nodes_used
    nodes0 = np.ascontiguousarray(bvh.nodes[:used])
    moved = animate(tris, 5)
    ref = orc.bvh_refit(nodes0, used, moved)[:used]
    branches = [i for i in range(used) if i != 1 and nodes0[i]["primitive_count"] == 0]
    leaves = [i for i in range(used) if i != 1 and nodes0[i]["primitive_count"] > 0]
    assert len(branches) > 8 and len(leaves) > 8

    def disjoint(a, chosen):  # neither a's ancestor nor its descendant
        anc = _ancestors_or_self(nodes0, used, [a])
        return all(c not in anc and a not in _ancestors_or_self(nodes0, used, [c]) for c in chosen)

    # four nodes in disjoint parts of the tree: branch x, leaf y, branch w, and a branch z below
    # w's children in index order (so that w's children pass z's index check)
    x = branches[len(branches) // 2]
    y = next(i for i in reversed(leaves) if disjoint(i, [x]))
    w = next(i for i in reversed(branches) if disjoint(i, [x, y]))
    z = next(i for i in branches if i < int(nodes0[w]["left_first"]) and disjoint(i, [x, y, w]))
    bad = nodes0.copy()
    bad[x]["left_first"] = x                                   # child index not above the branch
    bad[y]["primitive_count"] = np.uint32(len(tris) + 1)       # triangles past ntris
    bad[z]["left_first"] = bad[w]["left_first"]                # two branches claim the same children
    affected = _ancestors_or_self(nodes0, used, [x, y, z, w])
    with bt.Context(0) as ctx:
        d_nodes = ctx.to_device(bad)
        d_tris = ctx.to_device(moved)
        d_status = ctx.to_device(np.zeros(1, np.uint32))
        rc = ctx.lib.bvhgpu_refit_noalloc(d_nodes.ptr, used, d_tris.ptr, len(moved), ctx.stream, d_status.ptr)
        assert rc == 0
        ctx.sync()
        got = d_nodes.download(np.zeros(used, bt.NODE))
        status = int(d_status.download(np.zeros(1, np.uint32))[0])
    assert status == 1 | 2 | 4
    keep = [i for i in range(used) if i not in affected]
    assert len(keep) > used // 2
    assert got[keep].tobytes() == ref[keep].tobytes(), "nodes outside the corrupted chains differ from the oracle"
    untouched = _ancestors_or_self(nodes0, used, [x, y]) - _ancestors_or_self(nodes0, used, [z, w])
    for i in untouched:
        assert got[i].tobytes() == bad[i].tobytes(), f"node {i} on a corrupted chain was written"
