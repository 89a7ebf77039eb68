"""The product's host SAH build (BvhBuilder::build_for) against the oracle: identical node
arrays and identical triangle order, bit for bit.  CPU only."""
import numpy as np
import pytest

import bvhtracer_gb300 as bt
from bvhtracer_gb300 import scenes
from oracle import oracle as orc


def build_both(tris):
    tris = np.ascontiguousarray(tris, np.float32).reshape(-1, 9)
    mine = tris.copy()
    bvh = bt.BvhBuilder().build_for(mine)
    ref_tris, ref_nodes, ref_used = orc.bvh_build(tris)
    return mine, bvh, ref_tris, ref_nodes, ref_used


def assert_same(tris):
    mine, bvh, ref_tris, ref_nodes, ref_used = build_both(tris)
    assert bvh.nodes_used == ref_used
    assert mine.tobytes() == ref_tris.tobytes()
    assert bvh.nodes.tobytes() == ref_nodes.tobytes()


@pytest.mark.parametrize("n,seed", [(1, 0), (2, 1), (3, 2), (17, 3), (4096, 0), (4096, 11), (20000, 5)])
def test_soup(n, seed):
    assert_same(scenes.soup(n, seed))


@pytest.mark.parametrize("level", [0, 1, 3, 5])
def test_displaced_icosphere(level):
    assert_same(scenes.displaced_icosphere(level, seed=level).triangles())


def test_degenerate_meshes():
    # identical triangles: every axis is skipped (bounds_min == bounds_max), one leaf
    t = np.tile(np.array([0, 0, 0, 1, 0, 0, 0, 1, 0], np.float32), (64, 1))
    assert_same(t)
    # all centroids negative: the 1e-30 initial maximum of the reference is inside the range
    assert_same(scenes.soup(300, 9) - np.float32(20))
    # collinear centroids along one axis, zero extent on the others
    line = np.zeros((100, 9), np.float32)
    line[:, 0::3] = np.arange(100, dtype=np.float32)[:, None]
    assert_same(line)


def test_cube_fixture():
    import os
    d = np.load(os.path.join(os.path.dirname(__file__), "golden", "cube.npz"))
    assert_same(d["tris"])


def test_rejects_bad_mesh():
    with pytest.raises(ValueError):
        bt.BvhBuilder().build_for(np.zeros((4, 9), np.float64))
    with pytest.raises(bt.BvhGpuError):
        bt.BvhBuilder().build_for(np.zeros((0, 9), np.float32))


def random_mesh(rng, kind):
    n = int(rng.integers(1, 400))
    if kind == 0:    # uniform soup
        return rng.uniform(-10, 10, (n, 9)).astype(np.float32)
    if kind == 1:    # tight clusters with shared vertices
        c = rng.uniform(-5, 5, (int(rng.integers(1, 6)), 3))
        pts = c[rng.integers(0, len(c), n * 3)] + rng.normal(0, 1e-3, (n * 3, 3))
        return pts.reshape(n, 9).astype(np.float32)
    if kind == 2:    # coplanar (z = const) and axis-aligned edges
        t = rng.integers(-20, 20, (n, 9)).astype(np.float32) * np.float32(0.25)
        t[:, 2::3] = np.float32(rng.integers(-3, 3))
        return t
    if kind == 3:    # duplicates of a few triangles
        base = rng.uniform(-1, 1, (int(rng.integers(1, 5)), 9)).astype(np.float32)
        return base[rng.integers(0, len(base), n)]
    # mixed scales: tiny and huge triangles, negative-only coordinates
    s = np.float32(10.0) ** rng.integers(-3, 4, (n, 1)).astype(np.float32)
    return (rng.uniform(-1, 0, (n, 9)).astype(np.float32) * s).astype(np.float32)


def test_random_meshes_match_or_both_refuse():
    """300 random meshes of five kinds (soups, near-coincident clusters, coplanar grids, duplicates,
    mixed scales): the host build equals the oracle's bit for bit, or both refuse where the
    reference's build would panic."""
    rng = np.random.default_rng(2024)
    refused = 0
    for case in range(300):
        tris = random_mesh(rng, case % 5)
        try:
            ref_tris, ref_nodes, ref_used = orc.bvh_build(np.ascontiguousarray(tris))
        except orc.PanicError:
            with pytest.raises(bt.BvhGpuError) as e:
                bt.BvhBuilder().build_for(tris.copy())
            assert e.value.code == 6, f"case {case}"
            refused += 1
            continue
        mine = tris.copy()
        bvh = bt.BvhBuilder().build_for(mine)
        assert bvh.nodes_used == ref_used, f"case {case}"
        assert mine.tobytes() == ref_tris.tobytes(), f"case {case}"
        assert bvh.nodes.tobytes() == ref_nodes.tobytes(), f"case {case}"
    assert refused < 300


@pytest.mark.parametrize("kind", range(5))
def test_indexed_build_permutation(kind):
    """bvhgpu_build_bvh_host_indexed: the same nodes and order as the plain host build, and
    perm[i] the input index of the triangle at position i (so an indexed mesh's faces follow)."""
    import ctypes
    from bvhtracer_gb300 import _lib
    from bvhtracer_gb300._lib import ptr
    rng = np.random.default_rng(70 + kind)
    tris = np.ascontiguousarray(random_mesh(rng, kind))
    n = len(tris)
    try:
        ref_tris, ref_nodes, ref_used = orc.bvh_build(tris)
    except orc.PanicError:
        pytest.skip("the reference's build panics on this mesh")
    mesh = tris.copy()
    nodes = np.zeros(2 * n, bt.NODE)
    used = ctypes.c_uint32()
    perm = np.zeros(n, np.uint32)
    rc = _lib.load().bvhgpu_build_bvh_host_indexed(ptr(mesh), n, ptr(nodes), ctypes.byref(used), ptr(perm))
    assert rc == 0
    assert used.value == ref_used and nodes.tobytes() == ref_nodes.tobytes() and mesh.tobytes() == ref_tris.tobytes()
    assert sorted(perm.tolist()) == list(range(n))
    assert tris[perm].tobytes() == mesh.tobytes()
