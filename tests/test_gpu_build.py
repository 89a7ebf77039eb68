"""The GPU SAH build (BvhBuilder::build_for on the device) against the host build, which is itself
bit-identical to the oracle: the same node array, nodes_used, triangle order and permutation, bit
for bit, and the same refusal where the reference panics."""
import ctypes

import numpy as np
import pytest

import bvhtracer_gb300 as bt
from bvhtracer_gb300 import scenes
from bvhtracer_gb300 import _lib
from bvhtracer_gb300._lib import ptr

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = bt.Context(0)
    yield c
    c.close()


def host_build(tris):
    mesh = np.ascontiguousarray(tris, np.float32).reshape(-1, 9).copy()
    n = len(mesh)
    nodes = np.zeros(2 * n, bt.NODE)
    used = ctypes.c_uint32()
    perm = np.zeros(n, np.uint32)
    rc = _lib.load().bvhgpu_build_bvh_host_indexed(ptr(mesh), n, ptr(nodes), ctypes.byref(used), ptr(perm))
    return rc, mesh, nodes, used.value, perm


def assert_same_build(ctx, tris):
    rc, ref_mesh, ref_nodes, ref_used, ref_perm = host_build(tris)
    assert rc == 0
    mesh = np.ascontiguousarray(tris, np.float32).reshape(-1, 9).copy()
    bvh, perm = ctx.build_bvh(mesh, perm=True)
    assert bvh.nodes_used == ref_used
    assert bvh.nodes.tobytes() == ref_nodes.tobytes(), "node array differs"
    assert mesh.tobytes() == ref_mesh.tobytes(), "triangle order differs"
    assert np.array_equal(perm, ref_perm)
    return bvh


@pytest.mark.parametrize("n,seed", [(1, 0), (2, 1), (3, 2), (17, 3), (4096, 0), (4096, 11), (20000, 5),
                                    (150000, 8)])
def test_soup(ctx, n, seed):
    assert_same_build(ctx, scenes.soup(n, seed))


@pytest.mark.parametrize("level", [0, 1, 3, 5, 6])
def test_displaced_icosphere(ctx, level):
    bvh = assert_same_build(ctx, scenes.displaced_icosphere(level, seed=level).triangles())
    if level == 6:
        assert bvh.nodes_used == 48  # the flat tree of the reference's zero-box bins


def test_degenerate_meshes(ctx):
    t = np.tile(np.array([0, 0, 0, 1, 0, 0, 0, 1, 0], np.float32), (64, 1))  # one leaf, no axis
    assert_same_build(ctx, t)
    assert_same_build(ctx, scenes.soup(300, 9) - np.float32(20))          # centroids below 1e-30
    line = np.zeros((100, 9), np.float32)
    line[:, 0::3] = np.arange(100, dtype=np.float32)[:, None]
    assert_same_build(ctx, line)                                          # one axis binned
    assert_same_build(ctx, scenes.soup(5000, 4) + np.float32(50))         # away from the origin
    zeros = scenes.soup(2000, 6)
    zeros[::3, 0::3] = -0.0                                               # signed zeros in the folds
    zeros[1::3, 0::3] = 0.0
    assert_same_build(ctx, zeros)


def test_uneven_batch_scenes(ctx):
    ntris, _ = scenes.batch_specs(0, 64)
    for i in (0, 1, 2, 5, 10, 31):
        tris, _ = scenes.batch_scene(i, int(min(ntris[i], 400_000)), 64, 0)
        assert_same_build(ctx, tris)


def test_cube_fixture(ctx):
    import os
    d = np.load(os.path.join(os.path.dirname(__file__), "golden", "cube.npz"))
    assert_same_build(ctx, d["tris"])


def test_panicking_mesh_is_refused_like_the_host_build(ctx):
    # two triangles spanning +-3e38: the node area overflows to inf, so the leaf cost is inf and
    # the (absent) split is attempted with no binned axis -- the reference panics there
    big = np.array([[-3e38, -3e38, -3e38, 3e38, 3e38, 3e38, 0, 0, 0]] * 2, np.float32)
    rc = host_build(big)[0]
    assert rc == 6
    with pytest.raises(bt.BvhGpuError) as e:
        ctx.build_bvh(big.copy())
    assert e.value.code == 6


def test_blas_built_on_the_gpu_traces_like_the_host_built_one(ctx):
    tris, rays, _ = scenes.icosphere_frame(seed=2, width=96, height=64)
    host = np.ascontiguousarray(tris, np.float32).copy()
    bvh = bt.BvhBuilder().build_for(host)
    ref = ctx.upload_blas(bvh, host).intersect(rays)
    dev = np.ascontiguousarray(tris, np.float32).copy()
    bid = ctypes.c_uint32()
    ctx.check(ctx.lib.bvhgpu_blas_build(ctx.h, ptr(dev), len(dev), ctypes.byref(bid)))
    assert dev.tobytes() == host.tobytes()
    hits = np.zeros(len(rays), bt.HIT)
    ctx.check(ctx.lib.bvhgpu_blas_intersect(ctx.h, bid.value, ptr(np.ascontiguousarray(rays)), len(rays), ptr(hits)))
    assert hits.tobytes() == ref.tobytes()


def test_decoded_tri_file_builds_and_traces_on_the_gpu(ctx):
    """`.tri` text -> bvhgpu_mesh_decode -> GPU SAH build -> upload -> trace, against the oracle's
    build and traversal of the same decoded mesh."""
    from oracle import oracle as orc
    src = scenes.displaced_icosphere(4, seed=12).triangles()
    text = "\n".join(" ".join("{:.9g}".format(float(x)) for x in row) for row in src) + "\n"
    tris, normals, _ = bt.decode_mesh(text)
    assert tris.tobytes() == np.ascontiguousarray(src, np.float32).tobytes()
    mesh = tris.copy()
    bvh = ctx.build_bvh(mesh)
    blas = ctx.upload_blas(bvh, mesh)
    rays = scenes.look_at_rays(128, 96, (0.0, 0.0, -3.0), (0.0, 0.0, 0.0), 45.0)
    ref_tris, ref_nodes, ref_used = orc.bvh_build(tris)
    ref = orc.bvh_intersect(ref_nodes, ref_used, ref_tris, rays, threads=8)
    assert blas.intersect(rays).tobytes() == ref.tobytes()
    assert (ref["prim"] != bt.MISS).sum() > 1000
