"""Differentiable Lambertian render: the CUDA forward / adjoint (FP32) against the FP64 CPU
reference and FP64 central finite differences (eps 1e-3), with visibility held fixed.

Bars: hit ids identical to the oracle's traversal; gradient relative error <= 1e-3 (norm-wise,
||g - g_ref|| / ||g_ref|| over 64 sampled vertex coordinates) against FP64 central finite
differences and against the FP64 adjoint; every sampled coordinate within 1e-2.  The image is
compared with the FP64 shading within 1e-5 absolute (the GPU shades in FP32).
"""
import os

import numpy as np
import pytest

import bvhtracer_gb300 as bt
from bvhtracer_gb300 import scenes
from oracle import adjoint64, checks
from oracle import oracle as orc

pytestmark = pytest.mark.gpu
GRAD_TOL = 1e-3       # norm-wise relative error over the sampled coordinates
GRAD_TOL_EACH = 1e-2  # any single coordinate
JAC_TOL = 1e-3        # the FP32 Jacobian alone (FP64 adjoint fed the GPU's own residuals)
IMAGE_TOL = 1e-5


def rel_err(a, b):
    """|a - b| / max(|b|, 1e-3 * max|b|): relative error with a floor for near-zero entries."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    floor = 1e-3 * np.max(np.abs(b))
    return np.abs(a - b) / np.maximum(np.abs(b), floor)


@pytest.mark.parametrize("level,size", [(5, 128), (7, 512)])
def test_lambert_forward_adjoint_against_fp64(level, size):
    verts, faces, vn, tverts, rays, light = scenes.lambert_scene(seed=3, level=level, width=size, height=size)
    n = len(rays)
    with bt.Context(0) as ctx:
        m = bt.DiffMesh(ctx, verts, faces, vn)
        d_rays = ctx.to_device(rays)
        d_img = ctx.device_buffer(4 * n)
        d_tgt = ctx.device_buffer(4 * n)
        d_hits = ctx.device_buffer(bt.HIT.itemsize * n)
        d_grad = ctx.device_buffer(12 * len(verts))
        d_grad.zero()
        m.set_vertices(tverts)
        m.forward_async(d_rays, n, light, d_tgt, d_hits)
        ctx.sync()
        target = d_tgt.download(np.zeros(n, np.float32))
        m.set_vertices(verts)
        m.forward_async(d_rays, n, light, d_img, d_hits)
        m.adjoint_async(d_rays, n, light, d_hits, d_img, d_tgt, d_grad)
        ctx.sync()
        img = d_img.download(np.zeros(n, np.float32))
        hits = d_hits.download(np.zeros(n, bt.HIT))
        grad = d_grad.download(np.zeros((len(verts), 3), np.float32))
        loss_gpu = bt.mse_loss(ctx, d_img, d_tgt, n)

    # hits: the traversal is the exact one -- every pixel's hit record against the oracle's
    ref = orc.bvh_intersect(m.bvh.nodes, m.bvh.nodes_used, m.tris, rays, threads=len(os.sched_getaffinity(0)))
    r = checks.compare_hits(hits, ref)
    assert r["prim_mismatch"] == 0 and r["inst_mismatch"] == 0 and r["tuv_not_bit_identical"] == 0, r
    assert (hits["prim"] != bt.MISS).mean() > 0.2

    # forward image and loss against FP64
    img64 = adjoint64.render64(rays, hits["prim"], verts, m.faces, vn, light)
    assert np.max(np.abs(img.astype(np.float64) - img64)) <= IMAGE_TOL
    loss64 = adjoint64.loss64(img64, target)
    assert abs(loss_gpu - loss64) <= 1e-3 * loss64

    # gradient on 64 random coordinates of vertices the image sees, away from the terminator of
    # max(0, n.l) (every pixel of the vertex has n.l > 0.05), where the loss is smooth in the step
    g64 = adjoint64.adjoint64(rays, hits["prim"], verts, m.faces, vn, light, target)
    cos = adjoint64.shading_cosine64(rays, hits["prim"], verts, m.faces, vn, light)
    hit = np.nonzero(hits["prim"] != bt.MISS)[0]
    vmin = np.full(len(verts), np.inf)
    for k in range(3):
        np.minimum.at(vmin, m.faces[hits["prim"][hit], k], cos[hit])
    smooth = np.nonzero((vmin > 0.05) & np.isfinite(vmin) & np.any(g64 != 0.0, axis=1))[0]
    rng = np.random.default_rng(level)
    vids = rng.choice(smooth, size=64, replace=False)
    axes = rng.integers(0, 3, size=64)
    coords = list(zip(vids.tolist(), axes.tolist()))
    # central differences, eps 1e-3, and their Richardson extrapolation with eps / 2: the plain
    # difference carries an O(eps^2) truncation error that is ~1e-3 relative here (eps is not small
    # against triangles of 0.01-0.04), the extrapolated one cancels it
    fd, fd_r = adjoint64.richardson64(rays, hits["prim"], verts, m.faces, vn, light, target, coords, eps=1e-3)
    gpu = np.array([grad[v, a] for v, a in coords], np.float64)
    ref64 = np.array([g64[v, a] for v, a in coords])
    jac64 = adjoint64.adjoint64(rays, hits["prim"], verts, m.faces, vn, light, target, image=img)
    ref_jac = np.array([jac64[v, a] for v, a in coords])

    def norm_rel(a, b):
        return float(np.linalg.norm(a - b) / np.linalg.norm(b))

    n_fd, n_64, n_math, n_jac = norm_rel(gpu, fd_r), norm_rel(gpu, ref64), norm_rel(ref64, fd_r), norm_rel(gpu, ref_jac)
    print(f"level {level}: norm-wise rel. error GPU vs FD {n_fd:.2e} | GPU vs FP64 adjoint {n_64:.2e} | "
          f"FP64 adjoint vs FD {n_math:.2e} | FP32 Jacobian {n_jac:.2e} | worst coordinate GPU vs FD "
          f"{rel_err(gpu, fd_r).max():.2e} | plain FD (eps=1e-3, no extrapolation) median "
          f"{np.median(rel_err(gpu, fd)):.2e}")
    assert n_math <= GRAD_TOL, f"FP64 adjoint vs FD: {n_math:.2e}"
    assert n_fd <= GRAD_TOL, f"GPU adjoint vs FP64 FD: {n_fd:.2e}"
    assert n_64 <= GRAD_TOL, f"GPU adjoint vs FP64 adjoint: {n_64:.2e}"
    assert n_jac <= JAC_TOL, f"FP32 Jacobian: {n_jac:.2e}"
    assert rel_err(gpu, fd_r).max() <= GRAD_TOL_EACH


def test_descent_lowers_the_loss():
    verts, faces, vn, tverts, rays, light = scenes.lambert_scene(seed=4, level=4, width=96, height=96)
    n = len(rays)
    with bt.Context(0) as ctx:
        m = bt.DiffMesh(ctx, verts, faces, vn)
        d_rays = ctx.to_device(rays)
        d_img = ctx.device_buffer(4 * n)
        d_tgt = ctx.device_buffer(4 * n)
        d_hits = ctx.device_buffer(bt.HIT.itemsize * n)
        d_grad = ctx.device_buffer(12 * len(verts))
        d_grad.zero()
        m.set_vertices(tverts)
        m.forward_async(d_rays, n, light, d_tgt, d_hits)
        m.set_vertices(verts)
        # step size from the first gradient: the largest vertex move per step is 0.02 (of radius 10)
        m.forward_async(d_rays, n, light, d_img, d_hits)
        m.adjoint_async(d_rays, n, light, d_hits, d_img, d_tgt, d_grad)
        ctx.sync()
        g0 = d_grad.download(np.zeros((len(verts), 3), np.float32))
        d_grad.zero()
        lr = 0.02 / float(np.abs(g0).max())
        losses = []
        for _ in range(30):
            m.update_async()
            m.forward_async(d_rays, n, light, d_img, d_hits)
            losses.append(bt.mse_loss(ctx, d_img, d_tgt, n))
            m.adjoint_async(d_rays, n, light, d_hits, d_img, d_tgt, d_grad)
            m.sgd_step_async(d_grad, lr)
        ctx.sync()
    assert losses[-1] < 0.97 * losses[0], losses


def test_descent_resumes_from_a_checkpoint(tmp_path):
    """Three steps, a checkpoint, a fresh mesh resumed from it and three more steps: the resumed
    vertices equal the saved ones bit for bit, and the end state equals six uninterrupted steps
    (within 1e-5 relative: the adjoint scatters with atomics, whose summation order varies)."""
    verts, faces, vn, tverts, rays, light = scenes.lambert_scene(seed=4, level=4, width=96, height=96)
    n = len(rays)
    path = str(tmp_path / "descent.npz")

    def run(ctx, m, steps, d_rays, d_tgt):
        d_img = ctx.device_buffer(4 * n)
        d_hits = ctx.device_buffer(bt.HIT.itemsize * n)
        d_grad = ctx.device_buffer(12 * m.nverts)
        d_grad.zero()
        for _ in range(steps):
            m.update_async()
            m.forward_async(d_rays, n, light, d_img, d_hits)
            m.adjoint_async(d_rays, n, light, d_hits, d_img, d_tgt, d_grad)
            m.sgd_step_async(d_grad, 50.0)
        ctx.sync()

    with bt.Context(0) as ctx:
        d_rays = ctx.to_device(rays)
        d_tgt = ctx.device_buffer(4 * n)
        m = bt.DiffMesh(ctx, verts, faces, vn)
        m.set_vertices(tverts)
        m.forward_async(d_rays, n, light, d_tgt, ctx.device_buffer(bt.HIT.itemsize * n))
        m.set_vertices(verts)
        run(ctx, m, 6, d_rays, d_tgt)
        straight = m.vertices()
        m.set_vertices(verts)
        run(ctx, m, 3, d_rays, d_tgt)
        m.checkpoint(path, 3, [1.0], lr=50.0)
        saved = m.vertices()
        m2 = bt.DiffMesh(ctx, verts, faces, vn)
        state = m2.resume(path)
        assert state["step"] == 3 and m2.vertices().tobytes() == saved.tobytes()
        run(ctx, m2, 3, d_rays, d_tgt)
        resumed = m2.vertices()
    assert not np.array_equal(straight, verts)
    np.testing.assert_allclose(resumed, straight, rtol=1e-5, atol=1e-6)


def test_repeated_forward_passes_are_identical():
    """The persistent forward pass hands pixels to warps in whatever order the queue serves them: a
    second and third pass at the same vertices give bit-identical hit records and images."""
    verts, faces, vn, _, rays, light = scenes.lambert_scene(seed=5, level=5, width=128, height=128)
    n = len(rays)
    with bt.Context(0) as ctx:
        m = bt.DiffMesh(ctx, verts, faces, vn)
        d_rays = ctx.to_device(rays)
        out = []
        for _ in range(3):
            d_img = ctx.device_buffer(4 * n)
            d_hits = ctx.device_buffer(bt.HIT.itemsize * n)
            m.forward_async(d_rays, n, light, d_img, d_hits)
            ctx.sync()
            out.append((d_img.download(np.zeros(n, np.float32)).tobytes(),
                        d_hits.download(np.zeros(n, bt.HIT)).tobytes()))
    assert out[0] == out[1] == out[2]


def test_forward_schedule_across_ray_counts_and_orders():
    """The forward pass serves the rays its previous pass found long first (a per-mesh schedule that
    the previous pass writes).  Passes over a prefix of the rays, over the rays reversed, over a
    larger batch (the schedule grows) and replays of a captured pass must each trace every ray exactly
    once: hit records and images equal, ray by ray, those of the first (unscheduled) pass."""
    verts, faces, vn, _, rays, light = scenes.lambert_scene(seed=6, level=7, width=256, height=256)
    n = len(rays)
    with bt.Context(0) as ctx:
        m = bt.DiffMesh(ctx, verts, faces, vn)

        def forward(rs):
            k = len(rs)
            d_rays = ctx.to_device(np.ascontiguousarray(rs))
            d_img = ctx.device_buffer(4 * k)
            d_hits = ctx.device_buffer(bt.HIT.itemsize * k)
            d_img.zero()
            d_hits.zero()
            m.forward_async(d_rays, k, light, d_img, d_hits)
            ctx.sync()
            return d_img.download(np.zeros(k, np.float32)), d_hits.download(np.zeros(k, bt.HIT))

        img0, hits0 = forward(rays)
        assert (hits0["prim"] != bt.MISS).mean() > 0.2
        cases = [(rays, slice(None)), (rays, slice(None)), (rays[: n // 3], slice(0, n // 3)),
                 (rays[::-1], slice(None, None, -1)), (rays, slice(None)), (rays, slice(None))]
        for rs, sel in cases:
            img, hits = forward(rs)
            assert img.tobytes() == img0[sel].tobytes() and hits.tobytes() == hits0[sel].tobytes()
        both = np.concatenate([rays, rays[::-1]])
        img, hits = forward(both)
        assert img.tobytes() == np.concatenate([img0, img0[::-1]]).tobytes()
        assert hits.tobytes() == np.concatenate([hits0, hits0[::-1]]).tobytes()

        # a captured pass replays with the schedule on the device (its epoch advances per replay)
        d_rays = ctx.to_device(rays)
        d_img = ctx.device_buffer(4 * n)
        d_hits = ctx.device_buffer(bt.HIT.itemsize * n)
        ctx.graph_begin()
        m.forward_async(d_rays, n, light, d_img, d_hits)
        gid = ctx.graph_end()
        for _ in range(3):
            d_img.zero()
            d_hits.zero()
            ctx.graph_launch(gid)
            ctx.sync()
            assert d_img.download(np.zeros(n, np.float32)).tobytes() == img0.tobytes()
            assert d_hits.download(np.zeros(n, bt.HIT)).tobytes() == hits0.tobytes()
        ctx.graph_free(gid)
