"""GPU parity: the CUDA library through its C ABI against the CPU oracle.

Bar: identical hit primitive / instance ids and bit-identical t, u, v (the kernels follow
the reference's f32 operation order, so no tolerance is needed; the path's stated tolerance
of 1e-5 relative is asserted as well for the record), bit-identical refit nodes and TLAS
nodes, identical images.
"""
import numpy as np
import pytest

import bvhtracer_gb300 as bt
from bvhtracer_gb300 import scenes
from oracle import oracle as orc

pytestmark = pytest.mark.gpu
REL_TOL = 1e-5  # the stated tolerance for t/u/v; the kernels are expected to be bit-exact


@pytest.fixture(scope="module")
def ctx():
    c = bt.Context(0)
    yield c
    c.close()


def assert_hits_equal(gpu, ref, what=""):
    assert len(gpu) == len(ref)
    bad = np.nonzero(gpu["prim"] != ref["prim"])[0]
    assert len(bad) == 0, f"{what}: {len(bad)} rays with different primitive ids, first {bad[:10]}"
    assert np.array_equal(gpu["inst"], ref["inst"]), what
    hit = ref["prim"] != bt.MISS
    for k in ("t", "u", "v"):
        g, r = gpu[k][hit].astype(np.float64), ref[k][hit].astype(np.float64)
        assert np.all(np.abs(g - r) <= REL_TOL * np.maximum(np.abs(r), 1e-30) + 1e-30), f"{what} {k} tolerance"
        assert np.array_equal(gpu[k], ref[k]), f"{what}: {k} not bit-identical"


def build(tris):
    tris = np.ascontiguousarray(tris, np.float32).copy()
    bvh = bt.BvhBuilder().build_for(tris)
    return tris, bvh


# ---- known answers of the reference tests, through the GPU ---------------------------------

def test_known_answers_one_triangle(ctx):
    s3 = np.sqrt(np.float32(3))
    tri = np.array([[0, 0.5, 0, -1 / s3, -0.5, 0, 1 / s3, -0.5, 0]], np.float32)
    tris, bvh = build(tri)
    blas = ctx.upload_blas(bvh, tris)
    o = np.array([0, 0, 5], np.float32)
    targets = [np.zeros(3, np.float32), tri[0, 0:3], tri[0, 3:6], tri[0, 6:9],
               tri[0, 0:3] + np.array([0, 0.5, 0], np.float32)]
    rays = orc.make_rays(np.tile(o, (5, 1)), [orc.normalize(t - o) for t in targets])
    h = blas.intersect(rays)
    assert h["t"][0] == np.float32(5)                           # test_triangle_intersection.rs:67-80
    assert h["t"][1] == np.sqrt(np.float32(101) / np.float32(4))  # :82-95
    assert h["t"][2] == np.sqrt(np.float32(307) / np.float32(12))
    assert h["t"][3] == np.sqrt(np.float32(307) / np.float32(12))
    assert h["prim"][4] == bt.MISS


def test_cube_scene_known_answers(ctx):
    import os
    d = np.load(os.path.join(os.path.dirname(__file__), "golden", "cube.npz"))
    tris, bvh = build(d["tris"])
    blas = ctx.upload_blas(bvh, tris)
    xf = np.eye(4, dtype=np.float32)
    xf[:3, :3] *= 2
    xf[3, :3] = -1
    inv = np.eye(4, dtype=np.float32)
    inv[:3, :3] *= 0.5
    inv[3, :3] = 0.5
    sc = ctx.scene([blas], xf.reshape(1, 16), inv.reshape(1, 16))
    o = np.array([0, 4, 0], np.float32)
    targets = [np.array([0.5, 1.0, -0.5], np.float32), np.array([-0.5, 1.0, 0.5], np.float32)]
    rays = orc.make_rays(np.tile(o, (2, 1)), [orc.normalize(t - o) for t in targets])
    h = sc.intersect(rays)
    expect = np.sqrt(np.float32(19) / np.float32(2))
    assert np.all(np.abs(h["t"].astype(np.float64) - float(expect)) <= 1e-6)  # test_scene_cube.rs:96-108
    assert list(h["prim"]) == [6, 9]                                           # :124-136, :215-227
    assert list(h["inst"]) == [0, 0]


# ---- plain traversal --------------------------------------------------------------------------

def test_soup_full_frame(ctx):
    tris, rays = scenes.soup_frame(seed=0)
    tris, bvh = build(tris)
    blas = ctx.upload_blas(bvh, tris)
    gpu = blas.intersect(rays)
    ref = orc.bvh_intersect(bvh.nodes, bvh.nodes_used, tris, rays, threads=8)
    assert_hits_equal(gpu, ref, "soup_frame")
    assert (ref["prim"] != bt.MISS).mean() > 0.2


def test_icosphere_frame_sampled(ctx):
    tris, rays, _ = scenes.icosphere_frame(seed=1, width=480, height=272)
    tris, bvh = build(tris)
    blas = ctx.upload_blas(bvh, tris)
    gpu = blas.intersect(rays)
    ref = orc.bvh_intersect(bvh.nodes, bvh.nodes_used, tris, rays, threads=8)
    assert_hits_equal(gpu, ref, "icosphere_frame")


def test_incoherent_rays_and_edge_cases(ctx):
    tris, bvh = build(scenes.soup(3000, 4))
    blas = ctx.upload_blas(bvh, tris)
    rays = scenes.sphere_rays(50000, 3, box=6.0)
    # axis-aligned directions (1/d = inf, slab NaNs), zero direction, tiny t, huge origins
    extra = orc.make_rays([[0, 0, -10], [0, 0, -10], [1, 2, 3], [0, 0, -10], [1e30, 0, 0], [0.5, 0.5, -10]],
                          [[0, 0, 1], [0, 1, 0], [0, 0, 0], [1e-30, 0, 1], [-1, 0, 0], [0, 0, 1]],
                          t=[np.finfo(np.float32).max, 3.0, 1.0, 5.0, np.finfo(np.float32).max, 1e-5])
    rays = np.concatenate([rays, extra])
    ref = orc.bvh_intersect(bvh.nodes, bvh.nodes_used, tris, rays, threads=8)
    assert_hits_equal(blas.intersect(rays), ref, "incoherent")


def test_empty_and_single_ray(ctx):
    tris, bvh = build(scenes.soup(64, 1))
    blas = ctx.upload_blas(bvh, tris)
    assert len(blas.intersect(np.zeros(0, bt.RAY))) == 0
    r = scenes.plane_rays(1, 1, (0, 0, -18), -15, 1, 1)
    assert_hits_equal(blas.intersect(r), orc.bvh_intersect(bvh.nodes, bvh.nodes_used, tris, r))


def test_async_device_path_matches_host_path(ctx):
    tris, rays = scenes.soup_frame(seed=2)
    tris, bvh = build(tris)
    blas = ctx.upload_blas(bvh, tris)
    d_rays = ctx.to_device(rays)
    d_hits = ctx.device_buffer(len(rays) * bt.HIT.itemsize)
    blas.intersect_async(d_rays, len(rays), d_hits)
    ctx.sync()
    out = d_hits.download(np.zeros(len(rays), bt.HIT))
    assert out.tobytes() == blas.intersect(rays).tobytes()


# ---- bounce -------------------------------------------------------------------------------------

def test_bounce_rays_and_hits(ctx):
    tris, rays, _ = scenes.icosphere_frame(seed=3, width=320, height=184)
    tris, bvh = build(tris)
    blas = ctx.upload_blas(bvh, tris)
    seed = 1234
    ref0 = orc.bvh_intersect(bvh.nodes, bvh.nodes_used, tris, rays, threads=8)
    ref_b, ref_valid = orc.bounce_rays(rays, ref0, tris, seed)
    gpu_b, gpu_valid = blas.bounce_rays(rays, seed)
    assert np.array_equal(gpu_valid, ref_valid)
    assert gpu_b[ref_valid].tobytes() == ref_b[ref_valid].tobytes(), "bounce rays not bit-identical"
    ref1 = np.zeros(len(rays), orc.HIT)
    ref1["t"] = np.finfo(np.float32).max
    ref1["prim"] = ref1["inst"] = bt.MISS
    ref1[ref_valid] = orc.bvh_intersect(bvh.nodes, bvh.nodes_used, tris, ref_b[ref_valid], threads=8)
    for mode in (bt.MODE_PLAIN, bt.MODE_PERSISTENT):
        h0, h1, nb = blas.trace_bounce(rays, seed, mode)
        assert_hits_equal(h0, ref0, f"primary mode {mode}")
        assert_hits_equal(h1, ref1, f"bounce mode {mode}")
        assert nb == int((ref0["prim"] != bt.MISS).sum())


@pytest.mark.parametrize("mode", [bt.MODE_PLAIN, bt.MODE_PERSISTENT])
@pytest.mark.parametrize("pinned", [False, True])
def test_host_call_equals_device_launch(ctx, mode, pinned):
    """bvhgpu_blas_trace_bounce with host buffers -- staged through device copies, or read and
    written in place when every buffer is page-locked -- and its device-side bounce count give
    what the device-buffer launch gives."""
    tris, rays, _ = scenes.icosphere_frame(seed=5, width=960, height=544)
    tris, bvh = build(tris)
    blas = ctx.upload_blas(bvh, tris)
    n = len(rays)
    if pinned:
        pr, p0, p1 = ctx.pinned((n,), bt.RAY), ctx.pinned((n,), bt.HIT), ctx.pinned((n,), bt.HIT)
        pr.array[:] = rays
        import ctypes
        from bvhtracer_gb300._lib import ptr
        nb_c = ctypes.c_uint32()
        ctx.check(ctx.lib.bvhgpu_blas_trace_bounce(ctx.h, blas.id, ptr(pr.array), n, 77, mode, ptr(p0.array),
                                                   ptr(p1.array), ctypes.byref(nb_c)))
        h0, h1, nb = p0.array.copy(), p1.array.copy(), nb_c.value
    else:
        h0, h1, nb = blas.trace_bounce(rays, 77, mode)
    d_rays = ctx.to_device(rays)
    d0 = ctx.device_buffer(n * bt.HIT.itemsize)
    d1 = ctx.device_buffer(n * bt.HIT.itemsize)
    blas.trace_bounce_async(d_rays, n, 77, mode, d0, d1)
    ctx.sync()
    g0 = d0.download(np.zeros(n, bt.HIT))
    g1 = d1.download(np.zeros(n, bt.HIT))
    assert h0.tobytes() == g0.tobytes() and h1.tobytes() == g1.tobytes()
    assert nb == int((g0["prim"] != bt.MISS).sum())


def test_near_tie_rays_counted_and_identical(ctx):
    """The parity rule counts rays whose two nearest hits lie within 1e-5 relative in t apart.  The
    traversal keeps the reference's visit order and strict `<`, so even exact ties (duplicated
    triangles) resolve to the reference's primitive: near-tie rays match bit for bit too."""
    base = scenes.soup(3000, 21)
    tris, bvh = build(np.concatenate([base, base[::7], base[5::11]]))
    blas = ctx.upload_blas(bvh, tris)
    rays = np.concatenate([scenes.plane_rays(320, 320, (0.0, 0.0, -18.0), -15.0, 1.0, 1.0),
                           scenes.sphere_rays(20000, 4, box=6.0)])
    ref = orc.bvh_intersect(bvh.nodes, bvh.nodes_used, tris, rays, threads=8)
    ties = orc.near_ties(bvh.nodes, tris, rays)
    print(f"near-tie rays: {int(ties.sum())} of {int((ref['prim'] != bt.MISS).sum())} hits")
    assert ties.sum() > 1000
    gpu = blas.intersect(rays)
    assert_hits_equal(gpu[~ties], ref[~ties], "rays without a near tie")
    assert_hits_equal(gpu[ties], ref[ties], "near-tie rays")


@pytest.mark.parametrize("mode", [bt.LIST_CLOSEST, bt.LIST_MUT])
def test_triangle_list_matches_oracle(ctx, mode):
    """Triangle::intersect / intersect_mut over a list (no BVH), incl. duplicated triangles and a
    list that is not a multiple of the 128-triangle tile; LIST_MUT keeps the reference's
    overwrite of u, v by a later, farther hit."""
    base = scenes.soup(700, 9)
    tris = np.ascontiguousarray(np.concatenate([base, base[::13]]), np.float32)
    rays = np.concatenate([scenes.plane_rays(96, 96, (0.0, 0.0, -18.0), -15.0, 1.0, 1.0),
                           scenes.sphere_rays(3000, 2, box=6.0)])
    ref = orc.triangles_intersect(tris, rays, mode)
    gpu = ctx.triangles_intersect(tris, rays, mode)
    assert (ref["prim"] != bt.MISS).sum() > 1000
    assert gpu.tobytes() == ref.tobytes()
    if mode == bt.LIST_MUT:
        closest = orc.triangles_intersect(tris, rays, 0)
        assert (closest["prim"] != ref["prim"]).sum() > 0  # the overwrite quirk is exercised
    assert ctx.triangles_intersect(tris[:0], rays[:5], mode)["prim"].tolist() == [bt.MISS] * 5


# ---- refit -------------------------------------------------------------------------------------

def test_refit_bit_exact(ctx):
    mesh = scenes.displaced_icosphere(4, seed=5)
    tris0 = mesh.triangles()
    tris, bvh = build(tris0)
    blas = ctx.upload_blas(bvh, tris)
    # refit of the unchanged mesh is the identity (test_bvh_refit.rs:46-54)
    blas.refit()
    assert blas.download_nodes().tobytes() == bvh.nodes[:bvh.nodes_used].tobytes()
    # animate (radial wobble), refit on GPU vs oracle, then idempotence (:56-65)
    rng = np.random.default_rng(0)
    moved = tris.reshape(-1, 3, 3) * (1 + 0.05 * rng.standard_normal((len(tris), 3, 1))).astype(np.float32)
    moved = np.ascontiguousarray(moved.reshape(-1, 9), np.float32)
    blas.update_vertices(moved)
    blas.refit()
    gpu = blas.download_nodes()
    ref = orc.bvh_refit(bvh.nodes, bvh.nodes_used, moved)[:bvh.nodes_used]
    assert gpu.tobytes() == ref.tobytes()
    blas.refit()
    assert blas.download_nodes().tobytes() == gpu.tobytes()
    # traversal after refit still matches the oracle on the refitted tree
    rays = scenes.look_at_rays(128, 128, (0, 0, -3), (0, 0, 0), 45.0)
    assert_hits_equal(blas.intersect(rays), orc.bvh_intersect(ref, bvh.nodes_used, moved, rays), "after refit")


def test_refit_single_leaf_root(ctx):
    tris, bvh = build(scenes.soup(1, 0))
    blas = ctx.upload_blas(bvh, tris)
    moved = tris + np.float32(0.25)
    blas.update_vertices(moved)
    blas.refit()
    ref = orc.bvh_refit(bvh.nodes, bvh.nodes_used, moved)[:bvh.nodes_used]
    assert blas.download_nodes().tobytes() == ref.tobytes()


# ---- TLAS / scene --------------------------------------------------------------------------------

def random_instances(n, seed):
    rng = np.random.default_rng(seed)
    q = rng.standard_normal((n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    w, x, y, z = q.T
    R = np.stack([np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)], -1),
                  np.stack([2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)], -1),
                  np.stack([2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)], -1)], 1)
    s = rng.uniform(0.5, 2.0, n)
    t = rng.uniform(-20, 20, (n, 3))
    M = np.zeros((n, 4, 4))
    M[:, :3, :3] = R * s[:, None, None]
    M[:, :3, 3] = t
    M[:, 3, 3] = 1
    inv = np.linalg.inv(M)
    # column-major 16 floats: element [col*4 + row]
    return (np.ascontiguousarray(M.transpose(0, 2, 1).reshape(n, 16), np.float32),
            np.ascontiguousarray(inv.transpose(0, 2, 1).reshape(n, 16), np.float32))


def test_tlas_rebuild_and_scene_trace(ctx):
    blases, host = [], []
    for lvl, sd in ((2, 1), (3, 2), (4, 3)):
        tris, bvh = build(scenes.displaced_icosphere(lvl, sd).triangles())
        blases.append(ctx.upload_blas(bvh, tris))
        host.append((bvh.nodes[:bvh.nodes_used], bvh.nodes_used, tris))
    n = 96
    blas_of = np.arange(n) % 3
    xf, inv = random_instances(n, 7)
    sc = ctx.scene([blases[i] for i in blas_of], xf, inv)
    gpu_nodes, gpu_used = sc.download_tlas()
    omin = np.zeros((n, 3), np.float32)
    omax = np.zeros((n, 3), np.float32)
    for i in range(n):
        nd = host[blas_of[i]][0]
        omin[i], omax[i] = orc.object_bounds(nd[0]["bounds_min"], nd[0]["bounds_max"], xf[i])
    ref_nodes, ref_used = orc.tlas_build(omin, omax)
    assert gpu_used == ref_used
    assert gpu_nodes.tobytes() == ref_nodes.tobytes(), "TLAS not bit-identical to Tlas::rebuild"
    rays = np.concatenate([scenes.look_at_rays(160, 96, (0, 0, -60), (0, 0, 0), 60.0),
                           scenes.sphere_rays(20000, 5, box=25.0)])
    sa = orc.SceneArrays(host, blas_of, inv)
    ref = orc.scene_intersect(ref_nodes, ref_used, sa, rays)
    assert_hits_equal(sc.intersect(rays), ref, "scene")
    assert (ref["prim"] != bt.MISS).sum() > 1000


@pytest.mark.parametrize("n,dup", [(1, 0), (2, 0), (3, 0), (37, 0), (300, 3), (1000, 0), (1000, 2), (4096, 0),
                                   (4097, 0), (12000, 5)])
def test_tlas_rebuild_sizes_and_ties(ctx, n, dup):
    """TLAS nodes bit-identical to Tlas::rebuild from 1 object to 12,000 (above 4,096 the rebuild
    keeps its state in global instead of shared memory); with dup > 0 every dup-th object copies
    object 0's transform, so find_best_match meets exact area ties (decided by list position) and
    zero-area merges."""
    tris, bvh = build(scenes.displaced_icosphere(2, 5).triangles())
    blas = ctx.upload_blas(bvh, tris)
    xf, inv = random_instances(n, 100 + n)
    if dup:
        xf[::dup] = xf[0]
        inv[::dup] = inv[0]
    sc = ctx.scene([blas] * n, xf, inv)
    gpu_nodes, gpu_used = sc.download_tlas()
    root = bvh.nodes[0]
    omin = np.zeros((n, 3), np.float32)
    omax = np.zeros((n, 3), np.float32)
    for i in range(n):
        omin[i], omax[i] = orc.object_bounds(root["bounds_min"], root["bounds_max"], xf[i])
    ref_nodes, ref_used = orc.tlas_build(omin, omax)
    assert gpu_used == ref_used
    assert gpu_nodes.tobytes() == ref_nodes.tobytes(), "TLAS not bit-identical to Tlas::rebuild"
    sc.free()


def test_scene_above_the_object_limit_is_rejected(ctx):
    """A TLAS of n objects has 2n nodes in 16-bit indices (LeftRightIndex): 32,768 objects at most."""
    tris, bvh = build(scenes.displaced_icosphere(1, 5).triangles())
    blas = ctx.upload_blas(bvh, tris)
    xf, inv = random_instances(32769, 7)
    with pytest.raises(bt.BvhGpuError):
        ctx.scene([blas] * 32769, xf, inv)


# ---- render ----------------------------------------------------------------------------------------

def test_render_quad_viewport_matches_oracle(ctx):
    quad = np.array([[-1, -1, 0, 1, 1, 0, -1, 1, 0], [-1, -1, 0, 1, -1, 0, 1, 1, 0]], np.float32)
    tris, bvh = build(quad)
    blas = ctx.upload_blas(bvh, tris)
    cam = bt.Camera((-1, 1, -1, 1, 1, 100), (0, 0, 2), (0, 0, -1), (1, 0, 0), (0, 1, 0))
    acc = [1, 1, 1, 0, 0, 0]
    sh = [255, 255, 255, 255, 0, 0, 0, 255]
    rgba, n = blas.render(cam, 640, 640, bt.ACC_INTERSECTION, bt.SHADER_INTERSECTION, acc, sh)
    ref, _ = orc.render(cam.corners(), cam.view_inv, 640, 640, bvh.nodes, bvh.nodes_used, tris,
                        orc.ACC_INTERSECTION, orc.SH_INTERSECTION, acc_params=acc, shader_params=sh)
    assert n == 640 * 640
    assert np.array_equal(rgba, ref)


@pytest.mark.parametrize("acc,shader", [(bt.ACC_DEPTH, bt.SHADER_DEPTH), (bt.ACC_UV, bt.SHADER_RADIANCE),
                                        (bt.ACC_NORMAL, bt.SHADER_RADIANCE)])
def test_render_shaders_match_oracle(ctx, acc, shader):
    mesh = scenes.displaced_icosphere(4, seed=9)
    tris0 = mesh.triangles()
    # per-corner normals = unit directions of the vertices, permuted like the triangles
    nrm0 = np.ascontiguousarray(mesh.dirs[mesh.faces].reshape(-1, 9).astype(np.float32))
    tris = tris0.copy()
    bvh = bt.BvhBuilder().build_for(tris)
    order = {t.tobytes(): i for i, t in enumerate(tris0)}
    perm = np.array([order[t.tobytes()] for t in tris])
    nrm = nrm0[perm]
    blas = ctx.upload_blas(bvh, tris)
    cam = bt.Camera((-0.5, 0.5, -0.5, 0.5, 1, 100), (0, 0, -3), (0, 0, 1), (-1, 0, 0), (0, 1, 0))
    ap = np.eye(4, dtype=np.float32).reshape(16) if acc == bt.ACC_NORMAL else None
    sp = [40.0, 2.0] if shader == bt.SHADER_DEPTH else None
    rgba, _ = blas.render(cam, 256, 192, acc, shader, ap, sp, nrm if acc == bt.ACC_NORMAL else None)
    ref, _ = orc.render(cam.corners(), cam.view_inv, 256, 192, bvh.nodes, bvh.nodes_used, tris, acc, shader,
                        acc_params=ap, shader_params=sp, normals=nrm if acc == bt.ACC_NORMAL else None)
    assert np.array_equal(rgba, ref)
    assert (rgba[..., :3] != 0).any()


def test_render_texture_material_matches_oracle(ctx):
    """TextureMaterialAccumulator: per-corner spherical texture coordinates (some outside [0, 1],
    exercising the `as usize` saturation and the modulo wrap) on an RGB8 texture."""
    mesh = scenes.displaced_icosphere(4, seed=10)
    tris0 = mesh.triangles()
    d = mesh.dirs.astype(np.float64)
    uv_v = np.stack([np.arctan2(d[:, 2], d[:, 0]) / (2 * np.pi) * 3.0 + 0.5,
                     np.arccos(np.clip(d[:, 1], -1, 1)) / np.pi * 2.0 - 0.25], 1).astype(np.float32)
    tc0 = np.ascontiguousarray(uv_v[mesh.faces].reshape(-1, 6))
    tris = tris0.copy()
    bvh = bt.BvhBuilder().build_for(tris)
    order = {t.tobytes(): i for i, t in enumerate(tris0)}
    tc = tc0[np.array([order[t.tobytes()] for t in tris])]
    rng = np.random.default_rng(5)
    texels = rng.integers(0, 256, (37, 53, 3), dtype=np.uint8)
    blas = ctx.upload_blas(bvh, tris)
    cam = bt.Camera((-0.5, 0.5, -0.5, 0.5, 1, 100), (0, 0, -3), (0, 0, 1), (-1, 0, 0), (0, 1, 0))
    rgba, rays = blas.render_textured(cam, 200, 150, tc, texels)
    ref, _ = orc.render(cam.corners(), cam.view_inv, 200, 150, bvh.nodes, bvh.nodes_used, tris,
                        bt.ACC_TEXTURE, bt.SHADER_RADIANCE, tex_coords=tc, texels=texels)
    assert rays == 200 * 150
    assert np.array_equal(rgba, ref)
    assert len(np.unique(rgba.reshape(-1, 4), axis=0)) > 100


# ---- uneven batch ------------------------------------------------------------------------------------

def test_uneven_batch_persistent_equals_plain_equals_oracle(ctx):
    specs = [(scenes.soup(1000, 1), 5000), (scenes.displaced_icosphere(3, 2).triangles(), 30000),
             (scenes.soup(7000, 3, scale=1.5), 1000), (scenes.displaced_icosphere(1, 4).triangles(), 64)]
    items, rays_all, refs = [], [], []
    off = 0
    for k, (t, nr) in enumerate(specs):
        tris, bvh = build(t)
        b = ctx.upload_blas(bvh, tris)
        rays = np.concatenate([scenes.look_at_rays(nr // 2 // 8 * 8 or 8, 2, (0, 0, -25), (0, 0, 0), 40.0),
                               scenes.sphere_rays(nr - (nr // 2 // 8 * 8 or 8) * 2, 10 + k)])
        items.append((b.id, off, len(rays), 0))
        rays_all.append(rays)
        refs.append(orc.bvh_intersect(bvh.nodes, bvh.nodes_used, tris, rays, threads=8))
        off += len(rays)
        specs[k] = (t, nr, b)
    rays = np.concatenate(rays_all)
    ref = np.concatenate(refs)
    items = np.array(items, dtype=bt.BATCH_ITEM)
    plain = ctx.trace_batch(items, rays, bt.MODE_PLAIN)
    pers = ctx.trace_batch(items, rays, bt.MODE_PERSISTENT)
    assert_hits_equal(plain, ref, "batch plain")
    assert_hits_equal(pers, ref, "batch persistent")


def test_persistent_batch_in_a_graph_needs_a_known_item_list(ctx):
    """A persistent batch sets up its item table synchronously, which a stream capture cannot
    record: under capture a new item list is refused (status 1, nothing recorded, the capture still
    ends cleanly); a list traced once before capture replays from the graph with the same hits."""
    t1, b1 = build(scenes.soup(800, 31))
    t2, b2 = build(scenes.displaced_icosphere(2, 32).triangles())
    blas1, blas2 = ctx.upload_blas(b1, t1), ctx.upload_blas(b2, t2)
    rays = np.concatenate([scenes.sphere_rays(3000, 33), scenes.sphere_rays(2000, 34, box=3.0)])
    items = np.array([(blas1.id, 0, 3000, 0), (blas2.id, 3000, 2000, 0)], dtype=bt.BATCH_ITEM)
    new_items = np.array([(blas2.id, 0, 2500, 0), (blas1.id, 2500, 2500, 0)], dtype=bt.BATCH_ITEM)
    d_rays = ctx.to_device(rays)
    d_hits = ctx.device_buffer(len(rays) * bt.HIT.itemsize)
    expect = ctx.trace_batch(items, rays, bt.MODE_PERSISTENT)        # sets up `items`
    ctx.graph_begin()
    with pytest.raises(bt.BvhGpuError) as e:
        ctx.trace_batch_async(new_items, d_rays, len(rays), bt.MODE_PERSISTENT, d_hits)
    assert e.value.code == 1
    ctx.trace_batch_async(items, d_rays, len(rays), bt.MODE_PERSISTENT, d_hits)
    gid = ctx.graph_end()
    d_hits.zero()
    ctx.graph_launch(gid)
    ctx.sync()
    got = d_hits.download(np.zeros(len(rays), bt.HIT))
    ctx.graph_free(gid)
    assert got.tobytes() == expect.tobytes()


# ---- errors -----------------------------------------------------------------------------------------

def test_invalid_inputs_are_rejected(ctx):
    tris, bvh = build(scenes.soup(100, 1))
    bad = bvh.nodes.copy()
    bad[0]["left_first"] = 10 ** 6   # child index out of range
    with pytest.raises(bt.BvhGpuError) as e:
        ctx.upload_blas(bt.Bvh(bad, bvh.nodes_used), tris)
    assert e.value.code == 1
    with pytest.raises(bt.BvhGpuError):
        ctx.upload_blas(bvh, tris[:10])   # leaves address triangles past the end
    with pytest.raises(bt.BvhGpuError):
        ctx.scene([])


def test_stack_overflow_is_reported_not_faulted(ctx):
    # A valid but degenerate tree deeper than the largest compiled stack (256): a chain of
    # nested identical boxes whose far child is always pushed (the leaf triangles lie off the
    # ray, so no hit ever shrinks the ray and culls the chain).
    depth = 300
    nodes = np.zeros(2 * depth + 2, bt.NODE)
    tri = np.array([[5, 5, 0, 6, 5, 0, 5, 6, 0]], np.float32)
    tris = np.repeat(tri, depth + 1, axis=0)
    box_min, box_max = np.array([-1, -1, 0], np.float32), np.array([1, 1, 0], np.float32)
    used = 2
    cur = 0
    for lvl in range(depth):
        # equal entry distances send the traversal to the right child first (bvh.rs:271-275),
        # so the chain continues on the right and every left leaf is pushed
        l, r = used, used + 1
        used += 2
        nodes[cur]["left_first"] = l
        nodes[cur]["primitive_count"] = 0
        nodes[cur]["bounds_min"], nodes[cur]["bounds_max"] = box_min, box_max
        nodes[l]["left_first"], nodes[l]["primitive_count"] = lvl, 1
        nodes[l]["bounds_min"], nodes[l]["bounds_max"] = box_min, box_max
        cur = r
    nodes[cur]["left_first"], nodes[cur]["primitive_count"] = depth, 1
    nodes[cur]["bounds_min"], nodes[cur]["bounds_max"] = box_min, box_max
    blas = ctx.upload_blas(bt.Bvh(nodes, used), tris)
    rays = orc.make_rays([[0, 0, -5]], [[0, 0, 1]])
    with pytest.raises(bt.BvhGpuError) as e:
        blas.intersect(rays)
    assert e.value.code == 4
    # the context stays usable
    t2, b2 = build(scenes.soup(50, 2))
    ok = ctx.upload_blas(b2, t2).intersect(rays)
    assert len(ok) == 1
