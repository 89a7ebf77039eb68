"""Hidden trees under large leaves: the exact in-leaf culling gives the reference's results bit for
bit.

Leaves of at least 16 triangles get a hidden tree of boxes over their triangles (spatial order,
leaves of at most 4 triangles), and a box is skipped for a ray only when provably no triangle in it
is accepted at or below the ray's closest t.  These cases aim at what could break that: rays at
edges and vertices, exact ties between duplicate triangles in different hidden leaves (lowest
triangle index must win, but never against an equal t from an earlier leaf), boxes refreshed after
vertex updates and refits, non-finite vertices, axis-aligned and
denormal directions, short rays, instanced (transformed) BLASes and the plain and persistent bounce
kernels.  Everything is compared with the oracle's in-order leaf loop."""
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


def same(gpu, ref, what):
    bad = np.nonzero(gpu["prim"] != ref["prim"])[0]
    assert len(bad) == 0, f"{what}: {len(bad)} rays with different primitives, first {bad[:8]}"
    assert gpu.tobytes() == ref.tobytes(), f"{what}: hit records differ"


def one_leaf_bvh(tris):
    """A BVH whose root is one leaf holding every triangle (the reference's flat extreme)."""
    nodes = np.zeros(2, bt.NODE)
    v = tris.reshape(-1, 3)
    nodes[0]["bounds_min"] = v.min(0)
    nodes[0]["bounds_max"] = v.max(0)
    nodes[0]["primitive_count"] = len(tris)
    nodes[0]["left_first"] = 0
    return bt.Bvh(nodes, 2)


def edge_rays(tris, n, seed, eye_dist=6.0):
    """Rays from random eyes aimed exactly at triangle vertices, edge midpoints and centroids."""
    rng = np.random.default_rng(seed)
    k = rng.integers(0, len(tris), n)
    t = tris[k].reshape(n, 3, 3).astype(np.float64)
    pick = rng.integers(0, 4, n)
    a = np.where(pick[:, None] == 0, t[:, 0], np.where(pick[:, None] == 1, 0.5 * (t[:, 0] + t[:, 1]),
                 np.where(pick[:, None] == 2, 0.5 * (t[:, 1] + t[:, 2]), t.mean(1))))
    eye = rng.standard_normal((n, 3))
    eye = eye / np.linalg.norm(eye, axis=1, keepdims=True) * eye_dist
    d = a - eye
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return orc.make_rays(eye.astype(np.float32), d.astype(np.float32))


def test_flat_leaf_edges_vertices_and_random(ctx):
    tris = scenes.displaced_icosphere(4, 7).triangles().copy()  # 5,120 triangles in one leaf
    bvh = one_leaf_bvh(tris)
    blas = ctx.upload_blas(bvh, tris)
    h = blas.hidden()
    assert h["pairs"] >= len(tris) // 2 and h["depth"] >= 5  # 4-wide levels
    rays = np.concatenate([edge_rays(tris, 20000, 1), scenes.sphere_rays(20000, 2, box=4.0)])
    ref = orc.bvh_intersect(bvh.nodes, bvh.nodes_used, tris, rays, threads=8)
    same(blas.intersect(rays), ref, "flat leaf")


def test_reference_bvh_leaves_get_hidden_trees(ctx):
    tris = scenes.displaced_icosphere(6, 0).triangles().copy()
    bvh = bt.BvhBuilder().build_for(tris)
    blas = ctx.upload_blas(bvh, tris)
    assert blas.hidden()["pairs"] >= len(tris) // 2  # the reference's leaves of 1.7k-3.4k triangles
    rays = edge_rays(tris, 30000, 3, eye_dist=4.0)
    same(blas.intersect(rays), orc.bvh_intersect(bvh.nodes, bvh.nodes_used, tris, rays, threads=8), "ref bvh")


def test_duplicate_triangles_in_different_hidden_leaves_tie_to_lowest_index(ctx):
    rng = np.random.default_rng(5)
    base = np.array([[-1, -1, 0, 1, -1, 0, 0, 1, 0]], np.float32)
    other = rng.uniform(-3, 3, (600, 9)).astype(np.float32)
    other[:, 2::3] += np.float32(4.0)  # all behind the duplicates (z = 0) as seen from -z
    tris = np.concatenate([other[:300], np.repeat(base, 200, 0), other[300:]])  # 200 exact copies
    perm = rng.permutation(len(tris))
    tris = np.ascontiguousarray(tris[perm])
    bvh = one_leaf_bvh(tris)
    blas = ctx.upload_blas(bvh, tris)
    assert blas.hidden()["nodes"] > 100
    o = np.tile(np.array([0.05, -0.1, -5], np.float32), (64, 1))
    d = np.tile(np.array([0, 0, 1], np.float32), (64, 1))
    d[:, :2] = rng.uniform(-0.05, 0.05, (64, 2))
    rays = orc.make_rays(o, np.array([orc.normalize(x) for x in d]))
    ref = orc.bvh_intersect(bvh.nodes, bvh.nodes_used, tris, rays)
    copies = np.nonzero((tris == base[0]).all(1))[0]
    assert np.all(ref["prim"] == copies.min())
    same(blas.intersect(rays), ref, "duplicates")


@pytest.mark.parametrize("left_nearer", [False, True])
def test_equal_t_in_a_later_leaf_is_not_taken(ctx, left_nearer):
    """The same triangle in two reference leaves (indices 20 and 45): the leaf visited first keeps
    the hit, whatever the indices -- the reference's strict `<` across leaves."""
    rng = np.random.default_rng(21)
    tris = rng.uniform(-3, 3, (64, 9)).astype(np.float32)
    tris[:, 2::3] = rng.uniform(2, 6, (64, 3)).astype(np.float32)  # behind z = 0
    d = np.array([-1, -1, 0, 1, -1, 0, 0, 1, 0], np.float32)
    tris[20] = d
    tris[45] = d
    v = tris.reshape(-1, 3)
    nodes = np.zeros(4, bt.NODE)
    nodes[0]["bounds_min"], nodes[0]["bounds_max"] = v.min(0), v.max(0)
    nodes[0]["left_first"] = 2
    for i, first in ((2, 0), (3, 32)):
        nodes[i]["bounds_min"], nodes[i]["bounds_max"] = v.min(0), v.max(0)
        nodes[i]["left_first"] = first
        nodes[i]["primitive_count"] = 32
    if left_nearer:
        nodes[2]["bounds_min"][2] -= np.float32(0.5)
    bvh = bt.Bvh(nodes, 4)
    blas = ctx.upload_blas(bvh, tris)
    assert blas.hidden()["pairs"] >= 32
    rays = orc.make_rays(np.tile(np.array([0.05, -0.2, -5], np.float32), (8, 1)),
                         np.tile(np.array([0, 0, 1], np.float32), (8, 1)))
    ref = orc.bvh_intersect(bvh.nodes, bvh.nodes_used, tris, rays)
    assert np.all(ref["prim"] == (20 if left_nearer else 45))
    same(blas.intersect(rays), ref, "equal t across leaves")


def test_hidden_boxes_follow_vertex_updates_and_refit(ctx):
    tris, bvh = scenes.displaced_icosphere(5, 2).triangles().copy(), None
    bvh = bt.BvhBuilder().build_for(tris)
    blas = ctx.upload_blas(bvh, tris)
    rays = edge_rays(tris, 20000, 4)
    rng = np.random.default_rng(8)
    moved = (tris * np.float32(1.3) + rng.uniform(-0.02, 0.02, tris.shape).astype(np.float32)).astype(np.float32)
    blas.update_vertices(moved)
    blas.refit()
    nodes = orc.bvh_refit(bvh.nodes, bvh.nodes_used, moved)
    rays2 = edge_rays(moved, 20000, 5)
    for r in (rays, rays2):
        same(blas.intersect(r), orc.bvh_intersect(nodes, bvh.nodes_used, moved, r, threads=8), "after refit")


def test_non_finite_vertices_and_odd_rays(ctx):
    tris = scenes.displaced_icosphere(4, 3).triangles().copy()
    tris[17, 0] = np.nan
    tris[900, 4] = np.inf
    tris[2000, 8] = -np.inf
    tris[3001:3005] = np.float32(1e20)
    bvh = one_leaf_bvh(np.nan_to_num(tris, nan=0.0, posinf=1e20, neginf=-1e20))
    blas = ctx.upload_blas(bvh, tris)
    rays = np.concatenate([scenes.sphere_rays(20000, 6, box=4.0), edge_rays(tris[:3000], 5000, 7)])
    f32max = np.finfo(np.float32).max
    extra = orc.make_rays([[0, 0, -10], [0, 0, -10], [0.1, 0.2, -10], [0, 0, -10], [0.3, 0.1, -10], [1e30, 0, 0],
                           [0.2, 0.2, -3]],
                          [[0, 0, 1], [1e-40, 0, 1], [-1e-30, 1e-38, 1], [0, 1, 0], [0, 0, 1], [-1, 0, 0], [0, 0, 1]],
                          t=[f32max, f32max, f32max, 3.0, 9.3, f32max, 1e-5])
    rays = np.concatenate([rays, extra])
    ref = orc.bvh_intersect(bvh.nodes, bvh.nodes_used, tris, rays, threads=8)
    same(blas.intersect(rays), ref, "non-finite")


def test_short_rays_stop_at_their_t(ctx):
    tris = scenes.displaced_icosphere(5, 4).triangles().copy()
    bvh = bt.BvhBuilder().build_for(tris)
    blas = ctx.upload_blas(bvh, tris)
    rays = edge_rays(tris, 20000, 9)
    full = orc.bvh_intersect(bvh.nodes, bvh.nodes_used, tris, rays, threads=8)
    hit = full["prim"] != bt.MISS
    # limit every ray to exactly its closest t, to just below it and to a random fraction
    rng = np.random.default_rng(10)
    for lim in (full["t"], np.nextafter(full["t"], np.float32(0)), full["t"] * rng.uniform(0.5, 1.5, len(rays))):
        r = rays.copy()
        r["t"] = np.where(hit, lim, np.finfo(np.float32).max).astype(np.float32)
        same(blas.intersect(r), orc.bvh_intersect(bvh.nodes, bvh.nodes_used, tris, r, threads=8), "short rays")


def test_bounce_kernels_with_hidden_trees(ctx):
    tris = scenes.displaced_icosphere(6, 1).triangles().copy()
    bvh = bt.BvhBuilder().build_for(tris)
    blas = ctx.upload_blas(bvh, tris)
    prim = scenes.look_at_rays(160, 120, (0, 0, -3.2), (0, 0, 0), 50.0)
    ref0 = orc.bvh_intersect(bvh.nodes, bvh.nodes_used, tris, prim, threads=8)
    b2, valid = orc.bounce_rays(prim, ref0, tris, 99)
    ref1 = np.zeros(len(prim), orc.HIT)
    ref1["t"] = np.finfo(np.float32).max
    ref1["prim"] = ref1["inst"] = bt.MISS
    ref1[valid] = orc.bvh_intersect(bvh.nodes, bvh.nodes_used, tris, b2[valid], threads=8)
    for mode in (bt.MODE_PLAIN, bt.MODE_PERSISTENT):
        h0, h1, _ = blas.trace_bounce(prim, 99, mode)
        same(h0, ref0, f"primaries, mode {mode}")
        same(h1, ref1, f"bounces, mode {mode}")


def test_instanced_scene_with_hidden_trees(ctx):
    tris = scenes.displaced_icosphere(5, 6).triangles().copy()
    bvh = bt.BvhBuilder().build_for(tris)
    blas = ctx.upload_blas(bvh, tris)
    assert blas.hidden()["pairs"] > 0
    n = 24
    rng = np.random.default_rng(11)
    xf = np.zeros((n, 16), np.float32)
    inv = np.zeros((n, 16), np.float32)
    for i in range(n):
        s = rng.uniform(0.5, 2.0)
        m = np.eye(4) * s
        m[3, 3] = 1
        m[:3, 3] = rng.uniform(-6, 6, 3)
        xf[i] = m.T.reshape(16)
        inv[i] = np.linalg.inv(m).T.reshape(16)
    sc = ctx.scene([blas] * n, xf, inv)
    tl, used = sc.download_tlas()
    rays = scenes.sphere_rays(30000, 12, box=12.0)
    sa = orc.SceneArrays([(bvh.nodes[:bvh.nodes_used], bvh.nodes_used, tris)], np.zeros(n, np.int64), inv)
    ref = orc.scene_intersect(tl, used, sa, rays, threads=8)
    same(sc.intersect(rays), ref, "scene")


@pytest.mark.parametrize("hidden", [500, 100000])
def test_large_triangles_far_camera_with_normal_cones(ctx, hidden):
    """The sphere at 10x scale seen from distance 30 and 300 (margins set by the leaves' normal
    cones), with rays at vertices and edges from every side -- including the grazing ones at the
    silhouette, where the cone gives no bound -- at a moderate and an unlimited margin."""
    verts, faces, _, _, cam, _ = scenes.lambert_scene(seed=0, level=5, width=96, height=96)
    tris = np.ascontiguousarray(verts[faces].reshape(-1, 9), np.float32)
    bvh = bt.BvhBuilder().build_for(tris)
    blas = ctx.upload_blas(bvh, tris)
    saved = ctx.tune_get(bt.K_TRACE_BLAS)
    try:
        ctx.tune_set(bt.K_TRACE_BLAS, hidden=hidden)
        rays = np.concatenate([cam, edge_rays(tris, 20000, 31, eye_dist=30.0), edge_rays(tris, 20000, 32, eye_dist=300.0)])
        ref = orc.bvh_intersect(bvh.nodes, bvh.nodes_used, tris, rays, threads=8)
        assert (ref["prim"] != bt.MISS).sum() > 30000
        same(blas.intersect(rays), ref, f"cones, hidden {hidden}")
    finally:
        ctx.tune_set(bt.K_TRACE_BLAS, **saved)


def test_trace_counts_measure_the_culled_work(ctx):
    """The counting traversal returns the plain call's hits, and its counters show what the hidden
    trees save: triangles tested per ray far below the reference's (the oracle's counters)."""
    tris = scenes.displaced_icosphere(6, 0).triangles().copy()
    bvh = bt.BvhBuilder().build_for(tris)
    blas = ctx.upload_blas(bvh, tris)
    rays = scenes.look_at_rays(256, 192, (0, 0, -3.2), (0, 0, 0), 50.0)
    n = len(rays)
    d_rays = ctx.to_device(rays)
    d_h = ctx.device_buffer(n * bt.HIT.itemsize)
    c = blas.trace_counts(d_rays, n, d_h)
    got = d_h.download(np.zeros(n, bt.HIT))
    assert got.tobytes() == blas.intersect(rays).tobytes()
    ref, cnt = orc.bvh_intersect(bvh.nodes, bvh.nodes_used, tris, rays, counters=True)
    assert got.tobytes() == ref.tobytes()
    assert c["ref_nodes"] == int(cnt["interior"].sum())  # the reference's own node visits
    tested = 2 * c["hidden_pairs"] + c["lane_tris"] + c["warp_tris"]
    assert c["hidden_entries"] > 0 and tested < 0.05 * int(cnt["tris"].sum())


F32 = np.float32
U0 = F32(5.9604645e-8)
HUGE = F32(1e15)
HIDDEN_LEAF, HIDDEN_INTERIOR, CONE_MASK = 0x80000000, 0x40000000, 0x0FFFFFFF


def group_seal(lo, hi, e1m, e2m, finite):
    """The leaf seal of cull.cuh (group_seal) in float32: the raw bounds of v0, v0 + e1, v0 + e2
    rounded outward by 4 u0, Q = (max |e1_i| + max |e2_i|) (1 + 4 u0), B = the largest |bound|."""
    one_up, one_dn = F32(1) + F32(4) * U0, F32(1) - F32(4) * U0
    ok = finite and e1m < HUGE and e2m < HUGE and np.all(np.abs(lo) < HUGE) and np.all(np.abs(hi) < HUGE)
    clo = np.where(lo < 0, lo * one_up, lo * one_dn).astype(F32)
    chi = np.where(hi < 0, hi * one_dn, hi * one_up).astype(F32)
    b = F32(max(0.0, float(np.abs(clo).max()), float(np.abs(chi).max())))
    if not ok:
        return np.zeros(3, F32), np.zeros(3, F32), F32(np.inf), F32(0)
    return clo, chi, F32((F32(e1m) + F32(e2m)) * one_up), b


def check_hidden_records(blas, tris, min_valid_share=0.0):
    """Every hidden node's box and every cone record's Q, B against group_seal over the node's own
    triangles (restated here in float32: exact, since they are minima and maxima), and every cone
    (axis, cos_phi, nmin) against the triangles it covers in float64."""
    hd = blas.hidden_download()
    nodes, cones, slots, table = hd["nodes"], hd["cones"], hd["slots"], hd["table"]
    ui = nodes.view(np.uint32)
    nused = blas.nodes_used
    p0 = (len(tris) + 1) // 2
    v = tris.reshape(-1, 3, 3).astype(F32)
    v0, e1, e2 = v[:, 0], (v[:, 1] - v[:, 0]).astype(F32), (v[:, 2] - v[:, 0]).astype(F32)
    p1, p2 = (v0 + e1).astype(F32), (v0 + e2).astype(F32)
    memo = {}

    def tri_set(first, count):
        """Triangles under a hidden entry (first, count)."""
        key = (first, count)
        if key in memo:
            return memo[key]
        if count & HIDDEN_LEAF:
            ids = slots[first - p0: first - p0 + (count & ~HIDDEN_LEAF)].ravel()
            out = ids[ids != 0xFFFFFFFF]
        else:
            k = ((count >> 28) & 3) + 1
            out = np.concatenate([tri_set(int(ui[first - nused + c, 3]), int(ui[first - nused + c, 7]))
                                  for c in range(k)])
        memo[key] = out
        return out

    def seal_of(ids):
        lo = np.minimum(np.minimum(v0[ids], p1[ids]), p2[ids]).min(0)
        hi = np.maximum(np.maximum(v0[ids], p1[ids]), p2[ids]).max(0)
        finite = bool(np.isfinite(v0[ids]).all() and np.isfinite(e1[ids]).all() and np.isfinite(e2[ids]).all()
                      and np.isfinite(p1[ids]).all() and np.isfinite(p2[ids]).all())
        return group_seal(lo, hi, np.abs(e1[ids]).max(), np.abs(e2[ids]).max(), finite)

    checked_nodes = checked_cones = 0
    for i in range(len(nodes)):
        first, count = int(ui[i, 3]), int(ui[i, 7])
        lo, hi, _, _ = seal_of(tri_set(first, count))
        assert nodes[i, :3].tobytes() == lo.tobytes() and nodes[i, 4:7].tobytes() == hi.tobytes(), f"node {i}"
        checked_nodes += 1
    # cone records: at each hidden root (from the table) and at interior nodes; the count field of
    # an interior entry names the cone governing its subtree
    entries = [(int(f), int(c)) for f, c in table if c != 0]
    entries += [(int(ui[i, 3]), int(ui[i, 7])) for i in range(len(nodes)) if ui[i, 7] & HIDDEN_INTERIOR]
    valid = 0
    for first, count in entries:  # each interior entry names its own cone (the root's: the tree's)
        c = count & CONE_MASK
        ids = tri_set(first, count)
        _, _, q, b = seal_of(ids)
        assert cones[c, 6].tobytes() == q.tobytes() and cones[c, 7].tobytes() == b.tobytes(), f"cone {c} Q, B"
        n = np.cross(e1[ids].astype(np.float64), e2[ids].astype(np.float64))
        nl = np.linalg.norm(n, axis=1)
        a = cones[c, :3].astype(np.float64)
        if cones[c, 3] > 0:  # a valid cone: every normal line within the cone, no normal shorter than nmin
            cos = np.abs(n @ a) / (nl * np.linalg.norm(a))
            assert (cos >= cones[c, 3] * (1 - 1e-9)).all(), f"cone {c}"
            assert (nl >= cones[c, 5] * (1 - 1e-9)).all(), f"cone {c} nmin"
            valid += 1
        checked_cones += 1
    assert checked_nodes == len(nodes) and checked_cones == len(cones) and valid >= min_valid_share * len(cones)
    return checked_nodes, checked_cones


def test_hidden_records_equal_the_restated_seal_after_upload_and_updates(ctx):
    """The refresh (chunks of pairs per warp, combined in order) writes the boxes and Q, B that the
    seal gives over each node's triangles, bit for bit, and cones that hold every covered normal:
    after the upload and after two vertex updates (radial wobble, then a larger move)."""
    mesh = scenes.displaced_icosphere(6, 4)
    tris = mesh.triangles().copy()
    bvh = bt.BvhBuilder().build_for(tris)
    blas = ctx.upload_blas(bvh, tris)
    check_hidden_records(blas, tris, min_valid_share=0.5)
    rng = np.random.default_rng(9)
    for amp in (0.002, 0.01):  # 4 % and 20 % of an edge, per corner
        moved = (tris.reshape(-1, 3, 3) * (1 + amp * rng.standard_normal((len(tris), 3, 1)))).astype(F32)
        moved = np.ascontiguousarray(moved.reshape(-1, 9))
        blas.update_vertices(moved)
        tris = moved
        check_hidden_records(blas, tris)
