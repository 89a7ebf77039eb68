"""The parity checker (oracle/checks.py) on planted differences, CPU only."""
import numpy as np

from oracle import checks
from oracle import oracle as orc


def _hits(n, seed=0):
    rng = np.random.default_rng(seed)
    h = checks.miss_hits(n)
    hit = rng.random(n) < 0.6
    h["t"][hit] = rng.uniform(1, 10, hit.sum()).astype(np.float32)
    h["u"][hit] = rng.uniform(0, 0.5, hit.sum()).astype(np.float32)
    h["v"][hit] = rng.uniform(0, 0.5, hit.sum()).astype(np.float32)
    h["prim"][hit] = rng.integers(0, 1000, hit.sum())
    h["inst"][hit] = 0
    return h


def test_identical_hits_pass():
    ref = _hits(1000)
    r = checks.compare_hits(ref.copy(), ref, np.zeros(1000, bool))
    assert r["prim_mismatch"] == r["inst_mismatch"] == r["tuv_not_bit_identical"] == 0
    assert r["mismatch_outside_near_ties"] == 0 and r["max_rel_tuv"] == 0.0 and checks.passed(r)


def test_planted_differences_are_counted():
    ref = _hits(1000)
    gpu = ref.copy()
    hit = np.nonzero(ref["prim"] != orc.MISS)[0]
    gpu["prim"][hit[0]] += 1                                   # an id mismatch
    gpu["t"][hit[1]] = np.nextafter(gpu["t"][hit[1]], np.float32(np.inf))  # 1 ulp: in tolerance
    gpu["u"][hit[2]] *= np.float32(1.001)                      # out of tolerance
    gpu["inst"][hit[3]] = 5
    near = np.zeros(1000, bool)
    near[hit[3]] = True                                        # a near-tie ray, counted apart
    r = checks.compare_hits(gpu, ref, near)
    assert r["prim_mismatch"] == 1 and r["inst_mismatch"] == 1
    assert r["tuv_not_bit_identical"] == 2 and r["tuv_out_of_tolerance"] == 1
    assert r["near_tie_rays"] == 1 and r["near_tie_mismatch"] == 1
    assert r["mismatch_outside_near_ties"] == 2 and not checks.passed(r)
    assert 9e-4 < r["max_rel_tuv"] < 1.1e-3


def test_merge_sums_and_keeps_max():
    a = {"rays_checked": 3, "prim_mismatch": 1, "max_rel_tuv": 1e-7, "near_tie_rays": 2}
    b = {"rays_checked": 4, "prim_mismatch": 0, "max_rel_tuv": 3e-7, "near_tie_rays": None}
    m = checks.merge([a, b])
    assert m == {"rays_checked": 7, "prim_mismatch": 1, "max_rel_tuv": 3e-7, "near_tie_rays": None}


def test_frame_with_bounce_matches_separate_calls():
    from bvhtracer_gb300 import scenes
    tris, rays, _ = scenes.icosphere_frame(seed=1, width=64, height=48)
    t, nodes, used = orc.bvh_build(tris)
    h0, b, valid, h1 = checks.frame_with_bounce(nodes, used, t, rays, 7)
    assert h0.tobytes() == orc.bvh_intersect(nodes, used, t, rays).tobytes()
    assert valid.sum() == (h0["prim"] != orc.MISS).sum() > 0
    assert h1[valid].tobytes() == orc.bvh_intersect(nodes, used, t, b[valid]).tobytes()
    assert np.all(h1["prim"][~valid] == orc.MISS)


def test_descent_checkpoint_round_trip(tmp_path):
    """save_descent_state / load_descent_state: vertices bit for bit, step, losses and rate."""
    import bvhtracer_gb300 as bt
    rng = np.random.default_rng(2)
    verts = rng.standard_normal((100, 3)).astype(np.float32)
    path = str(tmp_path / "descent.npz")
    bt.save_descent_state(path, verts, 40, [3.0, 2.5, 2.25], lr=0.01)
    st = bt.load_descent_state(path)
    assert st["verts"].tobytes() == verts.tobytes() and st["step"] == 40
    assert st["losses"] == [3.0, 2.5, 2.25] and st["lr"] == 0.01
    bt.save_descent_state(path, verts * 2, 50)  # overwrite in place
    st = bt.load_descent_state(path)
    assert st["step"] == 50 and st["lr"] is None and st["losses"] == []
    assert [p.name for p in tmp_path.iterdir()] == ["descent.npz"]
