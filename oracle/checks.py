"""Parity checks of GPU results against the oracle, shared by the tests and bench.py.

TEST INFRASTRUCTURE ONLY: these helpers run the oracle (``oracle/bvh_oracle.cpp``, the CPU
restatement of the reference's traversal) and compare.  Only the tests, the smoke check and the
CPU-baseline / parity leg of ``bench.py`` call them; the product library never does.

The parity rule for the ray-BVH path: identical primitive and instance ids on every ray; t, u, v
within 1e-5 relative (the kernels follow the reference's f32 operation order, so they are expected
to be bit-identical, and that is counted too); rays whose two nearest hits lie within 1e-5
relative in t are counted apart ("near ties"), because a 1-ulp change of t could swap which
triangle is closest there.
"""
from __future__ import annotations

import numpy as np

from . import oracle as orc

REL_TOL = 1e-5


def miss_hits(n: int) -> np.ndarray:
    """n miss records (the reference's Option::None): t = FLT_MAX, u = v = 0, ids = MISS."""
    h = np.zeros(n, orc.HIT)
    h["t"] = orc.FLT_MAX
    h["prim"] = h["inst"] = orc.MISS
    return h


def compare_hits(gpu: np.ndarray, ref: np.ndarray, near: np.ndarray | None = None) -> dict:
    """Counts of differences between two hit arrays of the same rays.

    prim_mismatch / inst_mismatch: rays whose ids differ; tuv_not_bit_identical: rays with the
    same ids whose t, u or v differ in any bit; tuv_out_of_tolerance: those beyond REL_TOL;
    max_rel_tuv: the largest relative difference of t, u, v over rays with equal ids.  With a
    near-tie mask, mismatches on near-tie rays are also counted separately, and
    mismatch_outside_near_ties is what the parity bar forbids."""
    gpu = np.asarray(gpu)
    ref = np.asarray(ref)
    if len(gpu) != len(ref):
        raise ValueError(f"hit arrays differ in length: {len(gpu)} vs {len(ref)}")
    prim_bad = gpu["prim"] != ref["prim"]
    inst_bad = gpu["inst"] != ref["inst"]
    same = ~(prim_bad | inst_bad)
    max_rel = 0.0
    tol_bad = np.zeros(len(ref), bool)
    bits_bad = np.zeros(len(ref), bool)
    hit = same & (ref["prim"] != orc.MISS)
    for k in ("t", "u", "v"):
        g = gpu[k].astype(np.float64)
        r = ref[k].astype(np.float64)
        bits_bad |= same & (gpu[k].view(np.uint32) != ref[k].view(np.uint32))
        if hit.any():
            with np.errstate(invalid="ignore", over="ignore"):
                rel = np.abs(g[hit] - r[hit]) / np.maximum(np.abs(r[hit]), 1e-30)
            rel = np.nan_to_num(rel, nan=np.inf)
            max_rel = max(max_rel, float(rel.max()))
            idx = np.nonzero(hit)[0]
            tol_bad[idx] |= rel > REL_TOL
    bad = prim_bad | inst_bad | tol_bad
    out = {
        "rays_checked": int(len(ref)),
        "hits": int((ref["prim"] != orc.MISS).sum()),
        "prim_mismatch": int(prim_bad.sum()),
        "inst_mismatch": int(inst_bad.sum()),
        "tuv_not_bit_identical": int(bits_bad.sum()),
        "tuv_out_of_tolerance": int(tol_bad.sum()),
        "max_rel_tuv": max_rel,
    }
    if near is not None:
        near = np.asarray(near, bool)
        out["near_tie_rays"] = int(near.sum())
        out["near_tie_mismatch"] = int((bad & near).sum())
        out["mismatch_outside_near_ties"] = int((bad & ~near).sum())
    else:
        out["near_tie_rays"] = None
        out["mismatch_outside_near_ties"] = int(bad.sum())
    return out


def merge(parts: list[dict]) -> dict:
    """Sum of several compare_hits results (max of max_rel_tuv; near ties None if any is None)."""
    out: dict = {}
    for p in parts:
        for k, v in p.items():
            if k == "max_rel_tuv":
                out[k] = max(out.get(k, 0.0), v)
            elif v is None or out.get(k, 0) is None:
                out[k] = None
            else:
                out[k] = out.get(k, 0) + v
    return out


def passed(result: dict) -> bool:
    """The parity bar: no id or tolerance mismatch outside the near-tie rays."""
    return result.get("mismatch_outside_near_ties", 1) == 0


def frame_with_bounce(nodes, nodes_used, tris, rays, seed: int, threads: int = 1):
    """The oracle's primary hits, bounce rays (valid mask) and bounce hits in pixel order (a miss
    where the primary missed) of a single-BLAS frame: what bvhgpu_blas_trace_bounce returns."""
    h0 = orc.bvh_intersect(nodes, nodes_used, tris, rays, threads=threads)
    b, valid = orc.bounce_rays(rays, h0, tris, seed)
    h1 = miss_hits(len(rays))
    if valid.any():
        h1[valid] = orc.bvh_intersect(nodes, nodes_used, tris, b[valid], threads=threads)
    return h0, b, valid, h1


def frame_near_ties(nodes, tris, rays, bounce_rays, valid, threads: int = 1):
    """Near-tie masks of a frame's primaries and (in pixel order) of its bounce rays."""
    n0 = orc.near_ties(nodes, tris, rays, threads=threads)
    n1 = np.zeros(len(rays), bool)
    if valid.any():
        n1[valid] = orc.near_ties(nodes, tris, bounce_rays[valid], threads=threads)
    return n0, n1


def scene_state_reference(blas_states, blas_of, xf, inv):
    """The oracle's TLAS (Tlas::rebuild over the objects' world bounds) and scene arrays for a scene
    whose BLASes are given as (nodes, nodes_used, tris) and whose objects have the transforms xf /
    inverses inv (16 floats each, column-major)."""
    n = len(blas_of)
    omin = np.zeros((n, 3), np.float32)
    omax = np.zeros((n, 3), np.float32)
    for i in range(n):
        root = blas_states[blas_of[i]][0][0]
        omin[i], omax[i] = orc.object_bounds(root["bounds_min"], root["bounds_max"], xf[i])
    tlas, used = orc.tlas_build(omin, omax)
    return tlas, used, orc.SceneArrays(blas_states, blas_of, inv)


def scene_frame_with_bounce(tlas, tlas_used, sa, rays, seed: int, threads: int = 1):
    """Primary hits, bounce rays (valid mask) and bounce hits in pixel order of a scene frame: what
    bvhgpu_scene_trace_bounce_async writes."""
    h0 = orc.scene_intersect(tlas, tlas_used, sa, rays, threads=threads)
    b, valid = orc.scene_bounce_rays(sa, rays, h0, seed)
    h1 = miss_hits(len(rays))
    if valid.any():
        h1[valid] = orc.scene_intersect(tlas, tlas_used, sa, b[valid], threads=threads)
    return h0, b, valid, h1
