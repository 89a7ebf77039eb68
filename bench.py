"""Benchmark: Mrays/s of the ray-BVH hot path on one GB300; batched vs plain traversal with exact hit
ids checked against the oracle; adjoint ms/step.

Default run (one JSON line): the headline workload -- the displaced icosphere with 6 subdivisions
(81,920 triangles, the reference's SAH BVH), camera at distance 3, 1920 x 1080 primary rays plus one
cosine-weighted diffuse bounce per hit pixel, one step = one frame traced by one persistent
work-stealing launch (the plain trace / compact / trace pipeline timed beside it) -- with the other
three workloads attached as sub-objects: ``batch`` (uneven 64-scene batch, one persistent launch vs
one plain launch per scene), ``instanced`` (256 instances of 3 BLASes, 60 animated 1280 x 720
frames, each one CUDA graph) and ``adjoint`` (differentiable Lambertian render of 327,680 triangles
at 512 x 512, adjoint ms/step).  Inputs are resident on the device in the timed regions; the L2 is
flushed between steps.  Every line carries a ``parity`` object: the timed outputs compared with the
oracle (the CPU restatement of the reference's traversal) -- the whole frame for the headline;
a run with any mismatch outside the near-tie rays exits 1.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload default|icosphere|batch|instanced|lambert] [--mode persistent|plain]

``--impl reference`` times the CPU restatement of the reference's traversal (the reference is Rust
and cannot be built here) on the host cores, on a fixed sample of the headline frame, without
loading the CUDA library.  ``--gpus N`` without torchrun starts N ranks itself (one per GPU).
"""
from __future__ import annotations

import argparse
import ctypes
import importlib.util
import json
import os
import socket
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Mrays/s, 1 GB300: batched vs plain traversal, exact hit IDs; adjoint ms/step"
WORKLOAD = "displaced icosphere (6 subdivisions, 81,920 tris) 1920x1080 primaries + 1 diffuse bounce"
SEED = 0
BOUNCE_SEED = 12345


def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(
        os.environ.get("LOCAL_RANK", "0"))


def host_threads() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def load_scenes():
    """The seeded workload generator (bvhtracer_gb300/scenes.py) loaded by file path as a module of
    its own, so that code which must not touch the CUDA library (the reference arm) can use it."""
    path = os.path.join(ROOT, "bvhtracer_gb300", "scenes.py")
    spec = importlib.util.spec_from_file_location("bvh_workloads", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


# ---- clocks during the timed regions ------------------------------------------------------------------

class Clocks:
    """SM clock and clock-event reasons sampled while a timed region runs.

    Reads NVML directly (libnvidia-ml, every `period` seconds, read-only queries) so that short timed
    regions still get many samples; falls back to `nvidia-smi -lms 200`.  The device is the one the
    process sees as CUDA device `local_rank` (CUDA_VISIBLE_DEVICES honoured)."""

    REASON_BITS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown", 0x40: "hw_thermal_slowdown"}
    SMI_FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                  "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                  "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, local_rank: int, period: float = 0.001):
        self.local_rank = local_rank
        self.period = period
        self.samples = []  # (time, sm_mhz, max_mhz, reasons set)
        self.source = None
        self._stop = threading.Event()
        self._thread = None
        self._proc = None

    def _device_ident(self):
        vis = os.environ.get("CUDA_VISIBLE_DEVICES")
        if vis:
            ids = [v.strip() for v in vis.split(",") if v.strip()]
            if self.local_rank < len(ids):
                return ids[self.local_rank]
        return str(self.local_rank)

    def _nvml_open(self):
        nv = ctypes.CDLL("libnvidia-ml.so.1")
        if nv.nvmlInit_v2() != 0:
            return None
        h = ctypes.c_void_p()
        ident = self._device_ident()
        if ident.startswith("GPU-") or ident.startswith("MIG-"):
            rc = nv.nvmlDeviceGetHandleByUUID(ident.encode(), ctypes.byref(h))
        else:
            rc = nv.nvmlDeviceGetHandleByIndex_v2(int(ident), ctypes.byref(h))
        if rc != 0:
            return None
        reasons = getattr(nv, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            nv.nvmlDeviceGetCurrentClocksThrottleReasons
        return nv, h, reasons

    def start(self):
        try:
            opened = self._nvml_open()
        except (OSError, AttributeError, ValueError):
            opened = None
        if opened:
            self.source = f"NVML every {self.period * 1e3:.0f} ms"
            nv, h, reasons_fn = opened
            mx = ctypes.c_uint()
            nv.nvmlDeviceGetMaxClockInfo(h, 1, ctypes.byref(mx))  # NVML_CLOCK_SM = 1

            def run():
                clk, rs = ctypes.c_uint(), ctypes.c_ulonglong()
                while not self._stop.is_set():
                    if nv.nvmlDeviceGetClockInfo(h, 1, ctypes.byref(clk)) == 0 and \
                            reasons_fn(h, ctypes.byref(rs)) == 0:
                        names = {n for bit, n in self.REASON_BITS.items() if rs.value & bit}
                        self.samples.append((time.perf_counter(), float(clk.value), float(mx.value), names))
                    time.sleep(self.period)
            self._thread = threading.Thread(target=run, daemon=True)
            self._thread.start()
            return
        try:
            self._proc = subprocess.Popen(["nvidia-smi", f"--id={self._device_ident()}",
                                           f"--query-gpu={self.SMI_FIELDS}", "--format=csv,noheader,nounits",
                                           "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL,
                                          text=True)
        except OSError:
            return
        self.source = "nvidia-smi every 200 ms"
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]

        def read():
            for line in self._proc.stdout:
                p = [x.strip() for x in line.split(",")]
                try:
                    self.samples.append((time.perf_counter(), float(p[1]), float(p[2]),
                                         {n for n, v in zip(names, p[5:9]) if v.lower() == "active"}))
                except (ValueError, IndexError):
                    continue
        self._thread = threading.Thread(target=read, daemon=True)
        self._thread.start()
        t0 = time.perf_counter()
        while not self.samples and self._proc.poll() is None and time.perf_counter() - t0 < 3.0:
            time.sleep(0.01)

    def stop(self):
        self._stop.set()
        if self._proc:
            self._proc.terminate()
            try:
                self._proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self._proc.kill()
        if self._thread:
            self._thread.join(timeout=2)

    def summary(self, t0: float | None = None, t1: float | None = None):
        """Median SM clock, max clock and the union of reasons over the samples taken in [t0, t1]."""
        s = [x for x in self.samples if (t0 is None or x[0] >= t0) and (t1 is None or x[0] <= t1)]
        if not s:
            return None
        reasons = set()
        for x in s:
            reasons |= x[3]
        return {"sm_mhz": statistics.median(x[1] for x in s), "sm_max_mhz": max(x[2] for x in s),
                "reasons": sorted(reasons), "samples": len(s), "source": self.source}


class ClockedRegion:
    """with ClockedRegion(local_rank) as c: ... -> c.result: the clocks sampled inside the block."""

    def __init__(self, local_rank: int):
        self.clocks = Clocks(local_rank)
        self.result = None

    def __enter__(self):
        self.clocks.start()
        self.t0 = time.perf_counter()
        return self

    def __exit__(self, *exc):
        t1 = time.perf_counter()
        self.clocks.stop()
        self.result = self.clocks.summary(self.t0, t1)


# ---- shared helpers ---------------------------------------------------------------------------------------

TUNE_FIELDS = ("block", "min_blocks", "stack", "big_leaf", "refill", "hidden")


def apply_tune_args(ctx, args) -> dict:
    """Launch configs given with --tune KERNEL=block,min_blocks,stack,big_leaf,refill,hidden
    (e.g. the picks printed by an earlier tuned run), set on the context before any launch."""
    import bvhtracer_gb300 as bt
    given = {}
    for spec in args.tune or []:
        name, _, vals = spec.partition("=")
        if name not in bt._KERNELS:
            raise SystemExit(f"--tune: unknown kernel {name!r} (one of {', '.join(bt._KERNELS)})")
        try:
            nums = [int(v) for v in vals.split(",")]
        except ValueError:
            nums = []
        if len(nums) != len(TUNE_FIELDS):
            raise SystemExit(f"--tune {spec}: expected {len(TUNE_FIELDS)} values ({','.join(TUNE_FIELDS)})")
        cfg = dict(zip(TUNE_FIELDS, nums))
        ctx.tune_set(bt._KERNELS.index(name), **cfg)
        given[name] = dict(cfg, source="--tune")
    return given


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError, TypeError):
        return 6800.0, "fallback"


def count_bytes(c: dict, n: int) -> int:
    """Node and triangle bytes the traversal fetched for n rays with work counters c (summed):
    64 B per reference interior node (its two children), 32 B per hidden child box, 40 B per
    hidden-tree entry (table entry + root cone), 32 B per cone switch, 88 B per hidden pair (80 B
    pair + 8 B slot indices), 48 / 40 B per triangle tested by a lane / the warp, 32 B ray + 20 B hit."""
    node_b = 64 * c["ref_nodes"] + 32 * c["hidden_boxes"] + 40 * c["hidden_entries"] + 32 * c["cone_switches"]
    tri_b = 88 * c["hidden_pairs"] + 48 * c["lane_tris"] + 40 * c["warp_tris"]
    return node_b + tri_b + (32 + 20) * n


def fetched_bytes(ctx, blas, rays, seed):
    """Per-ray node and triangle bytes of the library's traversal, from bvhgpu_blas_trace_counts on
    the primaries and on their bounce rays (under the context's BVHGPU_K_TRACE_BLAS leaf policy:
    call inside leaf_policy() to count another kernel's policy)."""
    import bvhtracer_gb300 as bt
    out = {}
    b_rays, valid = blas.bounce_rays(rays, seed)
    for key, rs in (("primary", rays), ("bounce", b_rays[valid])):
        n = len(rs)
        d_r = ctx.to_device(rs)
        d_h = ctx.device_buffer(max(1, n) * bt.HIT.itemsize)
        c = blas.trace_counts(d_r, n, d_h)
        total = count_bytes(c, n)
        out[key] = {"rays": n, "bytes": total, "bytes_per_ray": total / max(1, n),
                    "per_ray": {k: v / max(1, n) for k, v in c.items()}}
    return out


class leaf_policy:
    """Temporarily gives BVHGPU_K_TRACE_BLAS (whose config the counting traversal follows) the leaf
    policy (big_leaf, hidden) of another kernel, so that the counted work is the timed kernel's."""

    def __init__(self, ctx, kernel):
        self.ctx, self.kernel = ctx, kernel

    def __enter__(self):
        import bvhtracer_gb300 as bt
        self.saved = self.ctx.tune_get(bt.K_TRACE_BLAS)
        src = self.ctx.tune_get(self.kernel)
        self.ctx.tune_set(bt.K_TRACE_BLAS, **dict(self.saved, big_leaf=src["big_leaf"], hidden=src["hidden"]))
        return src

    def __exit__(self, *exc):
        import bvhtracer_gb300 as bt
        self.ctx.tune_set(bt.K_TRACE_BLAS, **self.saved)


# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per launch of each workload's dominant
# kernel, from the ncu captures summarised under profiles/ (the command is in each summary).
NCU_TRAFFIC = {
    "persistent_bounce": (76.118528e6 + 49.763328e6, "ncu capture of the 1080p frame",
                          "profiles/k_persistent_bounce_icosphere_1080p_full.md"),
    "scene_bounce": (43.6e6 + 15.2e6, "ncu capture of one instanced 720p frame's trace launch",
                     "profiles/k_scene_persistent_bounce_instanced_720p_full.md"),
    # 8-scene capture: 584.9 MB for 10,057,687 rays; scaled to a launch by its ray count
    "trace_batch": (584.920064e6 / 10057687, "8-scene ncu capture, bytes per ray x rays",
                    "profiles/k_trace_batch_persistent_64_scene_batch.md"),
}


def parity_fail(line: dict) -> bool:
    """True when any parity object of the line (or of its sub-objects) has a mismatch outside the
    near-tie rays."""
    bad = False
    for key, val in line.items():
        if key == "parity" and isinstance(val, dict):
            for part in (val.get("checks") or {}).values():
                bad |= part.get("mismatch_outside_near_ties", 0) != 0
            bad |= val.get("identical_bvh") is False
        elif isinstance(val, dict) and key in ("batch", "instanced", "adjoint"):
            bad |= parity_fail(val)
    return bad


# ---- headline: the displaced-icosphere frame ----------------------------------------------------------------

def bench_icosphere(args, pg=None):
    import bvhtracer_gb300 as bt
    from bvhtracer_gb300 import scenes, shard
    rank, world, local_rank = dist_env()

    def barrier():
        if pg:
            pg.barrier()

    tris, rays, _ = scenes.icosphere_frame(seed=SEED)
    n = len(rays)
    # weak scaling: the job is `world` frames; rank r traces its contiguous range of the job's rays
    # (one frame each; the BVH is replicated, no collective on the data path)
    b0, b1 = shard.ray_range(world * n, rank, world)
    assert b1 - b0 == n
    tris_in = tris.copy()  # the build reorders its input in place; the oracle builds from the same input
    bvh = bt.BvhBuilder().build_for(tris)
    ctx = bt.Context(local_rank)
    given = apply_tune_args(ctx, args)
    blas = ctx.upload_blas(bvh, tris)
    d_rays = ctx.to_device(rays)
    d_h0 = ctx.device_buffer(n * bt.HIT.itemsize)
    d_h1 = ctx.device_buffer(n * bt.HIT.itemsize)
    mode = bt.MODE_PERSISTENT if args.mode == "persistent" else bt.MODE_PLAIN
    other = bt.MODE_PLAIN if mode == bt.MODE_PERSISTENT else bt.MODE_PERSISTENT
    mode_name = {bt.MODE_PERSISTENT: "persistent", bt.MODE_PLAIN: "plain"}

    h0 = np.zeros(n, bt.HIT)
    blas.trace_bounce_async(d_rays, n, BOUNCE_SEED, mode, d_h0, d_h1)
    ctx.sync()
    d_h0.download(h0)
    n_bounce = int((h0["prim"] != bt.MISS).sum())
    rays_per_step = n + n_bounce

    # autotune both pipelines on this frame (configs never change results, only speed)
    tuned, tune_s = dict(given), 0.0
    if not args.no_tune:
        t0 = time.perf_counter()
        cfg, ms_ = ctx.autotune(bt.K_PERSISTENT_BOUNCE, d_rays, n, d_h0, d_h1, target=blas.id, seed=BOUNCE_SEED,
                                reps=3)
        tuned["persistent_bounce"] = dict(cfg, ms=ms_)
        cfg, ms_ = ctx.autotune(bt.K_TRACE_BLAS, d_rays, n, d_h0, target=blas.id, reps=3)
        tuned["trace_blas"] = dict(cfg, ms=ms_)
        tune_s = time.perf_counter() - t0

    ev = [(ctx.event(), ctx.event()) for _ in range(args.steps)]

    def timed(m):
        for _ in range(args.warmup):
            ctx.flush_l2()
            blas.trace_bounce_async(d_rays, n, BOUNCE_SEED, m, d_h0, d_h1)
        ctx.sync()
        barrier()
        ctx.profile(True)
        ctx.profile_read()
        with ClockedRegion(local_rank) as clk:
            for s in range(args.steps):
                ctx.flush_l2()
                ev[s][0].record()
                blas.trace_bounce_async(d_rays, n, BOUNCE_SEED, m, d_h0, d_h1)
                ev[s][1].record()
            ctx.sync()
        barrier()
        ms = [a.elapsed_ms(b) for a, b in ev]
        prof = ctx.profile_read()
        ctx.profile(False)
        out = (d_h0.download(np.zeros(n, bt.HIT)), d_h1.download(np.zeros(n, bt.HIT)))
        return ms, prof, clk.result, out

    ms, prof, clk, hits_main = timed(mode)
    ms_other, prof_other, _, hits_other = timed(other)

    total_ms = sum(ms)
    if pg:
        from bvhtracer_gb300.shard import max_over_ranks
        total_ms = max_over_ranks(total_ms, pg)
    per_step_ms = total_ms / args.steps
    value = world * rays_per_step * args.steps / (total_ms / 1e3) / 1e6
    other_value = rays_per_step * len(ms_other) / (sum(ms_other) / 1e3) / 1e6

    # e2e: the C-ABI host-buffer call (rays in, both hit arrays out), wall clock per frame.
    # (1) page-locked host buffers, which the launch reads and writes in place over NVLink-C2C;
    # (2) ordinary (pageable) host memory, which the library stages through its own copies.
    from bvhtracer_gb300._lib import ptr
    nb = ctypes.c_uint32()

    def e2e(r_arr, h0_arr, h1_arr, steps):
        def once():
            ctx.check(ctx.lib.bvhgpu_blas_trace_bounce(ctx.h, blas.id, ptr(r_arr), n, BOUNCE_SEED, mode,
                                                       ptr(h0_arr), ptr(h1_arr), ctypes.byref(nb)))
        for _ in range(args.warmup):
            once()
        barrier()
        t0 = time.perf_counter()
        for _ in range(steps):
            once()
        return time.perf_counter() - t0

    pin_rays = ctx.pinned((n,), bt.RAY)
    pin_rays.array[:] = rays
    pin_h0 = ctx.pinned((n,), bt.HIT)
    pin_h1 = ctx.pinned((n,), bt.HIT)
    e2e_s = e2e(pin_rays.array, pin_h0.array, pin_h1.array, args.steps)
    e2e_value = world * rays_per_step * args.steps / e2e_s / 1e6
    e2e_identical = pin_h0.array.tobytes() == hits_main[0].tobytes() and \
        pin_h1.array.tobytes() == hits_main[1].tobytes()
    pg_rays = np.ascontiguousarray(rays)
    pg_h0, pg_h1 = np.zeros(n, bt.HIT), np.zeros(n, bt.HIT)
    e2e_pg_s = e2e(pg_rays, pg_h0, pg_h1, args.steps)
    e2e_pg_value = world * rays_per_step * args.steps / e2e_pg_s / 1e6
    e2e_identical = e2e_identical and pg_h0.tobytes() == hits_main[0].tobytes()

    kernel_launches = sum(v[1] for v in prof.values())
    result = {
        "metric": METRIC, "value": value, "unit": "Mrays/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": per_step_ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": {"workload": WORKLOAD, "mode": args.mode, "primary_rays": n, "bounce_rays": n_bounce,
                   "rays_per_step": rays_per_step, "triangles": int(len(tris)), "bvh_nodes": bvh.nodes_used,
                   "bvh_depth": blas.depth, "l2": "flushed between steps (256 MB memset)",
                   "parallelism": f"ray ranges of a {world}-frame job, one frame per GPU" if world > 1
                   else "1 GPU", "seed": SEED, "tuned": tuned, "tune_s": tune_s},
        "plain_vs_persistent": {
            mode_name[mode]: value / world, mode_name[other]: other_value,
            "ratio_persistent_over_plain": (value / world / other_value) if mode == bt.MODE_PERSISTENT
            else (other_value / (value / world)),
        },
        "e2e": {"value": e2e_value, "unit": "Mrays/s", "h2d_bytes_per_step": n * bt.RAY.itemsize,
                "d2h_bytes_per_step": 2 * n * bt.HIT.itemsize,
                "transfer": "page-locked host buffers, read and written in place by the launch (NVLink-C2C); "
                            "wall clock around bvhgpu_blas_trace_bounce"},
        "e2e_pageable": {"value": e2e_pg_value, "unit": "Mrays/s",
                         "transfer": "ordinary host memory (e.g. a Rust Vec), reused across calls: read and "
                                     "written in place by the launch on a GPU that accesses pageable memory "
                                     "coherently (Grace-attached GB300: yes), the hit pages touched by the CPU "
                                     "first, else staged through the library's page-locked copies; wall clock "
                                     "around bvhgpu_blas_trace_bounce"},
        "e2e_hits_identical_to_timed": bool(e2e_identical),
        "gpu_launches": kernel_launches,
        "clocks": clk,
        "kernel_ms": {k: {"ms_total": v[0], "launches": v[1]} for k, v in prof.items()},
    }

    if args.no_cpu_baseline or rank != 0:
        result["cpu_baseline"] = None
        result["roofline"] = None
        result["parity"] = None
        return result, ctx

    # ---- CPU leg: the oracle on the whole frame (all host threads): the CPU baseline, and the
    # parity check of both timed pipelines' outputs, every ray
    from oracle import checks
    from oracle import oracle as orc
    threads = host_threads()
    o_tris, o_nodes, o_used = orc.bvh_build(tris_in)
    identical_bvh = bool(o_used == bvh.nodes_used and o_nodes[:o_used].tobytes() == bvh.nodes[:o_used].tobytes()
                         and o_tris.tobytes() == np.ascontiguousarray(tris).tobytes())
    t0 = time.perf_counter()
    r0, rb, rvalid, r1 = checks.frame_with_bounce(o_nodes, o_used, o_tris, rays, BOUNCE_SEED, threads=threads)
    cpu_s = time.perf_counter() - t0
    cpu_traced = n + int(rvalid.sum())
    t0 = time.perf_counter()
    near0, near1 = checks.frame_near_ties(o_nodes, o_tris, rays, rb, rvalid, threads=threads)
    near_s = time.perf_counter() - t0
    par = {}
    for name, (g0, g1) in ((mode_name[mode], hits_main), (mode_name[other], hits_other)):
        par[f"{name}_primary"] = checks.compare_hits(g0, r0, near0)
        par[f"{name}_bounce"] = checks.compare_hits(g1, r1, near1)
    result["parity"] = {"scope": f"whole frame: {n} primaries + {int(rvalid.sum())} bounce rays, both pipelines",
                        "identical_bvh": identical_bvh, "checks": par,
                        "summary": checks.merge(list(par.values())), "oracle_s": cpu_s, "near_tie_pass_s": near_s}

    # single-thread figure (the reference is one scalar thread) on a bounded sample: every F-th 8x8
    # tile of the frame (spread over the image like the frame), F sized for a few seconds
    per_ray_1t = cpu_s * threads / cpu_traced
    f = max(1, int(np.ceil(n / max(64.0, 5.0 / max(per_ray_1t, 1e-9)))))
    one_rays = np.ascontiguousarray(rays.reshape(-1, 64)[::f].reshape(-1))
    k = len(one_rays)
    t0 = time.perf_counter()
    s0 = orc.bvh_intersect(o_nodes, o_used, o_tris, one_rays)
    sb, sv = orc.bounce_rays(one_rays, s0, o_tris, BOUNCE_SEED)
    orc.bvh_intersect(o_nodes, o_used, o_tris, sb[sv])
    one_s = time.perf_counter() - t0
    result["cpu_baseline"] = {
        "value": cpu_traced / cpu_s / 1e6, "unit": "Mrays/s", "cores": threads, "kind": "port",
        "sample": f"the whole frame: {n} primaries + their {int(rvalid.sum())} bounce rays, {threads} threads "
                  "over ray chunks (the same rays the GPU traces, also the parity check)",
        "seconds": cpu_s,
        "single_thread": {"value": (k + int(sv.sum())) / one_s / 1e6, "unit": "Mrays/s", "cores": 1,
                          "sample": f"every {f}th 8x8 tile of the frame ({k} primaries) + their {int(sv.sum())} "
                                    "bounce rays, one thread (the reference's scalar loop)", "seconds": one_s},
    }

    # ---- roofline of the dominant kernel
    peak, peak_kind = measured_peaks()
    dom_name, (dom_ms, dom_launches) = max(prof.items(), key=lambda kv: kv[1][0])
    per_launch_s = dom_ms / dom_launches / 1e3
    policy_kernel = bt.K_PERSISTENT_BOUNCE if mode == bt.MODE_PERSISTENT else bt.K_TRACE_BLAS
    with leaf_policy(ctx, policy_kernel) as pol:
        fetched = fetched_bytes(ctx, blas, rays, BOUNCE_SEED)
    if mode == bt.MODE_PERSISTENT:
        own_bytes = fetched["primary"]["bytes"] + fetched["bounce"]["bytes"]
    else:
        own_bytes = fetched["primary" if dom_name == "trace_blas" else "bounce"]["bytes"]
    # the reference algorithm's bytes per ray (brute-force leaves), from the oracle's counters on
    # every 64th ray and its bounce (single thread)
    sub = rays[::64]
    hs, cs = orc.bvh_intersect(o_nodes, o_used, o_tris, sub, counters=True)
    bs, vs = orc.bounce_rays(sub, hs, o_tris, BOUNCE_SEED)
    _, cb = orc.bvh_intersect(o_nodes, o_used, o_tris, bs[vs], counters=True)
    ref_bytes = n * float(orc.bytes_per_ray(cs).mean()) + n_bounce * float(orc.bytes_per_ray(cb).mean())
    achieved = own_bytes / per_launch_s / 1e9
    traffic, traffic_kind, traffic_src = NCU_TRAFFIC.get(dom_name, (None, None, None))
    result["roofline"] = {
        "bound": "hbm", "kernel": dom_name, "achieved": achieved, "peak": peak, "peak_kind": peak_kind,
        "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
        "traffic_kind": traffic_kind, "traffic_source": traffic_src,
        "basis": "bytes the kernel requested: node + triangle fetches of its traversal counted on the device "
                 "(bvhgpu_blas_trace_counts under the timed kernel's leaf policy, big_leaf "
                 f"{pol['big_leaf']}, hidden {pol['hidden']}) + 32 B ray + 20 B hit per ray, per launch / the "
                 "launch's CUDA-event time; these requests are served mostly by L1 / L2, so frac is a "
                 "data-movement rate against HBM bandwidth, not an HBM bound",
        "algorithmic_bytes_per_launch": own_bytes, "launch_ms": per_launch_s * 1e3, "fetched": fetched,
        "dram": None if traffic is None else {
            "bytes_per_launch": traffic, "gbs": traffic / per_launch_s / 1e9,
            "frac": traffic / per_launch_s / 1e9 / peak,
            "note": "DRAM bytes of the ncu capture / this run's launch time: the HBM fraction proper"},
        "reference_algorithm_bytes_per_launch": ref_bytes,
        "reference_algorithm_frac": ref_bytes / per_launch_s / 1e9 / peak,
        "reference_algorithm_note": "bytes the reference's brute-force leaf loop would fetch (oracle counters, "
                                    "every 64th ray): work the exact hidden-tree cull skips",
    }
    return result, ctx


# ---- uneven 64-scene batch ----------------------------------------------------------------------------------

WORKLOAD3 = ("uneven batch: 64 scenes, triangles log-uniform in [1k, 2M] (soup / displaced icosphere), "
             "rays log-uniform in [64k, 4M] (half pinhole primaries, half random)")


def setup_batch(nscenes: int = 64, seed: int = SEED):
    """The scenes of the uneven batch, generated and built (reference SAH, host) on host threads.
    Returns [(tris, bvh, rays)] and the triangles before the build's reordering."""
    import bvhtracer_gb300 as bt
    from concurrent.futures import ThreadPoolExecutor
    from bvhtracer_gb300 import scenes
    ntris, nrays = scenes.batch_specs(seed, nscenes)

    def make(i):
        tris, rays = scenes.batch_scene(i, int(ntris[i]), int(nrays[i]), seed)
        original = tris.copy()
        bvh = bt.BvhBuilder().build_for(tris)
        return tris, bvh, rays, original

    with ThreadPoolExecutor(max_workers=min(16, host_threads())) as ex:
        out = list(ex.map(make, range(nscenes)))
    return [(t, b, r) for t, b, r, _ in out], [o for *_, o in out]


def batch_sample_index(built, per_scene: int):
    """Ray indices (into the concatenated batch) of each scene's first `per_scene` primaries and first
    `per_scene` random rays (the second half of its rays)."""
    idx, off = [], 0
    for _, _, rays in built:
        half = len(rays) // 2
        k0 = min(per_scene, half)
        k1 = min(per_scene, len(rays) - half)
        idx.append(np.arange(off, off + k0))
        idx.append(np.arange(off + half, off + half + k1))
        off += len(rays)
    return np.concatenate(idx)


def bench_batch(args, local_rank: int, steps: int):
    import bvhtracer_gb300 as bt
    from bvhtracer_gb300._lib import ptr
    t0 = time.perf_counter()
    built, originals = setup_batch(args.scenes)
    setup_s = time.perf_counter() - t0
    ctx = bt.Context(local_rank)
    given = apply_tune_args(ctx, args)
    # the same SAH builds on the GPU (BvhBuilder::build_for on the device), checked bit for bit
    # against the host builds above
    t0 = time.perf_counter()
    gpu_builds = [(o.copy(), None) for o in originals]
    gpu_builds = [(m, ctx.build_bvh(m)) for m, _ in gpu_builds]
    gpu_build_s = time.perf_counter() - t0
    gpu_build_identical = all(m.tobytes() == t.tobytes() and g.nodes_used == b.nodes_used and
                              g.nodes.tobytes() == b.nodes.tobytes()
                              for (m, g), (t, b, _) in zip(gpu_builds, built))
    del gpu_builds
    blases = [ctx.upload_blas(bvh, tris) for tris, bvh, _ in built]
    rays = np.concatenate([r for _, _, r in built])
    items = np.zeros(len(built), bt.BATCH_ITEM)
    off = 0
    for i, (b, (_, _, r)) in enumerate(zip(blases, built)):
        items[i] = (b.id, off, len(r), 0)
        off += len(r)
    n = len(rays)
    d_rays = ctx.to_device(rays)
    d_hits = ctx.device_buffer(n * bt.HIT.itemsize)
    d_hits2 = ctx.device_buffer(n * bt.HIT.itemsize)
    ev = [(ctx.event(), ctx.event()) for _ in range(steps)]

    # autotune on a sample of every scene (its first primaries and first random rays)
    tuned, tune_s = dict(given), 0.0
    if not args.no_tune:
        t0 = time.perf_counter()
        s_items = np.zeros(len(built), bt.BATCH_ITEM)
        s_rays, off = [], 0
        for i, (b, (_, _, r)) in enumerate(zip(blases, built)):
            k, half = max(32, len(r) // 32), len(r) // 2
            sr = np.concatenate([r[:k], r[half:half + k]])
            s_items[i] = (b.id, off, len(sr), 0)
            s_rays.append(sr)
            off += len(sr)
        s_rays = np.concatenate(s_rays)
        d_srays = ctx.to_device(s_rays)
        for kernel, name in ((bt.K_TRACE_BATCH, "trace_batch"), (bt.K_TRACE_BLAS, "trace_blas")):
            cfg, ms_ = ctx.autotune(kernel, d_srays, len(s_rays), d_hits, items=s_items, reps=2)
            tuned[name] = dict(cfg, ms_on_sample=ms_)
        tuned["sample_rays"] = int(len(s_rays))
        del d_srays
        tune_s = time.perf_counter() - t0

    def timed(mode, out, k=None, clocked=False):
        k = k or steps
        for _ in range(min(3, args.warmup)):
            ctx.flush_l2()
            ctx.trace_batch_async(items, d_rays, n, mode, out)
        ctx.sync()
        ctx.profile(True)
        ctx.profile_read()
        region = ClockedRegion(local_rank) if clocked else None
        if region:
            region.__enter__()
        for s in range(k):
            ctx.flush_l2()
            ev[s][0].record()
            ctx.trace_batch_async(items, d_rays, n, mode, out)
            ev[s][1].record()
        ctx.sync()
        if region:
            region.__exit__()
        ms = [a.elapsed_ms(b) for a, b in ev[:k]]
        prof = ctx.profile_read()
        ctx.profile(False)
        return ms, prof, (region.result if region else None)

    ms_p, prof_p, clk = timed(bt.MODE_PERSISTENT, d_hits, clocked=True)
    ms_plain, prof_plain, _ = timed(bt.MODE_PLAIN, d_hits2)
    h_pers = d_hits.download(np.zeros(n, bt.HIT))
    h_plain = d_hits2.download(np.zeros(n, bt.HIT))
    value = n * steps / (sum(ms_p) / 1e3) / 1e6
    plain = n * steps / (sum(ms_plain) / 1e3) / 1e6
    # the textbook plain traversal: one launch per scene, one thread per ray, every leaf tested by
    # its own lane (no warp-cooperative leaves, no hidden trees), launch shape as tuned
    tb_cfg = ctx.tune_get(bt.K_TRACE_BLAS)
    ctx.tune_set(bt.K_TRACE_BLAS, **dict(tb_cfg, big_leaf=bt.BIG_LEAF_NEVER, hidden=0))
    tb_steps = max(1, min(2, steps))
    ms_tb, _, _ = timed(bt.MODE_PLAIN, d_hits2, k=tb_steps)
    ctx.tune_set(bt.K_TRACE_BLAS, **tb_cfg)
    h_tb = d_hits2.download(np.zeros(n, bt.HIT))
    textbook = n * tb_steps / (sum(ms_tb) / 1e3) / 1e6
    # e2e: bvhgpu_trace_batch with pinned host buffers
    pin_r = ctx.pinned((n,), bt.RAY)
    pin_r.array[:] = rays
    pin_h = ctx.pinned((n,), bt.HIT)
    its = np.ascontiguousarray(items)

    def e2e_once():
        ctx.check(ctx.lib.bvhgpu_trace_batch(ctx.h, ptr(its), len(its), ptr(pin_r.array), n, bt.MODE_PERSISTENT,
                                             ptr(pin_h.array)))
    e2e_once()
    e2e_steps = max(1, steps // 2)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        e2e_once()
    e2e_value = n * e2e_steps / (time.perf_counter() - t0) / 1e6
    same_cfg = {"persistent": {k: tuned.get("trace_batch", ctx.tune_get(bt.K_TRACE_BATCH)).get(k)
                               for k in ("big_leaf", "hidden")},
                "plain": {k: tuned.get("trace_blas", tb_cfg).get(k) for k in ("big_leaf", "hidden")}}
    result = {
        "metric": METRIC, "value": value, "unit": "Mrays/s", "steps": steps,
        "ms_per_step": sum(ms_p) / len(ms_p), "higher_is_better": True,
        "config": {"workload": WORKLOAD3, "scenes": len(built), "rays": n,
                   "triangles": int(sum(len(t) for t, _, _ in built)), "setup_s": setup_s,
                   "sah_build": {"host_s_incl_generation": setup_s, "gpu_s": gpu_build_s,
                                 "gpu_identical_to_host": gpu_build_identical},
                   "l2": "flushed between steps (256 MB memset)", "seed": SEED, "tuned": tuned, "tune_s": tune_s},
        "plain_vs_persistent": {
            "persistent": value, "plain": plain, "ratio_persistent_over_plain": value / plain,
            "leaf_policy": same_cfg,
            "note": "both arms have the same per-kernel features (warp-cooperative leaves, hidden trees), each "
                    "with its tuned knobs; only the launch model differs (one persistent launch vs one launch "
                    "per scene)",
            "plain_textbook_per_lane_leaves": textbook,
            "ratio_persistent_over_plain_textbook": value / textbook,
        },
        "e2e": {"value": e2e_value, "unit": "Mrays/s", "h2d_bytes_per_step": n * bt.RAY.itemsize,
                "d2h_bytes_per_step": n * bt.HIT.itemsize,
                "transfer": "page-locked host buffers; wall clock around bvhgpu_trace_batch"},
        "gpu_launches": sum(v[1] for v in prof_p.values()) // max(1, steps),
        "clocks": clk,
        "kernel_ms": {k: {"ms_total": v[0], "launches": v[1]} for k, v in prof_p.items()},
        "kernel_ms_plain": {k: {"ms_total": v[0], "launches": v[1]} for k, v in prof_plain.items()},
    }
    if args.no_cpu_baseline:
        result["cpu_baseline"] = result["roofline"] = result["parity"] = None
        return result, ctx, blases, built
    # oracle on each scene's first 4,096 primaries and first 4,096 random rays, scenes spread over
    # the host threads: the CPU baseline and the parity check of all three GPU arms on those rays
    from concurrent.futures import ThreadPoolExecutor
    from oracle import checks
    from oracle import oracle as orc
    threads = host_threads()
    per_scene = 4096
    idx = batch_sample_index(built, per_scene)

    def sample_of(r):
        half = len(r) // 2
        return np.concatenate([r[:min(per_scene, half)], r[half:half + min(per_scene, len(r) - half)]])

    def run(item):
        tris, bvh, r = item
        return orc.bvh_intersect(bvh.nodes, bvh.nodes_used, tris, sample_of(r))

    t0 = time.perf_counter()
    with ThreadPoolExecutor(max_workers=threads) as ex:
        refs = list(ex.map(run, built))
    cpu_s = time.perf_counter() - t0
    ref = np.concatenate(refs)

    def near(item):
        tris, bvh, r = item
        return orc.near_ties(bvh.nodes, tris, sample_of(r), threads=1)

    with ThreadPoolExecutor(max_workers=threads) as ex:
        near_mask = np.concatenate(list(ex.map(near, built)))
    checks_ = {"persistent": checks.compare_hits(h_pers[idx], ref, near_mask),
               "plain": checks.compare_hits(h_plain[idx], ref, near_mask),
               "plain_textbook": checks.compare_hits(h_tb[idx], ref, near_mask)}
    result["parity"] = {"scope": f"first {per_scene} primaries + first {per_scene} random rays of each of the "
                                 f"{len(built)} scenes ({len(idx)} rays), all three GPU arms",
                        "checks": checks_, "summary": checks.merge(list(checks_.values())),
                        "gpu_build_identical_to_host": gpu_build_identical,
                        "persistent_equals_plain_all_rays": bool(h_pers.tobytes() == h_plain.tobytes())}
    # single thread: the first 512 + 512 rays of each scene
    t0 = time.perf_counter()
    one = 0
    for tris, bvh, r in built:
        half = len(r) // 2
        s = np.concatenate([r[:512], r[half:half + 512]])
        orc.bvh_intersect(bvh.nodes, bvh.nodes_used, tris, s)
        one += len(s)
    one_s = time.perf_counter() - t0
    result["cpu_baseline"] = {
        "value": len(idx) / cpu_s / 1e6, "unit": "Mrays/s", "cores": threads, "kind": "port",
        "sample": f"{per_scene} primaries + {per_scene} random rays of each of the {len(built)} scenes, scenes "
                  f"spread over {threads} threads (also the parity check)", "seconds": cpu_s,
        "single_thread": {"value": one / one_s / 1e6, "unit": "Mrays/s", "cores": 1,
                          "sample": f"512 primaries + 512 random rays of each scene, one thread", "seconds": one_s}}
    # roofline: node + triangle bytes the persistent kernel's traversal requested, counted on the
    # device per scene under its leaf policy
    peak, peak_kind = measured_peaks()
    dom_ms, dom_n = prof_p["trace_batch"]
    per_launch_s = dom_ms / dom_n / 1e3
    own = 0
    with leaf_policy(ctx, bt.K_TRACE_BATCH) as pol:
        for b, (_, _, r) in zip(blases, built):
            d_r = ctx.to_device(r)
            d_h = ctx.device_buffer(len(r) * bt.HIT.itemsize)
            own += count_bytes(b.trace_counts(d_r, len(r), d_h), len(r))
            del d_r, d_h
    traffic = NCU_TRAFFIC["trace_batch"][0] * n
    achieved = own / per_launch_s / 1e9
    result["roofline"] = {
        "bound": "hbm", "kernel": "trace_batch", "achieved": achieved, "peak": peak, "peak_kind": peak_kind,
        "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
        "traffic_kind": NCU_TRAFFIC["trace_batch"][1], "traffic_source": NCU_TRAFFIC["trace_batch"][2],
        "basis": f"bytes the persistent kernel requested (device counters per scene, leaf policy big_leaf "
                 f"{pol['big_leaf']}, hidden {pol['hidden']}) per launch / launch time",
        "algorithmic_bytes_per_launch": own, "launch_ms": per_launch_s * 1e3,
        "dram": {"bytes_per_launch": traffic, "gbs": traffic / per_launch_s / 1e9,
                 "frac": traffic / per_launch_s / 1e9 / peak}}
    return result, ctx, blases, built


# ---- instanced animated frames ------------------------------------------------------------------------------

WORKLOAD2 = ("instanced animated scene: 3 displaced icospheres (5,120 / 20,480 / 81,920 tris), 256 instances, "
             "60 frames of 1280x720 primaries + 1 diffuse bounce; per frame wobble + refit x3, TLAS rebuild, trace, "
             "one CUDA graph")


def bench_instanced(args, local_rank: int, reps: int):
    import bvhtracer_gb300 as bt
    from bvhtracer_gb300 import scenes
    from bvhtracer_gb300.frames import AnimatedScene
    cfg = scenes.instanced_animation(seed=SEED)
    nframes = 60
    ctx = bt.Context(local_rank)
    given = apply_tune_args(ctx, args)
    sc = AnimatedScene(ctx, cfg)
    initial = [(m.bvh.nodes.copy(), m.bvh.nodes_used) for m in sc.meshes]
    n = sc.n
    for _ in range(3):
        sc.frame_async()
    ctx.sync()
    tuned, tune_s = dict(given), 0.0
    if not args.no_tune:  # tune the frame's trace kernel before the graph captures its launch
        t0 = time.perf_counter()
        cfg_t, ms_ = ctx.autotune(bt.K_SCENE_BOUNCE, sc.d_rays, n, sc.d_hits0, sc.d_hits1, target=sc.scene.id,
                                  seed=sc.seed, reps=3)
        tuned["scene_bounce"] = dict(cfg_t, ms=ms_)
        tune_s = time.perf_counter() - t0
    ctx.profile(True)
    ctx.profile_read()
    sc.frame_async()
    ctx.sync()
    prof = ctx.profile_read()
    ctx.profile(False)
    sc.capture()
    # rays per frame: primaries + the bounces of that frame's primary hits (counted in a first pass)
    sc.set_time(0.0)
    bounces = []
    for _ in range(nframes):
        sc.launch()
        ctx.sync()
        h0 = sc.d_hits0.download(np.zeros(n, bt.HIT))
        bounces.append(int((h0["prim"] != bt.MISS).sum()))
    total_rays = nframes * n + sum(bounces)
    evs = [(ctx.event(), ctx.event()) for _ in range(nframes)]
    best = None
    with ClockedRegion(local_rank) as clk:
        for _ in range(reps):
            sc.set_time(0.0)
            for f in range(nframes):
                ctx.flush_l2()
                evs[f][0].record()
                sc.launch()
                evs[f][1].record()
            ctx.sync()
            ms = [a.elapsed_ms(b) for a, b in evs]
            if best is None or sum(ms) < sum(best):
                best = ms
    total_ms = sum(best)
    value = total_rays / (total_ms / 1e3) / 1e6
    # e2e: per frame, the rays copied from page-locked host memory, the frame's graph, both hit
    # arrays copied back; wall clock over the 60 frames
    pin_r = ctx.pinned((n,), bt.RAY)
    pin_r.array[:] = cfg["rays"]
    pin_h0 = ctx.pinned((n,), bt.HIT)
    pin_h1 = ctx.pinned((n,), bt.HIT)
    from bvhtracer_gb300._lib import ptr
    sc.set_time(0.0)
    ctx.sync()
    t0 = time.perf_counter()
    for f in range(nframes):
        ctx.check(ctx.lib.bvhgpu_copy_to_device(ctx.h, sc.d_rays.ptr, ptr(pin_r.array), pin_r.array.nbytes, None))
        sc.launch()
        ctx.check(ctx.lib.bvhgpu_copy_to_host(ctx.h, ptr(pin_h0.array), sc.d_hits0.ptr, pin_h0.array.nbytes, None))
        ctx.check(ctx.lib.bvhgpu_copy_to_host(ctx.h, ptr(pin_h1.array), sc.d_hits1.ptr, pin_h1.array.nbytes, None))
        ctx.sync()
    e2e_s = time.perf_counter() - t0
    h0, h1 = sc.hits()
    result = {
        "metric": METRIC, "value": value, "unit": "Mrays/s", "steps": nframes, "ms_per_step": total_ms / nframes,
        "higher_is_better": True,
        "config": {"workload": WORKLOAD2, "frames": nframes, "primary_rays_per_frame": n,
                   "bounce_rays_total": sum(bounces), "instances": len(sc.blas_of),
                   "l2": "flushed between frames (256 MB memset)", "step": "one frame = one CUDA graph launch",
                   "repetitions": reps, "seed": SEED, "tuned": tuned, "tune_s": tune_s},
        "frame_ms": {"mean": total_ms / nframes, "max": max(best), "min": min(best)},
        "e2e": {"value": total_rays / e2e_s / 1e6, "unit": "Mrays/s", "h2d_bytes_per_step": n * bt.RAY.itemsize,
                "d2h_bytes_per_step": 2 * n * bt.HIT.itemsize,
                "transfer": "per frame: rays from page-locked host memory, graph launch, both hit arrays back"},
        "gpu_launches": 1, "clocks": clk.result,
        "kernel_ms_one_frame": {k: {"ms_total": v[0], "launches": v[1]} for k, v in prof.items()},
    }
    if args.no_cpu_baseline:
        result["cpu_baseline"] = result["roofline"] = result["parity"] = None
        return result, ctx
    # parity: the last frame's state (refit nodes, TLAS, primaries, bounce rays, bounce hits) against
    # the oracle run on that state; the oracle's trace of the frame is the CPU baseline
    from oracle import checks
    from oracle import oracle as orc
    threads = host_threads()
    blas_states, refit_ok = [], True
    for m, (nodes0, used) in zip(sc.meshes, initial):
        verts = m.vertices()
        tris = np.ascontiguousarray(verts[m.faces].reshape(-1, 9), np.float32)
        gpu_nodes = m.blas.download_nodes()
        ref_nodes = orc.bvh_refit(nodes0, used, tris)[:used]
        refit_ok &= gpu_nodes.tobytes() == ref_nodes.tobytes()
        blas_states.append((ref_nodes, used, tris))
    xf, inv = sc.scene.download_transforms()
    tlas, tused = sc.scene.download_tlas()
    ref_tlas, ref_used, sa = checks.scene_state_reference(blas_states, sc.blas_of, xf, inv)
    tlas_ok = tused == ref_used and tlas.tobytes() == ref_tlas.tobytes()
    t0 = time.perf_counter()
    r0, rb, rvalid, r1 = checks.scene_frame_with_bounce(ref_tlas, ref_used, sa, cfg["rays"], sc.seed,
                                                        threads=threads)
    cpu_s = time.perf_counter() - t0
    gb, gvalid = sc.scene.bounce_rays(cfg["rays"], sc.seed)
    bounce_rays_ok = bool(np.array_equal(gvalid, rvalid) and gb[rvalid].tobytes() == rb[rvalid].tobytes())
    par = {"primary": checks.compare_hits(h0, r0), "bounce": checks.compare_hits(h1, r1)}
    result["parity"] = {"scope": f"frame {nframes}: refit nodes of 3 BLASes, TLAS, {n} primaries, bounce rays, "
                                 f"{int(rvalid.sum())} bounce hits",
                        "refit_identical": bool(refit_ok), "tlas_identical": bool(tlas_ok),
                        "bounce_rays_identical": bounce_rays_ok, "checks": par,
                        "summary": checks.merge(list(par.values())),
                        "near_ties": "not computed for the two-level scene (the oracle's two-nearest pass is "
                                     "single-BLAS); every ray must match"}
    if not (refit_ok and tlas_ok and bounce_rays_ok):
        par["state"] = {"mismatch_outside_near_ties": 1}
    traced = n + int(rvalid.sum())
    result["cpu_baseline"] = {"value": traced / cpu_s / 1e6, "unit": "Mrays/s", "cores": threads, "kind": "port",
                              "sample": f"frame {nframes}: {n} primaries + {int(rvalid.sum())} bounce rays through "
                                        f"the TLAS, {threads} threads (also the parity check)", "seconds": cpu_s}
    # roofline on the reference algorithm's bytes (the tuned frame kernel walks no hidden trees here:
    # hidden = 0, so its leaves are tested in order like the reference's): oracle counters on every
    # 16th primary and its bounce
    peak, peak_kind = measured_peaks()
    sub = cfg["rays"][::16]
    hs, cs = orc.scene_intersect(ref_tlas, ref_used, sa, sub, counters=True)
    bs, vs = orc.scene_bounce_rays(sa, sub, hs, sc.seed)
    _, cb = orc.scene_intersect(ref_tlas, ref_used, sa, bs[vs], counters=True)
    bytes_frame = n * float(orc.bytes_per_ray(cs).mean()) + int(rvalid.sum()) * float(orc.bytes_per_ray(cb).mean())
    k_ms, k_n = prof.get("scene_bounce", (None, 0))
    if k_ms:
        per_launch_s = k_ms / k_n / 1e3
        result["roofline"] = {
            "bound": "hbm", "kernel": "scene_bounce", "achieved": bytes_frame / per_launch_s / 1e9, "peak": peak,
            "peak_kind": peak_kind, "unit": "GB/s", "frac": bytes_frame / per_launch_s / 1e9 / peak,
            "traffic": NCU_TRAFFIC["scene_bounce"][0], "traffic_kind": NCU_TRAFFIC["scene_bounce"][1],
            "traffic_source": NCU_TRAFFIC["scene_bounce"][2],
            "launch_ms": per_launch_s * 1e3, "algorithmic_bytes_per_launch": bytes_frame,
            "basis": "the reference algorithm's bytes per ray (oracle counters: 32 B x (1 + 2 x interior nodes) "
                     "+ 36 B x triangles + TLAS nodes + 48 B per BLAS entry + 44 B ray/hit), every 16th ray of "
                     "the last frame, over the frame kernel's launch time (one profiled frame)",
            "dram": {"bytes_per_launch": NCU_TRAFFIC["scene_bounce"][0],
                     "gbs": NCU_TRAFFIC["scene_bounce"][0] / per_launch_s / 1e9,
                     "frac": NCU_TRAFFIC["scene_bounce"][0] / per_launch_s / 1e9 / peak,
                     "note": "DRAM bytes of the ncu capture / this run's launch time: the HBM fraction proper"}}
    else:
        result["roofline"] = None
    return result, ctx


# ---- differentiable Lambertian render ---------------------------------------------------------------------

WORKLOAD4 = ("differentiable Lambertian render: displaced icosphere, 7 subdivisions (327,680 tris, "
             "163,842 vertices), 512x512, light (2,2,-3), target from N(0, 0.01^2) radial noise, all lengths x10 "
             "(the reference's |det| < 1e-4 test rejects every triangle of the unit sphere); "
             "step = update+refit, forward, adjoint, SGD (lr 1e-2)")


def bench_lambert(args, local_rank: int, steps: int):
    import bvhtracer_gb300 as bt
    from bvhtracer_gb300 import scenes
    from bvhtracer_gb300._lib import ptr
    verts, faces, vn, tverts, rays, light = scenes.lambert_scene(seed=SEED)
    n = len(rays)
    ctx = bt.Context(local_rank)
    given = apply_tune_args(ctx, args)
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
    lr = 1e-2

    def step(evs=None):
        if evs:
            evs[0].record()
        m.update_async()
        if evs:
            evs[1].record()
        m.forward_async(d_rays, n, light, d_img, d_hits)
        if evs:
            evs[2].record()
        m.adjoint_async(d_rays, n, light, d_hits, d_img, d_tgt, d_grad)
        if evs:
            evs[3].record()
        m.sgd_step_async(d_grad, lr)
        if evs:
            evs[4].record()

    for _ in range(args.warmup):
        ctx.flush_l2()
        step()
    ctx.sync()
    evs = [[ctx.event() for _ in range(5)] for _ in range(steps)]
    ctx.profile(True)
    ctx.profile_read()
    with ClockedRegion(local_rank) as clk:
        for s in range(steps):
            ctx.flush_l2()
            step(evs[s])
        ctx.sync()
    prof = ctx.profile_read()
    ctx.profile(False)
    upd = [e[0].elapsed_ms(e[1]) for e in evs]
    fwd = [e[1].elapsed_ms(e[2]) for e in evs]
    adj = [e[2].elapsed_ms(e[3]) for e in evs]
    tot = [e[0].elapsed_ms(e[4]) for e in evs]
    # e2e: a training step through the public calls with the rays copied from page-locked host
    # memory each step and the loss read back (wall clock)
    pin_r = ctx.pinned((n,), bt.RAY)
    pin_r.array[:] = rays
    ctx.sync()
    t0 = time.perf_counter()
    for _ in range(steps):
        ctx.check(ctx.lib.bvhgpu_copy_to_device(ctx.h, d_rays.ptr, ptr(pin_r.array), pin_r.array.nbytes, None))
        m.update_async()
        m.forward_async(d_rays, n, light, d_img, d_hits)
        bt.mse_loss(ctx, d_img, d_tgt, n)
        m.adjoint_async(d_rays, n, light, d_hits, d_img, d_tgt, d_grad)
        m.sgd_step_async(d_grad, lr)
    ctx.sync()
    e2e_ms = (time.perf_counter() - t0) / steps * 1e3
    # the descent from the start (outside the timed region): loss every 10 steps.  With --checkpoint the
    # state (vertices, step, losses) is saved every 10 steps and a run finding the file resumes there.
    m.set_vertices(verts)
    d_grad.zero()
    losses, start = [], 0
    ckpt = getattr(args, "checkpoint", None)
    if ckpt and os.path.exists(ckpt):
        state = m.resume(ckpt)
        start, losses = state["step"], state["losses"]
    for it in range(start, 101):
        m.update_async()
        m.forward_async(d_rays, n, light, d_img, d_hits)
        if it % 10 == 0:
            if len(losses) <= it // 10:
                losses.append(bt.mse_loss(ctx, d_img, d_tgt, n))
            if ckpt and it > start:
                m.checkpoint(ckpt, it, losses, lr)
        if it == 100:
            break
        m.adjoint_async(d_rays, n, light, d_hits, d_img, d_tgt, d_grad)
        m.sgd_step_async(d_grad, lr)
    ctx.sync()
    adj_ms = sum(adj) / len(adj)
    fwd_ms = sum(fwd) / len(fwd)
    result = {
        "metric": METRIC, "value": adj_ms, "unit": "ms/step (adjoint kernel)", "steps": steps,
        "ms_per_step": sum(tot) / len(tot), "higher_is_better": False,
        "config": {"workload": WORKLOAD4, "pixels": n, "triangles": int(len(faces)), "vertices": int(len(verts)),
                   "bvh_nodes": m.bvh.nodes_used, "l2": "flushed between steps (256 MB memset)", "seed": SEED,
                   "tuned": given},
        "adjoint": {"forward_ms": fwd_ms, "adjoint_ms": adj_ms, "update_refit_ms": sum(upd) / len(upd),
                    "step_ms": sum(tot) / len(tot), "adjoint_over_forward": adj_ms / fwd_ms,
                    "forward_mrays_per_s": n / fwd_ms / 1e3, "loss_every_10_steps": losses,
                    "loss_note": "lr 1e-2 moves the vertices by ~1e-9 per step (gradients ~1e-7 for a mean over "
                                 "262,144 pixels), so the loss stays flat at the configured rate"},
        "e2e": {"value": e2e_ms, "unit": "ms/step (whole training step)", "h2d_bytes_per_step": n * bt.RAY.itemsize,
                "d2h_bytes_per_step": 8,
                "transfer": "rays copied from page-locked host memory each step, loss (f64) read back"},
        "gpu_launches": sum(v[1] for v in prof.values()) // max(1, steps), "clocks": clk.result,
        "kernel_ms": {k: {"ms_total": v[0], "launches": v[1]} for k, v in prof.items()},
    }
    if args.no_cpu_baseline:
        result["cpu_baseline"] = result["parity"] = None
        return result, ctx
    # parity: a forward pass at the initial vertices (every hit against the oracle's traversal of the
    # same refit node array, the image against the FP64 shading)
    from oracle import adjoint64, checks
    from oracle import oracle as orc
    threads = host_threads()
    m.set_vertices(verts)
    m.forward_async(d_rays, n, light, d_img, d_hits)
    ctx.sync()
    hits = d_hits.download(np.zeros(n, bt.HIT))
    img = d_img.download(np.zeros(n, np.float32))
    cur = m.vertices()
    tris = np.ascontiguousarray(cur[m.faces].reshape(-1, 9), np.float32)
    nodes = m.blas.download_nodes()
    t0 = time.perf_counter()
    ref = orc.bvh_intersect(nodes, m.bvh.nodes_used, tris, rays, threads=threads)
    cpu_s = time.perf_counter() - t0
    near = orc.near_ties(nodes, tris, rays, threads=threads)
    img64 = adjoint64.render64(rays, hits["prim"], cur, m.faces, vn, light)
    par = {"forward_hits": checks.compare_hits(hits, ref, near)}
    result["parity"] = {"scope": f"every pixel of a forward pass ({n} rays); image vs FP64 shading",
                        "checks": par, "summary": par["forward_hits"],
                        "image_max_abs_vs_fp64": float(np.max(np.abs(img.astype(np.float64) - img64)))}
    result["cpu_baseline"] = {"value": n / cpu_s / 1e6, "unit": "Mrays/s", "cores": threads, "kind": "port",
                              "sample": f"the forward pass's {n} rays through the oracle's traversal, {threads} "
                                        "threads (also the parity check)", "seconds": cpu_s}
    return result, ctx


# ---- the reference arm -----------------------------------------------------------------------------------

def run_reference(args):
    """--impl reference: the CPU restatement of the reference's traversal (the Rust reference cannot be
    built here: no cargo), timed on all host threads.  Each step traces the same fixed sample of the
    headline frame: every ref_fraction-th 8x8 tile of its primaries (every 8th by default) and their
    bounce rays.  Nothing
    of the CUDA library is loaded: the BVH comes from the oracle's SAH build and the rays from the
    workload generator loaded on its own."""
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    from oracle import oracle as orc
    scenes = load_scenes()
    tris, rays, _ = scenes.icosphere_frame(seed=SEED)
    tris, nodes, used = orc.bvh_build(tris)
    threads = host_threads()
    # every F-th 8x8 tile of the frame (rays are in tile order, 64 per tile): spread over the image
    # like the whole frame, and the same rays every step
    sample = np.ascontiguousarray(rays.reshape(-1, 64)[::args.ref_fraction].reshape(-1))
    n = len(sample)
    times, traced = [], []
    for step in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        h0 = orc.bvh_intersect(nodes, used, tris, sample, threads=threads)
        b, v = orc.bounce_rays(sample, h0, tris, BOUNCE_SEED)
        orc.bvh_intersect(nodes, used, tris, b[v], threads=threads)
        dt = time.perf_counter() - t0
        if step >= args.warmup:
            times.append(dt)
            traced.append(n + int(v.sum()))
    value = sum(traced) / sum(times) / 1e6
    desc = (f"every {args.ref_fraction}th 8x8 tile of the frame ({n} primaries) + their {traced[0] - n} bounce "
            f"rays, the same rays every step, {threads} threads; the Rust reference cannot be built here (no "
            "cargo): the C++ restatement of its traversal (oracle/) is timed")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "Mrays/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / len(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "sample_per_step": desc, "seed": SEED},
        "cpu_baseline": {"value": value, "unit": "Mrays/s", "cores": threads, "kind": "port", "sample": desc},
        "e2e": {"value": value, "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ---- entry -------------------------------------------------------------------------------------------------

def free_port() -> int:
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def spawn_ranks(n: int) -> int:
    """`--gpus N` run without torchrun: start N ranks of this script with torch.distributed.run
    (one process per GPU, rendezvous on 127.0.0.1) and return the job's exit status."""
    argv = [a for a in sys.argv[1:]]
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={n}",
           "--master-addr=127.0.0.1", f"--master-port={free_port()}", os.path.abspath(__file__), *argv]
    return subprocess.call(cmd)


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--mode", choices=["persistent", "plain"], default="persistent")
    ap.add_argument("--workload", choices=["default", "icosphere", "instanced", "batch", "lambert"],
                    default="default",
                    help="default: the icosphere line with the batch, instanced and adjoint workloads as "
                         "sub-objects; icosphere: 81,920-triangle displaced icosphere, 1920x1080 primaries + "
                         "bounce; instanced: 256 instances of 3 BLASes, 60 animated 1280x720 frames in a CUDA "
                         "graph; batch: uneven 64-scene batch; lambert: differentiable render of 327,680 "
                         "triangles at 512x512 (adjoint ms/step)")
    ap.add_argument("--scenes", type=int, default=64,
                    help="batch: number of scenes (64 = the workload; fewer only for small profiling runs)")
    ap.add_argument("--no-tune", action="store_true", help="skip the autotuner (use the default launch configs)")
    ap.add_argument("--tune", action="append", metavar="KERNEL=B,M,S,L,R,H",
                    help="set a kernel's launch config (block, min_blocks, stack, big_leaf, refill, hidden) and "
                         "skip the autotuner, e.g. to profile the configs an earlier tuned run picked; repeatable")
    ap.add_argument("--ref-fraction", type=int, default=8,
                    help="--impl reference: each step traces every F-th 8x8 tile of the frame + its bounces")
    ap.add_argument("--checkpoint", metavar="PATH",
                    help="lambert: save the 100-step descent's state to PATH every 10 steps; resume from it if it "
                         "exists")
    ap.add_argument("--no-cpu-baseline", action="store_true",
                    help="skip the CPU-baseline and parity leg (outside the timed region), e.g. under a profiler")
    args = ap.parse_args(argv)
    if args.warmup < 3:
        args.warmup = 3
    if args.tune:
        args.no_tune = True
    rank, world, local_rank = dist_env()
    if "WORLD_SIZE" not in os.environ and args.gpus > 1:
        return spawn_ranks(args.gpus)
    if world != args.gpus:
        print(f"bench.py: --gpus {args.gpus} but WORLD_SIZE={world}", file=sys.stderr)
        return 2
    if args.impl == "reference":
        return run_reference(args)

    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        pg = dist

    sub_steps = max(3, min(args.steps, 10))
    if args.workload in ("default", "icosphere"):
        line, ctx = bench_icosphere(args, pg)
        ctx.close()
        if args.workload == "default":
            # the other workloads of the metric, each in its own context (per-rank replicas under N > 1)
            b, ctx, *_ = bench_batch(args, local_rank, sub_steps)
            ctx.close()
            line["batch"] = b
            inst, ctx = bench_instanced(args, local_rank, reps=max(1, args.steps // 10))
            ctx.close()
            line["instanced"] = inst
            lam, ctx = bench_lambert(args, local_rank, args.steps)
            ctx.close()
            line["adjoint"] = lam
    else:
        fn = {"batch": lambda: bench_batch(args, local_rank, args.steps)[0:2],
              "instanced": lambda: bench_instanced(args, local_rank, reps=max(1, args.steps // 10)),
              "lambert": lambda: bench_lambert(args, local_rank, args.steps)}[args.workload]
        line, ctx = fn()
        ctx.close()
        line.update({"n_gpus": world, "warmup": args.warmup, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                     "data": "synthetic (seeded)"})
    if rank != 0:
        return 0
    fail = parity_fail(line)
    line["parity_ok"] = not fail
    print(json.dumps(line), flush=True)
    return 1 if fail else 0


if __name__ == "__main__":
    sys.exit(main())
