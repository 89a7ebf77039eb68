"""bench.py host logic on the CPU: the --tune launch-config option and the byte basis of the
roofline (node + triangle bytes fetched per ray, from the device counters)."""
import importlib.util
import os

import numpy as np
import pytest

import bvhtracer_gb300 as bt

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


class FakeCtx:
    """Records tune_set calls; hands out placeholder device buffers."""

    def __init__(self):
        self.calls = []

    def tune_set(self, kernel, **cfg):
        self.calls.append((kernel, cfg))

    def to_device(self, arr):
        return ("device", len(arr))

    def device_buffer(self, nbytes):
        return ("buffer", nbytes)


class Args:
    def __init__(self, tune):
        self.tune = tune


def test_tune_option_sets_each_kernel(bench):
    ctx = FakeCtx()
    given = bench.apply_tune_args(ctx, Args(["trace_batch=128,6,256,16,8,100", "trace_blas=64,1,32,8,1,0"]))
    assert ctx.calls == [
        (bt.K_TRACE_BATCH, dict(block=128, min_blocks=6, stack=256, big_leaf=16, refill=8, hidden=100)),
        (bt.K_TRACE_BLAS, dict(block=64, min_blocks=1, stack=32, big_leaf=8, refill=1, hidden=0)),
    ]
    assert given["trace_batch"]["source"] == "--tune" and given["trace_blas"]["hidden"] == 0
    assert bench.apply_tune_args(FakeCtx(), Args(None)) == {}


@pytest.mark.parametrize("spec", ["no_such_kernel=128,5,256,16,8,2000", "trace_blas=128,5", "trace_blas"])
def test_tune_option_rejects_bad_specs(bench, spec):
    with pytest.raises(SystemExit):
        bench.apply_tune_args(FakeCtx(), Args([spec]))


def test_fetched_bytes_basis(bench):
    """64 B per reference node, 32 B per hidden box, 40 B per hidden-tree entry, 32 B per cone
    switch, 88 B per hidden pair, 48 / 40 B per lane / warp triangle, 52 B of ray + hit per ray."""
    counts = {"ref_nodes": 10, "hidden_boxes": 20, "hidden_entries": 1, "hidden_pairs": 3, "lane_tris": 2,
              "warp_tris": 5, "cone_switches": 4}

    class FakeBlas:
        def bounce_rays(self, rays, seed):
            valid = np.zeros(len(rays), bool)
            valid[:1] = True
            return rays.copy(), valid

        def trace_counts(self, d_rays, n, d_hits):
            return dict(counts)

    rays = np.zeros(2, bt.RAY)
    out = bench.fetched_bytes(FakeCtx(), FakeBlas(), rays, 0)
    per_call = 64 * 10 + 32 * 20 + 40 * 1 + 32 * 4 + 88 * 3 + 48 * 2 + 40 * 5
    assert out["primary"]["rays"] == 2 and out["primary"]["bytes"] == per_call + 52 * 2
    assert out["bounce"]["rays"] == 1 and out["bounce"]["bytes"] == per_call + 52
    assert out["primary"]["per_ray"]["hidden_boxes"] == 10.0


def test_reference_arm_loads_no_cuda_library():
    """--impl reference times the oracle only: the CUDA library is never loaded (checked on the
    process's own memory map) and the line carries the reference arm's keys."""
    import json
    import subprocess
    import sys
    code = ("import runpy, sys, json\n"
            "sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', '--warmup', '3', '--ref-fraction', '512']\n"
            "try:\n    runpy.run_path('bench.py', run_name='__main__')\n"
            "except SystemExit as e:\n    assert not e.code, e.code\n"
            "maps = open('/proc/self/maps').read()\n"
            "print(json.dumps({'bvhgpu': 'libbvhgpu' in maps, 'orc': 'liborc' in maps, "
            "'pkg': [m for m in sys.modules if m.startswith('bvhtracer_gb300')]}))\n")
    out = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    lines = [json.loads(x) for x in out.stdout.strip().splitlines()]
    line, probe = lines[0], lines[-1]
    assert line["impl"] == "reference" and line["value"] > 0 and line["e2e"]["h2d_bytes_per_step"] == 0
    assert line["cpu_baseline"]["kind"] == "port" and "every 512th 8x8 tile" in line["config"]["sample_per_step"]
    assert probe == {"bvhgpu": False, "orc": True, "pkg": []}


def test_parity_fail_reads_every_parity_object(bench):
    ok = {"checks": {"a": {"mismatch_outside_near_ties": 0}}, "identical_bvh": True}
    bad = {"checks": {"a": {"mismatch_outside_near_ties": 0}, "b": {"mismatch_outside_near_ties": 2}}}
    assert not bench.parity_fail({"parity": ok})
    assert bench.parity_fail({"parity": bad})
    assert bench.parity_fail({"parity": dict(ok, identical_bvh=False)})
    assert bench.parity_fail({"parity": ok, "batch": {"parity": bad}})
    assert not bench.parity_fail({"parity": ok, "batch": {"parity": ok}, "adjoint": {"parity": None}})


def test_gpus_flag_must_match_world_size(bench, monkeypatch):
    monkeypatch.setenv("WORLD_SIZE", "1")
    assert bench.main(["--gpus", "2", "--impl", "reference"]) == 2


def test_gpus_flag_starts_that_many_ranks():
    """`bench.py --gpus 2` run without torchrun starts two ranks itself (torch.distributed.run on
    127.0.0.1); the reference arm (the oracle stand-in, no GPU needed) then prints one line from
    rank 0 with n_gpus = 2."""
    import json
    import subprocess
    import sys
    pytest.importorskip("torch")
    env = {k: v for k, v in os.environ.items() if k not in ("RANK", "WORLD_SIZE", "LOCAL_RANK")}
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--gpus", "2", "--impl", "reference",
                          "--steps", "1", "--warmup", "3", "--ref-fraction", "1024"],
                         cwd=ROOT, capture_output=True, text=True, timeout=600, env=env)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [json.loads(x) for x in out.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1 and lines[0]["n_gpus"] == 2 and lines[0]["impl"] == "reference"
