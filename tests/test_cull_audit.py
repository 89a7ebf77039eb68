"""The exact in-leaf cull (csrc/cull.cuh), audited on the CPU with the library's own header.

Compiles tests/cull_audit.cpp with g++ (no fused multiply-add, like the kernels) and runs a few
million adversarial (ray, triangle group) pairs: no culled group may hold a triangle that the
reference's float test accepts at or below the ray's closest t, and the normal-cone bound on
|det| must never exceed the exact value.  A run that overclaims the cone bound by 0.1 % must be
caught, which shows the check is sensitive."""
import os
import re
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def audit(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    exe = str(tmp_path_factory.mktemp("cull") / "cull_audit")
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-pthread",
                    "-I", os.path.join(ROOT, "bvhtracer_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "cull_audit.cpp"), "-o", exe], check=True)
    return exe


def run(exe, iters, scale=1.0):
    out = subprocess.run([exe, str(iters), str(scale)], capture_output=True, text=True).stdout
    m = re.search(r"pairs (\d+) culled (\d+).*violations (\d+) \| cone bounds checked (\d+).*cone violations (\d+)",
                  out)
    assert m, out
    return {k: int(v) for k, v in zip(("pairs", "culled", "violations", "cone_checked", "cone_bad"), m.groups())}


def test_no_culled_group_holds_an_accepted_hit(audit):
    r = run(audit, 40000)
    assert r["pairs"] > 5_000_000 and r["culled"] > 500_000 and r["cone_checked"] > 500_000
    assert r["violations"] == 0 and r["cone_bad"] == 0


def test_overclaimed_cone_bound_is_caught(audit):
    r = run(audit, 40000, 1.001)
    assert r["cone_bad"] > 0
