"""The C-ABI library loads and exports every entry point include/bvhgpu.h declares.
CPU only: no compute call needs a GPU here."""
import ctypes
import os
import re

import pytest

from bvhtracer_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    with open(os.path.join(ROOT, "include", "bvhgpu.h")) as f:
        text = f.read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(bvhgpu_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_entry_points():
    names = declared()
    assert "bvhgpu_blas_intersect" in names and "bvhgpu_scene_rebuild" in names
    assert len(names) >= 40


def test_library_exports_every_declared_symbol():
    lib = _lib.load()
    missing = [n for n in declared() if not hasattr(lib, n)]
    assert not missing, f"missing exports: {missing}"


def test_binding_covers_header():
    assert set(declared()) <= set(_lib.SIGNATURES), set(declared()) - set(_lib.SIGNATURES)


def test_create_without_device_fails_cleanly():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    lib = _lib.load()
    h = ctypes.c_void_p()
    rc = lib.bvhgpu_create(ctypes.byref(h), 0)
    assert rc in (3, 7)
    assert not h.value


def test_host_entry_points_validate_arguments():
    lib = _lib.load()
    used = ctypes.c_uint32()
    assert lib.bvhgpu_build_bvh_host(None, 0, None, ctypes.byref(used)) == 1
    assert lib.bvhgpu_destroy(None) == 1
    assert lib.bvhgpu_sync(None) == 1


def test_every_entry_point_rejects_a_null_context():
    """Every entry point that takes a context returns BVHGPU_ERR_INVALID_ARG (1) for a null
    context and null / zero arguments, before touching the device: no crash, no CUDA call."""
    lib = _lib.load()
    no_ctx = {"bvhgpu_create", "bvhgpu_launch_count", "bvhgpu_tune_space", "bvhgpu_last_error",
              "bvhgpu_get_stream"}
    checked = 0
    for name, (res, args) in _lib.SIGNATURES.items():
        if name in no_ctx or not args:
            continue
        vals = [None if a in (ctypes.c_void_p, ctypes.c_char_p) else a(0) for a in args]
        assert getattr(lib, name)(*vals) == 1, name
        checked += 1
    assert checked >= 80
    assert lib.bvhgpu_get_stream(None) is None
    assert b"context" in lib.bvhgpu_last_error(None)


def test_tune_space_lists_every_compiled_variant():
    """bvhgpu_tune_space needs no device: 5 launch shapes x 3 stacks x 5 big-leaf values x 5
    hidden-tree margins, times 3 refill sizes for the persistent kernels."""
    from bvhtracer_gb300.api import Context
    import bvhtracer_gb300 as bt
    for kernel, n in ((bt.K_TRACE_BLAS, 375), (bt.K_TRACE_SCENE, 375), (bt.K_PERSISTENT_BOUNCE, 1125),
                      (bt.K_TRACE_BATCH, 1125), (bt.K_SCENE_BOUNCE, 1125)):
        space = Context.tune_space(kernel)
        assert len(space) == n
        assert {(c["block"], c["min_blocks"]) for c in space} == {(128, 1), (128, 5), (128, 6), (128, 8), (64, 1)}
        assert {c["stack"] for c in space} == {8, 32, 256}
        assert bt.BIG_LEAF_NEVER in {c["big_leaf"] for c in space}
        assert {c["hidden"] for c in space} == {0, 100, 250, 500, 1000}
    lib = _lib.load()
    assert lib.bvhgpu_tune_space(3, None, 0, None) == 1  # bounce generation has no variants


def test_rust_sys_binding_is_generated_from_the_header():
    """bvhgpu-sys/src/lib.rs is the generator's output for the current header (no cargo here to
    compile it; this keeps the Rust declarations in step with include/bvhgpu.h), and it declares
    every entry point of the header."""
    import subprocess
    import sys
    crate = os.path.join(ROOT, "bvhtracer_gb300", "rust", "bvhgpu-sys")
    rc = subprocess.run([sys.executable, os.path.join(crate, "gen_bindings.py"), "--check"]).returncode
    assert rc == 0, "bvhgpu-sys/src/lib.rs is stale: rerun gen_bindings.py"
    with open(os.path.join(crate, "src", "lib.rs")) as f:
        rs = f.read()
    rust_fns = set(re.findall(r"pub fn (bvhgpu_[a-z0-9_]+)\(", rs))
    assert rust_fns == set(declared()), set(declared()) ^ rust_fns
