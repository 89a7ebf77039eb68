"""Generate src/lib.rs (the raw Rust bindings of the bvhgpu C ABI) from include/bvhgpu.h.

    python bvhtracer_gb300/rust/bvhgpu-sys/gen_bindings.py          # rewrite src/lib.rs
    python bvhtracer_gb300/rust/bvhgpu-sys/gen_bindings.py --check  # exit 1 if src/lib.rs is stale

The header is plain C with a fixed style (one declaration per statement, `typedef struct name {...}
name;`, `#define NAME value`), so a small parser stands in for bindgen, which needs libclang."""
from __future__ import annotations

import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
HEADER = os.path.join(HERE, "..", "..", "..", "include", "bvhgpu.h")
OUT = os.path.join(HERE, "src", "lib.rs")

SCALARS = {"float": "f32", "double": "f64", "int": "c_int", "uint32_t": "u32", "uint64_t": "u64",
           "uint8_t": "u8", "size_t": "usize", "char": "c_char", "void": "c_void"}
U32_CONSTS = {"BVHGPU_MISS", "BVHGPU_BIG_LEAF_NEVER", "BVHGPU_NOALLOC_MAX_NODES"}


def strip_comments(text: str) -> str:
    text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
    return re.sub(r"//[^\n]*", " ", text)


def rust_type(ctype: str, array: bool = False) -> str:
    """C parameter / field type -> Rust type (a parameter declared as an array is a pointer)."""
    ctype = " ".join(ctype.split())
    const = ctype.startswith("const ")
    base = ctype[6:] if const else ctype
    stars = base.count("*") + (1 if array else 0)
    base = base.replace("*", "").strip()
    if base == "bvhgpu_stream":
        r = "bvhgpu_stream"
    else:
        r = SCALARS.get(base, base)
    for k in range(stars):
        innermost = k == 0
        r = ("*const " if (const and innermost) else "*mut ") + r
    return r


def parse_params(params: str):
    params = params.strip()
    if params in ("", "void"):
        return []
    out = []
    for p in params.split(","):
        p = p.strip()
        m = re.match(r"(.*?)([A-Za-z_][A-Za-z0-9_]*)\s*(\[[^\]]*\])?$", p)
        ctype, name, arr = m.group(1), m.group(2), m.group(3)
        if name in ("type", "ref", "fn", "mod", "loop", "move", "box", "in"):
            name = name + "_"
        out.append((name, rust_type(ctype, array=arr is not None)))
    return out


def generate() -> str:
    src = open(HEADER).read()
    defines = re.findall(r"^#define\s+(BVHGPU_[A-Z0-9_]+)\s+(.+?)\s*(?:/\*.*)?$", src, flags=re.M)
    body = strip_comments(src)
    lines = ["//! Raw bindings of the bvhgpu C ABI (include/bvhgpu.h), generated by gen_bindings.py -- do not",
             "//! edit by hand.  Every function returns a status (BVHGPU_OK = 0); see the header for each",
             "//! entry point's contract and the reference interface it replaces.",
             "#![allow(non_camel_case_types)]",
             "#![no_std]",
             "",
             "pub use core::ffi::{c_char, c_int, c_void};",
             "",
             "/// Opaque library context (one per host thread).",
             "#[repr(C)]",
             "pub struct bvhgpu_ctx {",
             "    _private: [u8; 0],",
             "}",
             "/// A cudaStream_t; null selects the context's own stream.",
             "pub type bvhgpu_stream = *mut c_void;",
             ""]
    for name, val in defines:
        if name == "BVHGPU_H":
            continue
        v = val.strip()
        m = re.match(r"\((\d+)u\s*<<\s*(\d+)\)", v)
        if m:
            v = f"{m.group(1)} << {m.group(2)}"
        v = v.rstrip("u").replace("0xFFFFFFFF", "0xFFFF_FFFF")
        ty = "u32" if name in U32_CONSTS else "c_int"
        lines.append(f"pub const {name}: {ty} = {v};")
    lines.append("")
    for m in re.finditer(r"typedef\s+struct\s+(\w+)\s*\{(.*?)\}\s*(\w+)\s*;", body, flags=re.S):
        name, fields = m.group(1), m.group(2)
        lines += ["#[repr(C)]", "#[derive(Copy, Clone, Debug, Default)]" if name != "bvhgpu_tune_job"
                  else "#[derive(Copy, Clone, Debug)]", f"pub struct {name} {{"]
        for decl in fields.split(";"):
            decl = " ".join(decl.split())
            if not decl:
                continue
            fm = re.match(r"(.*?)\s*((?:\*?\s*[A-Za-z_][A-Za-z0-9_]*(?:\[\d+\])?\s*,\s*)*\*?\s*[A-Za-z_][A-Za-z0-9_]*(?:\[\d+\])?)$",
                          decl)
            ctype = fm.group(1)
            for item in fm.group(2).split(","):
                item = item.strip()
                ptr = item.startswith("*")
                item = item.lstrip("*").strip()
                am = re.match(r"([A-Za-z_][A-Za-z0-9_]*)(?:\[(\d+)\])?$", item)
                fname, n = am.group(1), am.group(2)
                ty = rust_type(ctype + (" *" if ptr else ""))
                if n:
                    ty = f"[{ty}; {n}]"
                lines.append(f"    pub {fname}: {ty},")
        lines += ["}", ""]
    # tune_job holds raw pointers: no Default derive, give one by hand
    lines += ["impl Default for bvhgpu_tune_job {",
              "    fn default() -> Self {",
              "        Self { kernel: 0, target: 0, d_rays: core::ptr::null(), n: 0, seed: 0,",
              "               d_hits0: core::ptr::null_mut(), d_hits1: core::ptr::null_mut(),",
              "               items: core::ptr::null(), nitems: 0 }",
              "    }",
              "}", "",
              'extern "C" {']
    for m in re.finditer(r"^\s*(int|const char\s*\*|uint64_t|bvhgpu_stream)\s+(bvhgpu_\w+)\s*\(([^;]*?)\)\s*;",
                         body, flags=re.M | re.S):
        ret, name, params = m.group(1), m.group(2), m.group(3)
        rret = {"int": "c_int", "uint64_t": "u64", "bvhgpu_stream": "bvhgpu_stream"}.get(ret.strip(), "*const c_char")
        ps = ", ".join(f"{n}: {t}" for n, t in parse_params(params))
        lines.append(f"    pub fn {name}({ps}) -> {rret};")
    lines += ["}", ""]
    return "\n".join(lines)


if __name__ == "__main__":
    text = generate()
    if "--check" in sys.argv:
        cur = open(OUT).read() if os.path.exists(OUT) else ""
        sys.exit(0 if cur == text else 1)
    with open(OUT, "w") as f:
        f.write(text)
    print(f"wrote {OUT}")
