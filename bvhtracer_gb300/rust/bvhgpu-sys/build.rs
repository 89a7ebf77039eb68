//! Links libbvhgpu.so, which bvhtracer_gb300/build.py compiles in-tree with nvcc for sm_103a
//! (`python -c "import __graft_entry__ as g; g.build()"` at the repository root).  The library
//! links the CUDA runtime statically; the process needs only the NVIDIA driver at run time.
//! BVHGPU_LIB_DIR overrides the directory that holds libbvhgpu.so.
use std::env;
use std::path::PathBuf;

fn main() {
    let dir = match env::var("BVHGPU_LIB_DIR") {
        Ok(d) => PathBuf::from(d),
        Err(_) => PathBuf::from(env::var("CARGO_MANIFEST_DIR").expect("cargo sets CARGO_MANIFEST_DIR"))
            .join("..")
            .join("..")
            .join("_build"),
    };
    println!("cargo:rustc-link-search=native={}", dir.display());
    println!("cargo:rustc-link-lib=dylib=bvhgpu");
    println!("cargo:rerun-if-env-changed=BVHGPU_LIB_DIR");
    println!("cargo:rerun-if-changed=../../../include/bvhgpu.h");
    println!("cargo:rerun-if-changed=src/lib.rs");
}
