"""Compile the bvhgpu CUDA library (libbvhgpu.so) in-tree for sm_103a.

nvcc for the kernels (one -gencode, compute_103a / sm_103a), g++ for the host SAH build;
translation units are compiled in parallel.  Floating-point flags keep every step
IEEE round-to-nearest and unfused (parity with the reference's Rust arithmetic).
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libbvhgpu.so")
ROOT = os.path.dirname(HERE)

GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "--fmad=false", "-prec-div=true", "-prec-sqrt=true",
              "-ftz=false", "-Xcompiler", "-fPIC,-ffp-contract=off,-fno-fast-math", "-Xptxas", "-v"]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-Wall"]
CU_SOURCES = ["api.cu", "kernels_trace.cu", "kernels_scene.cu", "kernels_adjoint.cu", "refit_noalloc.cu", "tune.cu", "build_gpu.cu", "physics.cu"]
CPP_SOURCES = ["host_build.cpp", "loaders.cpp"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the bvhgpu library needs the CUDA toolkit")


def _cuda_include(nvcc: str) -> str:
    return os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc))), "include")


def _sources():
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps.append(os.path.join(ROOT, "include", "bvhgpu.h"))
    return deps


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(p) <= t for p in _sources())


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and up_to_date():
        return LIB
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    inc = ["-I", os.path.join(ROOT, "include"), "-I", CSRC]
    jobs = []
    objs = []
    for src in CU_SOURCES:
        obj = os.path.join(BUILD, src + ".o")
        objs.append(obj)
        jobs.append([nvcc, *GENCODE, *NVCC_FLAGS, *inc, "-c", os.path.join(CSRC, src), "-o", obj])
    for src in CPP_SOURCES:
        obj = os.path.join(BUILD, src + ".o")
        objs.append(obj)
        jobs.append(["g++", *CXX_FLAGS, *inc, "-I", _cuda_include(nvcc), "-c", os.path.join(CSRC, src), "-o", obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r

    with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        results = list(ex.map(run, jobs))
    log = []
    for cmd, r in results:
        log.append(" ".join(cmd) + "\n" + r.stdout + r.stderr)
        if r.returncode != 0:
            raise RuntimeError("bvhgpu build failed:\n" + log[-1])
    with open(os.path.join(BUILD, "build.log"), "w") as f:
        f.write("\n".join(log))
    tmp = LIB + f".tmp{os.getpid()}"
    link = [nvcc, *GENCODE, "-shared", "-o", tmp, *objs, "-lpthread"]
    r = subprocess.run(link, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("bvhgpu link failed:\n" + r.stdout + r.stderr)
    os.replace(tmp, LIB)
    if verbose:
        print("\n".join(log))
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
