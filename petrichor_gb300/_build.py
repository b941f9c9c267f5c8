"""Builds the CUDA library libpetrichor_gb300.so in-tree (sm_103a only).

nvcc compiles the kernels for ``-gencode arch=compute_103a,code=sm_103a``; the
host C++ is compiled by g++ with ``-ffp-contract=off`` (the reference's x86-64
rounding for the few host-derived floats). The kernels are compiled
with ``-fmad=false``: the replay kernel reproduces the reference's unfused float
arithmetic, and no code path's results depend on where the compiler would have
chosen to fuse. A throughput-path result computed by two kernels (the staged
shade kernel and the tail kernel, a single-job and a mixed wave) is then the same
bits in both; the fused multiply-adds the throughput path does use are written
out (``fmaf``), so they are the same in every kernel too.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT_DIR = os.path.join(PKG, "_lib")
OBJ_DIR = os.path.join(OUT_DIR, "obj")
LIB = os.path.join(OUT_DIR, "libpetrichor_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")

CU_SOURCES = ["replay.cu", "wavefront.cu", "noalloc.cu", "bvh_gpu.cu", "denoise.cu", "probe.cu"]
# The throughput kernels use approximate division and square root (a few ulps), except
# where the code asks for correctly rounded results (traversal reciprocals, the
# triangle test); the replay kernel keeps IEEE arithmetic throughout.
FAST_DIV_SQRT = {"wavefront.cu": ["-prec-div=false", "-prec-sqrt=false"]}
CPP_SOURCES = ["capi.cpp", "bvh_builder.cpp", "scheduler.cpp", "server.cpp", "cpp_api.cpp",
               "cpp_loaders.cpp"]


def _nvcc() -> str:
    p = shutil.which("nvcc") or os.path.join(CUDA_HOME, "bin", "nvcc")
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found; set CUDA_HOME")
    return p


def _sources():
    return [os.path.join(CSRC, s) for s in CU_SOURCES + CPP_SOURCES] + [
        os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".h", ".cuh"))
    ] + [os.path.join(ROOT, "include", "petrichor_gb300.h"),
          os.path.join(ROOT, "include", "petrichor_gb300", "Petrichor.hpp")]


def _stale(lib: str = LIB) -> bool:
    if not os.path.exists(lib):
        return True
    t = os.path.getmtime(lib)
    return any(os.path.getmtime(s) > t for s in _sources())


# The checked build (device-side bounds checks on every node, primitive and queue
# index, recorded as an error bit): a separate library, for the test suite.
CHECK_DIR = os.path.join(PKG, "_lib_check")


def build_checked(force: bool = False, verbose: bool = False) -> str:
    return build(force, verbose, defines=("PT_CHECK=1",), out_dir=CHECK_DIR)


def build(force: bool = False, verbose: bool = False, defines=(), out_dir: str = OUT_DIR) -> str:
    lib_path = os.path.join(out_dir, "libpetrichor_gb300.so")
    obj_dir = os.path.join(out_dir, "obj")
    if not force and not _stale(lib_path):
        return lib_path
    os.makedirs(obj_dir, exist_ok=True)
    nvcc = _nvcc()
    inc = ["-I", CSRC, "-I", os.path.join(ROOT, "include")]
    jobs = []
    for s in CU_SOURCES:
        o = os.path.join(obj_dir, s + ".o")
        jobs.append([nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-fmad=false",
                     *FAST_DIV_SQRT.get(s, []),
                     *[f"-D{d}" for d in defines],
                     "-Xcompiler", "-fPIC", "-Xptxas", "-warn-spills", *inc, "-c",
                     os.path.join(CSRC, s), "-o", o])
    for s in CPP_SOURCES:
        o = os.path.join(obj_dir, s + ".o")
        jobs.append(["g++", "-std=c++17", "-O3", "-ffp-contract=off", "-fno-fast-math", "-fPIC",
                     "-pthread", "-Wall", *[f"-D{d}" for d in defines], *inc, "-I", os.path.join(CUDA_HOME, "include"), "-c",
                     os.path.join(CSRC, s), "-o", o])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("compile failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr)
        return r

    with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        list(ex.map(run, jobs))
    objs = [os.path.join(obj_dir, s + ".o") for s in CU_SOURCES + CPP_SOURCES]
    tmp = lib_path + ".tmp"
    run([nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-lpthread"])
    os.replace(tmp, lib_path)
    return lib_path


if __name__ == "__main__":
    print(build(force=True, verbose=True))
