"""In-tree build of the dagc native libraries (no cmake, no torch).

Produces, under dag_compression_fast_gb300/_lib/:
  libdagc.so      the CUDA library behind include/dagc.h (sm_103a kernels,
                  C++ host orchestration, static CUDA runtime)
  libdagc_gen.so  the host-only synthetic fragment generators (include/dagc_gen.h)

Usage: python -m dag_compression_fast_gb300.build [--force]
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "_lib")
REPO = os.path.dirname(HERE)
INCLUDE = os.path.join(REPO, "include")

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                     "-Xcompiler", "-ffp-contract=off", f"-I{INCLUDE}", "--expt-relaxed-constexpr"]
CXX = os.environ.get("CXX", "g++")
CXX_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-pthread", "-Wall", "-Wextra", "-ffp-contract=off",
             f"-I{CUDA_HOME}/include", f"-I{INCLUDE}"]

CU_SOURCES = ["sort.cu", "dag_kernels.cu", "dedup.cu", "group.cu", "chunks.cu", "trace.cu", "voxelize.cu",
              "sort_noalloc.cu"]
# The tracer's and the voxelizer's float arithmetic must round once per
# operation (no FMA contraction) so that their results are reproducible on the CPU.
CU_EXTRA = {"trace.cu": ["--fmad=false"], "voxelize.cu": ["--fmad=false"]}
CPP_SOURCES = ["dagc.cpp", "serve.cpp", "io.cpp"]
GEN_SOURCES = ["generators.cpp"]

LIBDAGC = os.path.join(LIB, "libdagc.so")
LIBGEN = os.path.join(LIB, "libdagc_gen.so")


def _newer(target: str, deps) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return hs


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def build(force: bool = False, verbose: bool = False, ptxas_verbose: bool = False) -> None:
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIB, exist_ok=True)
    headers = _headers()
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if force or not _newer(o, [s] + headers):
            extra = ["-Xptxas", "-v"] if ptxas_verbose else []
            jobs.append([NVCC] + NVCC_FLAGS + CU_EXTRA.get(src, []) + extra + ["-c", s, "-o", o])
    for src in CPP_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if force or not _newer(o, [s] + headers):
            jobs.append([CXX] + CXX_FLAGS + ["-c", s, "-o", o])
    with ThreadPoolExecutor(max_workers=max(2, os.cpu_count() or 2)) as ex:
        outs = list(ex.map(_run, jobs))
    if verbose or ptxas_verbose:
        for o in outs:
            if o.strip():
                print(o)
    if force or jobs or not os.path.exists(LIBDAGC):
        _run([NVCC] + ARCH + ["-shared", "-cudart", "static", "-o", LIBDAGC] + objs + ["-ldl"])
    gen_srcs = [os.path.join(CSRC, f) for f in GEN_SOURCES]
    if force or not _newer(LIBGEN, gen_srcs + headers):
        _run([CXX] + CXX_FLAGS + ["-shared", "-o", LIBGEN] + gen_srcs)


def clean() -> None:
    shutil.rmtree(BUILD, ignore_errors=True)
    shutil.rmtree(LIB, ignore_errors=True)


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True, ptxas_verbose="--ptxas" in sys.argv)
    print("built", LIBDAGC, LIBGEN)
