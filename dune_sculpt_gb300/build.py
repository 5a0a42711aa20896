"""Builds libsculptgpu.so in-tree (dune_sculpt_gb300/lib/) with nvcc for sm_103a.

Kernels are compiled with -fmad=false and IEEE division/square root so that
every per-vertex formula rounds like the reference's scalar FP32 code; host
C++ is compiled with -ffp-contract=off for the same reason (the falloff table
and the PBVH build compare floats).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIBDIR, "libsculptgpu.so")
BUILD = os.path.join(HERE, "_build")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
                     "-fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false",
                     "--expt-relaxed-constexpr"]
CXX_FLAGS = ["-O2", "-fPIC", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-Wall"]

CU_SOURCES = ["kernels_team.cu", "kernels_wide.cu", "kernels_sym.cu", "kernels_lock.cu", "kernels.cu", "kernels_grids.cu",
              "kernels_ray.cu",
              "kernels_draw.cu", "noalloc.cu", "api.cu"]
CXX_SOURCES = ["host_pbvh.cpp", "host_draw.cpp"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _sources() -> list[str]:
    out = []
    for f in sorted(os.listdir(CSRC)):
        if f.endswith((".cu", ".cpp", ".h", ".cuh")):
            out.append(os.path.join(CSRC, f))
    return out


def _up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    deps = _sources() + [os.path.join(HERE, "..", "include", "sculpt_gpu.h"), __file__]
    return all(os.path.getmtime(p) <= t for p in deps if os.path.exists(p))


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and _up_to_date():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    nvcc = _nvcc()
    inc = ["-I", CSRC, "-I", os.path.join(HERE, "..", "include")]
    jobs = []
    for src in CU_SOURCES:
        obj = os.path.join(BUILD, src + ".o")
        jobs.append([nvcc] + NVCC_FLAGS + inc + ["-c", os.path.join(CSRC, src), "-o", obj])
    cuda_inc = os.path.join(os.path.dirname(os.path.dirname(nvcc)), "include")
    for src in CXX_SOURCES:
        obj = os.path.join(BUILD, src + ".o")
        jobs.append(["g++"] + CXX_FLAGS + inc + ["-I", cuda_inc, "-c", os.path.join(CSRC, src),
                                                "-o", obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if verbose or r.returncode != 0:
            sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
        return r.returncode

    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        codes = list(ex.map(run, jobs))
    if any(codes):
        raise RuntimeError("libsculptgpu compilation failed")
    objs = [os.path.join(BUILD, s + ".o") for s in CU_SOURCES + CXX_SOURCES]
    tmp = LIB + ".tmp"
    link = [nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-Xlinker", "--no-undefined"]
    if run(link) != 0:
        raise RuntimeError("libsculptgpu link failed")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
