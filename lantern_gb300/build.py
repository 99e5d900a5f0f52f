"""Build liblantern_gpu.so in-tree (lantern_gb300/_build) for sm_103a.

Beside it, liblantern_gpu_checked.so: the same objects with the kernels
compiled with -DLT_CHECKS=1 (device-side bound checks, LT_ERR_CHECK), for test
runs (lantern_gb300.native loads it when LANTERN_GPU_CHECKED=1).

nvcc compiles the kernels with -gencode arch=compute_103a,code=sm_103a and
-fmad=false (the integrator's arithmetic is spelled out operation by
operation; the traversal writes its fused multiply-adds explicitly); g++
compiles the host C++ with -ffp-contract=off for the same reason. Translation
units are compiled in parallel; the CUDA runtime is linked statically.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liblantern_gpu.so")
CHECKED_LIB = os.path.join(BUILD, "liblantern_gpu_checked.so")
CHECKED_SOURCE = "lt_kernels.cu"  # the translation unit that holds the checks

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-Xcompiler", "-fPIC,-ffp-contract=off",
                     "-I" + INCLUDE, "-I" + CSRC]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-Wno-unused-function",
             "-I" + INCLUDE, "-I" + CSRC, "-I" + os.path.join(CUDA_HOME, "include")]

CU_SOURCES = ["lt_kernels.cu", "lt_bvh_gpu.cu", "lt_noalloc.cu", "lt_resolve.cu", "lt_setup.cu"]
CPP_SOURCES = ["lt_api.cpp", "lt_scene.cpp", "lt_json.cpp", "lt_bvh8.cpp", "lt_image.cpp"]


def _sources():
    return [os.path.join(CSRC, f) for f in CU_SOURCES + CPP_SOURCES]


def _headers():
    return ([os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
            + [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")])


def up_to_date() -> bool:
    if not os.path.exists(LIB) or not os.path.exists(CHECKED_LIB):
        return False
    t = min(os.path.getmtime(LIB), os.path.getmtime(CHECKED_LIB))
    return all(os.path.getmtime(f) <= t for f in _sources() + _headers() + [__file__])


def build(force: bool = False, verbose: bool = False, extra_nvcc=()) -> str:
    if not force and up_to_date():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    cxx = os.environ.get("CXX", shutil.which("g++") or "g++")
    jobs = []
    objs = []
    for f in CU_SOURCES:
        o = os.path.join(BUILD, f + ".o")
        objs.append(o)
        jobs.append([NVCC] + NVCC_FLAGS + list(extra_nvcc) + ["-c", os.path.join(CSRC, f), "-o", o])
    checked_obj = os.path.join(BUILD, CHECKED_SOURCE + ".checked.o")
    jobs.append([NVCC] + NVCC_FLAGS + list(extra_nvcc) + ["-DLT_CHECKS=1", "-c", os.path.join(CSRC, CHECKED_SOURCE),
                                                          "-o", checked_obj])
    for f in CPP_SOURCES:
        o = os.path.join(BUILD, f + ".o")
        objs.append(o)
        jobs.append([cxx] + CXX_FLAGS + ["-c", os.path.join(CSRC, f), "-o", o])
    procs = [(j, subprocess.Popen(j, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)) for j in jobs]
    failed = []
    for j, p in procs:
        out, _ = p.communicate()
        if verbose and out:
            sys.stdout.write(out)
        if p.returncode != 0:
            failed.append((j, out))
    if failed:
        msg = "\n".join(" ".join(j) + "\n" + out for j, out in failed)
        raise RuntimeError("liblantern_gpu build failed:\n" + msg)
    plain_obj = os.path.join(BUILD, CHECKED_SOURCE + ".o")
    for lib, lib_objs in ((CHECKED_LIB, [checked_obj if o == plain_obj else o for o in objs]), (LIB, objs)):
        tmp = lib + f".{os.getpid()}.tmp"
        link = [NVCC] + ARCH + ["-shared", "-o", tmp] + lib_objs + ["-lpthread", "-ldl"]
        r = subprocess.run(link, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stdout + r.stderr)
        os.replace(tmp, lib)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv,
                extra_nvcc=["-Xptxas", "-v"] if "--ptxas" in sys.argv else []))
