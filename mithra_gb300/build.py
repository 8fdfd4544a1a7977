"""Build recipe of libmithra_gb300.so (in-tree, under mithra_gb300/_build/).

CUDA translation units are compiled with nvcc for sm_103a only; host C++ units with g++.
Units are compiled in parallel and skipped when their object is newer than every source and
header.  No cmake, no torch extension machinery: the library is a plain C-ABI shared object.
"""
from __future__ import annotations

import glob
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libmithra_gb300.so")
NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-I", os.path.join(REPO, "include")] + ARCH
# Translation units whose arithmetic must round like the host initialisation (no FMA contraction).
NO_FMA = {"init_kernels.cu"}
HOST_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-Wno-unused-function",
              "-I", os.path.join(REPO, "include")]


def _headers():
    return (glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h"))
            + glob.glob(os.path.join(CSRC, "host", "*.h")) + glob.glob(os.path.join(REPO, "include", "*.h")))


def _stale(obj, src, headers):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(p) > t for p in [src] + headers)


def _compile(job):
    cmd, obj = job
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return obj


def build(verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    headers = _headers()
    jobs, objs = [], []
    for src in sorted(glob.glob(os.path.join(CSRC, "*.cu"))):
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        objs.append(obj)
        if _stale(obj, src, headers):
            extra = ["--fmad=false"] if os.path.basename(src) in NO_FMA else []
            jobs.append(([NVCC] + CUDA_FLAGS + extra + ["-c", src, "-o", obj], obj))
    for src in sorted(glob.glob(os.path.join(CSRC, "host", "*.cpp"))):
        obj = os.path.join(BUILD, "host_" + os.path.basename(src) + ".o")
        objs.append(obj)
        if _stale(obj, src, headers):
            jobs.append((["g++"] + HOST_FLAGS + ["-c", src, "-o", obj], obj))
    if jobs:
        with ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            for o in ex.map(_compile, jobs):
                if verbose:
                    print("built", os.path.relpath(o, REPO))
    if jobs or not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        tmp = LIB + ".tmp%d" % os.getpid()
        cmd = [NVCC] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
