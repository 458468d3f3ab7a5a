"""Build recipe of libillum_gb300.so (sm_103a) — nvcc only, no CMake.

Each .cu is compiled in parallel and linked into illum_gb300/libillum_gb300.so
(in-tree, git-ignored). Translation units whose results must match the CPU
oracle bit for bit (geometry, horizons, visibility, direct insolation, host
set-up code) are compiled with -fmad=false; every host side is compiled with
-ffp-contract=off so aarch64 gcc does not fuse multiply-adds either.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "libillum_gb300.so")
BUILD = os.path.join(HERE, "_build")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off,-fno-fast-math",
                 "-Xptxas", "-warn-spills"]
EXACT = {"bvh.cu", "direct.cu", "capi.cu", "gauss_seidel.cu"}   # -fmad=false
SOURCES = ["primitives.cu", "bvh.cu", "direct.cu", "radiosity.cu", "conduction.cu", "capi.cu", "batch.cu",
           "gauss_seidel.cu"]
HEADERS = ["common.cuh", "internal.cuh", "geom.h"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    return "nvcc"


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(HERE, "..", "include", "illum_gb300.h")]
    jobs = []
    objs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _stale(o, [s] + hdrs):
            flags = COMMON + (["-fmad=false"] if src in EXACT else [])
            jobs.append([nvcc] + flags + ["-c", s, "-o", o])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r

    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for cmd, r in ex.map(run, jobs):
                if verbose or r.returncode:
                    sys.stderr.write(r.stdout + r.stderr)
                if r.returncode:
                    raise RuntimeError("nvcc failed: " + " ".join(cmd))
    if force or jobs or _stale(OUT, objs):
        cmd = [nvcc] + ARCH + ["-shared", "-o", OUT] + objs + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("link failed")
    return OUT


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
    print(OUT)
