"""Builds libwolkenbase_gb300.so in-tree with nvcc for sm_103a.

Each translation unit is compiled in parallel, then linked into one shared
library next to this file.  -fmad=false keeps every double expression free of
fused multiply-adds, so decoded coordinates, hypot and the tile sums round
exactly like the reference's x86-64 build.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libwolkenbase_gb300.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
SOURCES = ["wb_abi.cu", "wb_prims.cu", "wb_build.cu", "wb_tiles.cu", "wb_classify.cu", "wb_grid.cu", "wb_geom.cpp", "wb_serve.cpp", "wb_las.cu", "wb_lasio.cu", "wb_query.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _flags(src):
    f = ["-O3", "-std=c++17", "-lineinfo", "-fmad=false", "-Xcompiler", "-fPIC,-ffp-contract=off",
         "-I" + CSRC, "-I" + INCLUDE]
    if src.endswith(".cu"):
        f = ARCH + f + ["--expt-relaxed-constexpr"]
    return f


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, force=False):
    os.makedirs(OBJ, exist_ok=True)
    headers = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".h", ".cuh"))]
    headers.append(os.path.join(INCLUDE, "wolkenbase_gb300.h"))
    cc = nvcc()
    jobs = []
    objs = []
    for s in SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(OBJ, s + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            jobs.append([cc] + _flags(s) + ["-c", src, "-o", obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("compile failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        return r.stdout + r.stderr

    with cf.ThreadPoolExecutor(max_workers=min(8, max(1, len(jobs)))) as ex:
        for out in ex.map(run, jobs):
            if verbose and out.strip():
                print(out)
    if force or jobs or _stale(LIB, objs):
        cmd = [cc] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]
        run(cmd)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(verbose=True, force="--force" in sys.argv))
