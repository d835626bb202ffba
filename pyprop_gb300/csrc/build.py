"""Builds libgbprop.so in-tree (pyprop_gb300/libgbprop.so) for sm_103a with nvcc.

The translation units are compiled in parallel, then linked; no cmake, no torch
extension machinery.  Re-running is incremental on source mtimes.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(HERE)
ROOT = os.path.dirname(PKG)
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libgbprop.so")
SOURCES = ["gbprop_kernels.cu", "gbprop_solve.cu", "gbprop_cgs.cu", "gbprop_expm.cu", "gbprop_api.cpp",
           "gbprop_noalloc.cu", "gbprop_setup.cu", "gbprop_bound.cu"]
# per-file flags: the set-up kernels reproduce the host restatement's roundings (no FMA contraction)
EXTRA = {"gbprop_setup.cu": ["-fmad=false"]}
HEADERS = ["gbprop_internal.h", "gbprop_device.cuh", os.path.join(ROOT, "include", "gbprop.h")]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    return "nvcc"


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    hdrs = [os.path.join(HERE, h) if not os.path.isabs(h) else h for h in HEADERS]
    objs = []
    jobs = []
    for src in SOURCES:
        path = os.path.join(HERE, src)
        obj = os.path.join(BUILD, src + ".o")
        objs.append(obj)
        if force or _newer(obj, [path] + hdrs):
            lang = [] if src.endswith(".cu") else ["-x", "cu"]
            cmd = [nvcc] + ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
                                   "-I" + os.path.join(ROOT, "include"), "-c"] + EXTRA.get(src, []) + lang + \
                [path, "-o", obj]
            jobs.append(cmd)

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        return r

    with ThreadPoolExecutor(max_workers=len(jobs) or 1) as ex:
        list(ex.map(run, jobs))
    if force or jobs or _newer(LIB, objs):
        run([nvcc] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"])
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
