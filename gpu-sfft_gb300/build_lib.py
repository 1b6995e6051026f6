"""Builds libgsfft.so (sm_103a) and the gsfft_exec host driver in-tree.

    python gpu-sfft_gb300/build_lib.py [--verbose-ptxas] [--force]

Outputs go to gpu-sfft_gb300/build/ (git-ignored).  Every .cu file in csrc/ is
compiled in parallel with
    nvcc -gencode arch=compute_103a,code=sm_103a -O3 -lineinfo -std=c++17
and linked with the static CUDA runtime into one shared library.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "build")
OBJ = os.path.join(BUILD, "obj")
LIB = os.path.join(BUILD, "libgsfft.so")
EXE = os.path.join(BUILD, "gsfft_exec")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                     "-Xcompiler", "-fvisibility=hidden", "-I", INCLUDE, "-I", CSRC,
                     "--expt-relaxed-constexpr"]


def nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose_ptxas=False, force=False, quiet=True):
    os.makedirs(OBJ, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(INCLUDE, "gsfft.h"))
    sources = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))
    cc = nvcc()
    jobs = []
    for f in sources:
        src = os.path.join(CSRC, f)
        obj = os.path.join(OBJ, f[:-3] + ".o")
        if force or _newer(obj, [src] + headers):
            cmd = [cc] + NVCC_FLAGS + (["-Xptxas", "-v"] if verbose_ptxas else []) + \
                ["-c", src, "-o", obj]
            jobs.append((f, cmd))
    def run(job):
        name, cmd = job
        r = subprocess.run(cmd, capture_output=True, text=True)
        return name, r
    failed = False
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for name, r in ex.map(run, jobs):
            out = (r.stdout + r.stderr).strip()
            if r.returncode != 0:
                failed = True
                print(f"[build] {name} FAILED\n{out}", file=sys.stderr)
            elif out and (verbose_ptxas or not quiet):
                print(f"[build] {name}\n{out}", file=sys.stderr)
    if failed:
        raise RuntimeError("nvcc compilation failed")
    objs = [os.path.join(OBJ, f[:-3] + ".o") for f in sources]
    if force or jobs or _newer(LIB, objs):
        cmd = [cc] + ARCH + ["-shared", "-o", LIB] + objs + ["-cudart", "static",
                                                              "-Xlinker", "-Bsymbolic"]
        subprocess.check_call(cmd)
    exe_src = os.path.join(HERE, "host", "gsfft_exec.c")
    if os.path.exists(exe_src) and (force or _newer(EXE, [exe_src, LIB])):
        subprocess.check_call(["gcc", "-O2", "-std=gnu11", "-Wall", "-I", INCLUDE, exe_src,
                               "-o", EXE, "-L", BUILD, "-lgsfft", "-Wl,-rpath,$ORIGIN", "-lm"])
    return LIB


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--verbose-ptxas", action="store_true")
    ap.add_argument("--force", action="store_true")
    a = ap.parse_args()
    print(build(a.verbose_ptxas, a.force, quiet=False))
