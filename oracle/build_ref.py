"""Builds the reference implementation (pcdslab/gpu-sfft) as a parity checker.

TEST INFRASTRUCTURE ONLY: the product (gpu-sfft_gb300/) never links, calls or
runs anything this recipe makes.  Only tests/, tests/golden/make_ref_fixtures.py
and bench.py's reference-timing leg execute oracle/_ref/bin/ref_sfft.

Two steps:
  stage()  copies the reference's own C/CUDA sources from /root/reference into
           oracle/_ref/src/ and writes two stand-in headers for the CUDA-samples
           headers the reference includes but does not ship (helper_cuda.h:
           checkCudaErrors + <cassert>; helper_functions.h: empty).
           oracle/_ref/ is git-ignored: no reference source enters the history.
           The staged copy travels with the working tree to machines where
           /root/reference does not exist.
  build()  compiles the staged sources as they are (nvcc -O3 for .cu, gcc -O3
           -std=gnu99 for .c, the reference Makefile's flags without its
           CUDA-10.1 paths) for sm_103a, plus oracle/ref_harness.cu and the CPU
           oracle's parameter derivation, into oracle/_ref/bin/ref_sfft.

outerLoop.cu is compiled with -Douter_loop=ref_real_outer_loop so that the
harness can sit between the reference's experiment driver (run_experiment,
cuExperiment.cu:159-223) and its outer_loop (outerLoop.cu:65-190); no source
text is changed.

The reference's own build system (Makefile) is not used: it hard-codes
/usr/local/cuda-10.1 and the CUDA samples tree.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF_ROOT = "/root/reference"
OUT = os.path.join(HERE, "_ref")
SRC = os.path.join(OUT, "src")
SHIM = os.path.join(OUT, "shim")
OBJ = os.path.join(OUT, "obj")
BIN = os.path.join(OUT, "bin")
EXE = os.path.join(BIN, "ref_sfft")

# The files of the reference's sparse-FFT path and its experiment driver.
REF_FILES = ["cuExperiment.cu", "cudaFft.cu", "innerLoop.cu", "outerLoop.cu",
             "utils.c", "timer.c",
             "cudaFft.h", "experiment.h", "filters.h", "innerLoop.h", "outerLoop.h",
             "timer.h", "utils.h"]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

HELPER_CUDA = """\
// Stand-in for the CUDA samples' helper_cuda.h (not shipped with the reference).
#pragma once
#include <cassert>
#include <cstdio>
#include <cstdlib>
template <typename T>
inline void ref_check_status(T status, const char *what, const char *file, int line) {
  if ((int)status != 0) {
    fprintf(stderr, "reference: %s returned %d at %s:%d\\n", what, (int)status, file, line);
    exit(1);
  }
}
#define checkCudaErrors(call) ref_check_status((call), #call, __FILE__, __LINE__)
"""


def nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def staged():
    return all(os.path.exists(os.path.join(SRC, f)) for f in REF_FILES)


def stage():
    """Copies the reference sources into oracle/_ref/src (when they are here)."""
    if not os.path.isdir(REF_ROOT):
        return staged()
    os.makedirs(SRC, exist_ok=True)
    for f in REF_FILES:
        src, dst = os.path.join(REF_ROOT, f), os.path.join(SRC, f)
        if not os.path.exists(dst) or os.path.getmtime(src) > os.path.getmtime(dst):
            shutil.copyfile(src, dst)
    os.makedirs(SHIM, exist_ok=True)
    for name, text in (("helper_cuda.h", HELPER_CUDA), ("helper_functions.h", "#pragma once\n")):
        path = os.path.join(SHIM, name)
        if not os.path.exists(path) or open(path).read() != text:
            with open(path, "w") as fh:
                fh.write(text)
    return True


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(quiet=True, force=False):
    """Stages (if possible) and compiles oracle/_ref/bin/ref_sfft."""
    if not stage():
        raise RuntimeError("reference sources are not staged in oracle/_ref/src")
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(BIN, exist_ok=True)
    cc = nvcc()
    inc = ["-I", SRC, "-I", SHIM, "-I", HERE]
    headers = [os.path.join(SRC, f) for f in REF_FILES if f.endswith(".h")]
    units = []  # (source, object, command)
    for f in REF_FILES:
        src = os.path.join(SRC, f)
        if f.endswith(".cu"):
            obj = os.path.join(OBJ, f + ".o")
            extra = ["-Douter_loop=ref_real_outer_loop"] if f == "outerLoop.cu" else []
            cmd = [cc] + ARCH + ["-O3", "-lineinfo", "-w"] + extra + inc + ["-c", src, "-o", obj]
        elif f.endswith(".c"):
            obj = os.path.join(OBJ, f + ".o")
            cmd = ["gcc", "-O3", "-std=gnu99", "-w"] + inc + ["-c", src, "-o", obj]
        else:
            continue
        units.append((src, obj, cmd))
    harness = os.path.join(HERE, "ref_harness.cu")
    hobj = os.path.join(OBJ, "ref_harness.cu.o")
    units.append((harness, hobj, [cc] + ARCH + ["-O2", "-std=c++17"] + inc +
                  ["-c", harness, "-o", hobj]))
    osrc = os.path.join(HERE, "sfft_oracle.c")
    oobj = os.path.join(OBJ, "sfft_oracle.c.o")
    units.append((osrc, oobj, ["gcc", "-O2", "-std=gnu11", "-ffp-contract=off",
                               "-Wno-unknown-pragmas", "-I", HERE, "-c", osrc, "-o", oobj]))
    jobs = [(s, o, c) for s, o, c in units
            if force or _newer(o, [s] + headers + [os.path.join(HERE, "sfft_oracle.h")])]

    def run(job):
        s, o, c = job
        return s, subprocess.run(c, capture_output=True, text=True)

    failed = []
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for s, r in ex.map(run, jobs):
            if r.returncode != 0:
                failed.append(f"{os.path.basename(s)}:\n{(r.stdout + r.stderr).strip()}")
            elif not quiet and (r.stdout + r.stderr).strip():
                print(f"[build_ref] {os.path.basename(s)}\n{(r.stdout + r.stderr).strip()}",
                      file=sys.stderr)
    if failed:
        raise RuntimeError("reference build failed:\n" + "\n".join(failed))
    objs = [o for _, o, _ in units]
    if force or jobs or _newer(EXE, objs):
        subprocess.check_call([cc] + ARCH + ["-o", EXE] + objs + ["-lcufft", "-lm"])
    return EXE


if __name__ == "__main__":
    print(build(quiet=False, force="--force" in sys.argv))
