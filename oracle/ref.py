"""Python side of the reference harness (oracle/ref_harness.cu).

TEST INFRASTRUCTURE ONLY.  Runs the reference implementation (pcdslab/gpu-sfft,
built from its own sources by oracle/build_ref.py) as a child process and reads
back what it dumped: the signal and filter the reference's experiment produced,
and the candidate Nodes of its own outer_loop (outerLoop.cu:65-190).

Each run is a separate process, so the reference's exit(1) on a CUDA error and
its assert() aborts end that process only.
"""
from __future__ import annotations

import os
import re
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
EXE = os.path.join(HERE, "_ref", "bin", "ref_sfft")

NODE = np.dtype({"names": ["key", "x", "y"], "formats": ["<u4", "<f8", "<f8"],
                 "offsets": [0, 8, 16], "itemsize": 24})


def available():
    return os.path.exists(EXE)


def run(cfg, signal_seed=None, snr_db=None, outer_seed=None, reps=1, dump=None,
        candidate_bound=None, timeout=900):
    """Runs the reference experiment for cfg = (q, k, Bcst, loops_loc,
    loops_thresh, loops_est, RLFC_cst, RLFC_loops).  Returns its parsed report:
    per-run (I_F, wall ms), MISSED (estimation, result), MSE*k, the stdout."""
    if not available():
        raise RuntimeError("reference harness not built (oracle/build_ref.py)")
    q, k, Bcst, ll, lt, le, rc, rl = cfg
    cmd = [EXE, str(q), str(k), repr(float(Bcst)), str(ll), str(lt), str(le), str(int(rc)),
           str(rl)]
    if signal_seed is not None:
        cmd += ["--signal-seed", str(signal_seed)]
    if snr_db is not None:
        cmd += ["--snr-db", repr(float(snr_db))]
    if outer_seed is not None:
        cmd += ["--outer-seed", str(outer_seed)]
    if reps != 1:
        cmd += ["--reps", str(reps)]
    if dump is not None:
        os.makedirs(dump, exist_ok=True)
        cmd += ["--dump", dump]
    if candidate_bound is not None:
        cmd += ["--candidate-bound", str(int(candidate_bound))]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=timeout)
    if r.returncode != 0:
        raise RuntimeError(f"reference run failed ({r.returncode}): {r.stderr[-2000:]}")
    out = r.stdout
    runs = [(int(m.group(2)), float(m.group(3)))
            for m in re.finditer(r"^REF_RUN (\d+) (\d+) ([0-9.]+)$", out, re.M)]
    rep = {"runs": runs, "stdout": out}
    m = re.search(r"MISSED \(estimation, result\) = \((\d+), (\d+)\), MSE\*k = ([0-9.eE+-]+|nan|inf)",
                  out)
    if m:
        rep["missed"] = (int(m.group(1)), int(m.group(2)))
        rep["mse_k"] = float(m.group(3))
    m = re.search(r"Total GPU-SFFT time: ([0-9.eE+-]+)", out)
    if m:
        rep["reported_s"] = float(m.group(1))
    return rep


def load_dump(path):
    """Reads what one run with dump=path wrote."""
    vals = [int(v) for v in open(os.path.join(path, "params.txt")).read().split()]
    names = ["n", "w", "B", "B_thresh", "W_RLFC", "RLFC_loops", "loops_thresh", "loops_loc",
             "loops", "k"]
    prm = dict(zip(names, vals))
    n, w = prm["n"], prm["w"]
    d = {"params": prm,
         "x": np.fromfile(os.path.join(path, "x.bin"), dtype=np.complex128, count=n),
         "ft": np.fromfile(os.path.join(path, "ft.bin"), dtype=np.complex128, count=w),
         "ff": np.fromfile(os.path.join(path, "ff.bin"), dtype=np.complex128, count=n),
         "true_loc": np.fromfile(os.path.join(path, "true_loc.bin"), dtype=np.int32)}
    nodes = []
    r = 0
    while os.path.exists(os.path.join(path, f"nodes_{r}.bin")):
        raw = np.fromfile(os.path.join(path, f"nodes_{r}.bin"), dtype=np.uint8)
        count = int(raw[:4].view(np.int32)[0])
        nodes.append(raw[4:4 + 24 * count].view(NODE).copy())
        r += 1
    d["nodes"] = nodes
    return d


def stage(kind, meta, arrays, workdir, timeout=600):
    """Runs one reference stage function (ref_sfft stage KIND, see
    oracle/ref_harness.cu run_stage) on the given inputs in workdir and
    returns its output arrays.  meta: {name: int}; arrays: {file stem: numpy
    array} written as raw files (complex128 / int32)."""
    if not available():
        raise RuntimeError("reference harness not built (oracle/build_ref.py)")
    os.makedirs(workdir, exist_ok=True)
    with open(os.path.join(workdir, "meta.txt"), "w") as fh:
        for k, v in meta.items():
            fh.write(f"{k} {int(v)}\n")
    for stem, arr in arrays.items():
        arr = np.ascontiguousarray(arr)
        if np.iscomplexobj(arr):
            arr = arr.astype(np.complex128)
        else:
            arr = arr.astype(np.int32)
        arr.tofile(os.path.join(workdir, stem + ".bin"))
    r = subprocess.run([EXE, "stage", kind, workdir], capture_output=True, text=True,
                       timeout=timeout)
    if r.returncode != 0 or f"REF_STAGE {kind} ok" not in r.stdout:
        raise RuntimeError(f"reference stage {kind} failed ({r.returncode}): {r.stderr[-2000:]}")

    def ints(stem, count=-1):
        return np.fromfile(os.path.join(workdir, stem + ".bin"), dtype=np.int32, count=count)

    def cplx(stem, count=-1):
        return np.fromfile(os.path.join(workdir, stem + ".bin"), dtype=np.complex128, count=count)

    if kind == "cutoff":
        return {"J": ints("J")}
    if kind == "rlfc":
        return {"J2": ints("J2"), "offset": int(ints("offset")[0])}
    if kind == "perm":
        return {"bins_f": cplx("bins_f"), "J": ints("J")}
    if kind == "vote":
        return {"I": ints("I"), "vote": ints("vote")}
    if kind == "est":
        raw = np.fromfile(os.path.join(workdir, "nodes.bin"), dtype=np.uint8)
        return {"nodes": raw.view(NODE).copy()}
    raise ValueError(kind)
