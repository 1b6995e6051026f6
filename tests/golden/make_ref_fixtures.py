"""Generates the reference golden vectors tests/golden/ref_*.npz.

Runs the reference implementation itself (pcdslab/gpu-sfft, built from its own
sources by oracle/build_ref.py into oracle/_ref/bin/ref_sfft), so it needs a
GPU.  For each small configuration and seed the reference's experiment draws
its signal (cuExperiment.cu:84-111: k locations by drand48, values 1, inverse
cuFFT), designs its filter (make_multiple_t, cuExperiment.cu:248-448) and the
harness runs the reference's outer_loop (outerLoop.cu:65-190) three times with
glibc seeded identically before each run.  The signals carry the reference's
own additive noise (utils.c:187-219) at 30 dB, so that every bucket's |X|^2
lies far above FFT rounding and the cutoffs pick the same ids whichever FFT
computed them.  Stored per fixture:

  x, ft, ff_win      the signal, the w filter taps and the filter response on
                     the n/B + 1 bins around 0 that the estimate reads
                     (indices 0..n/2B and n-n/2B..n-1, in that order)
  true_loc           the k drawn locations (with repeats, as drawn)
  cfg, snr_db        the experiment arguments and the noise level
  outer_seed         the glibc seed of the runs
  keys_r, vals_r     each run's candidate keys and values (r = 0, 1, 2)

The reference's perm+filter races (innerLoop.cu:745-754: the residue thread
and the bucket threads update the same bins without atomics).  At these sizes
the bucket threads' read-modify-write chains overwrite every residue update,
the same way in every run, so the reference computes the bins without the
w mod B residue taps; the tests reproduce that by zeroing those taps.

ref_stage_*.npz hold single reference stage functions (innerLoop.h:32-50) run on
race-free inputs built by oracle/ref_cases.py, with their outputs.

    python tests/golden/make_ref_fixtures.py --out tests/golden
"""
from __future__ import annotations

import argparse
import os
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle import ref as R  # noqa: E402

# name, (q, k, Bcst, loops_loc, loops_thresh, loops_est, RLFC_cst, RLFC_loops), seed, SNR dB
FIXTURES = [
    ("ref_n15_k30_s1", (15, 30, 1.4, 2, 2, 5, 16, 2), 1, 30.0),
    ("ref_n15_k30_s2", (15, 30, 1.4, 2, 2, 5, 16, 2), 2, 30.0),
    ("ref_n16_k50_s1", (16, 50, 1.4, 2, 2, 5, 32, 2), 1, 30.0),
    ("ref_n16_k50_s2", (16, 50, 1.4, 2, 2, 5, 32, 2), 2, 30.0),
]
REPS = 3
# stage fixtures: inputs from oracle/ref_cases.py for this configuration
STAGE_CFG, STAGE_SEED = (15, 30, 1.4, 2, 2, 5, 16, 2), 1


def outer_seed(signal_seed):
    return 100 + signal_seed


def make_stages(out_dir):
    """tests/golden/ref_stage_<case>.npz: the case's meta and inputs (the
    filter response only on the window the estimate reads) and the reference
    stage's outputs (prefixed out_)."""
    from oracle import ref_cases
    cases = ref_cases.build(STAGE_CFG, STAGE_SEED)
    for name, (meta, arrays) in cases.items():
        with tempfile.TemporaryDirectory() as tmp:
            out = R.stage(ref_cases.kind_of(name), meta, arrays, tmp)
        store = {f"meta_{k}": np.array(v, dtype=np.int64) for k, v in meta.items()}
        for k, v in arrays.items():
            if k == "ff":
                n, B = meta["n"], meta["B"]
                half = n // (2 * B)
                v = v[np.r_[0:half + 1, n - half:n]]
                k = "ff_win"
            store[f"in_{k}"] = v
        for k, v in out.items():
            if k == "nodes":
                store["out_keys"] = v["key"].astype(np.uint32)
                store["out_vals"] = (v["x"] + 1j * v["y"]).astype(np.complex128)
            else:
                store[f"out_{k}"] = np.asarray(v)
        path = os.path.join(out_dir, f"ref_stage_{name}.npz")
        np.savez_compressed(path, **store)
        print(path, {k: np.shape(v) for k, v in store.items()})


def make(out_dir):
    os.makedirs(out_dir, exist_ok=True)
    make_stages(out_dir)
    for name, cfg, seed, snr_db in FIXTURES:
        with tempfile.TemporaryDirectory() as tmp:
            R.run(cfg, signal_seed=seed, snr_db=snr_db, outer_seed=outer_seed(seed), reps=REPS,
                  dump=tmp)
            d = R.load_dump(tmp)
        # candidates come back in atomic order: compare the runs as key -> value maps
        maps = [dict(zip(r["key"].tolist(), zip(r["x"].tolist(), r["y"].tolist())))
                for r in d["nodes"]]
        print(name, "runs identical:", all(m == maps[0] for m in maps[1:]))
        prm = d["params"]
        n, B = prm["n"], prm["B"]
        half = n // (2 * B)
        win = np.r_[0:half + 1, n - half:n]
        arrays = {"x": d["x"], "ft": d["ft"], "ff_win": d["ff"][win], "true_loc": d["true_loc"],
                  "cfg": np.array(cfg, dtype=np.float64), "snr_db": np.array(snr_db),
                  "outer_seed": np.array(outer_seed(seed), dtype=np.int64)}
        for r, nodes in enumerate(d["nodes"]):
            arrays[f"keys_{r}"] = nodes["key"].astype(np.uint32)
            arrays[f"vals_{r}"] = (nodes["x"] + 1j * nodes["y"]).astype(np.complex128)
        path = os.path.join(out_dir, name + ".npz")
        np.savez_compressed(path, **arrays)
        print(path, {k: v.shape for k, v in arrays.items()})


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=os.path.join(ROOT, "tests", "golden"))
    make(ap.parse_args().out)
