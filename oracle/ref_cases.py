"""Inputs for the reference stage comparisons (ref_sfft stage ...).

TEST INFRASTRUCTURE ONLY.  Builds, from seeded synthetic signals and the CPU
oracle, the inputs of each reference stage function (innerLoop.h:32-50) on
which the reference's kernels are race-free:

  cutoff  |v|^2 of `size` samples -> num ids (innerLoop.cu:484-616); one row
          with many exact ties (small integers) and one without.
  rlfc    noisy signal -> one RLFC block (innerLoop.cu:112-177); noise keeps
          every |X|^2 far above FFT rounding, so the selected ids do not
          depend on which FFT computed them.
  perm    noisy signal, w = (w // B) * B taps -> bins_f and J
          (innerLoop.cu:194-286).  With w a multiple of B the residue thread of
          permFilterTillKernel (innerLoop.cu:745-754) has nothing to add, so
          no two threads update one bin.
  vote    J of every location loop and J2 from an oracle run on a noisy
          signal -> candidates and votes (innerLoop.cu:300-384).
  est     that run's candidates, bins_f and permutations -> estimates
          (innerLoop.cu:396-466).

Every case carries the draws it used, so the engine can be run on the same
inputs.
"""
from __future__ import annotations

import numpy as np

from . import oracle as O


def _signal(n, k, seed, snr_db):
    import os
    import sys
    pkg = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "gpu-sfft_gb300")
    if pkg not in sys.path:
        sys.path.insert(0, pkg)
    from gsfft import synth
    x, loc, coef, X = synth.signal_numpy(n, k, seed, snr_db=snr_db)
    return x


def build(cfg, seed, snr_db=20.0):
    """Stage cases for cfg = (q, k, Bcst, loops_loc, loops_thresh, loops_est,
    RLFC_cst, RLFC_loops).  Returns {kind: (meta, arrays)}."""
    p, st = O.derive_params(*cfg)
    assert st == 0, cfg
    n, B, W, Bt = p.n, p.B, p.W_RLFC, p.B_thresh
    rng = np.random.Generator(np.random.PCG64(seed + 77))
    x = _signal(n, p.k, seed, snr_db)
    ft, ff = O.design_filter(p)
    cases = {}

    # cutoff: a tie-heavy row (|v|^2 in {0, 1, 4, ..., 36}) and a tie-free row
    size_t = max(256, (W // 4) // 256 * 256)
    v_ties = rng.integers(0, 7, size=size_t).astype(np.float64) + 0j
    cases["cutoff_ties"] = ({"size": size_t, "num": size_t // 6}, {"v": v_ties})
    v_free = rng.standard_normal(W) + 1j * rng.standard_normal(W)
    cases["cutoff_free"] = ({"size": W, "num": Bt}, {"v": v_free})

    # rlfc
    cases["rlfc"] = ({"n": n, "W_RLFC": W, "B_thresh": Bt, "seed": 1000 + seed}, {"x": x})

    # perm: one permutation, taps truncated to a whole number of tiles
    a = int(rng.integers(0, n // 2)) * 2 + 1
    ai = pow(a, -1, n)
    wt = (p.w // B) * B
    cases["perm"] = ({"n": n, "w": wt, "B": B, "B_thresh": Bt, "a": a, "ai": ai},
                     {"x": x, "ft": ft[:wt]})

    # vote + est from one oracle run (raw selection, as the reference selects)
    sig = np.random.Generator(np.random.PCG64(seed ^ 0xABC))
    offs = sig.integers(0, n // W, size=p.RLFC_loops).astype(np.int32)
    av = (sig.integers(0, n // 2, size=p.loops) * 2 + 1).astype(np.int64)
    aiv = np.array([pow(int(v), -1, n) for v in av], np.int64)
    o = O.outer_loop(x, p, ft, ff, offs, av.astype(np.int32), aiv.astype(np.int32),
                     want_stages=True, floor_rel=0.0)
    assert o["status"] == 0
    J = o["J"][:p.loops_loc].reshape(-1)
    J2 = np.unique(o["J2_blocks"].reshape(-1))
    cases["vote"] = ({"n": n, "B": B, "B_thresh": Bt, "W_RLFC": W, "RLFC_loops": p.RLFC_loops,
                      "loops_thresh": p.loops_thresh, "loops_loc": p.loops_loc,
                      "num_RLFC": J2.size},
                     {"J": J, "J2": J2, "a": av[:p.loops_loc], "ai": aiv[:p.loops_loc]})
    cand = o["nodes"]["key"].astype(np.int32)
    cases["est"] = ({"n": n, "B": B, "loops": p.loops, "loops_loc": p.loops_loc,
                     "I_F": cand.size},
                    {"I": cand, "bins_f": o["bins_f"].reshape(-1), "permute": aiv, "ff": ff})
    return cases


def kind_of(name):
    return name.split("_")[0]
