"""Shared helpers of the reference parity tests.

tests/test_ref_golden.py (CPU) checks the oracle, and tests/test_gpu_reference.py
(GPU) checks the engine, against outputs of the reference implementation
itself (pcdslab/gpu-sfft built from its own sources): the golden fixtures
tests/golden/ref_*.npz (made by tests/golden/make_ref_fixtures.py) and, on a
GPU machine with the reference harness built, live runs of the reference.

Comparison rules (the same for the oracle and the engine):
  cutoff, rlfc     selected ids identical (innerLoop.cu:551-642)
  perm             bins_f within 1e-12 x max|bins_f| (two FFT implementations
                   round differently), J identical
  vote             candidate multiset and vote table identical
                   (innerLoop.cu:783-817; the reference appends in atomic
                   order, so candidates are compared sorted)
  est              keys in input order identical, values within 1e-13 relative
                   (innerLoop.cu:825-870)
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
STAGE_CASES = ["cutoff_ties", "cutoff_free", "rlfc", "perm", "vote", "est"]
E2E_FIXTURES = ["ref_n15_k30_s1", "ref_n15_k30_s2", "ref_n16_k50_s1", "ref_n16_k50_s2"]

BINS_TOL = 1e-12
EST_TOL = 1e-13


def kind_of(case):
    return case.split("_")[0]


def expand_window(win, n, B):
    """Filter response on the n/B + 1 bins around 0 -> n bins (zero elsewhere)."""
    half = n // (2 * B)
    ff = np.zeros(n, np.complex128)
    ff[np.r_[0:half + 1, n - half:n]] = win
    return ff


def load_stage(case):
    z = np.load(os.path.join(GOLDEN, f"ref_stage_{case}.npz"))
    meta = {k[5:]: int(z[k]) for k in z.files if k.startswith("meta_")}
    inp = {k[3:]: z[k] for k in z.files if k.startswith("in_")}
    if "ff_win" in inp:
        inp["ff"] = expand_window(inp.pop("ff_win"), meta["n"], meta["B"])
    out = {k[4:]: z[k] for k in z.files if k.startswith("out_")}
    if "keys" in out:
        out["nodes_keys"], out["nodes_vals"] = out.pop("keys"), out.pop("vals")
    if "offset" in out:
        out["offset"] = int(out["offset"])
    return meta, inp, out


def from_live(out):
    """Reference stage output (oracle/ref.py stage) in the fixture's layout."""
    if "nodes" in out:
        nodes = out["nodes"]
        return {"nodes_keys": nodes["key"].copy(), "nodes_vals": nodes["x"] + 1j * nodes["y"]}
    return dict(out)


def cfg_tuple(arr):
    c = [float(v) for v in arr]
    return (int(c[0]), int(c[1]), c[2], int(c[3]), int(c[4]), int(c[5]), c[6], int(c[7]))


def load_e2e(O, name):
    """One end-to-end fixture with the oracle's parameters and the glibc draws
    the reference used; ft_dropped = the taps with the w mod B residue taps
    zeroed (what the reference computes at these sizes)."""
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    cfg = cfg_tuple(z["cfg"])
    p, st = O.derive_params(*cfg)
    assert st == 0
    ft = z["ft"]
    ft_dropped = ft.copy()
    ft_dropped[(p.w // p.B) * p.B:] = 0
    offs, a, ai = O.draw_glibc(int(z["outer_seed"]), p.n, p.W_RLFC, p.RLFC_loops, p.loops)
    reps = [dict(zip(z[f"keys_{r}"].tolist(), z[f"vals_{r}"].tolist())) for r in range(3)]
    return {"cfg": cfg, "p": p, "x": z["x"], "ft": ft, "ft_dropped": ft_dropped,
            "ff": expand_window(z["ff_win"], p.n, p.B), "ff_win": z["ff_win"],
            "true_loc": z["true_loc"], "draws": (offs, a, ai), "reps": reps}


# ---- stage runs --------------------------------------------------------------

def oracle_stage(O, kind, meta, inp):
    if kind == "cutoff":
        return {"J": O.cutoff(O.samples(inp["v"]), meta["num"], floor_rel=0.0)}
    if kind == "rlfc":
        lc = C.CDLL(None)
        lc.srand48(C.c_long(meta["seed"]))
        offset = int(np.floor(lc_drand48(lc) * (meta["n"] // meta["W_RLFC"])))
        return {"J2": O.rlfc(inp["x"], meta["n"], meta["W_RLFC"], meta["B_thresh"], offset,
                             floor_rel=0.0), "offset": offset}
    if kind == "perm":
        bins_t = O.perm_filter(inp["x"], meta["n"], inp["ft"], meta["B"], meta["ai"])
        bins_f = O.fft(bins_t)
        return {"bins_f": bins_f, "J": O.cutoff(O.samples(bins_f), meta["B_thresh"], 0.0)}
    if kind == "vote":
        n, Bt, L = meta["n"], meta["B_thresh"], meta["loops_loc"]
        vote, cand = None, None
        for l in range(L):
            cand, vote, st = O.reverse_hash(inp["J"][l * Bt:(l + 1) * Bt], inp["J2"], n, meta["B"],
                                            meta["W_RLFC"], int(inp["a"][l]), int(inp["ai"][l]),
                                            meta["loops_thresh"], vote=vote, cand=cand)
            assert st == 0
        return {"I": cand, "vote": vote}
    if kind == "est":
        nodes = O.estimate(inp["I"], inp["bins_f"], meta["loops"], meta["n"], inp["permute"],
                           meta["B"], inp["ff"])
        return {"nodes_keys": nodes["key"].copy(), "nodes_vals": nodes["x"] + 1j * nodes["y"]}
    raise ValueError(kind)


def lc_drand48(lc):
    lc.drand48.restype = C.c_double
    return lc.drand48()


def engine_stage(G, torch, kind, meta, inp):
    """The same stage through the engine's drop-ins with the reference's
    signatures (innerLoop.h:32-50), on device buffers."""
    L = G.lib()
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    if kind == "cutoff":
        d_v = dev(inp["v"].astype(np.complex128))
        d_out = torch.full((meta["num"],), -1, dtype=torch.int32, device="cuda")
        assert L.samples_indices(d_v.data_ptr(), meta["num"], meta["size"], d_out.data_ptr(),
                                 None) == 0, G.last_error()
        return {"J": d_out.cpu().numpy()}
    if kind == "rlfc":
        lc = C.CDLL(None)
        lc.srand48(C.c_long(meta["seed"]))
        d_x = dev(inp["x"])
        d_J2 = torch.full((meta["B_thresh"],), -1, dtype=torch.int32, device="cuda")
        assert L.restr_loc_freq_coeff(d_x.data_ptr(), meta["n"], meta["B_thresh"], meta["W_RLFC"],
                                      d_J2.data_ptr(), None) == 0, G.last_error()
        return {"J2": d_J2.cpu().numpy()}
    if kind == "perm":
        d_x, d_ft = dev(inp["x"]), dev(inp["ft"])
        d_bins = torch.zeros(meta["B"], dtype=torch.complex128, device="cuda")
        d_J = torch.full((meta["B_thresh"],), -1, dtype=torch.int32, device="cuda")
        assert L.perm_filter_cutoff(d_x.data_ptr(), meta["n"], d_ft.data_ptr(), meta["w"],
                                    meta["B_thresh"], meta["B"], meta["a"], meta["ai"],
                                    d_bins.data_ptr(), d_J.data_ptr(), None, None) == 0, \
            G.last_error()
        return {"bins_f": d_bins.cpu().numpy(), "J": d_J.cpu().numpy()}
    if kind == "vote":
        n, Bt, Lp = meta["n"], meta["B_thresh"], meta["loops_loc"]
        d_vote = torch.zeros(n, dtype=torch.int32, device="cuda")
        d_I = torch.full((524288,), -1, dtype=torch.int32, device="cuda")
        d_J2 = dev(inp["J2"].astype(np.int32))
        I_F = C.c_int(0)
        for l in range(Lp):
            d_J = dev(inp["J"][l * Bt:(l + 1) * Bt].astype(np.int32))
            assert L.reverse_hash(d_J.data_ptr(), n, Bt, meta["B"], int(inp["a"][l]),
                                  int(inp["ai"][l]), meta["loops_thresh"], d_vote.data_ptr(),
                                  d_I.data_ptr(), C.byref(I_F), None, d_J2.data_ptr(),
                                  meta["num_RLFC"], meta["W_RLFC"], meta["RLFC_loops"]) == 0, \
                G.last_error()
        torch.cuda.synchronize()
        return {"I": d_I[:I_F.value].cpu().numpy(), "vote": d_vote.cpu().numpy()}
    if kind == "est":
        d_I = dev(inp["I"].astype(np.int32))
        d_bins = dev(inp["bins_f"])
        d_ff = dev(inp["ff"])
        perm = np.ascontiguousarray(inp["permute"], np.int32)
        cnt = C.c_int(int(meta["I_F"]))
        ptr = L.estimate_values(d_I.data_ptr(), C.byref(cnt), d_bins.data_ptr(), meta["loops"],
                                meta["n"], perm.ctypes.data_as(C.c_void_p), meta["B"],
                                d_ff.data_ptr(), meta["loops_loc"])
        assert ptr, G.last_error()
        nodes = np.ctypeslib.as_array((C.c_char * (24 * cnt.value)).from_address(ptr)).view(
            G.NODE).copy()
        C.CDLL(None).free(C.c_void_p(ptr))
        return {"nodes_keys": nodes["key"].copy(), "nodes_vals": nodes["x"] + 1j * nodes["y"]}
    raise ValueError(kind)


def check_stage(kind, got, ref):
    if kind == "cutoff":
        np.testing.assert_array_equal(got["J"], ref["J"])
    elif kind == "rlfc":
        np.testing.assert_array_equal(got["J2"], ref["J2"])
    elif kind == "perm":
        scale = np.abs(ref["bins_f"]).max()
        assert np.abs(got["bins_f"] - ref["bins_f"]).max() <= BINS_TOL * scale
        np.testing.assert_array_equal(got["J"], ref["J"])
    elif kind == "vote":
        np.testing.assert_array_equal(np.sort(got["I"]), np.sort(ref["I"]))
        np.testing.assert_array_equal(got["vote"], ref["vote"])
    elif kind == "est":
        np.testing.assert_array_equal(got["nodes_keys"], ref["nodes_keys"])
        rv, gv = ref["nodes_vals"], got["nodes_vals"]
        floor = EST_TOL * np.abs(rv).max()
        assert (np.abs(gv - rv) <= EST_TOL * np.abs(rv) + floor).all(), \
            float((np.abs(gv - rv) / np.maximum(np.abs(rv), 1e-300)).max())
    else:
        raise ValueError(kind)


# ---- end to end --------------------------------------------------------------

def as_dict(nodes):
    return {int(k): complex(x, y) for k, x, y in zip(nodes["key"], nodes["x"], nodes["y"])}


def topk_keys(d, k):
    return set(sorted(d, key=lambda kk: (-abs(d[kk]), kk))[:k])


def compare_e2e(got, ref, k, value_tol):
    """got, ref: {key: value}.  Same candidate set, values within value_tol
    relative (floor: value_tol x the largest |value|), same top-k set."""
    assert set(got) == set(ref), (len(set(got) ^ set(ref)), len(got), len(ref))
    vmax = max(abs(v) for v in ref.values())
    bad = [kk for kk in ref if abs(got[kk] - ref[kk]) > value_tol * (abs(ref[kk]) + vmax)]
    assert not bad, (len(bad), max(abs(got[kk] - ref[kk]) / abs(ref[kk]) for kk in bad))
    assert topk_keys(got, k) == topk_keys(ref, k)
