"""ctypes binding of the CPU oracle (oracle/sfft_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, ``__graft_entry__.smoke()`` and
the cpu_baseline / ``--impl reference`` legs of bench.py, always as the checker
or the CPU baseline, never as the product path.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "build", "liboracle.so")

QUIRK_RESIDUE = 1
QUIRK_FILTER_RECURRENCE = 2
# the engine's default selection floor (samples below 1e-10 x max count as 0)
SELECTION_FLOOR = 1e-10

COMPLEX = np.dtype([("x", "<f8"), ("y", "<f8")])
NODE = np.dtype({"names": ["key", "x", "y"], "formats": ["<u4", "<f8", "<f8"],
                 "offsets": [0, 8, 16], "itemsize": 24})


class Params(C.Structure):
    _fields_ = [(f, C.c_int) for f in (
        "q", "n", "k", "B", "B_thresh", "W_RLFC", "RLFC_loops", "loops_loc",
        "loops_thresh", "loops_est", "loops", "b_f", "w")] + [
        (f, C.c_double) for f in ("Bcst", "RLFC_cst", "BB", "lobefrac", "tolerance", "t0")]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


def build():
    subprocess.check_call(["make", "-s", "-C", HERE])


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        P = C.c_void_p
        i, d = C.c_int, C.c_double
        L.oc_derive_params.argtypes = [i, i, d, i, i, i, d, i, d, C.POINTER(Params)]
        L.oc_draw_glibc.argtypes = [C.c_long, i, i, i, i, P, P, P]
        L.oc_draw_glibc.restype = None
        L.oc_fft.argtypes = [P, C.c_long, i]
        L.oc_design_filter.argtypes = [C.POINTER(Params), C.c_uint, P, P]
        L.oc_cutoff_f64.argtypes = [P, i, i, P]
        L.oc_cutoff_f64.restype = None
        L.oc_cutoff_f32.argtypes = [P, i, i, P]
        L.oc_cutoff_f32.restype = None
        L.oc_cutoff_floor_f64.argtypes = [P, i, i, d, P]
        L.oc_cutoff_floor_f64.restype = None
        L.oc_cutoff_floor_f32.argtypes = [P, i, i, d, P]
        L.oc_cutoff_floor_f32.restype = None
        L.oc_samples.argtypes = [P, i, P]
        L.oc_samples.restype = None
        L.oc_rlfc.argtypes = [P, i, i, i, i, d, P, P]
        L.oc_merge_j2.argtypes = [P, i]
        L.oc_perm_filter.argtypes = [P, i, P, i, i, i, C.c_uint, P]
        L.oc_perm_filter.restype = None
        L.oc_reverse_hash.argtypes = [P, i, P, i, i, i, i, i, i, i, P, P, P, i]
        L.oc_estimate.argtypes = [P, i, P, i, i, P, i, P, P]
        L.oc_estimate.restype = None
        L.oc_topk.argtypes = [P, i, i, P]
        L.oc_outer_loop.argtypes = [P, C.POINTER(Params), P, P, P, P, P, C.c_uint, d,
                                    P, i, P, P, P, P, P]
        L.oc_mod_inverse.argtypes = [i, i]
        L.oc_gcd.argtypes = [i, i]
        L.oc_floor_to_pow2.argtypes = [d]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def as_c128(x):
    return np.ascontiguousarray(x, dtype=np.complex128)


def derive_params(q, k, Bcst, loops_loc, loops_thresh, loops_est, RLFC_cst, RLFC_loops,
                  tolerance=1e-8):
    p = Params()
    st = lib().oc_derive_params(q, k, Bcst, loops_loc, loops_thresh, loops_est,
                                float(RLFC_cst), RLFC_loops, tolerance, C.byref(p))
    return p, st


def draw_glibc(seed, n, W, rlfc_loops, loops):
    off = np.zeros(rlfc_loops, np.int32)
    a = np.zeros(loops, np.int32)
    ai = np.zeros(loops, np.int32)
    lib().oc_draw_glibc(seed, n, W, rlfc_loops, loops, _p(off), _p(a), _p(ai))
    return off, a, ai


def fft(x, sign=-1):
    y = as_c128(x).copy()
    st = lib().oc_fft(_p(y), y.size, sign)
    assert st == 0
    return y


def design_filter(p, quirks=0):
    ft = np.zeros(p.w, np.complex128)
    ff = np.zeros(p.n, np.complex128)
    st = lib().oc_design_filter(C.byref(p), quirks, _p(ft), _p(ff))
    assert st == 0, st
    return ft, ff


def samples(v):
    v = as_c128(v)
    s = np.zeros(v.size, np.float64)
    lib().oc_samples(_p(v), v.size, _p(s))
    return s


def cutoff(s, num, floor_rel=0.0):
    out = np.zeros(num, np.int32)
    if s.dtype == np.float32:
        s = np.ascontiguousarray(s)
        lib().oc_cutoff_floor_f32(_p(s), s.size, num, floor_rel, _p(out))
    else:
        s = np.ascontiguousarray(s, dtype=np.float64)
        lib().oc_cutoff_floor_f64(_p(s), s.size, num, floor_rel, _p(out))
    return out


def rlfc(x, n, W, B_thresh, offset, want_spectrum=False, floor_rel=SELECTION_FLOOR):
    x = as_c128(x)
    J2 = np.zeros(B_thresh, np.int32)
    yf = np.zeros(W, np.complex128) if want_spectrum else None
    st = lib().oc_rlfc(_p(x), n, W, B_thresh, offset, floor_rel, _p(J2), _p(yf))
    assert st == 0
    return (J2, yf) if want_spectrum else J2


def merge_j2(blocks):
    J2 = np.ascontiguousarray(np.concatenate(blocks), dtype=np.int32)
    m = lib().oc_merge_j2(_p(J2), J2.size)
    return J2[:m].copy()


def perm_filter(x, n, filt, B, ai, quirks=0):
    x = as_c128(x)
    filt = as_c128(filt)
    out = np.zeros(B, np.complex128)
    lib().oc_perm_filter(_p(x), n, _p(filt), filt.size, B, ai, quirks, _p(out))
    return out


def reverse_hash(J, J2, n, B, W, a, ai, loops_thresh, vote=None, cand=None, cap=1 << 22):
    """One location loop; ``vote`` (n int32) and ``cand`` carry state across loops."""
    J = np.ascontiguousarray(J, np.int32)
    J2 = np.ascontiguousarray(J2, np.int32)
    if vote is None:
        vote = np.zeros(n, np.int32)
    buf = np.zeros(cap, np.int32)
    num = C.c_int(0)
    if cand is not None and len(cand):
        buf[:len(cand)] = cand
        num.value = len(cand)
    st = lib().oc_reverse_hash(_p(J), J.size, _p(J2), J2.size, n, B, W, a, ai,
                               loops_thresh, _p(vote), _p(buf), C.byref(num), cap)
    return buf[:min(num.value, cap)].copy(), vote, st


def estimate(cand, bins_f, loops, n, permute, B, filter_freq):
    cand = np.ascontiguousarray(cand, np.int32)
    bins_f = as_c128(bins_f)
    permute = np.ascontiguousarray(permute, np.int32)
    ff = as_c128(filter_freq)
    out = np.zeros(cand.size, NODE)
    lib().oc_estimate(_p(cand), cand.size, _p(bins_f), loops, n, _p(permute), B, _p(ff),
                      _p(out))
    return out


def topk(nodes, k):
    nodes = np.ascontiguousarray(nodes, NODE)
    out = np.zeros(min(k, nodes.size), NODE)
    c = lib().oc_topk(_p(nodes), nodes.size, k, _p(out))
    return out[:c]


def outer_loop(x, p, filter_time, filter_freq, offsets, a, ai, quirks=0, cap=1 << 22,
               want_stages=False, floor_rel=SELECTION_FLOOR):
    """The whole pipeline.  floor_rel: the engine's selection floor (default);
    0 gives the reference's raw cutoffs."""
    x = as_c128(x)
    ft, ff = as_c128(filter_time), as_c128(filter_freq)
    offsets = np.ascontiguousarray(offsets, np.int32)
    a = np.ascontiguousarray(a, np.int32)
    ai = np.ascontiguousarray(ai, np.int32)
    out = np.zeros(cap, NODE)
    I_F = C.c_int(0)
    nrl = C.c_int(0)
    J2 = np.zeros(p.RLFC_loops * p.B_thresh, np.int32) if want_stages else None
    bins = np.zeros(p.loops * p.B, np.complex128) if want_stages else None
    J = np.zeros(p.loops_loc * p.B_thresh, np.int32) if want_stages else None
    st = lib().oc_outer_loop(_p(x), C.byref(p), _p(ft), _p(ff), _p(offsets), _p(a), _p(ai),
                             quirks, floor_rel, _p(out), cap, C.byref(I_F), _p(J2), C.byref(nrl),
                             _p(bins), _p(J))
    res = {"status": st, "nodes": out[:min(I_F.value, cap)].copy(), "I_F": I_F.value,
           "num_RLFC": nrl.value}
    if want_stages:
        res.update(J2_blocks=J2.reshape(p.RLFC_loops, p.B_thresh), bins_f=bins.reshape(p.loops, p.B),
                   J=J.reshape(p.loops_loc, p.B_thresh))
    return res
