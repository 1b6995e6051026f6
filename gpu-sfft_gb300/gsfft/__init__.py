"""Host-side Python binding of libgsfft.so (include/gsfft.h) via ctypes.

This mirrors the reference's host interface for the sparse-FFT path
(outerLoop.h:35-38, innerLoop.h:32-50) plus the native plan API.  Device
buffers are passed as raw pointers (e.g. ``torch.Tensor.data_ptr()``); streams
as ``torch.cuda.Stream.cuda_stream`` integers (0 = default stream).

The CUDA library is required: every entry raises if libgsfft.so is missing.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(HERE)
LIB_PATH = os.path.join(PKG, "build", "libgsfft.so")
HEADER = os.path.join(os.path.dirname(PKG), "include", "gsfft.h")

FP64, MIXED = 0, 1
FLAG_QUIRK_RESIDUE = 1
FLAG_RAW_SELECTION = 2
FLAG_FORCE_GATHER = 4
FLAG_FORCE_STREAM = 8
FLAG_TC_BUCKET_FFT = 16
FLAG_TC_RLFC_FFT = 32
FLAG_CC_BUCKET_FFT = 64
SELECTION_FLOOR = 1e-10
OK, ERR_PARAM, ERR_CAPACITY, ERR_ALLOC, ERR_CUDA, ERR_UNSUPPORTED, ERR_STATE, ERR_TIMEOUT = range(8)

NODE = np.dtype({"names": ["key", "x", "y"], "formats": ["<u4", "<f8", "<f8"],
                 "offsets": [0, 8, 16], "itemsize": 24})


class GsfftError(RuntimeError):
    def __init__(self, status, what=""):
        self.status = status
        super().__init__(f"{what}: status {status} ({status_string(status)}) {last_error()}")


class Params(C.Structure):
    _fields_ = [(f, C.c_int) for f in (
        "q", "n", "k", "B", "B_thresh", "W_RLFC", "RLFC_loops", "loops_loc",
        "loops_thresh", "loops_est", "loops", "b_f", "w")] + [
        (f, C.c_double) for f in ("Bcst", "RLFC_cst", "BB", "lobefrac", "tolerance", "t0")]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class Tuning(C.Structure):
    """gsfft_plan_tuning: stage shapes of a plan (0 = the plan's rule)."""
    _fields_ = [(f, C.c_int) for f in ("perm_filter_form", "row_groups", "bucket_first_radix",
                                      "rlfc_first_radix", "select_form")]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


_lib = None


def build():
    import importlib.util
    spec = importlib.util.spec_from_file_location("gsfft_build_lib", os.path.join(PKG, "build_lib.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m.build()


def lib():
    """Loads libgsfft.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"libgsfft.so not built ({LIB_PATH}); run gpu-sfft_gb300/build_lib.py")
    L = C.CDLL(LIB_PATH)
    P, i, d, u = C.c_void_p, C.c_int, C.c_double, C.c_uint
    ll = C.c_longlong
    sig = {
        "gsfft_version": ([], C.c_char_p),
        "gsfft_last_error": ([], C.c_char_p),
        "gsfft_status_string": ([i], C.c_char_p),
        "gsfft_derive_params": ([i, i, d, i, i, i, d, i, d, C.POINTER(Params)], i),
        "gsfft_design_filter": ([C.POINTER(Params), P, P, P], i),
        "gsfft_plan_create": ([C.POINTER(Params), i, u, i, C.POINTER(P)], i),
        "gsfft_plan_create_tuned": ([C.POINTER(Params), i, u, i, C.POINTER(Tuning), C.POINTER(P)], i),
        "gsfft_plan_get_tuning": ([P, C.POINTER(Tuning)], i),
        "gsfft_autotune_plan": ([C.POINTER(Params), i, u, P, P, P, P, P, P, i, C.c_char_p,
                                 C.POINTER(Tuning), C.POINTER(C.c_float), P], i),
        "gsfft_plan_destroy": ([P], i),
        "gsfft_plan_set_filter": ([P, P, P, P], i),
        "gsfft_run": ([P, P, P, P, P, P], i),
        "gsfft_get_results": ([P, P, i, C.POINTER(i), P, i, C.POINTER(i), P], i),
        "gsfft_device_results": ([P, P, P, P, P], i),
        "gsfft_debug_stages": ([P, P, C.POINTER(i), P, P, P], i),
        "gsfft_plan_launches_per_run": ([P], i),
        "gsfft_plan_describe": ([P, C.POINTER(i), C.POINTER(i)], i),
        "gsfft_plan_tensor_core_ffts": ([P, C.POINTER(i), C.POINTER(i)], i),
        "gsfft_batch_create": ([C.POINTER(P), i, i, C.POINTER(P)], i),
        "gsfft_batch_destroy": ([P], i),
        "gsfft_run_batched": ([P, C.POINTER(P), P, P, P, P], i),
        "gsfft_batch_capture": ([P, C.POINTER(P), P, P, P], i),
        "gsfft_batch_launch": ([P, P], i),
        "gsfft_batch_set_persistent_tail": ([P, i], i),
        "gsfft_tc_dft64": ([P, P, i, P], i),
        "gsfft_alloc": ([C.POINTER(P), C.c_size_t], i),
        "gsfft_free": ([P], i),
        "gsfft_copy": ([P, P, C.c_size_t, P], i),
        "gsfft_sync": ([P], i),
        "gsfft_ingest": ([P, ll, i, P, P], i),
        "gsfft_convert_signal": ([P, P, ll, P], i),
        "gsfft_evaluate": ([P, P, P, i, C.POINTER(i), C.POINTER(i), C.POINTER(d), P], i),
        "gsfft_plan_enable_timing": ([P, i], i),
        "gsfft_plan_stage_times": ([P, C.POINTER(C.c_float), i, C.POINTER(i)], i),
        "gsfft_stage_name": ([i], C.c_char_p),
        "gsfft_fft": ([P, P, ll, i, i, i, P], i),
        "gsfft_fft_tc": ([P, P, ll, i, i, P], i),
        "gsfft_fft_tc64": ([P, P, ll, i, i, P], i),
        "gsfft_check_bounded_wait": ([ll, P], i),
        "gsfft_cutoff": ([P, i, i, i, i, P, P], i),
        "gsfft_cutoff_noalloc": ([P, i, i, i, i, P, P], i),
        "gsfft_cutoff_floor": ([P, i, i, i, i, d, P, P, P], i),
        "gsfft_stage_perm_filter": ([i, P, i, P, i, i, i, P, i, P, P], i),
        "gsfft_stage_perm_filter_stream": ([i, P, i, P, i, i, i, P, P, P], i),
        "gsfft_stage_reverse_hash": ([P, i, P, i, i, i, i, i, i, i, u, P, P, i,
                                      C.POINTER(i), P], i),
        "gsfft_stage_estimate": ([i, P, i, P, i, i, i, P, P, P, P], i),
        "outer_loop": ([P, i, P, P, i, i, i, i, i, i, i, i, C.POINTER(i), C.c_float], P),
        "restr_loc_freq_coeff": ([P, i, i, i, P, P], i),
        "samples_indices": ([P, i, i, P, P], i),
        "perm_filter_cutoff": ([P, i, P, i, i, i, i, i, P, P, P, P], i),
        "reverse_hash": ([P, i, i, i, i, i, i, P, P, C.POINTER(i), P, P, i, i, i], i),
        "estimate_values": ([P, C.POINTER(i), P, i, i, P, i, P, i], P),
        "timesmod": ([i, i, i], i),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    _lib = L
    return L


def version():
    return lib().gsfft_version().decode()


def last_error():
    return lib().gsfft_last_error().decode(errors="replace")


def status_string(s):
    return lib().gsfft_status_string(s).decode()


def check(status, what):
    if status != OK:
        raise GsfftError(status, what)


def exported_header_symbols():
    """Function names declared in include/gsfft.h."""
    import re
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    names = re.findall(r"^[A-Za-z_][\w \*]*?\b(\w+)\s*\(", txt, flags=re.M)
    return sorted(set(n for n in names if n not in ("if", "defined")))


def derive_params(q, k, Bcst, loops_loc, loops_thresh, loops_est, RLFC_cst, RLFC_loops,
                  tolerance=1e-8):
    p = Params()
    s = lib().gsfft_derive_params(q, k, Bcst, loops_loc, loops_thresh, loops_est, float(RLFC_cst),
                                  RLFC_loops, tolerance, C.byref(p))
    return p, s


def _np_ptr(a):
    return a.ctypes.data_as(C.c_void_p)


def design_filter(p, d_filter_time, d_filter_freq=0, stream=0):
    check(lib().gsfft_design_filter(C.byref(p), d_filter_time, d_filter_freq or None, stream or None),
          "gsfft_design_filter")


def fft(d_in, d_out, n, batch=1, sign=-1, precision=FP64, stream=0):
    check(lib().gsfft_fft(d_in, d_out, n, batch, sign, precision, stream or None), "gsfft_fft")


def fft_tc(d_in, d_out, n, batch=1, sign=-1, stream=0):
    """FP32 FFT with the tensor-core radix-4096 first pass (n = 2^17 .. 2^26)."""
    check(lib().gsfft_fft_tc(d_in, d_out, n, batch, sign, stream or None), "gsfft_fft_tc")


def fft_tc64(d_in, d_out, n, batch=1, sign=-1, stream=0):
    """FP32 FFT with the tensor-core radix-64 last pass (n = 2^13 .. 2^20)."""
    check(lib().gsfft_fft_tc64(d_in, d_out, n, batch, sign, stream or None), "gsfft_fft_tc64")


def cutoff(d_samples, size, num, batch, precision, d_out, stream=0):
    check(lib().gsfft_cutoff(d_samples, size, num, batch, precision, d_out, stream or None),
          "gsfft_cutoff")


MAX_LOOPS = 32        # GSFFT_MAX_LOOPS
MAX_RLFC_LOOPS = 8    # GSFFT_MAX_RLFC_LOOPS


class Batch:
    """gsfft_batch over existing Plan objects (kept alive by the batch)."""

    def __init__(self, plans, streams=8):
        self.plans = list(plans)
        arr = (C.c_void_p * len(self.plans))(*[pl.h for pl in self.plans])
        h = C.c_void_p()
        check(lib().gsfft_batch_create(arr, len(self.plans), streams, C.byref(h)), "gsfft_batch_create")
        self.h = h

    def _pack(self, d_xs, draws):
        n = len(self.plans)
        offs = np.zeros((n, MAX_RLFC_LOOPS), np.int32)
        a = np.zeros((n, MAX_LOOPS), np.int32)
        ai = np.zeros((n, MAX_LOOPS), np.int32)
        for i, (o, aa, ii) in enumerate(draws):
            offs[i, :len(o)] = o
            a[i, :len(aa)] = aa
            ai[i, :len(ii)] = ii
        xs = (C.c_void_p * n)(*[int(v) for v in d_xs])
        return xs, offs, a, ai

    def run(self, d_xs, draws, stream=0):
        """d_xs: device pointers, draws: per plan (offsets, a, ai)."""
        xs, offs, a, ai = self._pack(d_xs, draws)
        check(lib().gsfft_run_batched(self.h, xs, _np_ptr(offs), _np_ptr(a), _np_ptr(ai),
                                      stream or None), "gsfft_run_batched")

    def capture(self, d_xs, draws):
        """Record one batched run into a CUDA graph (replayed by launch())."""
        xs, offs, a, ai = self._pack(d_xs, draws)
        check(lib().gsfft_batch_capture(self.h, xs, _np_ptr(offs), _np_ptr(a), _np_ptr(ai)),
              "gsfft_batch_capture")

    def launch(self, stream=0):
        check(lib().gsfft_batch_launch(self.h, stream or None), "gsfft_batch_launch")

    def persistent_tail(self, on=True):
        """Voting of every plan in one persistent launch
        (gsfft_batch_set_persistent_tail); drops a captured graph."""
        check(lib().gsfft_batch_set_persistent_tail(self.h, int(on)),
              "gsfft_batch_set_persistent_tail")

    def close(self):
        if self.h:
            lib().gsfft_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def tc_dft64(d_in, d_out, nvec, stream=0):
    """nvec forward 64-point DFTs of complex64 vectors on the tensor cores."""
    check(lib().gsfft_tc_dft64(d_in, d_out, nvec, stream or None), "gsfft_tc_dft64")


def ingest(h_x, precision, d_x, stream=0):
    """Host complex128 signal -> device (complex128 for FP64, complex64 for MIXED)."""
    h_x = np.ascontiguousarray(h_x, dtype=np.complex128)
    check(lib().gsfft_ingest(_np_ptr(h_x), h_x.size, precision, d_x, stream or None), "gsfft_ingest")
    check(lib().gsfft_sync(stream or None), "gsfft_sync")


def convert_signal(d_in, d_out, n, stream=0):
    check(lib().gsfft_convert_signal(d_in, d_out, n, stream or None), "gsfft_convert_signal")


def cutoff_floor(d_samples, size, num, batch, precision, floor_rel, d_out, d_row_max=0,
                 stream=0):
    """gsfft_cutoff with the engine's selection floor (row maxima computed on
    the device when d_row_max is 0)."""
    check(lib().gsfft_cutoff_floor(d_samples, size, num, batch, precision, float(floor_rel),
                                   d_row_max or None, d_out, stream or None), "gsfft_cutoff_floor")


# limits of cutoff_noalloc (GSFFT_NOALLOC_MAX_SIZE / _BATCH in gsfft.h)
NOALLOC_MAX_SIZE = 1 << 24
NOALLOC_MAX_BATCH = 8


def cutoff_noalloc(d_samples, size, num, batch, precision, d_out, stream=0):
    """gsfft_cutoff without device allocation (fixed library scratch); queued
    on ``stream``, returns without waiting."""
    check(lib().gsfft_cutoff_noalloc(d_samples, size, num, batch, precision, d_out,
                                     stream or None), "gsfft_cutoff_noalloc")


def stage_perm_filter(precision, d_x, n, d_filter_time, w, B, ai, d_bins, quirk_residue=False,
                      stream=0):
    ai = np.ascontiguousarray(ai, np.int32)
    check(lib().gsfft_stage_perm_filter(precision, d_x, n, d_filter_time, w, B, ai.size,
                                        _np_ptr(ai), int(quirk_residue), d_bins, stream or None),
          "gsfft_stage_perm_filter")


def stage_perm_filter_stream(precision, d_x, n, d_filter_time, w, B, a, d_bins, stream=0):
    a = np.ascontiguousarray(a, np.int32)
    check(lib().gsfft_stage_perm_filter_stream(precision, d_x, n, d_filter_time, w, B, a.size,
                                               _np_ptr(a), d_bins, stream or None),
          "gsfft_stage_perm_filter_stream")


def stage_reverse_hash(d_J, B_thresh, d_J2, num_RLFC, n, B, W, a, ai, loops_thresh, epoch,
                       d_vote, d_cand, cap, count, stream=0):
    c = C.c_int(count)
    s = lib().gsfft_stage_reverse_hash(d_J, B_thresh, d_J2, num_RLFC, n, B, W, a, ai, loops_thresh,
                                       epoch, d_vote, d_cand, cap, C.byref(c), stream or None)
    return s, c.value


def stage_estimate(precision, d_cand, num, d_bins, loops, n, B, ai, d_filter_freq, d_out,
                   stream=0):
    ai = np.ascontiguousarray(ai, np.int32)
    check(lib().gsfft_stage_estimate(precision, d_cand, num, d_bins, loops, n, B, _np_ptr(ai),
                                     d_filter_freq, d_out, stream or None), "gsfft_stage_estimate")


def autotune_plan(params, precision, flags, d_x, d_filter_time, d_filter_freq, offsets, a, ai,
                  reps=5, cache_path=None, stream=0):
    """gsfft_autotune_plan: the fastest stage shapes for plans of these
    parameters, timed on this signal, filter and draws.  Returns (Tuning, ms)."""
    o, aa, ii = [np.ascontiguousarray(v, np.int32) for v in (offsets, a, ai)]
    t, ms = Tuning(), C.c_float(0.0)
    check(lib().gsfft_autotune_plan(C.byref(params), precision, flags, d_x, d_filter_time,
                                    d_filter_freq, _np_ptr(o), _np_ptr(aa), _np_ptr(ii), reps,
                                    cache_path.encode() if cache_path else None, C.byref(t),
                                    C.byref(ms), stream or None), "gsfft_autotune_plan")
    return t, ms.value


class Plan:
    """One reusable sparse-FFT plan (all device buffers allocated here)."""

    def __init__(self, params, precision=FP64, flags=0, max_candidates=0, tuning=None):
        self.params = params
        self.precision = precision
        h = C.c_void_p()
        check(lib().gsfft_plan_create_tuned(C.byref(params), precision, flags, max_candidates,
                                            C.byref(tuning) if tuning is not None else None,
                                            C.byref(h)), "gsfft_plan_create_tuned")
        self.h = h

    def tuning(self):
        t = Tuning()
        check(lib().gsfft_plan_get_tuning(self.h, C.byref(t)), "gsfft_plan_get_tuning")
        return t

    def close(self):
        if self.h:
            lib().gsfft_plan_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_filter(self, d_filter_time, d_filter_freq, stream=0):
        check(lib().gsfft_plan_set_filter(self.h, d_filter_time, d_filter_freq, stream or None),
              "gsfft_plan_set_filter")

    def run(self, d_x, offsets, a, ai, stream=0):
        self._draws = [np.ascontiguousarray(v, np.int32) for v in (offsets, a, ai)]
        o, aa, ii = self._draws
        check(lib().gsfft_run(self.h, d_x, _np_ptr(o), _np_ptr(aa), _np_ptr(ii), stream or None),
              "gsfft_run")

    def results(self, stream=0, cap=None):
        I_F = C.c_int(0)
        ntop = C.c_int(0)
        s = lib().gsfft_get_results(self.h, None, 0, C.byref(I_F), None, 0, C.byref(ntop),
                                    stream or None)
        if s not in (OK, ERR_CAPACITY):
            check(s, "gsfft_get_results")
        m = I_F.value if cap is None else min(cap, I_F.value)
        nodes = np.zeros(max(m, 1), NODE)
        top = np.zeros(max(ntop.value, 1), NODE)
        s = lib().gsfft_get_results(self.h, _np_ptr(nodes), m, C.byref(I_F), _np_ptr(top),
                                    ntop.value, C.byref(ntop), stream or None)
        return {"status": s, "I_F": I_F.value, "nodes": nodes[:min(m, I_F.value)],
                "topk": top[:ntop.value]}

    def debug_stages(self, stream=0):
        p = self.params
        J2 = np.zeros(p.RLFC_loops * p.B_thresh, np.int32)
        J = np.zeros(p.loops_loc * p.B_thresh, np.int32)
        bins = np.zeros(p.loops * p.B, np.complex128 if self.precision == FP64 else np.complex64)
        nr = C.c_int(0)
        check(lib().gsfft_debug_stages(self.h, _np_ptr(J2), C.byref(nr), _np_ptr(J),
                                       _np_ptr(bins), stream or None), "gsfft_debug_stages")
        return {"J2": J2[:nr.value], "J": J.reshape(p.loops_loc, p.B_thresh),
                "bins": bins.reshape(p.loops, p.B)}

    def enable_timing(self, on=True):
        check(lib().gsfft_plan_enable_timing(self.h, int(on)), "gsfft_plan_enable_timing")

    def stage_times(self):
        """{stage name: average ms} over the runs since the last call."""
        ms = (C.c_float * 16)()
        runs = C.c_int(0)
        check(lib().gsfft_plan_stage_times(self.h, ms, 16, C.byref(runs)), "gsfft_plan_stage_times")
        out = {}
        for i in range(16):
            name = lib().gsfft_stage_name(i).decode()
            if not name:
                break
            out[name] = ms[i]
        return out, runs.value

    def launches_per_run(self):
        return lib().gsfft_plan_launches_per_run(self.h)

    def evaluate(self, d_x_f, d_true_loc, k_true, stream=0):
        """Device-side MISSED (estimation, result) and MSE*k of the last run
        (d_true_loc: ascending distinct locations)."""
        me, mr, e = C.c_int(0), C.c_int(0), C.c_double(0.0)
        check(lib().gsfft_evaluate(self.h, d_x_f, d_true_loc, k_true, C.byref(me), C.byref(mr),
                                   C.byref(e), stream or None), "gsfft_evaluate")
        return {"missed_estimation": me.value, "missed_result": mr.value, "mse_k": e.value}

    def describe(self):
        """{'streaming': bool, 'row_groups': int} -- the perm+filter form chosen."""
        st, g = C.c_int(0), C.c_int(0)
        check(lib().gsfft_plan_describe(self.h, C.byref(st), C.byref(g)), "gsfft_plan_describe")
        return {"streaming": bool(st.value), "row_groups": g.value}

    def tensor_core_ffts(self):
        """{'bucket': bool, 'rlfc': bool} -- which FFTs have a tensor-core pass."""
        b, r = C.c_int(0), C.c_int(0)
        check(lib().gsfft_plan_tensor_core_ffts(self.h, C.byref(b), C.byref(r)),
              "gsfft_plan_tensor_core_ffts")
        return {"bucket": bool(b.value), "rlfc": bool(r.value)}
