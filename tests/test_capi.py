"""CPU-side checks of the C ABI: the library loads, exports every function
declared in include/gsfft.h, and its host-only entry points (parameter
derivation, version, status strings) behave.  No GPU calls."""
import ctypes as C

import pytest

from _cabi import check_binding


def test_exports_every_declared_symbol(G):
    declared = G.exported_header_symbols()
    assert "outer_loop" in declared and "gsfft_run" in declared
    L = G.lib()
    missing = [s for s in declared if not hasattr(L, s)]
    assert not missing, missing


def test_reference_dropin_symbols(G):
    # innerLoop.h:32-50 / outerLoop.h:35-38 names the reference's callers bind
    for s in ("outer_loop", "timesmod"):
        assert hasattr(G.lib(), s)


def test_version_and_status(G):
    assert G.version() == "0.1.0"
    assert G.status_string(0) == "ok"
    assert "capacity" in G.status_string(G.ERR_CAPACITY)


@pytest.mark.parametrize("args", [
    (27, 16000, 0.65, 2, 2, 7, 4096, 2),
    (20, 1000, 1.40, 2, 2, 5, 128, 2),
    (27, 43000, 0.8, 3, 2, 8, 32768, 2),
    (18, 100, 1.0, 3, 2, 6, 32, 2),
])
def test_derive_params_matches_oracle(G, O, args):
    pg, sg = G.derive_params(*args)
    po, so = O.derive_params(*args)
    assert sg == so == 0
    assert pg.as_dict() == po.as_dict()


def test_derive_params_rejects(G):
    _, s = G.derive_params(18, 4000, 1.0, 2, 2, 5, 128, 2)   # B_thresh >= B
    assert s == G.ERR_PARAM
    _, s = G.derive_params(20, 1000, 1.4, 1, 2, 5, 128, 2)   # loops_thresh > loops_loc
    assert s == G.ERR_PARAM
    _, s = G.derive_params(20, 1000, 1.4, 2, 2, 5, 0.001, 2)  # W_RLFC < 2 k
    assert s != 0


def test_timesmod(G):
    assert G.lib().timesmod(123456789, 987654321 % (1 << 30), 1 << 27) == \
        (123456789 * (987654321 % (1 << 30))) % (1 << 27)


def test_null_arguments_rejected(G):
    L = G.lib()
    assert L.gsfft_run(None, None, None, None, None, None) == G.ERR_PARAM
    assert L.gsfft_plan_destroy(None) == G.ERR_PARAM
    p = G.Params()
    assert L.gsfft_plan_create(C.byref(p), 0, 0, 0, None) == G.ERR_PARAM


def test_cutoff_arguments_rejected(G):
    """The cutoff's argument checks run before any device work, as the
    reference's asserts do (B_thresh < B: a cutoff keeps fewer than all)."""
    L = G.lib()
    fake = C.c_void_p(16)  # never dereferenced: every call below is rejected first
    assert L.gsfft_cutoff(fake, 100, 100, 1, G.FP64, fake, None) == G.ERR_PARAM  # num == size
    assert L.gsfft_cutoff(fake, 100, 101, 1, G.FP64, fake, None) == G.ERR_PARAM  # num > size
    assert L.gsfft_cutoff(fake, 100, 0, 1, G.FP64, fake, None) == G.ERR_PARAM    # num < 1
    assert L.gsfft_cutoff(fake, 0, 1, 1, G.FP64, fake, None) == G.ERR_PARAM      # empty row
    assert L.gsfft_cutoff(fake, 100, 10, 0, G.FP64, fake, None) == G.ERR_PARAM   # no rows
    assert L.gsfft_cutoff(None, 100, 10, 1, G.FP64, fake, None) == G.ERR_PARAM
    assert L.gsfft_cutoff(fake, 100, 10, 1, 7, fake, None) == G.ERR_PARAM         # no such precision


def test_binding_constants_match_header(G):
    """The Python binding's flags, status codes and limits are the header's."""
    import re
    text = open(G.HEADER).read()
    defines = {m.group(1): m.group(2) for m in
               re.finditer(r"#define (GSFFT_[A-Z0-9_]+) +(\(1 << \d+\)|\d+)u?", text)}

    def val(name):
        v = defines[name]
        m = re.fullmatch(r"\(1 << (\d+)\)", v)
        return 1 << int(m.group(1)) if m else int(v)

    for flag in ("QUIRK_RESIDUE", "RAW_SELECTION", "FORCE_GATHER", "FORCE_STREAM",
                 "TC_BUCKET_FFT", "TC_RLFC_FFT", "CC_BUCKET_FFT"):
        assert getattr(G, "FLAG_" + flag) == val("GSFFT_FLAG_" + flag), flag
    assert G.NOALLOC_MAX_SIZE == val("GSFFT_NOALLOC_MAX_SIZE")
    assert G.NOALLOC_MAX_BATCH == val("GSFFT_NOALLOC_MAX_BATCH")
    codes = dict(re.findall(r"\b(GSFFT_(?:OK|ERR_[A-Z]+)) = (\d+)", text))
    for name in ("OK", "ERR_PARAM", "ERR_CAPACITY", "ERR_ALLOC", "ERR_CUDA", "ERR_UNSUPPORTED",
                 "ERR_STATE", "ERR_TIMEOUT"):
        assert getattr(G, name) == int(codes["GSFFT_" + name]), name


def test_binding_signatures_match_header(G):
    """Every function of include/gsfft.h is bound in Python with the header's
    argument count and, per argument, the same width and signedness (or a
    pointer): an int passed where the header says long long would leave the
    upper half of the register undefined."""
    checked, unbound = check_binding(G.lib(), G.HEADER, handles=("gsfft_plan", "gsfft_batch"))
    assert checked == len(G.exported_header_symbols()) and not unbound, unbound


def test_noalloc_cutoff_arguments_and_limits(G):
    """The no-allocation cutoff checks its arguments like gsfft_cutoff and
    rejects requests beyond its fixed scratch with GSFFT_ERR_CAPACITY, all
    before any device work."""
    L = G.lib()
    fake = C.c_void_p(16)  # never dereferenced: every call below is rejected first
    nc = L.gsfft_cutoff_noalloc
    assert nc(fake, 100, 100, 1, G.FP64, fake, None) == G.ERR_PARAM   # num == size
    assert nc(fake, 100, 0, 1, G.FP64, fake, None) == G.ERR_PARAM     # num < 1
    assert nc(fake, 100, 10, 0, G.FP64, fake, None) == G.ERR_PARAM    # no rows
    assert nc(fake, 100, 10, 1, 7, fake, None) == G.ERR_PARAM         # no such precision
    assert nc(None, 100, 10, 1, G.FP64, fake, None) == G.ERR_PARAM
    assert nc(fake, 100, 10, 1, G.FP64, None, None) == G.ERR_PARAM
    assert nc(fake, G.NOALLOC_MAX_SIZE + 1, 10, 1, G.MIXED, fake, None) == G.ERR_CAPACITY
    assert b"exceed" in L.gsfft_last_error()
    assert nc(fake, 1000, 10, G.NOALLOC_MAX_BATCH + 1, G.FP64, fake, None) == G.ERR_CAPACITY


@pytest.mark.parametrize("field,value,status", [
    ("n", 3000, "ERR_PARAM"),            # not a power of two
    ("B", 3000, "ERR_PARAM"),
    ("B_thresh", 0, "ERR_PARAM"),
    ("B_thresh", 8192, "ERR_PARAM"),     # B_thresh >= B (the reference asserts B_thresh < B)
    ("loops_thresh", 3, "ERR_PARAM"),    # loops_thresh > loops_loc
    ("loops", 8, "ERR_PARAM"),           # loops != loops_loc + loops_est
    ("RLFC_loops", 0, "ERR_PARAM"),
    ("w", 0, "ERR_PARAM"),
    ("W_RLFC", 1 << 20, "ERR_UNSUPPORTED"),  # W_RLFC = n
    ("W_RLFC", 128, "ERR_PARAM"),            # B_thresh >= W_RLFC
])
def test_plan_create_rejects_params(G, field, value, status):
    """Plan parameters are checked before any allocation (n = 2^20 base case)."""
    p, st = G.derive_params(20, 1000, 1.40, 2, 2, 5, 128, 2)
    assert st == G.OK
    setattr(p, field, value)
    h = C.c_void_p()
    assert G.lib().gsfft_plan_create(C.byref(p), G.MIXED, 0, 0, C.byref(h)) == getattr(G, status)
    assert not h.value


def test_host_entry_points_reject_bad_arguments(G):
    """Argument checks of the batch, ingest, conversion, filter-design,
    evaluation and drop-in entry points, all before any device work."""
    L = G.lib()
    fake = C.c_void_p(16)  # never dereferenced: every call below is rejected first
    h = C.c_void_p()
    assert L.gsfft_batch_create(None, 1, 1, C.byref(h)) == G.ERR_PARAM
    plans = (C.c_void_p * 1)(None)
    assert L.gsfft_batch_create(plans, 0, 1, C.byref(h)) == G.ERR_PARAM
    assert L.gsfft_batch_create(plans, 1, 1, C.byref(h)) == G.ERR_PARAM  # a null plan
    assert L.gsfft_run_batched(None, None, None, None, None, None) == G.ERR_PARAM
    assert L.gsfft_ingest(None, 10, G.FP64, fake, None) == G.ERR_PARAM
    assert L.gsfft_ingest(fake, 0, G.FP64, fake, None) == G.ERR_PARAM
    assert L.gsfft_ingest(fake, 10, 7, fake, None) == G.ERR_PARAM
    assert L.gsfft_convert_signal(None, fake, 10, None) == G.ERR_PARAM
    assert L.gsfft_convert_signal(fake, fake, 0, None) == G.ERR_PARAM
    assert L.gsfft_design_filter(None, fake, fake, None) == G.ERR_PARAM
    i1, i2, d1 = C.c_int(), C.c_int(), C.c_double()
    assert L.gsfft_evaluate(None, fake, fake, 1, C.byref(i1), C.byref(i2), C.byref(d1),
                            None) == G.ERR_PARAM
    # the reference's outer_loop signature: NULL without an I_F pointer
    assert L.outer_loop(fake, 1 << 20, fake, fake, 123349, 8192, 2000, 16384, 2, 2, 2, 7,
                        None, 0.0) is None
