"""Plans with explicit stage shapes and the autotuner (through the C ABI).

Every shape must give the same sparse FFT: the same candidate list (the
selection floor settles rounding-level picks) and values within the
precision's rounding of the default plan's; shapes that a plan's sizes cannot
take are rejected with GSFFT_ERR_PARAM; the autotuner must return a shape the
plan accepts, reuse its cache, and its choice must give the same results."""
import os

import numpy as np
import pytest

from gsfft import synth

pytestmark = pytest.mark.gpu

# n = 2^22, B = 4096 (1024 signal rows), W_RLFC = 131072: every knob applies
CFG = (22, 500, 0.65, 2, 2, 5, 128, 2)
ONE_PASS_MAX = {0: 13, 1: 14}   # log2 of the largest one-pass FFT per precision
ROWS_PER_TILE = {0: 32, 1: 64}  # rows of the streaming pass's signal tiles


@pytest.fixture(scope="module")
def setup(G, torch_cuda):
    torch = torch_cuda
    p, st = G.derive_params(*CFG)
    assert st == 0
    x, loc, coef, X = synth.signal_numpy(p.n, p.k, seed=21)
    d_ft = torch.zeros(p.w, dtype=torch.complex128, device="cuda")
    d_ff = torch.zeros(p.n, dtype=torch.complex128, device="cuda")
    G.design_filter(p, d_ft.data_ptr(), d_ff.data_ptr())
    return {"p": p, "x64": torch.from_numpy(x).cuda(),
            "x32": torch.from_numpy(x.astype(np.complex64)).cuda(),
            "ft": d_ft, "ff": d_ff, "draws": synth.draws(21, p.n, p.W_RLFC, p.RLFC_loops, p.loops)}


def _run(G, s, prec, tuning=None):
    plan = G.Plan(s["p"], prec, 0, tuning=tuning)
    plan.set_filter(s["ft"].data_ptr(), s["ff"].data_ptr())
    x = s["x64"] if prec == G.FP64 else s["x32"]
    plan.run(x.data_ptr(), *s["draws"])
    r = plan.results()
    r["tuning"] = plan.tuning().as_dict()
    plan.close()
    assert r["status"] == 0
    return r


def _same(a, b, tol):
    np.testing.assert_array_equal(a["nodes"]["key"], b["nodes"]["key"])
    va = a["nodes"]["x"] + 1j * a["nodes"]["y"]
    vb = b["nodes"]["x"] + 1j * b["nodes"]["y"]
    assert np.abs(va - vb).max() <= tol * np.abs(vb).max()
    assert set(a["topk"]["key"].tolist()) == set(b["topk"]["key"].tolist())


def _applies(p, prec, shape):
    if "row_groups" in shape:
        g, nb = shape["row_groups"], p.n // p.B
        if g != 1 and nb // g < 4 * ROWS_PER_TILE[prec]:
            return False
    for key, size in (("bucket_first_radix", p.B), ("rlfc_first_radix", p.W_RLFC)):
        if key in shape:
            L, r, one = int(np.log2(size)), shape[key], ONE_PASS_MAX[prec]
            if L <= one or not (max(7, L - one) <= r <= min(one, L - 7)):
                return False
    return True


@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("shape", [
    dict(perm_filter_form=2),
    dict(perm_filter_form=1, row_groups=1),
    dict(perm_filter_form=1, row_groups=4),
    dict(perm_filter_form=1, row_groups=8),
    dict(bucket_first_radix=7),   # B = 2^12: one pass in both precisions
    dict(rlfc_first_radix=8),
    dict(rlfc_first_radix=10),
    dict(select_form=2),
])
def test_explicit_shapes_same_result(G, setup, prec, shape):
    p = setup["p"]
    t = G.Tuning(**shape)
    if not _applies(p, prec, shape):
        with pytest.raises(G.GsfftError) as e:
            G.Plan(p, prec, 0, tuning=t).close()
        assert e.value.status == G.ERR_PARAM
        return
    base = _run(G, setup, prec)
    got = _run(G, setup, prec, t)
    for k, v in shape.items():
        assert got["tuning"][k] == v, (k, got["tuning"])
    _same(got, base, 1e-12 if prec == 0 else 1e-5)


def test_bad_shapes_rejected(G, setup):
    p = setup["p"]
    for shape in (dict(row_groups=3, perm_filter_form=1), dict(rlfc_first_radix=3),
                  dict(select_form=7), dict(perm_filter_form=5)):
        with pytest.raises(G.GsfftError) as e:
            G.Plan(p, G.MIXED, 0, tuning=G.Tuning(**shape)).close()
        assert e.value.status == G.ERR_PARAM


@pytest.mark.parametrize("prec", [0, 1])
def test_autotune_plan_and_cache(G, setup, tmp_path, prec):
    s = setup
    cache = str(tmp_path / "tuning.txt")
    x = s["x64"] if prec == G.FP64 else s["x32"]
    t, ms = G.autotune_plan(s["p"], prec, 0, x.data_ptr(), s["ft"].data_ptr(), s["ff"].data_ptr(),
                            *s["draws"], reps=3, cache_path=cache)
    assert ms > 0 and os.path.exists(cache)
    lines = open(cache).read().splitlines()
    assert len(lines) == 1 and lines[0].startswith("gsfft-tune-v1 ")
    # a second call is answered from the cache (no new line, same shapes)
    t2, ms2 = G.autotune_plan(s["p"], prec, 0, x.data_ptr(), s["ft"].data_ptr(),
                              s["ff"].data_ptr(), *s["draws"], reps=3, cache_path=cache)
    assert t2.as_dict() == t.as_dict() and len(open(cache).read().splitlines()) == 1
    # the chosen shapes give the default plan's sparse FFT
    _same(_run(G, s, prec, t), _run(G, s, prec), 1e-12 if prec == 0 else 1e-5)
