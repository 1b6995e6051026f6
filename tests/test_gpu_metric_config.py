"""GPU against the oracle at the metric's own configuration, and the cutoff's
floored forms directly.

n = 2^27, k = 16000, Bcst 0.65, loops 2/2/7, RLFC 4096 x 2, tolerance 1e-8
(noiseless and 40 dB): the RLFC rows are 2^22 samples long, so the RLFC cutoff
takes the cooperative select form with the selection floor.  With identical
draws the FP64 path must give the oracle's J2, its candidate list (canonical
order), its top-k list and its values within 1e-9; the mixed path the same
top-k set with values within 1e-5 relative L2 (and, noiseless, the same
candidates).
"""
import numpy as np
import pytest

from gsfft import synth

pytestmark = pytest.mark.gpu

CFG = (27, 16000, 0.65, 2, 2, 7, 4096, 2)


@pytest.fixture(scope="module")
def metric_setup(G, O, torch_cuda):
    torch = torch_cuda
    p_g, st = G.derive_params(*CFG)
    assert st == 0
    p_o, st = O.derive_params(*CFG)
    assert st == 0
    # the filter designed on the GPU (checked against the oracle's design and
    # the reference's elsewhere) is the common input of both sides
    d_ft = torch.zeros(p_g.w, dtype=torch.complex128, device="cuda")
    d_ff = torch.zeros(p_g.n, dtype=torch.complex128, device="cuda")
    G.design_filter(p_g, d_ft.data_ptr(), d_ff.data_ptr())
    return {"p_g": p_g, "p_o": p_o, "d_ft": d_ft, "d_ff": d_ff,
            "ft": d_ft.cpu().numpy(), "ff": d_ff.cpu().numpy()}


def _run(G, torch, s, d_x, draws, prec):
    plan = G.Plan(s["p_g"], prec)
    plan.set_filter(s["d_ft"].data_ptr(), s["d_ff"].data_ptr())
    plan.run(d_x.data_ptr(), *draws)
    res = plan.results()
    res["stages"] = plan.debug_stages()
    plan.close()
    assert res["status"] == 0
    return res


@pytest.mark.parametrize("snr", [None, 40.0])
def test_metric_config_matches_oracle(G, O, torch_cuda, metric_setup, snr):
    torch = torch_cuda
    s = metric_setup
    p = s["p_o"]
    x64, loc, coef, X = synth.signal_torch(p.n, p.k, seed=11, snr_db=snr)
    del X
    draws = synth.draws(11, p.n, p.W_RLFC, p.RLFC_loops, p.loops)
    g64 = _run(G, torch, s, x64, draws, G.FP64)
    g32 = _run(G, torch, s, x64.to(torch.complex64), draws, G.MIXED)
    x = x64.cpu().numpy()
    del x64
    o = O.outer_loop(x, p, s["ft"], s["ff"], *draws, want_stages=True)
    assert o["status"] == 0
    # RLFC: same merged residue set (cooperative select with the floor)
    np.testing.assert_array_equal(g64["stages"]["J2"], O.merge_j2(list(o["J2_blocks"])))
    # location loops: same bucket ids
    np.testing.assert_array_equal(g64["stages"]["J"], o["J"])
    # candidates: the same list in the same canonical order
    np.testing.assert_array_equal(g64["nodes"]["key"], o["nodes"]["key"])
    vo = o["nodes"]["x"] + 1j * o["nodes"]["y"]
    vg = g64["nodes"]["x"] + 1j * g64["nodes"]["y"]
    assert np.abs(vg - vo).max() <= 1e-9 * np.abs(vo).max()
    # top-k: the same keys in the same order, values within 1e-9 relative
    top_o = O.topk(o["nodes"], p.k)
    np.testing.assert_array_equal(g64["topk"]["key"], top_o["key"])
    to = top_o["x"] + 1j * top_o["y"]
    tg = g64["topk"]["x"] + 1j * g64["topk"]["y"]
    assert (np.abs(tg - to) <= 1e-9 * np.abs(to)).all()
    # mixed: the same top-k set, values within 1e-5 relative L2.  Noiseless,
    # the floor settles every pick, so the candidate list is the same too;
    # with noise, buckets at the threshold differ by less than FP32 rounding
    # and a few candidates may differ.
    if snr is None:
        np.testing.assert_array_equal(g32["nodes"]["key"], o["nodes"]["key"])
    assert set(g32["topk"]["key"].tolist()) == set(top_o["key"].tolist())
    v32 = dict(zip(g32["topk"]["key"].tolist(), g32["topk"]["x"] + 1j * g32["topk"]["y"]))
    a32 = np.array([v32[kk] for kk in top_o["key"].tolist()])
    assert np.linalg.norm(a32 - to) <= 1e-5 * np.linalg.norm(to)


def _rows(rng, batch, size, prec, zero_frac):
    """Rows like |FFT|^2 of a noiseless signal: exact zeros, rounding-level
    samples (1e-22 relative) and significant samples (order 1)."""
    u = rng.random((batch, size))
    s = np.where(u < zero_frac, 0.0,
                 np.where(u < zero_frac + 0.3, 1e-22 * rng.random((batch, size)),
                          rng.random((batch, size)) ** 4 + 1e-6))
    return s.astype(np.float64 if prec == 0 else np.float32)


@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("size,batch", [(1 << 22, 2), (1 << 18, 3), (1 << 14, 9)])
@pytest.mark.parametrize("where", ["floored", "significant"])
def test_cutoff_floor_forms(G, O, torch_cuda, prec, size, batch, where):
    """Cooperative (rows > 2^18), cluster (<= 2^18, up to 8 rows) and
    multi-launch (more rows) select forms with the selection floor, the
    threshold either among the floored samples (ties resolved by index) or
    among the significant ones."""
    torch = torch_cuda
    rng = np.random.default_rng(size + batch + prec)
    s = _rows(rng, batch, size, prec, 0.4)
    sig = int((s > 1e-10 * s.max(axis=1, keepdims=True)).sum(axis=1).min())
    num = sig + size // 10 if where == "floored" else sig // 2
    d_s = torch.from_numpy(s).cuda()
    d_o = torch.full((batch, num), -1, dtype=torch.int32, device="cuda")
    G.cutoff_floor(d_s.data_ptr(), size, num, batch, prec, G.SELECTION_FLOOR, d_o.data_ptr())
    got = d_o.cpu().numpy()
    for r in range(batch):
        np.testing.assert_array_equal(got[r], O.cutoff(s[r], num, floor_rel=G.SELECTION_FLOOR))
