"""End-to-end parity of the GPU engine (through the C ABI) with the oracle."""
import ctypes as C

import numpy as np
import pytest

from gsfft import synth

pytestmark = pytest.mark.gpu

CFGS = {  # (q, k, Bcst, loops_loc, loops_thresh, loops_est, RLFC_cst, RLFC_loops)
    "n14": (14, 10, 2.5, 2, 2, 5, 16, 2),
    "n16": (16, 20, 1.0, 2, 2, 5, 8, 2),
    "n18_3loc": (18, 100, 1.0, 3, 2, 6, 32, 2),
    # three location loops, all three needed: vote counts reach 3 (the packed
    # tables' 2-bit maximum)
    "n18_3thr": (18, 100, 1.0, 3, 3, 6, 32, 2),
    "config1": (20, 1000, 1.40, 2, 2, 5, 128, 2),
}


def dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def recovered(top, loc):
    """True locations present in a top-k list."""
    return set(top["key"].tolist()) & set(int(v) for v in loc)


def assert_same_run(g, o, k, tol=1e-9):
    """GPU and oracle runs with identical draws: the same candidate list in
    the same canonical order, the same top-k list, values within tol.  With
    the selection floor (the default) bins that are zero in exact arithmetic
    tie and resolve by index on both sides, so no pick depends on rounding."""
    np.testing.assert_array_equal(g["nodes"]["key"], o["nodes"]["key"])
    vo = o["nodes"]["x"] + 1j * o["nodes"]["y"]
    vg = g["nodes"]["x"] + 1j * g["nodes"]["y"]
    assert np.abs(vg - vo).max() <= tol * np.abs(vo).max()
    top_o = O_topk(o["nodes"], k)
    np.testing.assert_array_equal(g["topk"]["key"], top_o["key"])


def O_topk(nodes, k):
    from oracle import oracle as O
    return O.topk(nodes, k)


def setup(G, O, torch, cfg, seed=0, snr_db=None):
    p_o, st = O.derive_params(*cfg)
    assert st == 0
    p_g, st = G.derive_params(*cfg)
    assert st == 0
    assert p_g.as_dict() == p_o.as_dict()
    x, loc, coef, X = synth.signal_numpy(p_o.n, p_o.k, seed=seed, snr_db=snr_db)
    ft, ff = O.design_filter(p_o)
    draws = synth.draws(seed, p_o.n, p_o.W_RLFC, p_o.RLFC_loops, p_o.loops)
    return p_o, p_g, x, loc, X, ft, ff, draws


def run_gpu(G, torch, p_g, x, ft, ff, draws, prec=0, flags=0):
    plan = G.Plan(p_g, prec, flags)
    d_ft, d_ff = dev(torch, ft), dev(torch, ff)
    plan.set_filter(d_ft.data_ptr(), d_ff.data_ptr())
    d_x = dev(torch, x.astype(np.complex128 if prec == 0 else np.complex64))
    plan.run(d_x.data_ptr(), *draws)
    res = plan.results()
    res["stages"] = plan.debug_stages()
    res["launches"] = plan.launches_per_run()
    plan.close()
    return res


@pytest.mark.parametrize("name", list(CFGS))
def test_fp64_pipeline_vs_oracle(G, O, torch_cuda, name):
    torch = torch_cuda
    cfg = CFGS[name]
    p, p_g, x, loc, X, ft, ff, (offs, a, ai) = setup(G, O, torch, cfg)
    g = run_gpu(G, torch, p_g, x, ft, ff, (offs, a, ai))
    assert g["status"] == 0
    o = O.outer_loop(x, p, ft, ff, offs, a, ai, want_stages=True)
    st = g["stages"]
    # J2 and J: the same ids (the floor settles the rounding-level picks)
    np.testing.assert_array_equal(st["J2"], O.merge_j2(list(o["J2_blocks"])))
    np.testing.assert_array_equal(st["J"], o["J"])
    # bucket spectra: FP64 FFT parity
    bins_o = o["bins_f"]
    assert np.abs(st["bins"] - bins_o).max() <= 1e-11 * np.abs(bins_o).max()
    # stage injection: the oracle's cutoff on the GPU's bins gives the GPU's J
    for l in range(p.loops_loc):
        np.testing.assert_array_equal(
            st["J"][l], O.cutoff(O.samples(st["bins"][l]), p.B_thresh, floor_rel=G.SELECTION_FLOOR))
    # stage injection: the oracle's vote on the GPU's J and J2 gives the GPU's
    # candidates in the same (canonical) order
    vote = np.zeros(p.n, np.int32)
    cand = []
    for l in range(p.loops_loc):
        c, vote, s = O.reverse_hash(st["J"][l], st["J2"], p.n, p.B, p.W_RLFC, int(a[l]), int(ai[l]),
                                    p.loops_thresh, vote=vote, cand=cand)
        cand = list(c)
    np.testing.assert_array_equal(g["nodes"]["key"], np.array(cand, np.uint32))
    est = O.estimate(np.array(cand, np.int32), st["bins"], p.loops, p.n, ai, p.B, ff)
    scale = max(1.0, np.abs(est["x"] + 1j * est["y"]).max())
    assert np.abs(g["nodes"]["x"] - est["x"]).max() <= 1e-12 * scale
    assert np.abs(g["nodes"]["y"] - est["y"]).max() <= 1e-12 * scale
    # end to end: the same candidates, top-k list and values (1e-9)
    assert_same_run(g, o, p.k)
    assert len(recovered(g["topk"], loc)) >= p.k - 3


def test_fp64_pipeline_noisy_exact(G, O, torch_cuda):
    """With 40 dB noise no RLFC pick sits at rounding level: the whole top-k
    list (keys and order) matches the oracle, values within 1e-9."""
    torch = torch_cuda
    p, p_g, x, loc, X, ft, ff, (offs, a, ai) = setup(G, O, torch, CFGS["config1"], seed=2,
                                                     snr_db=40.0)
    g = run_gpu(G, torch, p_g, x, ft, ff, (offs, a, ai))
    o = O.outer_loop(x, p, ft, ff, offs, a, ai)
    np.testing.assert_array_equal(g["nodes"]["key"], o["nodes"]["key"])
    top_o = O.topk(o["nodes"], p.k)
    np.testing.assert_array_equal(g["topk"]["key"], top_o["key"])
    vo = top_o["x"] + 1j * top_o["y"]
    vg = g["topk"]["x"] + 1j * g["topk"]["y"]
    assert np.abs(vg - vo).max() <= 1e-9 * np.abs(vo).max()


@pytest.mark.parametrize("name", ["n16", "config1"])
def test_fp64_residue_quirk(G, O, torch_cuda, name):
    """GSFFT_FLAG_QUIRK_RESIDUE reproduces permFilterTillKernel's tap indexing."""
    torch = torch_cuda
    p, p_g, x, loc, X, ft, ff, (offs, a, ai) = setup(G, O, torch, CFGS[name], seed=3)
    g = run_gpu(G, torch, p_g, x, ft, ff, (offs, a, ai), flags=G.FLAG_QUIRK_RESIDUE)
    o = O.outer_loop(x, p, ft, ff, offs, a, ai, quirks=O.QUIRK_RESIDUE, want_stages=True)
    assert np.abs(g["stages"]["bins"] - o["bins_f"]).max() <= 1e-11 * np.abs(o["bins_f"]).max()
    assert_same_run(g, o, p.k)


@pytest.mark.parametrize("prec", [0, 1])
def test_stream_and_gather_agree(G, O, torch_cuda, prec):
    """Both perm+filter forms (and both RLFC sub-sampling paths) give the same
    candidates; values agree to the precision's rounding."""
    torch = torch_cuda
    p, p_g, x, loc, X, ft, ff, draws = setup(G, O, torch, CFGS["config1"], seed=4)
    gs = run_gpu(G, torch, p_g, x, ft, ff, draws, prec=prec, flags=G.FLAG_FORCE_STREAM)
    gg = run_gpu(G, torch, p_g, x, ft, ff, draws, prec=prec, flags=G.FLAG_FORCE_GATHER)
    np.testing.assert_array_equal(gs["stages"]["J2"], gg["stages"]["J2"])
    np.testing.assert_array_equal(gs["nodes"]["key"], gg["nodes"]["key"])
    vs = gs["nodes"]["x"] + 1j * gs["nodes"]["y"]
    vg = gg["nodes"]["x"] + 1j * gg["nodes"]["y"]
    tol = 1e-12 if prec == 0 else 1e-5
    assert np.abs(vs - vg).max() <= tol * np.abs(vg).max()


@pytest.mark.parametrize("prec", [0, 1])
def test_deterministic_repeat(G, O, torch_cuda, prec):
    torch = torch_cuda
    p, p_g, x, loc, X, ft, ff, draws = setup(G, O, torch, CFGS["config1"], seed=5)
    plan = G.Plan(p_g, prec)
    d_ft, d_ff = dev(torch, ft), dev(torch, ff)
    d_x = dev(torch, x.astype(np.complex128 if prec == 0 else np.complex64))
    plan.set_filter(d_ft.data_ptr(), d_ff.data_ptr())
    outs = []
    for _ in range(3):
        plan.run(d_x.data_ptr(), *draws)
        outs.append(plan.results())
    for r in outs[1:]:
        assert r["nodes"].tobytes() == outs[0]["nodes"].tobytes()
        assert r["topk"].tobytes() == outs[0]["topk"].tobytes()
    plan.close()


@pytest.mark.parametrize("name,snr", [("n18_3loc", None), ("config1", None), ("config1", 40.0)])
def test_mixed_vs_fp64(G, O, torch_cuda, name, snr):
    """Mixed path: same recovered location set as FP64, value rel-L2 <= 1e-5."""
    torch = torch_cuda
    p, p_g, x, loc, X, ft, ff, draws = setup(G, O, torch, CFGS[name], seed=7, snr_db=snr)
    g64 = run_gpu(G, torch, p_g, x, ft, ff, draws, prec=0)
    g32 = run_gpu(G, torch, p_g, x, ft, ff, draws, prec=1)
    k64 = g64["topk"]["key"].tolist()
    # the selection floor makes rounding-level picks identical across precisions
    np.testing.assert_array_equal(g32["stages"]["J2"], g64["stages"]["J2"])
    np.testing.assert_array_equal(g32["nodes"]["key"], g64["nodes"]["key"])
    assert set(g32["topk"]["key"].tolist()) == set(k64)
    v64 = dict(zip(k64, g64["topk"]["x"] + 1j * g64["topk"]["y"]))
    common = [r for r in g32["topk"] if int(r["key"]) in v64]
    v32 = np.array([complex(r["x"], r["y"]) for r in common])
    ref = np.array([v64[int(r["key"])] for r in common])
    rel = np.linalg.norm(v32 - ref) / np.linalg.norm(ref)
    assert rel <= 1e-5, rel


def test_outer_loop_dropin(G, O, torch_cuda):
    """The reference-signature outer_loop (outerLoop.h:35-38) with glibc draws
    and the reference's raw cutoffs and residue tap index: on a 40 dB signal
    (no pick at rounding level) the oracle run the same way gives the same
    candidates and values."""
    torch = torch_cuda
    cfg = CFGS["config1"]
    p, p_g, x, loc, X, ft, ff, _ = setup(G, O, torch, cfg, seed=9, snr_db=40.0)
    offs, a, ai = O.draw_glibc(1234, p.n, p.W_RLFC, p.RLFC_loops, p.loops)
    O.lib().srand48(1234)
    O.lib().srandom(1234)
    d_x, d_ft, d_ff = dev(torch, x), dev(torch, ft), dev(torch, ff)
    I_F = C.c_int(0)
    ptr = G.lib().outer_loop(d_x.data_ptr(), p.n, d_ft.data_ptr(), d_ff.data_ptr(), p.w, p.B,
                             p.B_thresh, p.W_RLFC, p.RLFC_loops, p.loops_thresh, p.loops_loc,
                             p.loops, C.byref(I_F), C.c_float(0.0))
    assert ptr, G.last_error()
    nodes = np.ctypeslib.as_array((C.c_char * (24 * I_F.value)).from_address(ptr)).view(G.NODE).copy()
    C.CDLL(None).free(C.c_void_p(ptr))
    o = O.outer_loop(x, p, ft, ff, offs, a, ai, quirks=O.QUIRK_RESIDUE, floor_rel=0.0)
    assert I_F.value == o["I_F"]
    assert_same_run({"nodes": nodes, "topk": O.topk(nodes, p.k)}, o, p.k)


def test_filter_design_gpu(G, O, torch_cuda):
    torch = torch_cuda
    cfg = CFGS["n18_3loc"]
    p_o, _ = O.derive_params(*cfg)
    p_g, _ = G.derive_params(*cfg)
    ft_o, ff_o = O.design_filter(p_o)
    d_ft = torch.zeros(p_g.w, dtype=torch.complex128, device="cuda")
    d_ff = torch.zeros(p_g.n, dtype=torch.complex128, device="cuda")
    G.design_filter(p_g, d_ft.data_ptr(), d_ff.data_ptr())
    ft, ff = d_ft.cpu().numpy(), d_ff.cpu().numpy()
    assert np.abs(ff - ff_o).max() <= 1e-10
    assert np.abs(ft - ft_o).max() <= 1e-10 * np.abs(ft_o).max()


def test_plan_rejects_bad_draws(G, O, torch_cuda):
    torch = torch_cuda
    p, p_g, x, loc, X, ft, ff, (offs, a, ai) = setup(G, O, torch, CFGS["n16"])
    plan = G.Plan(p_g, 0)
    d_x, d_ft, d_ff = dev(torch, x), dev(torch, ft), dev(torch, ff)
    with pytest.raises(G.GsfftError):  # run before the filter is installed
        plan.run(d_x.data_ptr(), offs, a, ai)
    plan.set_filter(d_ft.data_ptr(), d_ff.data_ptr())
    bad = a.copy()
    bad[0] = 2  # even: not invertible mod 2^q
    with pytest.raises(G.GsfftError):
        plan.run(d_x.data_ptr(), offs, bad, ai)
    plan.close()


def test_candidate_capacity_overflow(G, O, torch_cuda):
    """A plan whose candidate capacity is far below the run's candidate count
    (MAXSIZE_HITS overflow, unchecked in innerLoop.cu:813): the run reports
    GSFFT_ERR_CAPACITY with the true count, returns exactly `cap` candidates
    -- the first `cap` of the full run, with the same values -- and writes
    nothing past them."""
    torch = torch_cuda
    p, p_g, x, loc, X, ft, ff, draws = setup(G, O, torch, CFGS["config1"], seed=6)
    full = run_gpu(G, torch, p_g, x, ft, ff, draws)
    assert full["status"] == 0
    total = full["I_F"]
    cap = total // 3
    plan = G.Plan(p_g, G.FP64, 0, max_candidates=cap)
    d_ft, d_ff = dev(torch, ft), dev(torch, ff)
    plan.set_filter(d_ft.data_ptr(), d_ff.data_ptr())
    d_x = dev(torch, x)
    plan.run(d_x.data_ptr(), *draws)
    h = np.zeros(total + 64, G.NODE)
    h["key"] = 0xFFFFFFFF
    h["x"] = np.nan
    I_F = C.c_int(0)
    st = G.lib().gsfft_get_results(plan.h, h.ctypes.data_as(C.c_void_p), h.size, C.byref(I_F),
                                   None, 0, None, None)
    plan.close()
    assert st == G.ERR_CAPACITY
    assert I_F.value == total
    assert (h["key"][cap:] == 0xFFFFFFFF).all() and np.isnan(h["x"][cap:]).all()
    np.testing.assert_array_equal(h["key"][:cap], full["nodes"]["key"][:cap])
    np.testing.assert_array_equal(h["x"][:cap], full["nodes"]["x"][:cap])
    np.testing.assert_array_equal(h["y"][:cap], full["nodes"]["y"][:cap])
