"""Tensor-core (tcgen05) 64-point DFT building block against numpy."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("nvec", [1, 64, 1000, 20000])
def test_tc_dft64_matches_numpy(G, torch_cuda, nvec):
    torch = torch_cuda
    rng = np.random.default_rng(nvec)
    x = (rng.normal(size=(nvec, 64)) + 1j * rng.normal(size=(nvec, 64))).astype(np.complex64)
    d_x = torch.from_numpy(x).cuda()
    d_y = torch.zeros_like(d_x)
    G.tc_dft64(d_x.data_ptr(), d_y.data_ptr(), nvec)
    torch.cuda.synchronize()
    got = d_y.cpu().numpy().astype(np.complex128)
    want = np.fft.fft(x.astype(np.complex128), axis=1)
    err = np.linalg.norm(got - want, axis=1) / np.linalg.norm(want, axis=1)
    # three-part bf16 split with fp32 accumulation: FP32-level accuracy
    assert err.max() < 2e-6, err.max()


def test_tc_bucket_fft_pipeline(G, O, torch_cuda):
    """Mixed engine with the tensor-core bucket FFT (B = 2^17: the plan's
    default for 2^17 <= B <= 2^20, and what GSFFT_FLAG_TC_BUCKET_FFT asks for)
    against the CUDA-core mixed engine (GSFFT_FLAG_CC_BUCKET_FFT) and the FP64
    engine, same draws."""
    from gsfft import synth
    torch = torch_cuda
    cfg = (24, 1600, 4.0, 2, 2, 5, 64, 2)
    p, st = G.derive_params(*cfg)
    assert st == 0 and p.B == 1 << 17
    x, loc, coef, X = synth.signal_numpy(p.n, p.k, seed=5)
    d_ft = torch.zeros(p.w, dtype=torch.complex128, device="cuda")
    d_ff = torch.zeros(p.n, dtype=torch.complex128, device="cuda")
    G.design_filter(p, d_ft.data_ptr(), d_ff.data_ptr())
    d64 = torch.from_numpy(x).cuda()
    d32 = d64.to(torch.complex64)
    draws = synth.draws(5, p.n, p.W_RLFC, p.RLFC_loops, p.loops)
    res = {}
    for name, prec, flags, xx in [("fp64", G.FP64, 0, d64), ("mixed", G.MIXED, G.FLAG_CC_BUCKET_FFT, d32),
                                  ("tc", G.MIXED, G.FLAG_TC_BUCKET_FFT, d32),
                                  ("default", G.MIXED, 0, d32)]:
        plan = G.Plan(p, prec, flags)
        tcf = plan.tensor_core_ffts()
        assert tcf["bucket"] == (name in ("tc", "default")) and not tcf["rlfc"]
        plan.set_filter(d_ft.data_ptr(), d_ff.data_ptr())
        plan.run(xx.data_ptr(), *draws)
        r = plan.results()
        assert r["status"] == 0
        r["bins"] = plan.debug_stages()["bins"]
        r["launches"] = plan.launches_per_run()
        plan.close()
        res[name] = r
    assert res["tc"]["launches"] == res["mixed"]["launches"]  # two bucket-FFT passes either way
    assert res["default"]["topk"].tobytes() == res["tc"]["topk"].tobytes()
    b_tc = res["tc"]["bins"].astype(np.complex128)
    b_cc = res["mixed"]["bins"].astype(np.complex128)
    assert np.linalg.norm(b_tc - b_cc) / np.linalg.norm(b_cc) < 1e-5
    k64 = res["fp64"]["topk"]["key"]
    ktc = res["tc"]["topk"]["key"]
    assert set(k64.tolist()) == set(ktc.tolist())
    v64 = dict(zip(k64.tolist(), res["fp64"]["topk"]["x"] + 1j * res["fp64"]["topk"]["y"]))
    vtc = dict(zip(ktc.tolist(), res["tc"]["topk"]["x"] + 1j * res["tc"]["topk"]["y"]))
    a = np.array([v64[kk] for kk in k64.tolist()])
    b = np.array([vtc[kk] for kk in k64.tolist()])
    assert np.linalg.norm(a - b) / np.linalg.norm(a) <= 1e-5


@pytest.mark.parametrize("n,batch,sign", [(1 << 17, 9, -1), (1 << 20, 2, -1), (1 << 22, 2, -1),
                                          (1 << 17, 1, 1), (1 << 17, 3, -1), (1 << 22, 5, -1),
                                          (1 << 20, 3, 1)])
def test_tc_fft_matches_numpy(G, torch_cuda, n, batch, sign):
    """The FP32 FFT whose radix-4096 first pass runs on the tensor cores (the
    bucket FFT's B = 2^17 shape and the RLFC FFT's W = 2^22 shape).  The
    pass is a two-tile pipeline per CTA: 2^17 x 3 gives one tile to each of
    48 CTAs, 2^22 x 5 about 34 tiles to each CTA (both buffers reused many
    times), 2^22 x 2 an odd number to some."""
    torch = torch_cuda
    rng = np.random.default_rng(n + batch)
    x = (rng.normal(size=(batch, n)) + 1j * rng.normal(size=(batch, n))).astype(np.complex64)
    d_x = torch.from_numpy(x).cuda()
    d_y = torch.zeros_like(d_x)
    G.fft_tc(d_x.data_ptr(), d_y.data_ptr(), n, batch, sign)
    got = d_y.cpu().numpy().astype(np.complex128)
    x64 = x.astype(np.complex128)
    want = np.fft.fft(x64, axis=1) if sign < 0 else np.fft.ifft(x64, axis=1) * n
    err = np.linalg.norm(got - want, axis=1) / np.linalg.norm(want, axis=1)
    assert err.max() < 2e-6, err.max()


@pytest.mark.parametrize("n,batch,sign", [(1 << 17, 9, -1), (1 << 13, 3, -1), (1 << 20, 2, -1),
                                          (1 << 18, 1, 1), (1 << 16, 400, -1)])
def test_tc64_fft_matches_numpy(G, torch_cuda, n, batch, sign):
    """The FP32 FFT whose radix-64 last pass runs on the tensor cores (the
    bucket FFT's plan for B = 2^13 .. 2^20): 2^13 x 3 gives 3 tiles of 128
    sub-transforms, 2^16 x 400 about 21 tiles per CTA."""
    torch = torch_cuda
    rng = np.random.default_rng(n + batch + 7)
    x = (rng.normal(size=(batch, n)) + 1j * rng.normal(size=(batch, n))).astype(np.complex64)
    d_x = torch.from_numpy(x).cuda()
    d_y = torch.zeros_like(d_x)
    G.fft_tc64(d_x.data_ptr(), d_y.data_ptr(), n, batch, sign)
    got = d_y.cpu().numpy().astype(np.complex128)
    x64 = x.astype(np.complex128)
    want = np.fft.fft(x64, axis=1) if sign < 0 else np.fft.ifft(x64, axis=1) * n
    err = np.linalg.norm(got - want, axis=1) / np.linalg.norm(want, axis=1)
    assert err.max() < 2e-6, err.max()
