"""Signal ingest, FP64 -> FP32 conversion, device-side evaluation and the
command-line driver, through the C ABI."""
import os
import re
import subprocess

import numpy as np
import pytest

from gsfft import synth

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
EXE = os.path.join(ROOT, "gpu-sfft_gb300", "build", "gsfft_exec")


def test_cli_usage_without_gpu(G):
    """The driver prints its usage (the reference's eight arguments) and fails
    without them; this needs no GPU."""
    if not os.path.exists(EXE):
        pytest.skip("gsfft_exec not built")
    r = subprocess.run([EXE], capture_output=True, text=True)
    assert r.returncode != 0
    assert "q k Bcst loops_loc loops_thresh loops_est RLFC_cst RLFC_loops" in r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [0, 1])
def test_ingest_matches_host(G, torch_cuda, prec):
    torch = torch_cuda
    rng = np.random.default_rng(3)
    n = 5 * (1 << 20) + 12345  # several staging chunks and a ragged tail
    h = rng.normal(size=n) + 1j * rng.normal(size=n)
    d = torch.zeros(n, dtype=torch.complex128 if prec == 0 else torch.complex64, device="cuda")
    G.ingest(h, prec, d.data_ptr())
    got = d.cpu().numpy()
    want = h if prec == 0 else h.astype(np.complex64)
    np.testing.assert_array_equal(got, want)
    if prec == 0:  # device conversion equals the host rounding
        d32 = torch.zeros(n, dtype=torch.complex64, device="cuda")
        G.convert_signal(d.data_ptr(), d32.data_ptr(), n)
        np.testing.assert_array_equal(d32.cpu().numpy(), h.astype(np.complex64))


@pytest.mark.gpu
def test_evaluate_matches_host(G, O, torch_cuda):
    torch = torch_cuda
    cfg = (20, 1000, 1.40, 2, 2, 5, 128, 2)
    p_g, st = G.derive_params(*cfg)
    p_o, _ = O.derive_params(*cfg)
    x, loc, coef, X = synth.signal_numpy(p_o.n, p_o.k, seed=11)
    ft, ff = O.design_filter(p_o)
    offs, a, ai = synth.draws(11, p_o.n, p_o.W_RLFC, p_o.RLFC_loops, p_o.loops)
    plan = G.Plan(p_g, 0, 0)
    d_ft = torch.from_numpy(ft).cuda()
    d_ff = torch.from_numpy(ff).cuda()
    plan.set_filter(d_ft.data_ptr(), d_ff.data_ptr())
    d_x = torch.from_numpy(x).cuda()
    plan.run(d_x.data_ptr(), offs, a, ai)
    res = plan.results()
    tl = np.sort(np.asarray(loc, np.int32))
    d_tl = torch.from_numpy(tl).cuda()
    d_X = torch.from_numpy(np.ascontiguousarray(X, np.complex128)).cuda()
    ev = plan.evaluate(d_X.data_ptr(), d_tl.data_ptr(), tl.size)
    plan.close()
    cand = set(res["nodes"]["key"].tolist())
    top = res["topk"]
    assert ev["missed_estimation"] == sum(1 for v in tl if int(v) not in cand)
    assert ev["missed_result"] == sum(1 for v in tl if int(v) not in set(top["key"].tolist()))
    xhat = np.zeros(p_o.n, np.complex128)
    xhat[top["key"]] = top["x"] + 1j * top["y"]
    err = float(np.sum(np.abs(xhat - X) ** 2))
    assert ev["mse_k"] == pytest.approx(err, rel=1e-9, abs=1e-12)


@pytest.mark.gpu
@pytest.mark.parametrize("mixed", [False, True])
def test_cli_runs_reference_report(G, torch_cuda, mixed):
    if not os.path.exists(EXE):
        pytest.skip("gsfft_exec not built")
    args = [EXE, "20", "1000", "1.40", "2", "2", "5", "128", "2", "--seed", "7", "--reps", "3"]
    if mixed:
        args.append("--mixed")
    r = subprocess.run(args, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    out = r.stdout
    assert "RLFC Filter: RLFC_loops: 2  B_thresh:2000 W_RLFC: 16384" in out
    assert "Filter: (numlobes=" in out and "b_f=136) B: 8192" in out
    assert "Time distribution: votetable  restr-loc-index  perm+filter reverse-hash  estimation FFT+Cutoff    other    total" in out
    m = re.search(r"MISSED \(estimation, result\) = \((\d+), (\d+)\), MSE\*k = (\S+),", out)
    assert m, out
    assert int(m.group(2)) <= 5  # the randomised method may lose a location or two
    assert float(m.group(3)) < 50.0
