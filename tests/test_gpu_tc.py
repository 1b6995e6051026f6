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
