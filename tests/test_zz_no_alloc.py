"""gsfft_cutoff_noalloc against gsfft_cutoff, through the C ABI.

The no-allocation cutoff keeps its scratch in one fixed device array that
every call shares and that keeps the previous call's contents, so the checks
run two different calls back to back (different row counts, sizes, num and
tie patterns) and compare each with the allocating entry point on the same
input.  This file is collected last so that it also runs after every other
test of the session; it passes alone in a fresh process as well.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _samples(rng, batch, size, ties, prec):
    if ties:
        s = rng.integers(0, 7, size=(batch, size)).astype(np.float64) ** 2
    else:
        s = np.abs(rng.normal(size=(batch, size))) ** 3
    return s.astype(np.float64 if prec == 0 else np.float32)


def _both(G, torch, s, num, prec):
    batch, size = s.shape
    d_s = torch.from_numpy(s).to("cuda")
    d_ref = torch.full((batch, num), -1, dtype=torch.int32, device="cuda")
    d_got = torch.full((batch, num), -1, dtype=torch.int32, device="cuda")
    G.cutoff(d_s.data_ptr(), size, num, batch, prec, d_ref.data_ptr())
    G.cutoff_noalloc(d_s.data_ptr(), size, num, batch, prec, d_got.data_ptr())
    torch.cuda.synchronize()
    return d_ref.cpu().numpy(), d_got.cpu().numpy()


@pytest.mark.parametrize("prec", [0, 1])
def test_noalloc_cutoff_matches_cutoff_twice(G, torch_cuda, prec):
    torch = torch_cuda
    rng = np.random.default_rng(4242 + prec)
    calls = [
        (_samples(rng, 5, 300_001, True, prec), 20_000),   # many ties at the threshold
        (_samples(rng, 2, 70_000, False, prec), 1_234),    # fewer, shorter rows afterwards
    ]
    for s, num in calls:
        ref, got = _both(G, torch, s, num, prec)
        np.testing.assert_array_equal(got, ref)
        assert (got >= 0).all()
        assert (np.diff(got, axis=1) > 0).all()  # ids ascending, distinct


def test_noalloc_cutoff_limits(G, torch_cuda):
    torch = torch_cuda
    d_s = torch.zeros(16, dtype=torch.float64, device="cuda")
    d_o = torch.zeros(16, dtype=torch.int32, device="cuda")
    L = G.lib()
    # beyond the fixed scratch: rejected before any device work
    assert L.gsfft_cutoff_noalloc(d_s.data_ptr(), G.NOALLOC_MAX_SIZE + 1, 4, 1, 0,
                                  d_o.data_ptr(), None) == 2
    assert b"exceed" in L.gsfft_last_error()
    assert L.gsfft_cutoff_noalloc(d_s.data_ptr(), 16, 4, G.NOALLOC_MAX_BATCH + 1, 0,
                                  d_o.data_ptr(), None) == 2
    # the largest accepted row count still matches the allocating cutoff
    rng = np.random.default_rng(77)
    s = _samples(rng, G.NOALLOC_MAX_BATCH, 50_000, True, 0)
    ref, got = _both(G, torch, s, 999, 0)
    np.testing.assert_array_equal(got, ref)
