"""gsfft_cutoff_noalloc against gsfft_cutoff, through the C ABI.

The no-allocation cutoff serves callers that must not allocate device memory
while they run (a cudaMalloc can wait for the whole device, or fail when
another allocator of the process holds the free HBM).  Its scratch is one
fixed device array that every call shares and that keeps the previous call's
contents, so the checks run different calls back to back (different row
counts, sizes, num and tie patterns, on the default stream and on another
stream) and compare each with the allocating entry point on the same input;
one check confirms that the device's free memory does not change across
calls.  This file is collected last so that it also runs after every other
test of the session; it passes alone in a fresh process as well.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _samples(rng, batch, size, ties, prec):
    if ties:
        s = rng.integers(0, 7, size=(batch, size)).astype(np.float64) ** 2
    else:
        s = np.abs(rng.normal(size=(batch, size))) ** 3
    return s.astype(np.float64 if prec == 0 else np.float32)


def _both(G, torch, s, num, prec, stream=None):
    batch, size = s.shape
    d_s = torch.from_numpy(s).to("cuda")
    d_ref = torch.full((batch, num), -1, dtype=torch.int32, device="cuda")
    d_got = torch.full((batch, num), -1, dtype=torch.int32, device="cuda")
    G.cutoff(d_s.data_ptr(), size, num, batch, prec, d_ref.data_ptr())
    torch.cuda.synchronize()
    if stream is None:
        G.cutoff_noalloc(d_s.data_ptr(), size, num, batch, prec, d_got.data_ptr())
    else:
        G.cutoff_noalloc(d_s.data_ptr(), size, num, batch, prec, d_got.data_ptr(),
                         stream=stream.cuda_stream)
    torch.cuda.synchronize()
    return d_ref.cpu().numpy(), d_got.cpu().numpy()


@pytest.mark.parametrize("prec", [0, 1])
def test_noalloc_cutoff_matches_cutoff_twice(G, torch_cuda, prec):
    torch = torch_cuda
    rng = np.random.default_rng(4242 + prec)
    side = torch.cuda.Stream()
    calls = [
        (_samples(rng, 5, 300_001, True, prec), 20_000, None),   # many ties at the threshold
        (_samples(rng, 2, 70_000, False, prec), 1_234, side),    # fewer, shorter rows, other stream
        (_samples(rng, 3, 1 << 22, False, prec), 30_000, None),  # rows of the cooperative form
    ]
    for s, num, stream in calls:
        ref, got = _both(G, torch, s, num, prec, stream)
        np.testing.assert_array_equal(got, ref)
        assert (got >= 0).all()
        assert (np.diff(got, axis=1) > 0).all()  # ids ascending, distinct


def test_noalloc_cutoff_allocates_nothing(G, torch_cuda):
    """After a first call (which looks up the array's address), further calls
    leave the device's free memory exactly as it was."""
    torch = torch_cuda
    rng = np.random.default_rng(9)
    s = _samples(rng, 4, 1 << 20, False, 0)
    d_s = torch.from_numpy(s).cuda()
    d_o = torch.full((4, 5000), -1, dtype=torch.int32, device="cuda")
    G.cutoff_noalloc(d_s.data_ptr(), 1 << 20, 5000, 4, 0, d_o.data_ptr())
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for num in (5000, 777):
        G.cutoff_noalloc(d_s.data_ptr(), 1 << 20, num, 4, 0, d_o.data_ptr())
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0


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


def test_noalloc_cutoff_second_device(G, torch_cuda):
    """A call on a second device after the first: its own array address and
    its own selection set-up."""
    torch = torch_cuda
    if torch.cuda.device_count() < 2:
        pytest.skip("one GPU visible")
    rng = np.random.default_rng(5)
    s = _samples(rng, 2, 1 << 21, False, 0)
    outs = []
    for dev in (0, 1):
        with torch.cuda.device(dev):
            d_s = torch.from_numpy(s).to(f"cuda:{dev}")
            d_o = torch.full((2, 4000), -1, dtype=torch.int32, device=f"cuda:{dev}")
            G.cutoff_noalloc(d_s.data_ptr(), 1 << 21, 4000, 2, 0, d_o.data_ptr())
            torch.cuda.synchronize(dev)
            outs.append(d_o.cpu().numpy())
    np.testing.assert_array_equal(outs[0], outs[1])
