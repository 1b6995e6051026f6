"""gsfft_run_batched: a batch of plans with different sizes, parameters and
precisions gives exactly the results of running each plan alone -- with
per-plan tails and with the persistent tail (every plan's voting and
estimation in one launch)."""
import numpy as np
import pytest

from gsfft import synth

pytestmark = pytest.mark.gpu

CASES = [  # (q, k, Bcst, loops_loc, loops_thresh, loops_est, RLFC_cst, RLFC_loops), precision
    ((14, 10, 2.5, 2, 2, 5, 16, 2), 0),
    ((16, 20, 1.0, 2, 2, 5, 8, 2), 1),
    ((18, 100, 1.0, 3, 2, 6, 32, 2), 1),
    ((16, 40, 1.2, 2, 2, 4, 16, 2), 0),
    ((20, 1000, 1.40, 2, 2, 5, 128, 2), 1),
    ((18, 60, 0.9, 2, 2, 5, 32, 2), 0),
]


def _setup(G, torch, cfg, prec, seed):
    p, st = G.derive_params(*cfg)
    assert st == 0
    d_ft = torch.zeros(p.w, dtype=torch.complex128, device="cuda")
    d_ff = torch.zeros(p.n, dtype=torch.complex128, device="cuda")
    G.design_filter(p, d_ft.data_ptr(), d_ff.data_ptr())
    plan = G.Plan(p, prec, 0)
    plan.set_filter(d_ft.data_ptr(), d_ff.data_ptr())
    x, loc, coef, X = synth.signal_numpy(p.n, p.k, seed=seed)
    d_x = torch.from_numpy(x.astype(np.complex128 if prec == 0 else np.complex64)).cuda()
    draws = synth.draws(seed, p.n, p.W_RLFC, p.RLFC_loops, p.loops)
    return plan, d_x, draws, (d_ft, d_ff)


@pytest.mark.parametrize("persistent", [False, True])
@pytest.mark.parametrize("streams", [1, 4])
def test_batched_equals_single(G, torch_cuda, streams, persistent):
    torch = torch_cuda
    items = [_setup(G, torch, cfg, prec, 100 + i) for i, (cfg, prec) in enumerate(CASES)]
    single = []
    for plan, d_x, draws, _ in items:
        plan.run(d_x.data_ptr(), *draws)
        single.append(plan.results())
    batch = G.Batch([it[0] for it in items], streams=streams)
    if persistent:
        batch.persistent_tail(True)
    batch.run([it[1].data_ptr() for it in items], [it[2] for it in items])
    torch.cuda.synchronize()
    for (plan, _, _, _), ref in zip(items, single):
        got = plan.results()
        assert got["I_F"] == ref["I_F"]
        np.testing.assert_array_equal(got["nodes"], ref["nodes"])
        np.testing.assert_array_equal(got["topk"], ref["topk"])
    batch.close()
    for it in items:
        it[0].close()


@pytest.mark.parametrize("persistent", [False, True])
def test_batch_graph_replays(G, torch_cuda, persistent):
    """A captured batch replays with one graph launch: on new signal contents
    written into the captured buffers, and twice in a row (each replay must
    count votes afresh), it gives exactly the single-plan results."""
    torch = torch_cuda
    items = [_setup(G, torch, cfg, prec, 200 + i) for i, (cfg, prec) in enumerate(CASES)]
    batch = G.Batch([it[0] for it in items], streams=4)
    if persistent:
        batch.persistent_tail(True)
    batch.capture([it[1].data_ptr() for it in items], [it[2] for it in items])
    stream = torch.cuda.Stream()
    for rep in range(2):
        # new signal contents in the captured buffers
        for i, (plan, d_x, draws, _) in enumerate(items):
            p = plan.params
            x, _, _, _ = synth.signal_numpy(p.n, p.k, seed=300 + 10 * rep + i)
            d_x.copy_(torch.from_numpy(x.astype(np.complex128 if plan.precision == 0 else np.complex64)))
        torch.cuda.synchronize()
        batch.launch(stream=stream.cuda_stream)
        stream.synchronize()
        got = [plan.results() for plan, _, _, _ in items]
        for (plan, d_x, draws, _), g in zip(items, got):
            plan.run(d_x.data_ptr(), *draws)
            ref = plan.results()
            assert g["I_F"] == ref["I_F"]
            np.testing.assert_array_equal(g["nodes"], ref["nodes"])
            np.testing.assert_array_equal(g["topk"], ref["topk"])
    batch.close()
    for it in items:
        it[0].close()


def test_bounded_wait_gives_up_and_context_survives(G, torch_cuda):
    """Failure detection without a GPU fault: a wait on an mbarrier that
    nothing arrives on (no copy or product in flight) gives up after its
    limit, the library reports GSFFT_ERR_TIMEOUT -- the status a run returns
    when one of its bounded waits gives up -- and the context keeps working
    (a cutoff right after returns the right ids)."""
    import numpy as np
    torch = torch_cuda
    L = G.lib()
    assert L.gsfft_check_bounded_wait(20_000_000, None) == G.ERR_TIMEOUT  # about 10 ms
    assert b"gave up" in L.gsfft_last_error()
    assert L.gsfft_check_bounded_wait(0, None) == G.ERR_PARAM
    s = np.arange(1000, dtype=np.float64)[::-1].copy()
    d_s = torch.from_numpy(s).cuda()
    d_o = torch.zeros(10, dtype=torch.int32, device="cuda")
    G.cutoff(d_s.data_ptr(), 1000, 10, 1, 0, d_o.data_ptr())
    np.testing.assert_array_equal(d_o.cpu().numpy(), np.arange(10))
