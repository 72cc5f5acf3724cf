"""four1 on device tensors captured into a CUDA graph and replayed.  The
library launches on the caller's current stream; calls made while that
stream captures leave the cross-call ordering to the graph.  After a warm-up
call (plans, twiddle tables and scratch exist), a capture of forward +
inverse transforms must replay to the same results as eager calls, and
replays on new input data must match the oracle (src/FFT_1.rs:5-107)."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def nr():
    pytest.importorskip("torch")
    import numrs_gb300 as m
    from numrs_gb300 import build
    build.build()
    return m


@pytest.mark.parametrize("log2n", [12, 16, 22])
@pytest.mark.parametrize("form", ["fp64", "fp32"])
def test_four1_graph_replay(nr, log2n, form):
    import torch
    import oracle as O
    from numrs_gb300 import workloads as W
    nn = 1 << log2n
    bar = 1e-12 if form == "fp64" else 1e-6
    x = W.normal(7000 + log2n, 2 * nn)
    d = torch.from_numpy(x).cuda()
    fwd = torch.empty_like(d)
    nr.set_async(True)
    try:
        def step():
            fwd.copy_(d)
            nr.four1(fwd, nn, 1, form=form)

        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            step()
        torch.cuda.current_stream().wait_stream(side)
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            step()
        for seed in (0, 1):
            y = W.normal(7100 + 10 * log2n + seed, 2 * nn)
            d.copy_(torch.from_numpy(y))
            g.replay()
            torch.cuda.synchronize()
            ref = y.copy()
            O.four1(ref, nn, 1)
            e = rel_l2(fwd.cpu().numpy(), ref)
            assert e <= bar, "graph replay %s 2^%d rel-L2 %.3e" % (form, log2n, e)
        # an eager call after the capture still works and agrees
        e2 = d.clone()
        nr.four1(e2, nn, 1, form=form)
        torch.cuda.synchronize()
        assert torch.equal(e2, fwd)
    finally:
        nr.set_async(False)
