"""The tensor-core batch form on tcgen05 (k_batch_umma: radix-16 sub-passes as
tcgen05.mma products with TMEM accumulators, the default) and on the
warp-level mma.sync kernel, each selected in process with the
GBFFT_DEBUG_TC_UMMA key.  Each transform must match the oracle within the
FP32-form bar (rel-L2 1e-6), in both directions, for single-pass bins and for
the two-pass bins whose pass-2 tiles wait on pass-1 counters."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", params=[1, 0], ids=["tcgen05", "mma_sync"])
def env(request):
    pytest.importorskip("torch")
    import numrs_gb300 as nr
    from numrs_gb300 import _lib as L
    from numrs_gb300 import build
    build.build()
    lib = L.load()
    assert lib.gbfft_debug_set(L.DEBUG_TC_UMMA, request.param) == L.OK
    yield nr, L, lib
    lib.gbfft_debug_set(L.DEBUG_TC_UMMA, 1)


@pytest.mark.parametrize("isign", [1, -1])
def test_tcgen05_batch_uneven(env, isign):
    import torch
    import oracle as O
    from numrs_gb300 import workloads as W
    nr, L, lib = env
    sizes = [16, 64, 256, 1 << 12, 1 << 13, 1 << 14, 1 << 16, 1 << 20, 32, 512, 1 << 15, 128] * 3
    host = [W.normal(8000 + i, 2 * n) * 10.0 ** ((i % 7) - 3) for i, n in enumerate(sizes)]
    refs = [a.copy() for a in host]
    O.fft_batch(refs, isign)
    dev = [torch.from_numpy(a).cuda() for a in host]
    nr.FFTBatch(dev, form="tc32").run(isign)
    torch.cuda.synchronize()
    for t, ref, n in zip(dev, refs, sizes):
        e = rel_l2(t.cpu().numpy(), ref)
        assert e <= 1e-6, "nn=%d rel-L2 %.3e" % (n, e)


def test_tcgen05_batch_c3_all_transforms(env):
    import torch
    import oracle as O
    from numrs_gb300 import workloads as W
    nr, L, lib = env
    sizes, u = W.batch_c3()
    host = W.batch_c3_data(sizes, u)
    refs = [a.copy() for a in host]
    O.set_threads(16)
    O.fft_batch(refs, 1)
    O.set_threads(1)
    ref = np.concatenate(refs)
    buf = torch.from_numpy(np.concatenate(host)).cuda()
    starts = np.concatenate([[0], np.cumsum(2 * sizes)[:-1]])
    views = [buf[int(s):int(s) + 2 * int(n)] for s, n in zip(starts, sizes)]
    nr.FFTBatch(views, form="tc32").run(1)
    torch.cuda.synchronize()
    got = buf.cpu().numpy()
    rel = np.sqrt(np.add.reduceat((got - ref) ** 2, starts)) / np.sqrt(np.add.reduceat(ref ** 2, starts))
    assert rel.max() <= 1e-6, rel.max()
