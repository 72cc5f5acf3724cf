"""gbfft_four1_noalloc against gbfft_four1.

The no-allocation entry point exists for callers that cannot call cudaMalloc
when they need a transform (for example while a CUDA graph is being captured,
or under a fixed memory budget).  It must give the same transform as the
ordinary entry point.  This file is collected last so that a failure here
leaves every other GPU test already run.
"""
import ctypes

import numpy as np
import pytest

from numrs_gb300 import workloads as W
from conftest import assert_fp64_close

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    from numrs_gb300 import build, _lib
    build.build()
    return torch, _lib, _lib.load()


@pytest.mark.parametrize("log2n", [12, 16, 20])
@pytest.mark.parametrize("isign", [1, -1])
def test_noalloc_matches_four1_twice(env, log2n, isign):
    torch, L, lib = env
    nn = 1 << log2n
    x = W.normal(9000 + log2n, 2 * nn)
    # the ordinary entry point, on device memory
    ref = torch.from_numpy(x.copy()).cuda()
    o = L.Opts()
    o.form, o.device_ptrs, o.stream, o.async_ = 0, 1, None, 0
    assert lib.gbfft_four1(ref.data_ptr(), nn, isign, ctypes.byref(o)) == L.OK, L.last_error()
    torch.cuda.synchronize()
    want = ref.cpu().numpy()
    # two calls in a row through the no-allocation entry point
    for call in range(2):
        t = torch.from_numpy(x.copy()).cuda()
        torch.cuda.synchronize()
        st = lib.gbfft_four1_noalloc(t.data_ptr(), nn, isign, None)
        assert st == L.OK, L.last_error()
        torch.cuda.synchronize()
        assert_fp64_close(t.cpu().numpy(), want, log2n, "four1_noalloc call %d" % call)


def test_noalloc_rejects_sizes_beyond_its_scratch(env):
    torch, L, lib = env
    t = torch.zeros(2 * (1 << 21), dtype=torch.float64, device="cuda")
    assert lib.gbfft_four1_noalloc(t.data_ptr(), 1 << 21, 1, None) == L.UNSUPPORTED_SIZE
    assert "2^20" in L.last_error()
    assert lib.gbfft_four1_noalloc(t.data_ptr(), 3, 1, None) == L.UNSUPPORTED_SIZE
    assert lib.gbfft_four1_noalloc(t.data_ptr(), 8, 0, None) == L.INVALID_ARG
