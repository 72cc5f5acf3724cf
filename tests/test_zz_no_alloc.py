"""gbfft_four1_noalloc against gbfft_four1 and the oracle.

The no-allocation entry point exists for callers that cannot call cudaMalloc
when they need a transform: hosts that fix their GPU memory budget up front
and plugins living inside another framework's memory pool.  It must give the
same transform as the ordinary entry point, call after call (its scratch is
one shared array that keeps the previous call's contents).  Every size it
accepts is run, which covers its one-pass tiles and every two-pass radix
split.  This file is collected last so that a failure here leaves every
other GPU test already run.
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


@pytest.mark.parametrize("log2n", list(range(0, 21)))
@pytest.mark.parametrize("isign", [1, -1])
def test_noalloc_matches_four1_twice(env, log2n, isign):
    torch, L, lib = env
    import oracle as O
    nn = 1 << log2n
    x = W.normal(9000 + log2n, 2 * nn)
    oracle_out = x.copy()
    O.four1(oracle_out, nn, isign)
    # the ordinary entry point, on device memory
    ref = torch.from_numpy(x.copy()).cuda()
    o = L.Opts()
    o.form, o.device_ptrs, o.stream, o.async_ = 0, 1, None, 0
    assert lib.gbfft_four1(ref.data_ptr(), nn, isign, ctypes.byref(o)) == L.OK, L.last_error()
    torch.cuda.synchronize()
    want = ref.cpu().numpy()
    assert_fp64_close(want, oracle_out, log2n, "four1 vs oracle")
    # two calls in a row through the no-allocation entry point
    for call in range(2):
        t = torch.from_numpy(x.copy()).cuda()
        torch.cuda.synchronize()
        st = lib.gbfft_four1_noalloc(t.data_ptr(), nn, isign, None)
        assert st == L.OK, L.last_error()
        torch.cuda.synchronize()
        got = t.cpu().numpy()
        assert_fp64_close(got, want, log2n, "four1_noalloc call %d vs four1" % call)
        assert_fp64_close(got, oracle_out, log2n, "four1_noalloc call %d vs oracle" % call)


def test_noalloc_rejects_sizes_beyond_its_scratch(env):
    torch, L, lib = env
    t = torch.zeros(2 * (1 << 21), dtype=torch.float64, device="cuda")
    assert lib.gbfft_four1_noalloc(t.data_ptr(), 1 << 21, 1, None) == L.UNSUPPORTED_SIZE
    assert "2^20" in L.last_error()
    assert lib.gbfft_four1_noalloc(t.data_ptr(), 3, 1, None) == L.UNSUPPORTED_SIZE
    assert lib.gbfft_four1_noalloc(t.data_ptr(), 8, 0, None) == L.INVALID_ARG
