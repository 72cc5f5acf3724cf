"""Failure paths, exercised without faulting or hanging a GPU.

* A bounded device wait that runs out: the persistent batch kernel's pass-2
  tiles poll a per-transform counter.  The test raises the count they wait
  for by one (so the wait cannot be met) and cuts the poll limit to 1000; the
  kernel must give up, return, and the call must report GBFFT_TIMEOUT.  The
  next normal call must succeed and match the oracle.
* A device allocation that fails: the k-th allocation after the setting is
  made to fail as if the GPU were out of memory.  The call must report
  GBFFT_OOM, and the library must work afterwards.
"""
import ctypes

import numpy as np
import pytest

from conftest import assert_fp64_close

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import numrs_gb300 as nr
    import oracle as O
    from numrs_gb300 import _lib as L
    from numrs_gb300 import build
    build.build()
    lib = L.load()
    yield torch, nr, O, L, lib
    lib.gbfft_debug_set(L.DEBUG_FAIL_ALLOC_AT, 0)
    lib.gbfft_debug_set(L.DEBUG_BATCH_SPIN_LIMIT, 0)
    lib.gbfft_debug_set(L.DEBUG_BATCH_NEED_EXTRA, 0)


def _device_batch(torch, sizes, seed):
    from numrs_gb300 import workloads as W
    host = [W.normal(seed + i, 2 * n) for i, n in enumerate(sizes)]
    dev = [torch.from_numpy(a).cuda() for a in host]
    return host, dev


def _batch_call(L, lib, dev, sizes, isign):
    ptrs = (ctypes.c_void_p * len(dev))(*[t.data_ptr() for t in dev])
    nn = (ctypes.c_size_t * len(sizes))(*sizes)
    o = L.Opts()
    o.form, o.device_ptrs, o.stream, o.async_ = 0, 1, None, 0
    return lib.gbfft_four1_batch(ptrs, nn, len(sizes), isign, ctypes.byref(o))


@pytest.mark.parametrize("form", ["fp64", "fp32"])
def test_batch_wait_runs_out_then_library_recovers(env, form):
    torch, nr, O, L, lib = env
    # 2^13 and 2^14 transforms take two passes in the persistent kernel, so
    # their pass-2 tiles wait on pass-1 counters
    sizes = [1 << 14, 1 << 13, 1 << 14, 256, 64, 1 << 13]
    host, dev = _device_batch(torch, sizes, 700)
    assert lib.gbfft_debug_set(L.DEBUG_BATCH_SPIN_LIMIT, 1000) == L.OK
    assert lib.gbfft_debug_set(L.DEBUG_BATCH_NEED_EXTRA, 1) == L.OK
    try:
        ptrs = (ctypes.c_void_p * len(dev))(*[t.data_ptr() for t in dev])
        nn = (ctypes.c_size_t * len(sizes))(*sizes)
        o = L.Opts()
        o.form, o.device_ptrs, o.stream, o.async_ = L.FORMS[form], 1, None, 0
        st = lib.gbfft_four1_batch(ptrs, nn, len(sizes), 1, ctypes.byref(o))
        assert st == L.TIMEOUT, (st, L.last_error())
        assert "bounded device wait" in L.last_error()
    finally:
        assert lib.gbfft_debug_set(L.DEBUG_BATCH_SPIN_LIMIT, 0) == L.OK
        assert lib.gbfft_debug_set(L.DEBUG_BATCH_NEED_EXTRA, 0) == L.OK
    torch.cuda.synchronize()  # the context is still usable
    host, dev = _device_batch(torch, sizes, 800)
    assert _batch_call(L, lib, dev, sizes, 1) == L.OK, L.last_error()
    refs = [a.copy() for a in host]
    O.fft_batch(refs, 1)
    for t, ref, n in zip(dev, refs, sizes):
        assert_fp64_close(t.cpu().numpy(), ref, int(np.log2(n)), "batch after timeout")


def test_allocation_failure_reports_oom_then_library_recovers(env):
    torch, nr, O, L, lib = env
    from numrs_gb300 import workloads as W
    x = W.normal(901, 1 << 20)
    resp = np.zeros(1 << 20)
    resp[:5] = [0.5, 0.25, 0.125, 0.0625, 0.25]
    st_ref, want = O.convlv(x, resp, 1)
    assert st_ref == 0
    failed = 0
    # fail the 1st, 2nd, ... allocation of a call that starts from released
    # buffers; every call either fails cleanly with GBFFT_OOM or (when it needs
    # fewer allocations) succeeds
    for k in range(1, 6):
        assert lib.gbfft_release() == L.OK
        assert lib.gbfft_debug_set(L.DEBUG_FAIL_ALLOC_AT, k) == L.OK
        out = np.zeros_like(x)
        st = lib.gbfft_convlv(x.ctypes.data, x.size, resp.ctypes.data, resp.size, 1,
                              out.ctypes.data, None)
        lib.gbfft_debug_set(L.DEBUG_FAIL_ALLOC_AT, 0)
        assert st in (L.OK, L.OOM), (k, st, L.last_error())
        if st == L.OOM:
            failed += 1
            assert "cudaMalloc" in L.last_error()
        else:
            assert_fp64_close(out, want, 20, "convlv with allocation %d failing" % k)
    assert failed >= 1
    # afterwards every form works
    for form in ("fp64", "df64", "fp32", "tc32"):
        got = nr.convlv(x, resp, 1, form=form)
        e = float(np.linalg.norm(got - want) / np.linalg.norm(want))
        assert e <= (1e-12 if form in ("fp64", "df64") else 2e-6), (form, e)


def test_twiddle_table_allocation_failure_leaves_no_half_table(env):
    torch, nr, O, L, lib = env
    from numrs_gb300 import workloads as W
    # whatever tables exist already, a call in every form after failing its
    # first and second allocations must still give correct results
    x = W.normal(902, 2 * 4096)
    ref = x.copy()
    O.four1(ref, 4096, 1)
    for form in ("fp64", "df64", "fp32", "tc32"):
        for k in (1, 2):
            assert lib.gbfft_release() == L.OK
            assert lib.gbfft_debug_set(L.DEBUG_FAIL_ALLOC_AT, k) == L.OK
            d = x.copy()
            o = L.Opts()
            o.form, o.device_ptrs, o.stream, o.async_ = L.FORMS[form], 0, None, 0
            st = lib.gbfft_four1(d.ctypes.data, 4096, 1, ctypes.byref(o))
            lib.gbfft_debug_set(L.DEBUG_FAIL_ALLOC_AT, 0)
            assert st in (L.OK, L.OOM), (form, k, st, L.last_error())
        d = x.copy()
        nr.four1(d, 4096, 1, form=form)
        if form in ("fp64", "df64"):
            assert_fp64_close(d, ref, 12, "four1 %s after failed allocations" % form)
        else:
            assert np.linalg.norm(d - ref) / np.linalg.norm(ref) <= 1e-6


def test_init_binds_one_device():
    """The library binds to the calling thread's current device at its first
    call (or to the device gbfft_init names); naming another device later is
    an argument error, and the bound device keeps working."""
    torch = pytest.importorskip("torch")
    from numrs_gb300 import _lib as L
    from numrs_gb300 import build
    build.build()
    lib = L.load()
    cur = torch.cuda.current_device()
    assert lib.gbfft_init(-1) == L.OK
    assert lib.gbfft_init(cur) == L.OK
    assert lib.gbfft_init(cur + 1) == L.INVALID_ARG
    assert "bound to device" in L.last_error()
    import numrs_gb300 as nr
    x = np.random.default_rng(11).standard_normal(2 * 64)
    d = x.copy()
    nr.four1(d, 64, 1)
    c = x[0::2] + 1j * x[1::2]
    ref = np.fft.ifft(c) * 64
    assert np.allclose(d[0::2] + 1j * d[1::2], ref, rtol=0, atol=1e-12 * np.abs(ref).max())
