"""CPU tests of the C-ABI library: it loads, exports every entry point that
include/gbfft.h declares, and rejects bad arguments before touching a GPU."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADERS = [os.path.join(ROOT, "include", f) for f in sorted(os.listdir(os.path.join(ROOT, "include")))
           if f.endswith(".h")]


def declared_symbols():
    names = []
    for h in HEADERS:
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names += re.findall(r"\b(gbfft_[a-z0-9_]+)\s*\(", text)
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib():
    from numrs_gb300 import build, _lib
    build.build()
    return _lib.load()


def test_header_declares_the_family():
    syms = declared_symbols()
    for name in ("gbfft_four1", "gbfft_four1_batch", "gbfft_twofft", "gbfft_realft",
                 "gbfft_fourn", "gbfft_rlft3", "gbfft_sinft", "gbfft_cosft1", "gbfft_cosft2",
                 "gbfft_convlv", "gbfft_correl"):
        assert name in syms


def test_every_declared_symbol_is_exported(lib):
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_argument_errors_need_no_gpu(lib):
    from numrs_gb300 import _lib as L
    x = np.zeros(8)
    p = x.ctypes.data
    # convlv check order, src/Convolve.rs:13-21
    assert lib.gbfft_convlv(p, 0, p, 1, 1, p, None) == L.EMPTY_INPUT
    assert lib.gbfft_convlv(p, 2, p, 3, 1, p, None) == L.RESPONSE_TOO_LONG
    assert lib.gbfft_convlv(p, 2, p, 1, 0, p, None) == L.INVALID_ISIGN
    assert lib.gbfft_convlv(p, 6, p, 1, 1, p, None) == L.UNSUPPORTED_SIZE
    # correl, src/Correlation.rs:10-16
    assert lib.gbfft_correl(p, 0, p, 1, p, None) == L.EMPTY_INPUT
    assert lib.gbfft_correl(p, 2, p, 1, p, None) == L.LENGTH_MISMATCH
    # fourn validate_inputs, src/Fourn.rs:367-378
    nn = (ctypes.c_size_t * 2)(8, 1)
    assert lib.gbfft_fourn(p, nn, 2, 2, 1, None) == L.INVALID_ARG
    assert lib.gbfft_fourn(p, nn, 2, 3, 1, None) == L.INVALID_ARG
    assert lib.gbfft_fourn(p, nn, 2, 1, 0, None) == L.INVALID_ARG
    # fourfs validate_inputs, src/Four_FS.rs:328-339 (as the reference's
    # test_invalid_inputs, src/Four_FS.rs:428-437)
    one = (ctypes.c_size_t * 1)(1)
    eight = (ctypes.c_size_t * 1)(8)
    assert lib.gbfft_fourfs(p, one, 1, 1, 1, None, None) == L.INVALID_ARG
    assert lib.gbfft_fourfs(p, eight, 1, 1, 0, None, None) == L.INVALID_ARG
    assert lib.gbfft_fourfs(p, eight, 1, 2, 1, None, None) == L.INVALID_ARG
    # sizes and signs
    assert lib.gbfft_four1(p, 3, 1, None) == L.UNSUPPORTED_SIZE
    assert lib.gbfft_four1(p, 4, 2, None) == L.INVALID_ARG
    assert lib.gbfft_four1(None, 4, 1, None) == L.INVALID_ARG
    assert lib.gbfft_realft(p, 6, 1, None) == L.UNSUPPORTED_SIZE
    assert lib.gbfft_rlft3(p, p, 2, 2, 2, 0, None) == L.INVALID_ARG
    msg = L.last_error()
    assert "isign" in msg
    # the local steps of the sharded transforms
    dims = (ctypes.c_size_t * 3)(2, 4, 8)
    assert lib.gbfft_fourn_axes(p, dims, 3, 0, 1, None) == L.INVALID_ARG      # no axis
    assert lib.gbfft_fourn_axes(p, dims, 3, 1 << 3, 1, None) == L.INVALID_ARG  # axis 3 of 3
    assert lib.gbfft_fourn_axes(p, dims, 3, 1, 2, None) == L.INVALID_ARG      # isign
    bad = (ctypes.c_size_t * 2)(3, 4)
    assert lib.gbfft_fourn_axes(p, bad, 2, 1, 1, None) == L.UNSUPPORTED_SIZE
    assert lib.gbfft_twiddle_lines(p, 2, 4, 0, 16, 1, None) == L.INVALID_ARG  # host data


def test_python_mirror_raises_reference_errors(lib):
    import numrs_gb300 as nr
    with pytest.raises(nr.ConvlvError.EmptyInput):
        nr.convlv([], [1.0], 1)
    with pytest.raises(nr.ConvlvError.ResponseTooLong):
        nr.convlv([1.0, 2.0], [1.0, 2.0, 3.0], 1)
    with pytest.raises(nr.ConvlvError.InvalidIsign):
        nr.convlv([1.0, 2.0], [1.0], 0)
    with pytest.raises(nr.CorrelError.EmptyInput):
        nr.correl([], [1.0])
    with pytest.raises(nr.CorrelError.LengthMismatch):
        nr.correl([1.0, 2.0], [1.0])
    with pytest.raises(ValueError):
        nr.fourn(np.zeros(4), [1], 1, 1)
    with pytest.raises(ValueError):
        nr.cosft2(np.zeros(8), 8, 0)


def test_unaligned_device_arrays_are_rejected_before_any_launch(lib):
    """Device arrays must start on a 16-byte boundary (the kernels move complex
    values as 16-byte vectors); an unaligned one is refused on the host, so no
    GPU is needed to check it.  The pointers are never dereferenced."""
    from numrs_gb300 import _lib as L
    o = L.Opts()
    o.form = 0
    o.device_ptrs = 1
    o.stream = None
    o.async_ = 0
    po = ctypes.byref(o)
    bad = 0x7F0000001008  # 8-byte aligned only
    assert lib.gbfft_four1(ctypes.c_void_p(bad), 8, 1, po) == L.INVALID_ARG
    assert "16-byte" in L.last_error()
    assert lib.gbfft_four1_many(ctypes.c_void_p(bad), 8, 2, 16, 1, po) == L.INVALID_ARG
    assert lib.gbfft_realft(ctypes.c_void_p(bad), 8, 1, po) == L.INVALID_ARG
    assert lib.gbfft_sinft(ctypes.c_void_p(bad), 8, po) == L.INVALID_ARG
    ptrs = (ctypes.c_void_p * 2)(0x7F0000002000, bad)
    nns = (ctypes.c_size_t * 2)(8, 8)
    assert lib.gbfft_four1_batch(ptrs, nns, 2, 1, po) == L.INVALID_ARG
    assert "16-byte" in L.last_error()
    assert lib.gbfft_four1_noalloc(ctypes.c_void_p(bad), 8, 1, None) == L.INVALID_ARG
    assert "16-byte" in L.last_error()


def test_batch_wrapper_errors_need_no_gpu(lib):
    """convlv_batch / correl_batch run convlv's and correl's checks item by item
    and return the first failure before any work."""
    from numrs_gb300 import _lib as L
    x = np.zeros(8)
    p = x.ctypes.data
    ptrs = (ctypes.c_void_p * 2)(p, p)
    outs = (ctypes.c_void_p * 2)(p, p)
    ns = (ctypes.c_size_t * 2)(8, 0)
    assert lib.gbfft_convlv_batch(ptrs, ns, 2, p, 3, 1, outs, None) == L.EMPTY_INPUT
    assert "item 1" in L.last_error()
    ns = (ctypes.c_size_t * 2)(8, 2)
    assert lib.gbfft_convlv_batch(ptrs, ns, 2, p, 3, 1, outs, None) == L.RESPONSE_TOO_LONG
    ns = (ctypes.c_size_t * 2)(8, 8)
    assert lib.gbfft_convlv_batch(ptrs, ns, 2, p, 3, 0, outs, None) == L.INVALID_ISIGN
    ns = (ctypes.c_size_t * 2)(8, 6)
    assert lib.gbfft_convlv_batch(ptrs, ns, 2, p, 3, 1, outs, None) == L.UNSUPPORTED_SIZE
    n1 = (ctypes.c_size_t * 2)(8, 8)
    n2 = (ctypes.c_size_t * 2)(8, 7)
    assert lib.gbfft_correl_batch(ptrs, n1, ptrs, n2, 2, outs, None) == L.LENGTH_MISMATCH
    n1 = (ctypes.c_size_t * 2)(0, 8)
    assert lib.gbfft_correl_batch(ptrs, n1, ptrs, n1, 2, outs, None) == L.EMPTY_INPUT
    assert lib.gbfft_convlv_batch(ptrs, ns, 0, p, 3, 1, outs, None) == L.OK
