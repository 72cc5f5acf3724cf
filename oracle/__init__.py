"""CPU oracle for the numrs FFT family -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline legs of
``bench.py`` use this package, and only as the checker or the timed CPU
baseline.  The shipped library (``numrs_gb300``) never imports it.

Every function here wraps the C++ restatement in ``nr_oracle.cpp`` (which cites
the reference file:line for each routine) and works on float64 numpy arrays
with the reference's 0-based layouts.
"""
import ctypes
import os

import numpy as np

from . import build as _build

_lib = None

_dp = ctypes.POINTER(ctypes.c_double)
_sz = ctypes.c_size_t


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = ctypes.CDLL(path)
        L.orc_set_threads.argtypes = [ctypes.c_int]
        L.orc_get_threads.restype = ctypes.c_int
        L.orc_four1.argtypes = [_dp, _sz, _sz, ctypes.c_int]
        L.orc_four1_optimized.argtypes = [_dp, _sz, _sz, ctypes.c_int]
        L.orc_four1_nr.argtypes = [_dp, _sz, ctypes.c_int]
        L.orc_fft_batch.argtypes = [ctypes.POINTER(_dp), ctypes.POINTER(_sz), _sz, ctypes.c_int]
        L.orc_realft.argtypes = [_dp, _sz, ctypes.c_int]
        L.orc_twofft.argtypes = [_dp, _dp, _dp, _dp, _sz]
        L.orc_fourn.argtypes = [_dp, ctypes.POINTER(_sz), _sz, _sz, ctypes.c_int]
        L.orc_fourn.restype = ctypes.c_int
        L.orc_rlft3.argtypes = [_dp, _dp, _sz, _sz, _sz, ctypes.c_int]
        L.orc_sinft.argtypes = [_dp, _sz]
        L.orc_cosft1.argtypes = [_dp, _sz]
        L.orc_cosft2.argtypes = [_dp, _sz, ctypes.c_int]
        L.orc_cosft2.restype = ctypes.c_int
        L.orc_convlv.argtypes = [_dp, _sz, _dp, _sz, ctypes.c_int, _dp]
        L.orc_convlv.restype = ctypes.c_int
        L.orc_correl.argtypes = [_dp, _sz, _dp, _sz, _dp]
        L.orc_correl.restype = ctypes.c_int
        L.orc_correl_normalized.argtypes = [_dp, _sz, _dp, _sz, _dp, ctypes.c_int]
        L.orc_correl_normalized.restype = ctypes.c_int
        L.orc_magnitude_spectrum.argtypes = [_dp, _sz, _dp]
        L.orc_power_spectrum.argtypes = [_dp, _sz, _dp]
        L.orc_dft_ld.argtypes = [_dp, _sz, ctypes.c_int, _dp]
        L.orc_dft_bins.argtypes = [_dp, _sz, ctypes.c_int, ctypes.POINTER(_sz), _sz, _dp]
        _lib = L
    return _lib


def _ptr(a):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_dp)


def set_threads(n: int) -> None:
    lib().orc_set_threads(int(n))


def get_threads() -> int:
    return lib().orc_get_threads()


def four1(data, nn, isign):
    """In place, ``src/FFT_1.rs:5`` (hybrid twiddles); loops bounded by len(data)."""
    lib().orc_four1(_ptr(data), data.size, nn, isign)


def four1_optimized(data, nn, isign):
    """In place, ``src/FFT_1.rs:110`` (recurrence twiddles)."""
    lib().orc_four1_optimized(_ptr(data), data.size, nn, isign)


def four1_nr(data, nn, isign):
    """In place, the private copy ``src/Real_FT.rs:430``."""
    lib().orc_four1_nr(_ptr(data), nn, isign)


def fft_batch(arrays, isign):
    """``FFTProcessor::fft_batch`` (``src/FFT_1.rs:185``), in place on each array."""
    n = len(arrays)
    ptrs = (_dp * n)(*[_ptr(a) for a in arrays])
    lens = (_sz * n)(*[a.size for a in arrays])
    lib().orc_fft_batch(ptrs, lens, n, isign)


def realft(data, n, isign):
    lib().orc_realft(_ptr(data), n, isign)


def twofft(data1, data2):
    n = data1.size
    f1 = np.zeros(2 * n + 2)
    f2 = np.zeros(2 * n + 2)
    lib().orc_twofft(_ptr(data1), _ptr(data2), _ptr(f1), _ptr(f2), n)
    return f1, f2


def fourn(data, nn, isign, ndim=None):
    nn_arr = (_sz * len(nn))(*nn)
    nd = len(nn) if ndim is None else ndim
    return lib().orc_fourn(_ptr(data), nn_arr, len(nn), nd, isign)


def rlft3(data, speq, nn1, nn2, nn3, isign):
    lib().orc_rlft3(_ptr(data), _ptr(speq), nn1, nn2, nn3, isign)


def sinft(y, n):
    lib().orc_sinft(_ptr(y), n)


def cosft1(y, n):
    lib().orc_cosft1(_ptr(y), n)


def cosft2(y, n, isign):
    return lib().orc_cosft2(_ptr(y), n, isign)


def convlv(data, respns, isign):
    """Returns (status, ans); status follows ConvlvError order (0 = ok)."""
    data = np.ascontiguousarray(data, dtype=np.float64)
    respns = np.ascontiguousarray(respns, dtype=np.float64)
    n = data.size
    ans = np.zeros(max(n, 1))
    st = lib().orc_convlv(_ptr(data) if n else None, n, _ptr(respns) if respns.size else None,
                          respns.size, isign, _ptr(ans))
    return st, ans[:n]


def correl(data1, data2):
    """Returns (status, ans); status follows CorrelError order (0 = ok)."""
    data1 = np.ascontiguousarray(data1, dtype=np.float64)
    data2 = np.ascontiguousarray(data2, dtype=np.float64)
    n = data1.size
    ans = np.zeros(max(n, 1))
    st = lib().orc_correl(_ptr(data1) if n else None, n, _ptr(data2) if data2.size else None,
                          data2.size, _ptr(ans))
    return st, ans[:n]


def correl_normalized(data1, data2, fast=False):
    """Returns (status, ans); status 5 = ZeroStdDev."""
    data1 = np.ascontiguousarray(data1, dtype=np.float64)
    data2 = np.ascontiguousarray(data2, dtype=np.float64)
    n = data1.size
    ans = np.zeros(max(n, 1))
    st = lib().orc_correl_normalized(_ptr(data1) if n else None, n,
                                     _ptr(data2) if data2.size else None, data2.size, _ptr(ans),
                                     1 if fast else 0)
    return st, ans[:n]


def magnitude_spectrum(c):
    """``src/FFT_1.rs:206``: chunks(2); an odd-length input's last half chunk gives 0.0."""
    out = np.zeros(c.size // 2 + (c.size & 1))
    if c.size >= 2:
        lib().orc_magnitude_spectrum(_ptr(c), c.size // 2, _ptr(out))
    return out


def power_spectrum(c):
    """``src/FFT_1.rs:218``, as magnitude_spectrum."""
    out = np.zeros(c.size // 2 + (c.size & 1))
    if c.size >= 2:
        lib().orc_power_spectrum(_ptr(c), c.size // 2, _ptr(out))
    return out


def dft_ld(data, nn, isign):
    out = np.zeros(2 * nn)
    lib().orc_dft_ld(_ptr(data), nn, isign, _ptr(out))
    return out


def dft_bins(data, nn, isign, bins):
    """Bins X_k (k in ``bins``) of the direct DFT of ``data`` (nn interleaved
    complex values), each a compensated sum accurate to about one rounding.
    Returns a complex128 array.  Uses the oracle's thread pool."""
    bins = [int(b) for b in bins]
    arr = (_sz * len(bins))(*bins)
    out = np.zeros(2 * len(bins))
    lib().orc_dft_bins(_ptr(data), nn, isign, arr, len(bins), _ptr(out))
    return out[0::2] + 1j * out[1::2]
