"""ctypes binding of libgbfft.so (the C ABI declared in include/gbfft.h).

The shared library is loaded from the package directory.  There is no
fallback: if the library is missing or no CUDA device is present, calls raise.
"""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libgbfft.so")

OK = 0
INVALID_ARG = 1
UNSUPPORTED_SIZE = 2
CUDA_ERROR = 3
TIMEOUT = 4
OOM = 5
EMPTY_INPUT = 10
RESPONSE_TOO_LONG = 11
INVALID_ISIGN = 12
LENGTH_MISMATCH = 13
ZERO_STD_DEV = 14

FORMS = {"fp64": 0, "fp32": 1, "df64": 2, "tc32": 3}


class Opts(ctypes.Structure):
    _fields_ = [("form", ctypes.c_int), ("device_ptrs", ctypes.c_int),
                ("stream", ctypes.c_void_p), ("async_", ctypes.c_int)]


_dp = ctypes.POINTER(ctypes.c_double)
_vp = ctypes.c_void_p
_sz = ctypes.c_size_t
_op = ctypes.POINTER(Opts)

# name -> argtypes; every entry point returns int (gbfft_status)
SIGNATURES = {
    "gbfft_init": [ctypes.c_int],
    "gbfft_four1": [_vp, _sz, ctypes.c_int, _op],
    "gbfft_four1_batch": [ctypes.POINTER(_vp), ctypes.POINTER(_sz), _sz, ctypes.c_int, _op],
    "gbfft_four1_many": [_vp, _sz, _sz, _sz, ctypes.c_int, _op],
    "gbfft_four1_spectrum": [_vp, _sz, ctypes.c_int, ctypes.c_int, _vp, _op],
    "gbfft_twofft": [_vp, _vp, _vp, _vp, _sz, _op],
    "gbfft_realft": [_vp, _sz, ctypes.c_int, _op],
    "gbfft_fourn": [_vp, ctypes.POINTER(_sz), _sz, _sz, ctypes.c_int, _op],
    "gbfft_fourfs": [_vp, ctypes.POINTER(_sz), _sz, _sz, ctypes.c_int, _vp, _op],
    "gbfft_rlft3": [_vp, _vp, _sz, _sz, _sz, ctypes.c_int, _op],
    "gbfft_sinft": [_vp, _sz, _op],
    "gbfft_cosft1": [_vp, _sz, _op],
    "gbfft_cosft2": [_vp, _sz, ctypes.c_int, _op],
    "gbfft_convlv": [_vp, _sz, _vp, _sz, ctypes.c_int, _vp, _op],
    "gbfft_correl": [_vp, _sz, _vp, _sz, _vp, _op],
    "gbfft_convlv_batch": [_vp, _vp, _sz, _vp, _sz, ctypes.c_int, _vp, _op],
    "gbfft_correl_batch": [_vp, _vp, _vp, _vp, _sz, _vp, _op],
    "gbfft_correl_normalized": [_vp, _sz, _vp, _sz, _vp, ctypes.c_int, _op],
    "gbfft_magnitude_spectrum": [_vp, _sz, _vp, _op],
    "gbfft_power_spectrum": [_vp, _sz, _vp, _op],
    "gbfft_twiddle_lines": [_vp, _sz, _sz, _sz, _sz, ctypes.c_int, _op],
    "gbfft_fourn_axes": [_vp, ctypes.POINTER(_sz), _sz, ctypes.c_ulonglong, ctypes.c_int, _op],
    "gbfft_release": [],
    "gbfft_four1_noalloc": [_vp, _sz, ctypes.c_int, _vp],
    "gbfft_profile": [ctypes.c_int],
    "gbfft_set_autotune": [ctypes.c_int],
    "gbfft_profile_read": [ctypes.c_int, _dp, ctypes.POINTER(ctypes.c_longlong), _dp, _dp],
    "gbfft_debug_set": [ctypes.c_int, ctypes.c_longlong],
    "gbfft_set_spectral_path": [ctypes.c_int],
}

# gbfft_debug_set keys (failure injection for tests)
DEBUG_FAIL_ALLOC_AT = 1
DEBUG_BATCH_SPIN_LIMIT = 2
DEBUG_BATCH_NEED_EXTRA = 3
DEBUG_BATCH_FIRST_RADIX_DELTA = 4
DEBUG_FUSED_TWIST = 5
DEBUG_TC_UMMA = 6
DEBUG_CLUSTER_PASS = 7
DEBUG_TOP_TWIDDLES = 8

_lib = None


def load():
    """Load libgbfft.so once; raises OSError if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise OSError("libgbfft.so is not built (run numrs_gb300.build.build())")
        L = ctypes.CDLL(LIB_PATH)
        for name, args in SIGNATURES.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = ctypes.c_int
        L.gbfft_last_error.restype = ctypes.c_char_p
        L.gbfft_last_error.argtypes = []
        L.gbfft_version.restype = ctypes.c_int
        L.gbfft_scratch_bytes.restype = ctypes.c_size_t
        L.gbfft_launch_count.restype = ctypes.c_longlong
        L.gbfft_launch_count.argtypes = [ctypes.c_int]
        _lib = L
    return _lib


def last_error() -> str:
    return load().gbfft_last_error().decode(errors="replace")
