"""numrs_gb300 -- the FFT family of the numrs crate on one GB300.

Python mirror of the crate's public FFT API over the C ABI of libgbfft.so
(include/gbfft.h).  Names, argument meaning and error behaviour follow the
Rust functions:

    four1(data, nn, isign)                 src/FFT_1.rs:5
    FFTProcessor().fft / .fft_batch        src/FFT_1.rs:143-190
    twofft(data1, data2, fft1, fft2)       src/FFT_2.rs:3
    realft(data, n, isign)                 src/Real_FT.rs:4
    fourn(data, nn, ndim, isign)           src/Fourn.rs:278 (in-memory contract)
    rlft3(data, speq, nn1, nn2, nn3, isign) src/Real_FT3.rs:8
    cosft1(y, n), cosft2(y, n, isign), sinft(y, n)
    convlv(data, respns, isign) -> array   src/Convolve.rs:8
    correl(data1, data2) -> array          src/Correlation.rs:8
    magnitude_spectrum / power_spectrum    src/FFT_1.rs:206,218

Arrays are float64: numpy arrays (host memory; copied to and from the GPU
inside the call) or torch CUDA tensors (device memory; no copies).  In-place
routines modify their argument.  Every call runs on the GPU; there is no CPU
path.  ``form`` selects the arithmetic: "fp64" (default, the crate's),
"fp32", "df64" (double-float pairs, FP64-class accuracy) or "tc32" (FP32 with
the radix-16 stages as 3xTF32 tensor-core products).
"""
import ctypes

import numpy as np

from . import _lib
from ._lib import FORMS

__all__ = [
    "four1", "four1_optimized", "FFTProcessor", "twofft", "realft", "fourn", "rlft3",
    "cosft1", "cosft2", "sinft", "convlv", "correl", "convlv_batch", "correl_batch",
    "autocorrel", "magnitude_spectrum", "power_spectrum", "real_to_complex",
    "complex_to_real", "ConvlvError", "CorrelError", "GbfftError", "launch_count",
    "FFTBatch", "four1_many", "set_async", "profile", "profile_read", "four1_noalloc",
    "four1_spectrum", "set_spectral_path", "fourfs", "twiddle_lines", "fourn_axes",
    "correl_normalized", "correl_normalized_fast", "autocorrel_fast", "ConvlvProcessor",
    "RealFTProcessor", "TwoFFTProcessor",
]


class GbfftError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("gbfft status %d: %s" % (status, msg))
        self.status = status


class ConvlvError(Exception):
    """Mirror of ``ConvlvError`` (src/Convolve.rs:226-238)."""

    class EmptyInput(Exception):
        pass

    class ResponseTooLong(Exception):
        pass

    class InvalidIsign(Exception):
        pass


class CorrelError(Exception):
    """Mirror of ``CorrelError`` (src/Correlation.rs:389-399)."""

    class EmptyInput(Exception):
        pass

    class LengthMismatch(Exception):
        pass

    class ZeroStdDev(Exception):
        pass


def _check(status):
    if status != _lib.OK:
        raise GbfftError(status, _lib.last_error())


# ---------------------------------------------------------------------------
# argument marshalling
# ---------------------------------------------------------------------------
def _is_torch(a):
    return type(a).__module__.startswith("torch")


class _Arg:
    """A float64 buffer as (pointer, number of doubles, on-device flag)."""

    def __init__(self, a, writable):
        if _is_torch(a):
            import torch
            if a.dtype != torch.float64:
                raise TypeError("expected a float64 tensor")
            if not a.is_contiguous():
                raise ValueError("tensor must be contiguous")
            self.dev = a.is_cuda
            if not self.dev:
                a = a.numpy()
            else:
                self.ptr = a.data_ptr()
                self.size = a.numel()
                self.obj = a
                return
        if not isinstance(a, np.ndarray):
            if writable:
                raise TypeError("in-place routines need a float64 numpy array or tensor")
            a = np.ascontiguousarray(a, dtype=np.float64)
        if a.dtype != np.float64:
            if writable:
                raise TypeError("expected a float64 array")
            a = a.astype(np.float64)
        if not a.flags.c_contiguous:
            if writable:
                raise ValueError("array must be C-contiguous")
            a = np.ascontiguousarray(a)
        if writable and not a.flags.writeable:
            raise ValueError("array is read-only")
        self.dev = False
        self.obj = a
        self.size = a.size
        self.ptr = a.ctypes.data if a.size else None


_ASYNC = [False]


def set_async(flag):
    """Device-tensor calls return without synchronising when set (work is
    ordered on the current torch stream).  Host-array calls always wait."""
    _ASYNC[0] = bool(flag)


def _opts(args, form, stream=None):
    devs = {a.dev for a in args}
    if len(devs) > 1:
        raise ValueError("mixing host arrays and device tensors in one call")
    o = _lib.Opts()
    o.form = FORMS[form] if isinstance(form, str) else int(form)
    o.device_ptrs = 1 if devs == {True} else 0
    o.stream = stream
    o.async_ = 1 if (o.device_ptrs and _ASYNC[0]) else 0
    if o.device_ptrs and stream is None:
        import torch
        o.stream = torch.cuda.current_stream().cuda_stream
    return o


def _new_like(proto, n):
    if proto.dev:
        import torch
        return torch.empty(n, dtype=torch.float64, device=proto.obj.device)
    return np.empty(n, dtype=np.float64)


# ---------------------------------------------------------------------------
# complex FFT
# ---------------------------------------------------------------------------
def four1(data, nn, isign, form="fp64"):
    """In-place complex FFT of nn points (``src/FFT_1.rs:5``).

    ``data`` holds 2*nn interleaved doubles.  isign=+1 uses exp(+2 pi i jk/N).
    """
    a = _Arg(data, True)
    if a.size < 2 * nn:
        raise ValueError("data holds %d doubles, need 2*nn=%d" % (a.size, 2 * nn))
    o = _opts([a], form)
    _check(_lib.load().gbfft_four1(a.ptr, nn, isign, ctypes.byref(o)))


def four1_noalloc(data, nn, isign, stream=None):
    """four1 on a CUDA float64 tensor without any GPU memory allocation.

    For callers that cannot allocate when they transform (fixed GPU memory
    budgets, plugins inside another framework's memory pool): scratch and
    tables are fixed arrays inside the library, so nn <= 2^20.  The first call
    on a device sets it up and must not be made under stream capture.  Calls
    that overlap on the GPU share that scratch; order them.
    """
    a = _Arg(data, True)
    if not a.dev:
        raise ValueError("four1_noalloc works on device tensors only")
    if stream is None:
        import torch
        stream = torch.cuda.current_stream().cuda_stream
    _check(_lib.load().gbfft_four1_noalloc(a.ptr, nn, isign, stream))


def four1_spectrum(data, nn, isign, kind="magnitude", form="fp64", out=None):
    """four1 in place, plus its magnitude (or power) spectrum written by the
    transform's last pass: ``FFTProcessor::fft`` then ``magnitude_spectrum`` /
    ``power_spectrum`` (src/FFT_1.rs:166,206,218) without a second pass over
    the data.  Returns the spectrum (nn doubles)."""
    a = _Arg(data, True)
    if a.size < 2 * nn:
        raise ValueError("data holds %d doubles, need 2*nn=%d" % (a.size, 2 * nn))
    k = {"magnitude": 0, "power": 1}[kind]
    if out is None:
        out = _new_like(a, nn)
    o = _opts([a, _Arg(out, True)], form)
    _check(_lib.load().gbfft_four1_spectrum(a.ptr, nn, isign, k, _Arg(out, True).ptr,
                                            ctypes.byref(o)))
    return out


def four1_optimized(data, nn, isign, form="fp64"):
    """``src/FFT_1.rs:110`` -- same transform as four1 (twiddles are exact on the GPU)."""
    four1(data, nn, isign, form)


def four1_many(data, nn, count, isign, dist=None, form="fp64"):
    """``count`` transforms of nn points, ``dist`` doubles apart (default 2*nn)."""
    a = _Arg(data, True)
    dist = 2 * nn if dist is None else dist
    o = _opts([a], form)
    _check(_lib.load().gbfft_four1_many(a.ptr, nn, count, dist, isign, ctypes.byref(o)))


def twiddle_lines(data, lines, length, line0, n, isign):
    """Four-step twiddle of a transform of n points split across ranks (see
    ``numrs_gb300.dist``): element k of line c of ``data`` (a CUDA float64
    tensor of ``lines`` lines of ``length`` complex values) times
    exp(isign 2 pi i ((line0 + c) k mod n) / n)."""
    a = _Arg(data, True)
    if not a.dev:
        raise ValueError("twiddle_lines takes a CUDA tensor")
    if a.size < 2 * lines * length:
        raise ValueError("data holds %d doubles, need %d" % (a.size, 2 * lines * length))
    o = _opts([a], "fp64")
    _check(_lib.load().gbfft_twiddle_lines(a.ptr, lines, length, line0, n, isign, ctypes.byref(o)))


class FFTProcessor:
    """Mirror of ``FFTProcessor`` (src/FFT_1.rs:143-190)."""

    def __init__(self, form="fp64"):
        self.max_threads = 0
        self.use_optimized = True
        self.form = form

    def with_threads(self, threads):
        self.max_threads = threads  # the reference stores and ignores it as well
        return self

    def with_optimized(self, use_optimized):
        self.use_optimized = use_optimized
        return self

    def fft(self, data, isign):
        n = data.size if isinstance(data, np.ndarray) else data.numel()
        four1(data, n // 2, isign, self.form)

    def fft_batch(self, batches, isign):
        """All transforms in one library call; sizes may differ."""
        if not batches:
            return
        args = [_Arg(b, True) for b in batches]
        o = _opts(args, self.form)
        n = len(args)
        ptrs = (ctypes.c_void_p * n)(*[x.ptr for x in args])
        nns = (ctypes.c_size_t * n)(*[x.size // 2 for x in args])
        _check(_lib.load().gbfft_four1_batch(ptrs, nns, n, isign, ctypes.byref(o)))


class FFTBatch:
    """A fixed list of arrays transformed together, the marshalling done once.

    ``FFTBatch(arrays).run(isign)`` is ``FFTProcessor().fft_batch(arrays, isign)``
    without rebuilding the pointer tables; the library caches the device plan
    and a CUDA graph of it, so repeated runs on the same device tensors are one
    graph launch each.
    """

    def __init__(self, arrays, form="fp64"):
        self.args = [_Arg(a, True) for a in arrays]
        self.form = form
        n = len(self.args)
        self.n = n
        self.ptrs = (ctypes.c_void_p * n)(*[x.ptr for x in self.args])
        self.nns = (ctypes.c_size_t * n)(*[x.size // 2 for x in self.args])

    def run(self, isign):
        o = _opts(self.args, self.form)
        _check(_lib.load().gbfft_four1_batch(self.ptrs, self.nns, self.n, isign, ctypes.byref(o)))


def twofft(data1, data2, fft1, fft2, form="fp64"):
    """Spectra of two real arrays from one complex FFT (``src/FFT_2.rs:3``).

    fft1 and fft2 have length 2n+2 (as asserted at src/FFT_2.rs:6-7).
    """
    a1, a2 = _Arg(data1, False), _Arg(data2, False)
    n = a1.size
    if a2.size != n:
        raise ValueError("data2 length must equal data1 length")
    f1, f2 = _Arg(fft1, True), _Arg(fft2, True)
    if f1.size != 2 * n + 2 or f2.size != 2 * n + 2:
        raise ValueError("fft1 and fft2 must have length 2*n + 2")
    o = _opts([a1, a2, f1, f2], form)
    _check(_lib.load().gbfft_twofft(a1.ptr, a2.ptr, f1.ptr, f2.ptr, n, ctypes.byref(o)))


def realft(data, n, isign, form="fp64"):
    """In-place real FFT of n reals (``src/Real_FT.rs:4``), packed output."""
    if n % 2 != 0:
        raise ValueError("n must be even")
    a = _Arg(data, True)
    if a.size < n:
        raise ValueError("data length must be at least n")
    o = _opts([a], form)
    _check(_lib.load().gbfft_realft(a.ptr, n, isign, ctypes.byref(o)))


def fourn(data, nn, ndim, isign, form="fp64"):
    """In-place N-D complex FFT, row-major (``src/Fourn.rs:278`` contract).

    Raises ValueError for the inputs ``validate_inputs`` rejects
    (src/Fourn.rs:367-378).
    """
    a = _Arg(data, True)
    nn = list(nn)
    arr = (ctypes.c_size_t * max(len(nn), 1))(*nn)
    o = _opts([a], form)
    st = _lib.load().gbfft_fourn(a.ptr, arr, len(nn), ndim, isign, ctypes.byref(o))
    if st == _lib.INVALID_ARG:
        raise ValueError(_lib.last_error())
    _check(st)


def fourn_axes(data, nn, axes, isign, form="fp64"):
    """fourn (row-major, ``src/Fourn.rs:278`` contract) along the listed axes
    only (axis 0 slowest): the local steps of an N-D transform split across
    ranks (``numrs_gb300.dist.fourn_sharded``)."""
    a = _Arg(data, True)
    nn = list(nn)
    total = 1
    for v in nn:
        total *= int(v)
    if a.size < 2 * total:
        raise ValueError("data holds %d doubles, need %d" % (a.size, 2 * total))
    mask = 0
    for ax in axes:
        if not 0 <= int(ax) < len(nn):
            raise ValueError("axis %r out of range" % (ax,))
        mask |= 1 << int(ax)
    arr = (ctypes.c_size_t * max(len(nn), 1))(*nn)
    o = _opts([a], form)
    st = _lib.load().gbfft_fourn_axes(a.ptr, arr, len(nn), mask, isign, ctypes.byref(o))
    if st == _lib.INVALID_ARG:
        raise ValueError(_lib.last_error())
    _check(st)


def fourfs(data, nn, ndim, isign, work=None, form="fp64"):
    """Out-of-core N-D FFT (``FourFS::fourfs``, src/Four_FS.rs:55): ``data`` is
    a host float64 array (it may be larger than the GPU's memory) transformed
    in place; every pass reads and writes host memory over the CPU-GPU link.
    ``work``: optional host scratch holding at least len(data) doubles (16
    bytes per complex element); None allocates one for the call."""
    a = _Arg(data, True)
    if a.dev:
        raise ValueError("fourfs works on host arrays (fourn takes device tensors)")
    nn = list(nn)
    arr = (ctypes.c_size_t * max(len(nn), 1))(*nn)
    w = None if work is None else _Arg(work, True)
    o = _opts([a], form)
    st = _lib.load().gbfft_fourfs(a.ptr, arr, len(nn), ndim, isign, None if w is None else w.ptr,
                                  ctypes.byref(o))
    if st == _lib.INVALID_ARG:
        raise ValueError(_lib.last_error())
    _check(st)


def rlft3(data, speq, nn1, nn2, nn3, isign, form="fp64"):
    """3-D real FFT (``src/Real_FT3.rs:8``); speq holds nn1 x 2*nn2 doubles."""
    if isign not in (1, -1):
        raise ValueError("isign must be 1 or -1")
    a, s = _Arg(data, True), _Arg(speq, True)
    if a.size != nn1 * nn2 * nn3:
        raise ValueError("data dimensions mismatch")
    if s.size != nn1 * 2 * nn2:
        raise ValueError("speq dimensions mismatch")
    o = _opts([a, s], form)
    _check(_lib.load().gbfft_rlft3(a.ptr, s.ptr, nn1, nn2, nn3, isign, ctypes.byref(o)))


def sinft(y, n, form="fp64"):
    a = _Arg(y, True)
    o = _opts([a], form)
    _check(_lib.load().gbfft_sinft(a.ptr, n, ctypes.byref(o)))


def cosft1(y, n, form="fp64"):
    """``src/Cos_FT.rs:7``; y holds n+1 values (0-based)."""
    a = _Arg(y, True)
    o = _opts([a], form)
    _check(_lib.load().gbfft_cosft1(a.ptr, n, ctypes.byref(o)))


def cosft2(y, n, isign, form="fp64"):
    """``src/Cos_FT2.rs:7``; y holds n values (0-based)."""
    if isign not in (1, -1):
        raise ValueError("Invalid isign value: %d. Must be 1 or -1" % isign)
    a = _Arg(y, True)
    o = _opts([a], form)
    _check(_lib.load().gbfft_cosft2(a.ptr, n, isign, ctypes.byref(o)))


# ---------------------------------------------------------------------------
# spectral routines
# ---------------------------------------------------------------------------
def convlv(data, respns, isign, form="fp64", out=None):
    """Convolution / deconvolution (``src/Convolve.rs:8``); returns n reals.

    Raises ConvlvError.EmptyInput / ResponseTooLong / InvalidIsign in the
    order the reference checks them.  ``out`` may supply the result array.
    """
    a, r = _Arg(data, False), _Arg(respns, False)
    n, m = a.size, r.size
    if out is None:
        out = _new_like(a, n)
    o_arg = _Arg(out, True) if n else a
    o = _opts([a, r], form)
    st = _lib.load().gbfft_convlv(a.ptr, n, r.ptr, m, isign, o_arg.ptr if n else None,
                                  ctypes.byref(o))
    if st == _lib.EMPTY_INPUT:
        raise ConvlvError.EmptyInput(_lib.last_error())
    if st == _lib.RESPONSE_TOO_LONG:
        raise ConvlvError.ResponseTooLong(_lib.last_error())
    if st == _lib.INVALID_ISIGN:
        raise ConvlvError.InvalidIsign(_lib.last_error())
    _check(st)
    return out


def correl(data1, data2, form="fp64", out=None):
    """Correlation (``src/Correlation.rs:8``); returns n reals."""
    a, b = _Arg(data1, False), _Arg(data2, False)
    n = a.size
    if out is None:
        out = _new_like(a, max(n, 1))
    o_arg = _Arg(out, True)
    o = _opts([a, b], form)
    st = _lib.load().gbfft_correl(a.ptr, n, b.ptr, b.size, o_arg.ptr, ctypes.byref(o))
    if st == _lib.EMPTY_INPUT:
        raise CorrelError.EmptyInput(_lib.last_error())
    if st == _lib.LENGTH_MISMATCH:
        raise CorrelError.LengthMismatch(_lib.last_error())
    _check(st)
    return out[:n]


def _correl_norm(data1, data2, fast, form, out):
    a, b = _Arg(data1, False), _Arg(data2, False)
    n = a.size
    if out is None:
        out = _new_like(a, max(n, 1))
    o_arg = _Arg(out, True)
    o = _opts([a, b], form)
    st = _lib.load().gbfft_correl_normalized(a.ptr, n, b.ptr, b.size, o_arg.ptr, 1 if fast else 0,
                                             ctypes.byref(o))
    if st == _lib.EMPTY_INPUT:
        raise CorrelError.EmptyInput(_lib.last_error())
    if st == _lib.LENGTH_MISMATCH:
        raise CorrelError.LengthMismatch(_lib.last_error())
    if st == _lib.ZERO_STD_DEV:
        raise CorrelError.ZeroStdDev(_lib.last_error())
    _check(st)
    return out[:n]


def correl_normalized(data1, data2, form="fp64", out=None):
    """Pearson-normalised correlation (``src/Correlation.rs:189``)."""
    return _correl_norm(data1, data2, False, form, out)


def correl_normalized_fast(data1, data2, form="fp64", out=None):
    """One-pass-statistics variant (``src/Correlation.rs:226``)."""
    return _correl_norm(data1, data2, True, form, out)


def autocorrel_fast(data, form="fp64"):
    """``autocorrel_fast`` (src/Correlation.rs:286): the autocorrelation, as autocorrel."""
    return correl(data, data, form)


class ConvlvProcessor:
    """Mirror of ``ConvlvProcessor`` (src/Convolve.rs:253-339)."""

    def __init__(self, form="fp64"):
        self.use_optimized = True
        self.parallel_threshold = 1024
        self.form = form

    def with_optimized(self, use_optimized):
        self.use_optimized = use_optimized
        return self

    def with_threshold(self, threshold):
        self.parallel_threshold = threshold
        return self

    def process(self, data, respns, isign):
        return convlv(data, respns, isign, self.form)

    def process_batch(self, data_batch, respns, isign):
        """``process_batch`` (src/Convolve.rs:333): every branch of process()
        computes convlv, so the batch is one convlv_batch call."""
        return convlv_batch(data_batch, respns, isign, self.form)


class RealFTProcessor:
    """Mirror of ``RealFTProcessor`` (src/Real_FT.rs:332-370)."""

    def __init__(self, form="fp64"):
        self.use_optimized = True
        self.parallel_threshold = 1024
        self.form = form

    def with_optimized(self, use_optimized):
        self.use_optimized = use_optimized
        return self

    def with_threshold(self, threshold):
        self.parallel_threshold = threshold
        return self

    def process(self, data, n, isign):
        realft(data, n, isign, self.form)

    def process_batch(self, batches):
        for data, n, isign in batches:
            self.process(data, n, isign)


class TwoFFTProcessor:
    """Mirror of ``TwoFFTProcessor`` (src/FFT_2.rs:222-265)."""

    def __init__(self, form="fp64"):
        self.use_optimized = True
        self.parallel_threshold = 1024
        self.form = form

    def with_optimized(self, use_optimized):
        self.use_optimized = use_optimized
        return self

    def with_threshold(self, threshold):
        self.parallel_threshold = threshold
        return self

    def process(self, data1, data2, fft1, fft2):
        twofft(data1, data2, fft1, fft2, self.form)

    def process_batch(self, batches):
        for data1, data2, fft1, fft2 in batches:
            self.process(data1, data2, fft1, fft2)


def _ptr_table(args):
    return (ctypes.c_void_p * max(len(args), 1))(*[x.ptr for x in args])


def _size_table(sizes):
    return (ctypes.c_size_t * max(len(sizes), 1))(*sizes)


def convlv_batch(data_batch, respns, isign, form="fp64"):
    """``convlv_batch`` (src/Convolve.rs:241): one library call for the whole
    batch; items of equal length share one response spectrum.  Raises the
    ConvlvError of the first failing item."""
    if len(data_batch) == 0:
        return []
    args = [_Arg(d, False) for d in data_batch]
    r = _Arg(respns, False)
    outs = [_new_like(a, a.size) for a in args]
    oargs = [_Arg(o, True) for o in outs]
    o = _opts(args + [r], form)
    st = _lib.load().gbfft_convlv_batch(_ptr_table(args), _size_table([a.size for a in args]),
                                        len(args), r.ptr, r.size, isign, _ptr_table(oargs),
                                        ctypes.byref(o))
    if st == _lib.EMPTY_INPUT:
        raise ConvlvError.EmptyInput(_lib.last_error())
    if st == _lib.RESPONSE_TOO_LONG:
        raise ConvlvError.ResponseTooLong(_lib.last_error())
    if st == _lib.INVALID_ISIGN:
        raise ConvlvError.InvalidIsign(_lib.last_error())
    _check(st)
    return outs


def correl_batch(pairs, form="fp64"):
    """``correl_batch`` (src/Correlation.rs:273): one library call for all
    pairs.  Raises the CorrelError of the first failing pair."""
    if len(pairs) == 0:
        return []
    a1 = [_Arg(a, False) for a, _ in pairs]
    a2 = [_Arg(b, False) for _, b in pairs]
    outs = [_new_like(a, a.size) for a in a1]
    oargs = [_Arg(o, True) for o in outs]
    o = _opts(a1 + a2, form)
    st = _lib.load().gbfft_correl_batch(_ptr_table(a1), _size_table([a.size for a in a1]),
                                        _ptr_table(a2), _size_table([a.size for a in a2]),
                                        len(a1), _ptr_table(oargs), ctypes.byref(o))
    if st == _lib.EMPTY_INPUT:
        raise CorrelError.EmptyInput(_lib.last_error())
    if st == _lib.LENGTH_MISMATCH:
        raise CorrelError.LengthMismatch(_lib.last_error())
    _check(st)
    return outs


def autocorrel(data, form="fp64"):
    """``autocorrel`` (src/Correlation.rs:281)."""
    return correl(data, data, form)


def _spectrum(fn, c, form):
    """The crate maps chunks(2) of the input: an odd-length input ends with a
    half chunk, whose entry is 0.0 (src/FFT_1.rs:206-228)."""
    a = _Arg(c, False)
    nn = a.size // 2
    out = _new_like(a, nn + (a.size & 1))
    if nn:
        o = _opts([a], form)
        _check(getattr(_lib.load(), fn)(a.ptr, nn, _Arg(out, True).ptr, ctypes.byref(o)))
    if a.size & 1:
        out[nn] = 0.0
    return out


def magnitude_spectrum(c, form="fp64"):
    """``magnitude_spectrum`` (src/FFT_1.rs:206): |c_k| of interleaved complex data."""
    return _spectrum("gbfft_magnitude_spectrum", c, form)


def power_spectrum(c, form="fp64"):
    """``power_spectrum`` (src/FFT_1.rs:218): |c_k|^2 of interleaved complex data."""
    return _spectrum("gbfft_power_spectrum", c, form)


def real_to_complex(x):
    """``src/FFT_1.rs:193``: interleave with zero imaginary parts (host helper)."""
    x = np.asarray(x, dtype=np.float64)
    out = np.zeros(2 * x.size)
    out[0::2] = x
    return out


def complex_to_real(c):
    """``src/FFT_1.rs:202``: the real parts (host helper)."""
    return np.asarray(c, dtype=np.float64)[0::2].copy()


def launch_count(reset=False):
    """Kernel launches issued by the library since the last reset."""
    return _lib.load().gbfft_launch_count(1 if reset else 0)


def set_spectral_path(path):
    """How convlv / correl transform their two real inputs: "realft" (two
    n/2-point realft lines, the default) or "twofft" (packed as one n-point
    complex FFT, src/FFT_2.rs:3-17, with a fused split-product-twist step)."""
    _check(_lib.load().gbfft_set_spectral_path({"realft": 0, "twofft": 1}[path]))


def set_autotune(enable=True):
    """Choose each plan's tile size by timing candidates on its first use."""
    _check(_lib.load().gbfft_set_autotune(1 if enable else 0))


PROFILE_KINDS = {"pass": 0, "twist": 1, "spectral": 2, "other": 3}


def profile(enable):
    """Start (and clear) or stop event timing of every library launch."""
    _check(_lib.load().gbfft_profile(1 if enable else 0))


def profile_read(kind):
    """(total ms, launches, algorithmic bytes, nominal flops) of one kernel kind."""
    ms = ctypes.c_double()
    n = ctypes.c_longlong()
    by = ctypes.c_double()
    fl = ctypes.c_double()
    _check(_lib.load().gbfft_profile_read(PROFILE_KINDS[kind], ctypes.byref(ms), ctypes.byref(n),
                                          ctypes.byref(by), ctypes.byref(fl)))
    return ms.value, n.value, by.value, fl.value
