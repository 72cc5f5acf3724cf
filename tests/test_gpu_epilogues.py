"""GPU parity of the work fused into a transform's first or last pass.

* four1_spectrum: FFTProcessor::fft followed by magnitude_spectrum or
  power_spectrum (src/FFT_1.rs:166,206,218) with the spectrum written by the
  last pass.  The transform must equal four1's and the spectrum the oracle's
  spectrum of the oracle's transform; it must launch no kernel beyond
  four1's.
"""
import numpy as np
import pytest

from conftest import assert_fp64_close, rel_l2

pytestmark = pytest.mark.gpu

FORMS = ["fp64", "df64", "fp32", "tc32"]
EXACT = {"fp64": True, "df64": True, "fp32": False, "tc32": False}


@pytest.fixture(scope="module")
def nr():
    pytest.importorskip("torch")
    import numrs_gb300 as m
    from numrs_gb300 import build
    build.build()
    return m


def _close(form, got, ref, log2n, what, factor=1.0):
    if EXACT[form]:
        if factor == 1.0:
            assert_fp64_close(got, ref, log2n, what)
        else:
            e = rel_l2(got, ref)
            assert e <= factor * 1e-12, "%s rel-L2 %.3e" % (what, e)
    else:
        e = rel_l2(got, ref)
        assert e <= factor * 1e-6, "%s rel-L2 %.3e" % (what, e)


@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("log2n", [0, 1, 3, 4, 9, 10, 12, 13, 16, 20, 22])
@pytest.mark.parametrize("kind", ["magnitude", "power"])
def test_four1_spectrum_host(nr, form, log2n, kind):
    import oracle as O
    from numrs_gb300 import workloads as W
    nn = 1 << log2n
    x = W.normal(3000 + log2n, 2 * nn)
    ref = x.copy()
    O.four1(ref, nn, 1)
    want = O.magnitude_spectrum(ref) if kind == "magnitude" else O.power_spectrum(ref)
    e = x.copy()
    nr.four1(e.copy(), nn, 1, form=form)  # first use of the form fills its twiddle table
    nr.launch_count(reset=True)
    nr.four1(e, nn, 1, form=form)
    n_plain = nr.launch_count(reset=True)
    d = x.copy()
    got = nr.four1_spectrum(d, nn, 1, kind=kind, form=form)
    n_spec = nr.launch_count(reset=True)
    assert n_spec <= max(n_plain, 1), (n_spec, n_plain)
    _close(form, d, ref, log2n, "four1_spectrum data")
    # |X|^2 doubles the relative error of X
    _close(form, got, want, log2n, "four1_spectrum %s" % kind, 2.0 if kind == "power" else 1.0)


@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("log2n", [5, 12, 14, 21])
def test_four1_spectrum_device(nr, form, log2n):
    import torch
    import oracle as O
    from numrs_gb300 import workloads as W
    nn = 1 << log2n
    x = W.normal(3100 + log2n, 2 * nn)
    ref = x.copy()
    O.four1(ref, nn, -1)
    want = O.power_spectrum(ref)
    d = torch.from_numpy(x).cuda()
    got = nr.four1_spectrum(d, nn, -1, kind="power", form=form)
    torch.cuda.synchronize()
    _close(form, d.cpu().numpy(), ref, log2n, "four1_spectrum device data")
    _close(form, got.cpu().numpy(), want, log2n, "four1_spectrum device power", 2.0)


def test_four1_spectrum_rejects_bad_kind(nr):
    from numrs_gb300 import _lib as L
    lib = L.load()
    x = np.zeros(16)
    s = np.zeros(8)
    assert lib.gbfft_four1_spectrum(x.ctypes.data, 8, 1, 2, s.ctypes.data, None) == L.INVALID_ARG
    assert lib.gbfft_four1_spectrum(x.ctypes.data, 6, 1, 0, s.ctypes.data, None) == L.UNSUPPORTED_SIZE


# ---------------------------------------------------------------------------
# twofft-packed convlv / correl (src/FFT_2.rs:3-17 applied to the forward
# transforms of src/Convolve.rs:66-77 and src/Correlation.rs:53-55)
# ---------------------------------------------------------------------------
@pytest.fixture
def twofft_path(nr):
    nr.set_spectral_path("twofft")
    yield
    nr.set_spectral_path("realft")


def _composite_bar(form):
    # three transforms in sequence
    return 1e-12 if EXACT[form] else 3 ** 0.5 * 1e-6


@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("n,m", [(4, 3), (8, 1), (64, 64), (1024, 257), (4096, 3), (1 << 16, 257),
                                 (1 << 20, 257)])
def test_convlv_twofft_path(nr, twofft_path, form, n, m):
    import oracle as O
    from numrs_gb300 import workloads as W
    x = W.normal(4000 + n % 101, n)
    taps = W.normal(4050 + m, m)  # m taps in wrap-around order
    st, want = O.convlv(x, taps, 1)
    assert st == 0
    got = nr.convlv(x, taps, 1, form=form)
    e = rel_l2(got, want)
    assert e <= _composite_bar(form), "convlv twofft %s n=%d rel-L2 %.3e" % (form, n, e)
    # deconvolution of the same input (the convolution's oracle output)
    st, back = O.convlv(want, taps, -1)
    assert st == 0
    got_back = nr.convlv(want, taps, -1, form=form)
    if EXACT[form]:
        e = rel_l2(got_back, back)
        assert e <= 1e-10, "deconvolution twofft %s n=%d rel-L2 %.3e" % (form, n, e)


@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("n", [64, 4096, 1 << 20])
def test_correl_twofft_path(nr, twofft_path, form, n):
    import oracle as O
    from numrs_gb300 import workloads as W
    a = W.normal(4100 + n % 97, n)
    b = W.normal(4200 + n % 89, n)
    st, want = O.correl(a, b)
    assert st == 0
    got = nr.correl(a, b, form=form)
    e = rel_l2(got, want)
    assert e <= _composite_bar(form), "correl twofft %s n=%d rel-L2 %.3e" % (form, n, e)


def test_twofft_path_device_tensors(nr, twofft_path):
    import torch
    import oracle as O
    from numrs_gb300 import workloads as W
    x = W.normal(4300, 1 << 18)
    taps = W.normal(4301, 33)
    st, want = O.convlv(x, taps, 1)
    got = nr.convlv(torch.from_numpy(x).cuda(), torch.from_numpy(taps).cuda(), 1)
    assert rel_l2(got.cpu().numpy(), want) <= 1e-12


# ---------------------------------------------------------------------------
# realft and rlft3 with the twist fused into a pass: results as the oracle's,
# and no separate twist kernel in the launch list
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("log2n", [2, 3, 5, 9, 11, 13, 14, 18, 21, 23])
@pytest.mark.parametrize("isign", [1, -1])
def test_realft_fused_twist(nr, form, log2n, isign):
    import oracle as O
    from numrs_gb300 import workloads as W
    n = 1 << log2n
    x = W.normal(6000 + log2n, n)
    if isign == -1:
        O.realft(x, n, 1)  # a packed spectrum as input
    ref = x.copy()
    O.realft(ref, n, isign)
    d = x.copy()
    nr.realft(d.copy(), n, isign, form=form)  # tables of the form
    nr.launch_count(reset=True)
    nr.realft(d, n, isign, form=form)
    launches = nr.launch_count(reset=True)
    _close(form, d, ref, log2n, "realft %d isign %d" % (n, isign))
    # the transform's passes only: 2^(log2n-1) complex points in at most 3 passes
    assert launches <= 3, launches


@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("shape", [(2, 2, 4), (4, 8, 16), (16, 8, 4), (8, 4, 64), (32, 64, 128),
                                   (64, 2, 32), (2, 128, 8)])
def test_rlft3_fused_twist(nr, form, shape):
    import oracle as O
    from numrs_gb300 import workloads as W
    n1, n2, n3 = shape
    x = W.plane_waves(shape, count=4).ravel()
    ref, rs = x.copy(), np.zeros(n1 * 2 * n2)
    O.rlft3(ref, rs, n1, n2, n3, 1)
    log2n = int(np.log2(n1 * n2 * n3))
    d = x.copy()
    sp = np.zeros(n1 * 2 * n2)
    nr.rlft3(d.copy(), sp.copy(), n1, n2, n3, 1, form=form)
    nr.launch_count(reset=True)
    nr.rlft3(d, sp, n1, n2, n3, 1, form=form)
    fwd_launches = nr.launch_count(reset=True)
    _close(form, np.concatenate([d, sp]), np.concatenate([ref, rs]), log2n, "rlft3 fwd %s" % (shape,))
    # shapes whose twist passes qualify: one pass per axis, no speq gather or
    # twist kernel
    if shape in ((32, 64, 128), (64, 2, 32)):
        assert fwd_launches <= 3, fwd_launches
    d2, s2 = ref.copy(), rs.copy()
    nr.launch_count(reset=True)
    nr.rlft3(d2, s2, n1, n2, n3, -1, form=form)
    inv_launches = nr.launch_count(reset=True)
    O.rlft3(ref, rs, n1, n2, n3, -1)
    _close(form, d2, ref, log2n, "rlft3 inverse %s" % (shape,))
    if shape in ((32, 64, 128), (2, 128, 8)):
        assert inv_launches <= 3, inv_launches
