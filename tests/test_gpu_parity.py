"""GPU parity: every routine through the C ABI against the CPU oracle.

Bars (written into each check):
  FP64 and DF64 forms: rel-L2 <= 1e-12 and max-abs <= 1e-12 * ||X_ref||_inf * log2 N
  FP32 and tensor-core (3xTF32) forms: rel-L2 <= 1e-6 per transform.  A
  convolution or correlation is three transforms in sequence (two forward, one
  inverse) whose independent errors add in quadrature, so its bar is
  sqrt(3) * 1e-6 (check_composite).
"""
import os

import numpy as np
import pytest

import oracle as O
from numrs_gb300 import workloads as W
from conftest import rel_l2, assert_fp64_close

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden", "golden.npz")
FORMS = ["fp64", "df64", "fp32", "tc32"]


@pytest.fixture(scope="module")
def nr():
    import numrs_gb300
    from numrs_gb300 import build
    build.build()
    return numrs_gb300


def check(got, ref, log2n, form, what=""):
    if form in ("fp32", "tc32"):
        e = rel_l2(got, ref)
        assert e <= 1e-6, "%s %s rel-L2 %.3e > 1e-6" % (what, form, e)
    else:
        assert_fp64_close(got, ref, log2n, "%s %s" % (what, form))


def check_composite(got, ref, log2n, form, what="", transforms=3):
    """Bar of a result made of `transforms` transforms in sequence: FP64/DF64 as
    check(); FP32/TC32 at sqrt(transforms) * 1e-6 rel-L2."""
    if form in ("fp32", "tc32"):
        bar = 1e-6 * transforms ** 0.5
        e = rel_l2(got, ref)
        assert e <= bar, "%s %s rel-L2 %.3e > %.2e" % (what, form, e, bar)
    else:
        assert_fp64_close(got, ref, log2n, "%s %s" % (what, form))


def oracle_four1(x, nn, isign):
    d = x.copy()
    O.four1(d, nn, isign)
    return d


@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("log2n", list(range(0, 15)))
def test_four1_small_sizes(nr, form, log2n):
    nn = 1 << log2n
    for isign in (1, -1):
        x = W.uniform_pm1(1000 + log2n, 2 * nn)
        d = x.copy()
        nr.four1(d, nn, isign, form=form)
        check(d, oracle_four1(x, nn, isign), log2n, form, "four1 nn=%d isign=%d" % (nn, isign))


@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("log2n", [13, 15, 16, 19, 20, 22])
def test_four1_multipass(nr, form, log2n):
    nn = 1 << log2n
    x = W.normal(2000 + log2n, 2 * nn)
    d = x.copy()
    nr.four1(d, nn, 1, form=form)
    check(d, oracle_four1(x, nn, 1), log2n, form, "four1 nn=%d" % nn)


def test_four1_roundtrip_c1(nr):
    # the N=4096 configuration: +1 then -1, scaled by 1/N
    x = W.four1_c1()
    d = x.copy()
    nr.four1(d, 4096, 1)
    nr.four1(d, 4096, -1)
    d /= 4096
    assert_fp64_close(d, x, 12, "four1 round trip")


def test_four1_device_tensor(nr):
    torch = pytest.importorskip("torch")
    nn = 1 << 12
    x = W.normal(7, 2 * nn)
    t = torch.from_numpy(x.copy()).cuda()
    nr.four1(t, nn, 1)
    torch.cuda.synchronize()
    assert_fp64_close(t.cpu().numpy(), oracle_four1(x, nn, 1), 12, "four1 tensor")


def test_four1_golden(nr):
    g = np.load(GOLD)
    d = g["four1_4096_in"].copy()
    nr.four1(d, 4096, 1)
    assert_fp64_close(d, g["four1_4096_out_p"], 12, "golden four1 +1")
    d = g["four1_4096_in"].copy()
    nr.four1(d, 4096, -1)
    assert_fp64_close(d, g["four1_4096_out_m"], 12, "golden four1 -1")
    for nn in (1, 2, 4, 8, 16, 32, 64, 128):
        d = g["four1_small_%d_in" % nn].copy()
        nr.four1(d, nn, 1)
        assert_fp64_close(d, g["four1_small_%d_out" % nn], max(1, nn.bit_length() - 1), "golden small")


@pytest.mark.parametrize("form", FORMS)
def test_four1_many(nr, form):
    nn, count = 256, 37
    x = W.normal(11, 2 * nn * count)
    d = x.copy()
    nr.four1_many(d, nn, count, 1, form=form)
    ref = x.copy().reshape(count, 2 * nn)
    for r in ref:
        O.four1(r, nn, 1)
    check(d, ref.ravel(), 8, form, "four1_many")


@pytest.mark.parametrize("form", FORMS)
def test_fft_batch_uneven(nr, form):
    sizes, u = W.batch_c3(count=300)
    data = W.batch_c3_data(sizes, u)
    work = [a.copy() for a in data]
    nr.FFTProcessor(form=form).fft_batch(work, 1)
    for a, w, s in zip(data, work, sizes):
        ref = a.copy()
        (O.four1_optimized if s >= 512 else O.four1)(ref, int(s), 1)
        check(w, ref, int(s).bit_length() - 1, form, "fft_batch nn=%d" % s)


@pytest.mark.parametrize("form", [f for f in FORMS if f != "fp64"])
def test_fft_batch_prefetch_kernel(nr, form, monkeypatch):
    """The opt-in prefetching persistent kernel (bulk copies of the next tile
    into shared memory) against the oracle, single- and two-pass bins."""
    torch = pytest.importorskip("torch")
    monkeypatch.setenv("GBFFT_BATCH_PREFETCH", "1")
    sizes = [64, 8192, 128, 16384, 4096, 256, 2, 8192, 512, 32] * 4
    data = [W.normal(700 + i, 2 * s) for i, s in enumerate(sizes)]
    tens = [torch.from_numpy(a.copy()).cuda() for a in data]
    b = nr.FFTBatch(tens, form=form)
    for sg in (-1, -1):
        for t, a in zip(tens, data):
            t.copy_(torch.from_numpy(a))
        b.run(sg)
        torch.cuda.synchronize()
        for a, t, s in zip(data, tens, sizes):
            ref = a.copy()
            O.four1(ref, s, sg)
            check(t.cpu().numpy(), ref, max(1, s.bit_length() - 1), form,
                  "prefetch batch nn=%d isign=%d" % (s, sg))


@pytest.mark.parametrize("form", FORMS)
def test_fft_batch_device_graph_replay(nr, form):
    """Device tensors through the persistent batched launch: the first call
    builds and captures the plan, a repeated call replays the graph, a call in
    the other direction rebuilds it; every call is checked against the oracle,
    including 2^13 / 2^14 sizes (two passes with completion counters) and a
    size above the persistent limit."""
    torch = pytest.importorskip("torch")
    sizes = [64, 8192, 128, 16384, 4096, 1 << 21, 256, 16384, 2, 1, 8192, 512] * 3
    data = [W.normal(400 + i, 2 * s) for i, s in enumerate(sizes)]
    tens = [torch.from_numpy(a.copy()).cuda() for a in data]
    b = nr.FFTBatch(tens, form=form)
    for sg in (1, 1, -1, 1):
        for t, a in zip(tens, data):
            t.copy_(torch.from_numpy(a))
        b.run(sg)
        torch.cuda.synchronize()
        for a, t, s in zip(data, tens, sizes):
            ref = a.copy()
            O.four1(ref, s, sg)
            check(t.cpu().numpy(), ref, max(1, s.bit_length() - 1), form,
                  "batch nn=%d isign=%d" % (s, sg))


@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("log2n", [1, 2, 3, 4, 8, 10, 12, 13, 16, 20])
def test_realft(nr, form, log2n):
    n = 1 << log2n
    x = W.normal(3000 + log2n, n)
    d = x.copy()
    nr.realft(d, n, 1, form=form)
    ref = x.copy()
    O.realft(ref, n, 1)
    check(d, ref, log2n, form, "realft n=%d" % n)
    # inverse from the oracle's spectrum
    d2 = ref.copy()
    nr.realft(d2, n, -1, form=form)
    ref2 = ref.copy()
    O.realft(ref2, n, -1)
    check(d2, ref2, log2n, form, "realft inverse n=%d" % n)


def test_realft_golden(nr):
    g = np.load(GOLD)
    d = g["realft_1024_in"].copy()
    nr.realft(d, 1024, 1)
    assert_fp64_close(d, g["realft_1024_out"], 10, "golden realft")


@pytest.mark.parametrize("n", [4, 256, 4096])
def test_twofft(nr, n):
    a, b = W.normal(5, n), W.normal(6, n)
    f1 = np.full(2 * n + 2, 7.0)
    f2 = np.full(2 * n + 2, 7.0)
    nr.twofft(a, b, f1, f2)
    r1, r2 = O.twofft(a, b)
    log2n = n.bit_length() - 1
    assert_fp64_close(f1[:2 * n], r1[:2 * n], log2n, "twofft fft1")
    assert_fp64_close(f2[:2 * n], r2[:2 * n], log2n, "twofft fft2")
    assert f1[2 * n] == 7.0 and f2[2 * n + 1] == 7.0  # tail left untouched


@pytest.mark.parametrize("form", ["fp32", "tc32", "df64"])
@pytest.mark.parametrize("n", [4, 256, 4096, 1 << 16, 1 << 20])
def test_twofft_forms(nr, form, n):
    """twofft (src/FFT_2.rs:3) in the other forms: both spectra against the
    oracle's at the form's bar."""
    a, b = W.normal(5, n), W.normal(6, n)
    f1 = np.zeros(2 * n + 2)
    f2 = np.zeros(2 * n + 2)
    nr.twofft(a, b, f1, f2, form=form)
    r1, r2 = O.twofft(a, b)
    bar = 1e-12 if form == "df64" else 1e-6
    for got, ref, what in ((f1, r1, "fft1"), (f2, r2, "fft2")):
        e = rel_l2(got[:2 * n], ref[:2 * n])
        assert e <= bar, "twofft %s %s n=%d rel-L2 %.3e" % (form, what, n, e)


@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("shape", [(8, 16, 32), (4, 4), (2, 8192), (8192, 4), (64, 2, 128), (16, 16, 16, 16)])
def test_fourn(nr, form, shape):
    total = int(np.prod(shape))
    x = W.uniform_pm1(total, 2 * total)
    for isign in (1, -1):
        d = x.copy()
        nr.fourn(d, shape, len(shape), isign, form=form)
        ref = x.copy()
        assert O.fourn(ref, shape, isign) == 0
        check(d, ref, int(np.log2(total)), form, "fourn %s" % (shape,))


def test_fourn_golden(nr):
    g = np.load(GOLD)
    d = g["fourn_8x16x32_in"].copy()
    nr.fourn(d, (8, 16, 32), 3, 1)
    assert_fp64_close(d, g["fourn_8x16x32_out"], 12, "golden fourn")


@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("shape", [(8, 8, 16), (4, 8, 16), (2, 4, 2), (1, 1, 8), (16, 8, 4), (8, 4, 64)])
def test_rlft3(nr, form, shape):
    n1, n2, n3 = shape
    x = W.plane_waves(shape, count=4).ravel()
    d = x.copy()
    sp = np.zeros(n1 * 2 * n2)
    nr.rlft3(d, sp, n1, n2, n3, 1, form=form)
    rd, rs = x.copy(), np.zeros(n1 * 2 * n2)
    O.rlft3(rd, rs, n1, n2, n3, 1)
    log2n = int(np.log2(n1 * n2 * n3))
    check(d, rd, log2n, form, "rlft3 fwd data")
    check(sp, rs, log2n, form, "rlft3 fwd speq")
    d2, s2 = rd.copy(), rs.copy()
    nr.rlft3(d2, s2, n1, n2, n3, -1, form=form)
    O.rlft3(rd, rs, n1, n2, n3, -1)
    check(d2, rd, log2n, form, "rlft3 inverse")


def test_rlft3_golden(nr):
    g = np.load(GOLD)
    d = g["rlft3_8x8x16_in"].copy()
    sp = np.zeros(128)
    nr.rlft3(d, sp, 8, 8, 16, 1)
    assert_fp64_close(d, g["rlft3_8x8x16_out"], 10, "golden rlft3")
    assert_fp64_close(sp, g["rlft3_8x8x16_speq"], 10, "golden rlft3 speq")


@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("n,m", [(16, 5), (1024, 257), (4096, 3), (64, 64), (8, 1), (32, 4), (2, 1), (4, 3)])
def test_convlv(nr, form, n, m):
    x = W.normal(n + 1, n)
    r = W.normal(m + 2, m)
    got = nr.convlv(x, r, 1, form=form)
    st, ref = O.convlv(x, r, 1)
    assert st == 0
    check_composite(got, ref, max(1, n.bit_length() - 1), form, "convlv n=%d m=%d" % (n, m))
    got2 = nr.convlv(ref, r, -1, form=form)
    st, ref2 = O.convlv(ref, r, -1)
    check_composite(got2, ref2, max(1, n.bit_length() - 1), form, "deconvolve n=%d m=%d" % (n, m))


@pytest.mark.parametrize("form", FORMS)
def test_convlv_c2_full_size(nr, form):
    # N = 2^20 signal, m = 257 taps in a length-N wrap-around buffer
    x, r = W.convlv_c2()
    got = nr.convlv(x, r, 1, form=form)
    st, ref = O.convlv(x, r, 1)
    assert st == 0
    check_composite(got, ref, 20, form, "convlv C2")


def test_convlv_golden(nr):
    g = np.load(GOLD)
    got = nr.convlv(g["convlv_1024_data"], g["convlv_1024_resp"], 1)
    assert_fp64_close(got, g["convlv_1024_out"], 10, "golden convlv")
    got = nr.convlv(g["convlv_1024_data"], g["convlv_1024_taps"], 1)
    assert_fp64_close(got, g["convlv_1024_out"], 10, "golden convlv taps")


@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("n", [1, 2, 4, 31, 32, 64, 1024, 1 << 20])
def test_correl(nr, form, n):
    a, b = W.normal(n + 3, n), W.normal(n + 4, n)
    got = nr.correl(a, b, form=form)
    st, ref = O.correl(a, b)
    assert st == 0
    check_composite(got, ref, max(1, n.bit_length() - 1), form, "correl n=%d" % n)


def test_correl_kats(nr):
    # src/Correlation.rs:406-418,464-478,493-502 (direct branch, n <= 32)
    r = nr.correl([1.0, 2.0, 3.0, 4.0], [1.0, 2.0, 3.0, 4.0])
    assert abs(r[0] - 30.0) < 1e-10 and r[0] > r[1]
    assert np.allclose(nr.correl([1.0, 2.0], [1.0, 2.0]), [5.0, 2.0], atol=1e-10)
    res = nr.correl_batch([([1.0, 2.0], [1.0, 2.0]), ([3.0, 4.0], [3.0, 4.0])])
    assert abs(res[0][0] - 5.0) < 1e-10 and abs(res[1][0] - 25.0) < 1e-10


@pytest.mark.parametrize("fast", [False, True])
@pytest.mark.parametrize("n", [4, 16, 32, 64, 4096])
def test_correl_normalized(nr, fast, n):
    a, b = W.normal(n + 30, n), W.normal(n + 31, n) + 0.5
    fn = nr.correl_normalized_fast if fast else nr.correl_normalized
    got = fn(a, b)
    st, ref = O.correl_normalized(a, b, fast=fast)
    assert st == 0
    assert_fp64_close(got, ref, max(1, n.bit_length() - 1), "correl_normalized n=%d" % n)
    assert abs(nr.correl_normalized_fast([1.0, 2.0, 3.0, 4.0], [1.0, 2.0, 3.0, 4.0])[0] - 1.0) < 1e-10
    with pytest.raises(nr.CorrelError.ZeroStdDev):
        nr.correl_normalized([2.0, 2.0, 2.0], [1.0, 2.0, 3.0])


def test_processors(nr):
    x = W.normal(3, 1024)
    d = x.copy()
    nr.RealFTProcessor().process(d, 1024, 1)
    ref = x.copy()
    O.realft(ref, 1024, 1)
    assert_fp64_close(d, ref, 10, "RealFTProcessor")
    r = W.normal(4, 33)
    got = nr.ConvlvProcessor().process_batch([x, x[::-1].copy()], r, 1)
    for g_, xx in zip(got, [x, x[::-1].copy()]):
        assert_fp64_close(g_, O.convlv(xx, r, 1)[1], 10, "ConvlvProcessor")
    f1, f2 = np.zeros(2050), np.zeros(2050)
    nr.TwoFFTProcessor().process(x, x * 2, f1, f2)
    r1, r2 = O.twofft(x, x * 2)
    assert_fp64_close(f1[:2048], r1[:2048], 10, "TwoFFTProcessor")


def test_correl_golden(nr):
    g = np.load(GOLD)
    got = nr.correl(g["convlv_1024_data"], g["correl_1024_b"])
    assert_fp64_close(got, g["correl_1024_out"], 10, "golden correl")


def _exact_trig(kind, y, n, isign=1):
    import scipy.fft as sf
    if kind == "sinft":
        ref = np.zeros(n)
        ref[1:] = sf.dst(y[1:], type=1) / 2
        return ref
    if kind == "cosft1":
        return sf.dct(y, type=1) / 2
    return sf.dct(y, type=2 if isign == 1 else 3) / 2


@pytest.mark.parametrize("form", ["fp32", "tc32"])
@pytest.mark.parametrize("n", [4, 64, 1024, 4096, 1 << 16, 1 << 20])
def test_sine_cosine_transforms_fp32_forms(nr, form, n):
    """sinft, cosft1 and cosft2 (both directions) in the FP32-pipe forms
    against the exact transforms (scipy).  The algorithm (src/Cos_FT.rs:7-68,
    src/Cos_FT2.rs:7-173, and the sine transform) turns realft outputs into
    running sums over n/2 terms, which grow each output's rounding error like
    sqrt(n): the FP64 path shows the same growth relative to its unit
    roundoff (1.7e-13, about 1500 units, at 2^20).  The bar is that growth
    in FP32 units, 4 * 2^-24 * sqrt(n) (at least the FFT bar 1e-6)."""
    bar = max(1e-6, 4 * 2.0 ** -24 * np.sqrt(n))
    cases = [("sinft", W.normal(n + 5, n), None), ("cosft1", W.normal(n + 6, n + 1), None),
             ("cosft2", W.normal(n + 7, n), 1), ("cosft2", W.normal(n + 7, n), -1)]
    for kind, y, isign in cases:
        d = y.copy()
        y0 = y.copy()
        if kind == "sinft":
            nr.sinft(d, n, form=form)
            y0[0] = 0.0
        elif kind == "cosft1":
            nr.cosft1(d, n, form=form)
        else:
            nr.cosft2(d, n, isign, form=form)
        e = rel_l2(d, _exact_trig(kind, y0, n, isign or 1))
        assert e <= bar, "%s %s n=%d isign=%s rel-L2 %.3e (bar %.1e)" % (form, kind, n, isign, e, bar)


@pytest.mark.parametrize("form", ["fp64", "df64"])
@pytest.mark.parametrize("n", [2, 4, 8, 64, 1024, 4096, 1 << 16, 1 << 20])
def test_sine_cosine_transforms(nr, form, n):
    """Up to 4096 points: against the oracle at the FP64 bar.  Above, the
    oracle's Numerical Recipes twiddle recurrences (the crate's own method)
    drift from the exact transform by up to ~7e-12 at 2^20, so the GPU result
    is held to the FP64 bar against the exact transform (scipy) and to the
    oracle within the oracle's own measured drift plus 1e-12."""
    log2n = n.bit_length() - 1
    cases = [("sinft", W.normal(n + 5, n), None), ("cosft1", W.normal(n + 6, n + 1), None),
             ("cosft2", W.normal(n + 7, n), 1), ("cosft2", W.normal(n + 7, n), -1)]
    for kind, y, isign in cases:
        d, ref = y.copy(), y.copy()
        if kind == "sinft":
            nr.sinft(d, n, form=form)
            O.sinft(ref, n)
        elif kind == "cosft1":
            nr.cosft1(d, n, form=form)
            O.cosft1(ref, n)
        else:
            nr.cosft2(d, n, isign, form=form)
            O.cosft2(ref, n, isign)
        what = "%s n=%d isign=%s" % (kind, n, isign)
        if n <= 4096:
            check(d, ref, log2n, form, what)
        else:
            y0 = y.copy()
            if kind == "sinft":
                y0[0] = 0.0
            exact = _exact_trig(kind, y0, n, isign or 1)
            if kind == "cosft2" and isign == -1:
                # The inverse divides by 2 sin(pi (2i+1)/(4n)) (k_cosft2_inv_post;
                # the crate's inverse_transform, src/Cos_FT2.rs:89-173, does the
                # same), which multiplies one rounding of its inputs by up to
                # 0.5/sin(pi/(4n)) (6.7e5 at n = 2^20) at the two ends.  The
                # max-abs bar adds that conditioning, element by element.
                e = rel_l2(d, exact)
                assert e <= 1e-12, "%s rel-L2 %.3e" % (what, e)
                i = np.arange(n)
                kappa = 0.5 / np.sin(np.pi * (2 * np.minimum(i, n - 1 - i) + 1) / (4 * n))
                amax = np.abs(exact).max()
                bound = 1e-12 * amax * log2n + 8 * 2.2e-16 * kappa * amax * log2n
                worst = int(np.argmax(np.abs(d - exact) / bound))
                assert np.abs(d[worst] - exact[worst]) <= bound[worst], "%s at %d" % (what, worst)
            else:
                assert_fp64_close(d, exact, log2n, what + " vs exact " + form)
            drift = rel_l2(ref, exact)
            assert rel_l2(d, ref) <= drift + 1e-12, what


def test_sine_cosine_golden(nr):
    g = np.load(GOLD)
    for name, fn in (("sinft", lambda y: nr.sinft(y, 64)), ("cosft1", lambda y: nr.cosft1(y, 64)),
                     ("cosft2", lambda y: nr.cosft2(y, 64, 1))):
        y = g[name + "_64_in"].copy()
        fn(y)
        assert_fp64_close(y, g[name + "_64_out"], 6, "golden " + name)
    y = g["cosft2_64_in"].copy()
    nr.cosft2(y, 64, -1)
    assert_fp64_close(y, g["cosft2_64_inv_out"], 6, "golden cosft2 inverse")


def test_spectra(nr):
    x = W.normal(9, 2048)
    m = nr.magnitude_spectrum(x)
    p = nr.power_spectrum(x)
    assert_fp64_close(m, O.magnitude_spectrum(x), 10, "magnitude")
    assert_fp64_close(p, O.power_spectrum(x), 10, "power")
    # odd length: the crate's chunks(2) ends with a half chunk, whose entry is 0.0
    y = W.normal(10, 2049)
    m = nr.magnitude_spectrum(y)
    assert m.size == 1025 and m[-1] == 0.0
    assert_fp64_close(m, O.magnitude_spectrum(y), 10, "magnitude, odd length")
    assert list(nr.power_spectrum(np.array([3.0]))) == [0.0]


def test_large_roundtrip_properties(nr):
    # size-independent checks at a large size: round trip and Parseval
    nn = 1 << 24
    x = W.normal(77, 2 * nn)
    d = x.copy()
    nr.four1(d, nn, 1)
    e_t = float(np.dot(x, x))
    e_f = float(np.dot(d, d)) / nn
    assert abs(e_f - e_t) / e_t < 1e-12
    nr.four1(d, nn, -1)
    d /= nn
    assert rel_l2(d, x) < 1e-13


def test_host_and_device_paths_agree(nr):
    """Host arrays (read and written by the kernels directly where the device
    supports it, staged otherwise) and device tensors give the same results."""
    torch = pytest.importorskip("torch")
    for n in (64, 4096, 1 << 16, 1 << 20):
        x, r = W.normal(n + 50, n), W.normal(n + 51, n)
        h = nr.convlv(x, r, 1)
        d = nr.convlv(torch.from_numpy(x).cuda(), torch.from_numpy(r).cuda(), 1).cpu().numpy()
        assert_fp64_close(h, d, n.bit_length() - 1, "convlv host vs device n=%d" % n)
        hc = nr.correl(x, r)
        dc = nr.correl(torch.from_numpy(x).cuda(), torch.from_numpy(r).cuda()).cpu().numpy()
        assert_fp64_close(hc, dc, n.bit_length() - 1, "correl host vs device n=%d" % n)
        z = W.normal(n + 52, 2 * n)
        zh = z.copy()
        nr.four1(zh, n, -1)
        zd = torch.from_numpy(z.copy()).cuda()
        nr.four1(zd, n, -1)
        assert_fp64_close(zh, zd.cpu().numpy(), n.bit_length() - 1, "four1 host vs device n=%d" % n)


def test_repeat_calls_bit_identical(nr):
    x = W.normal(5, 1 << 16)
    a, b = x.copy(), x.copy()
    nr.four1(a, 1 << 15, 1)
    nr.four1(b, 1 << 15, 1)
    assert np.array_equal(a, b)


def _unaligned(n):
    """A float64 array of n values that starts 8 bytes past a 16-byte boundary
    (as a Rust subslice data[1..] can)."""
    buf = np.empty(n + 2)
    off = 1 if buf.ctypes.data % 16 == 0 else 0
    a = buf[off:off + n]
    assert a.ctypes.data % 16 == 8
    return a


@pytest.mark.parametrize("form", FORMS)
def test_unaligned_host_arrays(nr, form):
    """Host arrays on an 8-byte boundary take the staged path (the direct host
    path moves 16-byte vectors) and give the same results."""
    nn = 4096
    x = W.normal(900, 2 * nn)
    a = _unaligned(2 * nn)
    a[:] = x
    nr.four1(a, nn, 1, form=form)
    ref = x.copy()
    O.four1(ref, nn, 1)
    check(a, ref, 12, form, "unaligned four1")

    n = 1 << 14
    d = _unaligned(n)
    d[:] = W.normal(901, n)
    r = W.normal(902, 33)
    out = _unaligned(n)
    nr.convlv(d, r, 1, form=form, out=out)
    st, ref = O.convlv(np.array(d), r, 1)
    assert st == 0
    check_composite(out, ref, 14, form, "unaligned convlv")

    e = _unaligned(n)
    e[:] = W.normal(903, n)
    out2 = _unaligned(n)
    nr.correl(d, e, form=form, out=out2)
    st, ref = O.correl(np.array(d), np.array(e))
    assert st == 0
    check_composite(out2, ref, 14, form, "unaligned correl")

    # a batch mixing aligned and unaligned arrays
    sizes = [64, 8192, 256, 4096, 16384, 512]
    pairs = []
    for i, s in enumerate(sizes):
        x = W.normal(910 + i, 2 * s)
        arr = _unaligned(2 * s) if i % 2 else np.empty(2 * s)
        arr[:] = x
        pairs.append((x, arr))
    nr.FFTProcessor(form=form).fft_batch([arr for _, arr in pairs], -1)
    for (x, arr), s in zip(pairs, sizes):
        ref = x.copy()
        O.four1(ref, s, -1)
        check(arr, ref, s.bit_length() - 1, form, "unaligned batch nn=%d" % s)


@pytest.mark.parametrize("form", FORMS)
def test_batch_host_arrays_direct(nr, form):
    """Aligned host arrays within the persistent limit are read and written in
    place by the batched kernel; a repeat call replays the cached plan."""
    sizes = [64, 8192, 128, 16384, 4096, 256, 2, 1, 8192, 512] * 3
    data = [W.normal(950 + i, 2 * s) for i, s in enumerate(sizes)]
    work = [np.empty(2 * s) for s in sizes]
    assert all(w.ctypes.data % 16 == 0 for w in work)
    proc = nr.FFTProcessor(form=form)
    for rep in range(2):
        for w, x in zip(work, data):
            w[:] = x
        proc.fft_batch(work, 1)
        for w, x, s in zip(work, data, sizes):
            ref = x.copy()
            O.four1(ref, s, 1)
            check(w, ref, max(1, s.bit_length() - 1), form, "direct batch nn=%d rep %d" % (s, rep))


def test_unaligned_device_tensor_is_rejected(nr):
    torch = pytest.importorskip("torch")
    t = torch.zeros(2 * 64 + 1, dtype=torch.float64, device="cuda")
    v = t[1:]
    assert v.data_ptr() % 16 == 8
    with pytest.raises(nr.GbfftError) as ei:
        nr.four1(v, 64, 1)
    assert "16-byte" in str(ei.value)


@pytest.mark.parametrize("form", FORMS)
def test_convlv_batch_shared_response(nr, form):
    """convlv_batch over items of mixed lengths (one shared response spectrum per
    length) against the oracle's convlv of each item; deconvolution of the
    results gives the inputs back."""
    lengths = [1024, 4096, 1024, 1 << 16, 16, 8, 4096, 1024]
    data = [W.normal(1200 + i, n) for i, n in enumerate(lengths)]
    r = W.normal(1300, 7)
    got = nr.convlv_batch(data, r, 1, form=form)
    assert len(got) == len(data)
    for x, y, n in zip(data, got, lengths):
        st, ref = O.convlv(x, r, 1)
        assert st == 0
        check_composite(y, ref, max(1, n.bit_length() - 1), form, "convlv_batch n=%d" % n)
    back = nr.ConvlvProcessor(form=form).process_batch(
        [np.asarray(y) for y in got], r, -1)
    for y, b, n in zip(got, back, lengths):
        st, ref = O.convlv(np.asarray(y), r, -1)
        check_composite(b, ref, max(1, n.bit_length() - 1), form, "deconvolve batch n=%d" % n)


def test_convlv_batch_device_and_errors(nr):
    torch = pytest.importorskip("torch")
    lengths = [2048, 2048, 512]
    data = [W.normal(1400 + i, n) for i, n in enumerate(lengths)]
    r = W.normal(1500, 31)
    got = nr.convlv_batch([torch.from_numpy(x).cuda() for x in data], torch.from_numpy(r).cuda(), 1)
    for x, y, n in zip(data, got, lengths):
        st, ref = O.convlv(x, r, 1)
        assert_fp64_close(y.cpu().numpy(), ref, n.bit_length() - 1, "device convlv_batch")
    with pytest.raises(nr.ConvlvError.ResponseTooLong):
        nr.convlv_batch([data[0], np.zeros(16)], r, 1)
    with pytest.raises(nr.ConvlvError.EmptyInput):
        nr.convlv_batch([data[0], np.zeros(0)], r, 1)


@pytest.mark.parametrize("form", FORMS)
def test_correl_batch(nr, form):
    """correl_batch over pairs of mixed lengths, including the direct n <= 32
    branch, against the oracle's correl of each pair."""
    lengths = [1, 5, 32, 64, 4096, 64, 1 << 15, 32]
    pairs = [(W.normal(1600 + i, n), W.normal(1700 + i, n)) for i, n in enumerate(lengths)]
    got = nr.correl_batch(pairs, form=form)
    for (a, b), y, n in zip(pairs, got, lengths):
        st, ref = O.correl(a, b)
        assert st == 0
        check_composite(y, ref, max(1, n.bit_length() - 1), form, "correl_batch n=%d" % n)
    with pytest.raises(nr.CorrelError.LengthMismatch):
        nr.correl_batch([pairs[3], (np.ones(8), np.ones(9))], form=form)


@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("n", [16, 64, 4096, 1 << 20])
def test_autocorrel(nr, form, n):
    """autocorrel / autocorrel_fast (src/Correlation.rs:281-286): one forward
    transform whose spectrum is both operands, against the oracle's correl(x, x)."""
    x = W.normal(1800 + n, n)
    st, ref = O.correl(x, x)
    assert st == 0
    check_composite(nr.autocorrel(x, form=form), ref, max(1, n.bit_length() - 1), form,
                    "autocorrel n=%d" % n, transforms=2)
    check_composite(nr.autocorrel_fast(x, form=form), ref, max(1, n.bit_length() - 1), form,
                    "autocorrel_fast n=%d" % n, transforms=2)
    if form == "fp64":
        torch = pytest.importorskip("torch")
        xd = torch.from_numpy(x).cuda()
        got = nr.autocorrel(xd).cpu().numpy()
        assert_fp64_close(got, ref, max(1, n.bit_length() - 1), "device autocorrel n=%d" % n)


def test_async_calls_on_two_streams_are_ordered(nr):
    """Asynchronous device calls on different streams share the library's work
    buffers; the library orders each after the previous one, so back-to-back
    convolutions on two streams both come out right."""
    torch = pytest.importorskip("torch")
    n = 1 << 16
    xs = [W.normal(2000 + i, n) for i in range(4)]
    r = W.normal(2100, 33)
    refs = [O.convlv(x, r, 1)[1] for x in xs]
    rd = torch.from_numpy(r).cuda()
    xd = [torch.from_numpy(x).cuda() for x in xs]
    outs = [torch.empty(n, dtype=torch.float64, device="cuda") for _ in xs]
    streams = [torch.cuda.Stream(), torch.cuda.Stream()]
    torch.cuda.synchronize()
    nr.set_async(True)
    try:
        for i in range(4):
            with torch.cuda.stream(streams[i % 2]):
                nr.convlv(xd[i], rd, 1, out=outs[i])
    finally:
        nr.set_async(False)
    torch.cuda.synchronize()
    for i in range(4):
        assert_fp64_close(outs[i].cpu().numpy(), refs[i], 16, "two-stream convlv %d" % i)


def test_convlv_device_paths(nr):
    """Device-array convolution and correlation: aligned arrays take the
    copy-free path (inputs read through a pointer table), 8-byte-aligned views
    and lengths beyond two passes take the copying path; all match the oracle."""
    torch = pytest.importorskip("torch")
    n = 1 << 14
    x, y = W.normal(2200, n), W.normal(2201, n)
    r = W.normal(2202, 65)
    st, ref_c = O.convlv(x, r, 1)
    st2, ref_r = O.correl(x, y)
    for off in (0, 1):  # off = 1: views that start 8 bytes past a 16-byte boundary
        bx = torch.zeros(n + 2, dtype=torch.float64, device="cuda")
        by = torch.zeros(n + 2, dtype=torch.float64, device="cuda")
        bo = torch.zeros(n + 2, dtype=torch.float64, device="cuda")
        xv, yv, ov = bx[off:off + n], by[off:off + n], bo[off:off + n]
        xv.copy_(torch.from_numpy(x))
        yv.copy_(torch.from_numpy(y))
        assert (xv.data_ptr() % 16 == 0) == (off == 0)
        nr.convlv(xv, torch.from_numpy(r).cuda(), 1, out=ov)
        assert_fp64_close(ov.cpu().numpy(), ref_c, 14, "device convlv off=%d" % off)
        nr.correl(xv, yv, out=ov)
        assert_fp64_close(ov.cpu().numpy(), ref_r, 14, "device correl off=%d" % off)
    # 2^22 points: three passes per transform, beyond the copy-free path
    big = 1 << 22
    xb = W.normal(2203, big)
    st, ref_b = O.convlv(xb, r, 1)
    got = nr.convlv(torch.from_numpy(xb).cuda(), torch.from_numpy(r).cuda(), 1).cpu().numpy()
    assert_fp64_close(got, ref_b, 22, "device convlv 2^22")


@pytest.mark.parametrize("form", ["fp64", "df64"])
@pytest.mark.parametrize("log2n", [21, 22])
@pytest.mark.parametrize("isign", [1, -1])
def test_top_twiddle_level(nr, form, log2n, isign):
    """The last pass of a long FP64 axis reads its twiddles from a dense copy
    of their level (the default) or forms them as products of two table
    entries (debug key off; the double-float form always does): both within
    the FP64 bar of the oracle's four1."""
    from numrs_gb300 import _lib as L
    lib = L.load()
    nn = 1 << log2n
    x = W.normal(8000 + log2n, 2 * nn)
    ref = x.copy()
    O.four1(ref, nn, isign)
    got = {}
    for top in (1, 0):
        assert lib.gbfft_debug_set(L.DEBUG_TOP_TWIDDLES, top) == L.OK
        try:
            d = x.copy()
            nr.four1(d, nn, isign, form=form)
        finally:
            lib.gbfft_debug_set(L.DEBUG_TOP_TWIDDLES, 1)
        check(d, ref, log2n, form, "four1 2^%d %s top=%d" % (log2n, form, top))
        got[top] = d
    # the two twiddle paths differ by the rounding of one product
    assert rel_l2(got[1], got[0]) <= 1e-13
    # gbfft_release frees the dense level; the next transform rebuilds it
    assert lib.gbfft_release() == L.OK
    d = x.copy()
    nr.four1(d, nn, isign, form=form)
    assert np.array_equal(d, got[1])
