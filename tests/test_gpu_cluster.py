"""The FP32 form's two-pass schedule on four-CTA clusters (k_pass_cl) for
unit-stride axes of 2^22..2^28 points.  Each pass is a radix-2^11..2^14
Stockham pass (src/FFT_1.rs:47-107 reorganised) whose R-point DFTs are split
over a cluster: every CTA computes the R/4-point DFTs of its decimated rows,
then one radix-4 step reads the four CTAs' results over distributed shared
memory.  The schedule is opt-in (slower than the three per-CTA passes on
GB300); the tests select it with the debug key.  Every case must match the
oracle (or the FP64 form, which the parity tests hold to the oracle at 1e-12)
within the FP32 bar, take two launches, and agree with the three-pass
per-CTA schedule."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

BAR = 1e-6


@pytest.fixture(scope="module")
def env():
    pytest.importorskip("torch")
    import numrs_gb300 as nr
    from numrs_gb300 import _lib as L
    from numrs_gb300 import build
    build.build()
    lib = L.load()
    assert lib.gbfft_debug_set(L.DEBUG_CLUSTER_PASS, 1) == L.OK
    yield nr, L, lib
    lib.gbfft_debug_set(L.DEBUG_CLUSTER_PASS, 0)


@pytest.mark.parametrize("log2n", [22, 23])
@pytest.mark.parametrize("isign", [1, -1])
def test_cluster_four1_vs_oracle(env, log2n, isign):
    import oracle as O
    from numrs_gb300 import workloads as W
    nr, L, lib = env
    nn = 1 << log2n
    x = W.normal(5000 + log2n, 2 * nn)
    ref = x.copy()
    O.four1(ref, nn, isign)
    nr.four1(x.copy(), nn, isign, form="fp32")  # the form's twiddle table
    d = x.copy()
    nr.launch_count(reset=True)
    nr.four1(d, nn, isign, form="fp32")
    assert nr.launch_count(reset=True) == 2
    e = rel_l2(d, ref)
    assert e <= BAR, "four1 2^%d fp32 cluster rel-L2 %.3e" % (log2n, e)


@pytest.mark.parametrize("log2n", [24, 25, 26, 27])
@pytest.mark.parametrize("isign", [1, -1])
def test_cluster_four1_vs_fp64_form(env, log2n, isign):
    import torch
    from numrs_gb300 import workloads as W
    nr, L, lib = env
    nn = 1 << log2n
    x = torch.from_numpy(W.normal(5100 + log2n, 2 * nn)).cuda()
    ref = x.clone()
    nr.four1(ref, nn, isign, form="fp64")
    d = x.clone()
    nr.four1(d, nn, isign, form="fp32")
    torch.cuda.synchronize()
    e = float(torch.linalg.vector_norm(d - ref) / torch.linalg.vector_norm(ref))
    assert e <= BAR, "four1 2^%d fp32 cluster vs fp64 rel-L2 %.3e" % (log2n, e)
    # the three-pass per-CTA schedule gives the same transform to FP32 accuracy
    assert lib.gbfft_debug_set(L.DEBUG_CLUSTER_PASS, 0) == L.OK
    try:
        d3 = x.clone()
        nr.four1(d3, nn, isign, form="fp32")
        torch.cuda.synchronize()
    finally:
        lib.gbfft_debug_set(L.DEBUG_CLUSTER_PASS, 1)
    e3 = float(torch.linalg.vector_norm(d3 - ref) / torch.linalg.vector_norm(ref))
    assert e3 <= BAR
    del x, ref, d, d3
    torch.cuda.empty_cache()


def test_cluster_fourn_lines(env):
    """fourn with a 2^22-point last axis (four contiguous lines on the cluster
    schedule) and a short strided first axis."""
    import torch
    from numrs_gb300 import workloads as W
    nr, L, lib = env
    dims = [4, 1 << 22]
    n = dims[0] * dims[1]
    x = torch.from_numpy(W.normal(5200, 2 * n)).cuda()
    ref = x.clone()
    nr.fourn(ref, dims, 2, 1, form="fp64")
    d = x.clone()
    nr.fourn(d, dims, 2, 1, form="fp32")
    torch.cuda.synchronize()
    e = float(torch.linalg.vector_norm(d - ref) / torch.linalg.vector_norm(ref))
    assert e <= BAR, "fourn 4 x 2^22 fp32 rel-L2 %.3e" % e


@pytest.mark.parametrize("kind", ["magnitude", "power"])
def test_cluster_spectrum_epilogue(env, kind):
    import oracle as O
    from numrs_gb300 import workloads as W
    nr, L, lib = env
    log2n = 22
    nn = 1 << log2n
    x = W.normal(5300, 2 * nn)
    ref = x.copy()
    O.four1(ref, nn, 1)
    want = O.magnitude_spectrum(ref) if kind == "magnitude" else O.power_spectrum(ref)
    d = x.copy()
    got = nr.four1_spectrum(d, nn, 1, kind=kind, form="fp32")
    assert rel_l2(d, ref) <= BAR
    assert rel_l2(got, want) <= (2.0 if kind == "power" else 1.0) * BAR


def test_cluster_realft_round_trip(env):
    """realft of 2^23 points: a 2^22-point complex FFT on the cluster schedule
    with the twist in a kernel of its own."""
    import oracle as O
    from numrs_gb300 import workloads as W
    nr, L, lib = env
    n = 1 << 23
    x = W.normal(5400, n)
    ref = x.copy()
    O.realft(ref, n, 1)
    d = x.copy()
    nr.realft(d, n, 1, form="fp32")
    assert rel_l2(d, ref) <= BAR
    nr.realft(d, n, -1, form="fp32")
    assert rel_l2(d * (2.0 / n), x) <= 2 * BAR


def test_cluster_convlv_twofft_path(env):
    """convlv of 2^23 points on the twofft-packed path: its forward transform
    reads the two inputs through a per-line pointer table."""
    import oracle as O
    from numrs_gb300 import workloads as W
    nr, L, lib = env
    n, m = 1 << 23, 257
    x = W.normal(5500, n)
    taps = W.normal(5501, m)
    st, want = O.convlv(x, taps, 1)
    assert st == 0
    for path in ("realft", "twofft"):
        nr.set_spectral_path(path)
        try:
            got = nr.convlv(x, taps, 1, form="fp32")
        finally:
            nr.set_spectral_path("realft")
        e = rel_l2(got, want)
        assert e <= 3 ** 0.5 * BAR, "convlv 2^23 fp32 %s rel-L2 %.3e" % (path, e)
