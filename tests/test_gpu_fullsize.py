"""Parity at the benchmark configurations' full sizes.

The CUDA path is compared with the CPU oracle on the same seeded inputs at
the sizes the benchmark runs:

  large 1-D four1   nn = 2^28 complex (4 GiB), i.i.d. N(0,1)        (FFT_1.rs:5-107)
  batched four1     all 20,000 transforms of 2^6..2^14 points,
                    amplitudes 10^u, u ~ U[-3, 3]                     (FFT_1.rs:185-190)
  fourn             256 x 256 x 512 complex, uniform + 32 plane waves (Fourn.rs:278)
  rlft3             512^3 real + speq, uniform + 32 plane waves       (Real_FT3.rs:8-141)

FP64 and double-float results must match the oracle within rel-L2 1e-12 and
max-abs 1e-12 * ||X_ref||_inf * log2 N; FP32 and tensor-core results within
rel-L2 1e-6 (per transform for the batch).  At 2^28 the oracle itself is
also checked against exact compensated direct sums of 32 bins
(oracle.dft_bins), which involve no FFT at all.
"""
import math
import os

import numpy as np
import pytest

from conftest import assert_fp64_close, rel_l2

pytestmark = pytest.mark.gpu

FORMS = ["fp64", "df64", "fp32", "tc32"]
EXACT = {"fp64": True, "df64": True, "fp32": False, "tc32": False}


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import numrs_gb300 as nr
    import oracle as O
    from numrs_gb300 import build
    build.build()
    O.set_threads(os.cpu_count() or 1)
    yield torch, nr, O
    O.set_threads(1)


def _check(form, got, ref, log2n, what):
    if EXACT[form]:
        assert_fp64_close(got, ref, log2n, what)
    else:
        e = rel_l2(got, ref)
        assert e <= 1e-6, "%s rel-L2 %.3e > 1e-6" % (what, e)


# ---------------------------------------------------------------------------
# four1, nn = 2^28
# ---------------------------------------------------------------------------
@pytest.fixture(scope="module")
def large(env):
    torch, nr, O = env
    from numrs_gb300 import workloads as W
    log2n = 28
    nn = 1 << log2n
    x = W.normal(W.BASE_SEED + 5, 2 * nn)
    ref = x.copy()
    O.four1(ref, nn, 1)
    rng = np.random.default_rng(2028)
    bins = sorted(set([0, 1, nn // 2, nn - 1] + [int(b) for b in rng.integers(0, nn, 28)]))
    exact = O.dft_bins(x, nn, 1, bins)
    return x, ref, bins, exact, log2n


def test_large_oracle_matches_exact_bins(large):
    x, ref, bins, exact, log2n = large
    refc = ref[0::2][bins] + 1j * ref[1::2][bins]
    scale = np.abs(ref).max()
    err = np.abs(refc - exact).max()
    assert err <= 1e-12 * scale * log2n, "oracle vs exact bins %.3e" % (err / scale)


@pytest.mark.parametrize("form", FORMS)
def test_large_four1_2p28(env, large, form):
    torch, nr, O = env
    x, ref, bins, exact, log2n = large
    nn = 1 << log2n
    d = torch.from_numpy(x).cuda()
    nr.four1(d, nn, 1, form=form)
    torch.cuda.synchronize()
    got = d.cpu().numpy()
    _check(form, got, ref, log2n, "four1 2^28 %s vs oracle" % form)
    gotc = got[0::2][bins] + 1j * got[1::2][bins]
    tol = (1e-12 * log2n if EXACT[form] else 1e-5) * np.abs(ref).max()
    assert np.abs(gotc - exact).max() <= tol, "four1 2^28 %s vs exact bins" % form
    # round trip: the inverse transform scaled by 1/nn gives the input back
    nr.four1(d, nn, -1, form=form)
    d.mul_(1.0 / nn)
    torch.cuda.synchronize()
    xd = torch.from_numpy(x).cuda()
    e = float((d - xd).norm() / xd.norm())
    assert e <= (1e-13 if EXACT[form] else 2e-6), "four1 2^28 %s round trip %.3e" % (form, e)
    del d, xd
    torch.cuda.empty_cache()


# ---------------------------------------------------------------------------
# 20,000 uneven transforms
# ---------------------------------------------------------------------------
@pytest.fixture(scope="module")
def batch(env):
    torch, nr, O = env
    from numrs_gb300 import workloads as W
    sizes, u = W.batch_c3()
    host = W.batch_c3_data(sizes, u)
    refs = [a.copy() for a in host]
    O.fft_batch(refs, 1)
    return sizes, host, np.concatenate(refs)


@pytest.mark.parametrize("form", FORMS)
def test_batch_all_20000_transforms(env, batch, form):
    torch, nr, O = env
    sizes, host, ref = batch
    total = int(sum(2 * s for s in sizes))
    buf = torch.from_numpy(np.concatenate(host)).cuda()
    views, off = [], 0
    for s in sizes:
        views.append(buf[off:off + 2 * int(s)])
        off += 2 * int(s)
    assert off == total
    nr.FFTBatch(views, form=form).run(1)
    torch.cuda.synchronize()
    got = buf.cpu().numpy()
    starts = np.concatenate([[0], np.cumsum(2 * sizes)[:-1]])
    num = np.sqrt(np.add.reduceat((got - ref) ** 2, starts))
    den = np.sqrt(np.add.reduceat(ref ** 2, starts))
    rel = num / den
    worst = int(np.argmax(rel))
    if EXACT[form]:
        assert rel.max() <= 1e-12, "transform %d (nn=%d) rel-L2 %.3e" % (worst, sizes[worst], rel[worst])
        mabs = np.maximum.reduceat(np.abs(got - ref), starts)
        bound = 1e-12 * np.maximum.reduceat(np.abs(ref), starts) * np.log2(sizes)
        bad = np.nonzero(mabs > bound)[0]
        assert bad.size == 0, "transform %d exceeds the max-abs bound" % bad[0]
    else:
        assert rel.max() <= 1e-6, "transform %d (nn=%d) rel-L2 %.3e" % (worst, sizes[worst], rel[worst])


# ---------------------------------------------------------------------------
# fourn 256 x 256 x 512 and rlft3 512^3
# ---------------------------------------------------------------------------
@pytest.fixture(scope="module")
def fourn_case(env):
    torch, nr, O = env
    from numrs_gb300 import workloads as W
    shape = (256, 256, 512)
    re = W.plane_waves_torch(shape, "cuda").reshape(-1)
    im = W.plane_waves_torch(shape, "cuda", seed=W.BASE_SEED + 40).reshape(-1)
    d = torch.stack([re, im], dim=1).reshape(-1).contiguous()
    x = d.cpu().numpy()
    del re, im, d
    ref = x.copy()
    assert O.fourn(ref, shape, 1) == 0
    return shape, x, ref


@pytest.mark.parametrize("form", FORMS)
def test_fourn_256x256x512(env, fourn_case, form):
    torch, nr, O = env
    shape, x, ref = fourn_case
    n = int(np.prod(shape))
    d = torch.from_numpy(x).cuda()
    nr.fourn(d, shape, 3, 1, form=form)
    torch.cuda.synchronize()
    _check(form, d.cpu().numpy(), ref, int(math.log2(n)), "fourn 256x256x512 %s" % form)
    nr.fourn(d, shape, 3, -1, form=form)
    d.mul_(1.0 / n)
    xd = torch.from_numpy(x).cuda()
    e = float((d - xd).norm() / xd.norm())
    assert e <= (1e-13 if EXACT[form] else 2e-6), "fourn round trip %.3e" % e


@pytest.fixture(scope="module")
def rlft3_case(env):
    torch, nr, O = env
    from numrs_gb300 import workloads as W
    nn = (512, 512, 512)
    x = W.plane_waves_torch(nn, "cuda").reshape(-1).cpu().numpy()
    ref = x.copy()
    speq = np.zeros(nn[0] * 2 * nn[1])
    O.rlft3(ref, speq, nn[0], nn[1], nn[2], 1)
    return nn, x, ref, speq


@pytest.mark.parametrize("form", FORMS)
def test_rlft3_512cubed(env, rlft3_case, form):
    torch, nr, O = env
    nn, x, ref, speq = rlft3_case
    n = int(np.prod(nn))
    d = torch.from_numpy(x).cuda()
    sp = torch.zeros(nn[0] * 2 * nn[1], dtype=torch.float64, device="cuda")
    nr.launch_count(reset=True)
    nr.rlft3(d, sp, nn[0], nn[1], nn[2], 1, form=form)
    torch.cuda.synchronize()
    # one pass per axis; the twist and the speq plane ride on the last one
    assert nr.launch_count(reset=True) <= 4
    got = np.concatenate([d.cpu().numpy(), sp.cpu().numpy()])
    _check(form, got, np.concatenate([ref, speq]), int(math.log2(n)), "rlft3 512^3 %s" % form)
    nr.rlft3(d, sp, nn[0], nn[1], nn[2], -1, form=form)
    d.mul_(2.0 / n)
    xd = torch.from_numpy(x).cuda()
    e = float((d - xd).norm() / xd.norm())
    assert e <= (1e-13 if EXACT[form] else 2e-6), "rlft3 round trip %.3e" % e
