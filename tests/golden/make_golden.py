"""Generate the golden fixtures in this directory from the CPU oracle.

Run from the repository root:  python tests/golden/make_golden.py

Inputs come from the seeded counter-based generator in numrs_gb300.workloads,
outputs from the oracle (oracle/nr_oracle.cpp); every output is also checked
against numpy.fft / scipy.fft here before it is written.  The reference crate
cannot be built in this container (no Rust toolchain, and its FFT modules are
commented out of src/lib.rs), so these vectors pin the oracle's restatement;
the reference's own known answers are pinned in tests/test_oracle.py.
"""
import os
import sys

import numpy as np
import scipy.fft as sf

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle as O  # noqa: E402
from numrs_gb300 import workloads as W  # noqa: E402


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def main():
    out = {}
    # four1, N = 4096 (the CPU-runnable configuration), both directions
    x = W.four1_c1()
    z = x[0::2] + 1j * x[1::2]
    for s in (1, -1):
        d = x.copy()
        O.four1(d, 4096, s)
        ref = 4096 * np.fft.ifft(z) if s == 1 else np.fft.fft(z)
        got = d[0::2] + 1j * d[1::2]
        assert rel(got, ref) < 1e-14
        out["four1_4096_in"] = x
        out["four1_4096_out_%s" % ("p" if s == 1 else "m")] = d
    # four1 at small sizes (both signs)
    for nn in (1, 2, 4, 8, 16, 32, 64, 128):
        xi = W.uniform_pm1(W.BASE_SEED + 100 + nn, 2 * nn)
        d = xi.copy()
        O.four1(d, nn, 1)
        assert rel(d[0::2] + 1j * d[1::2], nn * np.fft.ifft(xi[0::2] + 1j * xi[1::2])) < 1e-14 or nn == 1
        out["four1_small_%d_in" % nn] = xi
        out["four1_small_%d_out" % nn] = d
    # realft n = 1024
    xr = W.normal(W.BASE_SEED + 7, 1024)
    d = xr.copy()
    O.realft(d, 1024, 1)
    X = np.conj(np.fft.rfft(xr))
    pk = np.empty(1024)
    pk[0], pk[1] = X[0].real, X[512].real
    pk[2::2], pk[3::2] = X[1:512].real, X[1:512].imag
    assert rel(d, pk) < 1e-14
    out["realft_1024_in"] = xr
    out["realft_1024_out"] = d
    # convlv n = 1024, m = 257 (C2 shape, scaled down)
    sig, resp = W.convlv_c2(n=1024, m=257, seed=W.BASE_SEED + 9)
    st, a = O.convlv(sig, resp, 1)
    assert st == 0
    ref = np.real(np.fft.ifft(np.fft.fft(sig) * np.fft.fft(resp)))
    assert rel(a, ref) < 1e-13
    out["convlv_1024_data"] = sig
    out["convlv_1024_resp"] = resp
    out["convlv_1024_out"] = a
    taps = np.concatenate([resp[:129], resp[-128:]])  # the 257 taps in wrap-around order
    st, a2 = O.convlv(sig, taps, 1)
    assert st == 0 and rel(a2, ref) < 1e-13
    out["convlv_1024_taps"] = taps
    # correl n = 1024
    s2 = W.normal(W.BASE_SEED + 11, 1024)
    st, c = O.correl(sig, s2)
    ref = np.array([np.dot(np.roll(sig, -k), s2) for k in range(1024)])
    assert st == 0 and rel(c, ref) < 1e-13
    out["correl_1024_b"] = s2
    out["correl_1024_out"] = c
    # twofft n = 256
    t1, t2 = W.normal(W.BASE_SEED + 12, 256), W.normal(W.BASE_SEED + 13, 256)
    f1, f2 = O.twofft(t1, t2)
    assert rel(f1[:512:2] + 1j * f1[1:512:2], 256 * np.fft.ifft(t1)) < 1e-14
    out["twofft_256_a"], out["twofft_256_b"] = t1, t2
    out["twofft_256_f1"], out["twofft_256_f2"] = f1, f2
    # fourn 8 x 16 x 32
    nn = (8, 16, 32)
    xf = W.uniform_pm1(W.BASE_SEED + 14, 2 * int(np.prod(nn)))
    d = xf.copy()
    assert O.fourn(d, nn, 1) == 0
    zz = (xf[0::2] + 1j * xf[1::2]).reshape(nn)
    assert rel((d[0::2] + 1j * d[1::2]).reshape(nn), np.prod(nn) * np.fft.ifftn(zz)) < 1e-14
    out["fourn_8x16x32_in"], out["fourn_8x16x32_out"] = xf, d
    # rlft3 8 x 8 x 16 with plane waves
    x3 = W.plane_waves((8, 8, 16), count=8)
    d = x3.ravel().copy()
    sp = np.zeros(8 * 2 * 8)
    O.rlft3(d, sp, 8, 8, 16, 1)
    H = np.conj(np.fft.rfftn(x3))
    assert rel((d[0::2] + 1j * d[1::2]).reshape(8, 8, 8), H[:, :, :8]) < 1e-14
    out["rlft3_8x8x16_in"], out["rlft3_8x8x16_out"], out["rlft3_8x8x16_speq"] = x3.ravel(), d, sp
    # sine / cosine transforms n = 64
    ys = W.normal(W.BASE_SEED + 15, 64)
    ys[0] = 0.0
    d = ys.copy()
    O.sinft(d, 64)
    assert rel(d[1:], sf.dst(ys[1:], type=1) / 2) < 1e-14
    out["sinft_64_in"], out["sinft_64_out"] = ys, d
    yc = W.normal(W.BASE_SEED + 16, 65)
    d = yc.copy()
    O.cosft1(d, 64)
    assert rel(d, sf.dct(yc, type=1) / 2) < 1e-14
    out["cosft1_64_in"], out["cosft1_64_out"] = yc, d
    y2 = W.normal(W.BASE_SEED + 17, 64)
    d = y2.copy()
    O.cosft2(d, 64, 1)
    assert rel(d, sf.dct(y2, type=2) / 2) < 1e-14
    out["cosft2_64_in"], out["cosft2_64_out"] = y2, d
    d = y2.copy()
    O.cosft2(d, 64, -1)
    assert rel(d, sf.dct(y2, type=3) / 2) < 1e-14
    out["cosft2_64_inv_out"] = d
    path = os.path.join(HERE, "golden.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, sum(v.nbytes for v in out.values()), "bytes raw")


if __name__ == "__main__":
    main()
