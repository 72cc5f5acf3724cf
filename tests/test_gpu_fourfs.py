"""The out-of-core N-D FFT (FourFS::fourfs, src/Four_FS.rs:55-73) on the GPU.

The data stay in host memory and every pass reads and writes host memory
directly, so the transform must equal the in-memory fourn's (the oracle's
fourn at the FP64 bar) while the library takes no device scratch for it.
"""
import numpy as np
import pytest

from conftest import assert_fp64_close, rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def nr():
    pytest.importorskip("torch")
    import numrs_gb300 as m
    from numrs_gb300 import build
    build.build()
    return m


@pytest.mark.parametrize("shape", [(1 << 20,), (1 << 24,), (64, 128, 256), (8, 1 << 16), (2, 2, 2)])
@pytest.mark.parametrize("isign", [1, -1])
def test_fourfs_matches_oracle_fourn(nr, shape, isign):
    import oracle as O
    from numrs_gb300 import _lib as L
    from numrs_gb300 import workloads as W
    n = int(np.prod(shape))
    x = W.normal(5000 + n % 113, 2 * n)
    ref = x.copy()
    O.set_threads(8)
    assert O.fourn(ref, shape, isign) == 0
    O.set_threads(1)
    lib = L.load()
    assert lib.gbfft_release() == L.OK
    d = x.copy()
    nr.fourfs(d, shape, len(shape), isign)
    assert_fp64_close(d, ref, int(np.log2(n)), "fourfs %s" % (shape,))
    # no device scratch proportional to the data
    assert lib.gbfft_scratch_bytes() == 0
    # a caller-supplied work array gives the same result
    d2 = x.copy()
    work = np.empty(2 * n)
    nr.fourfs(d2, shape, len(shape), isign, work=work)
    assert np.array_equal(d, d2)


@pytest.mark.parametrize("form", ["df64", "fp32", "tc32"])
def test_fourfs_forms(nr, form):
    import oracle as O
    from numrs_gb300 import workloads as W
    shape = (256, 4096)
    n = int(np.prod(shape))
    x = W.normal(5100, 2 * n)
    ref = x.copy()
    assert O.fourn(ref, shape, 1) == 0
    d = x.copy()
    nr.fourfs(d, shape, 2, 1, form=form)
    e = rel_l2(d, ref)
    assert e <= (1e-12 if form == "df64" else 1e-6), (form, e)


def test_fourfs_rejects_device_data(nr):
    import torch
    t = torch.zeros(64, dtype=torch.float64, device="cuda")
    with pytest.raises(ValueError):
        nr.fourfs(t, (32,), 1, 1)
