"""The autotuner of the persistent batch launch: for every bin of the batch
it chooses the radix split of two-pass transforms and the resident CTAs per
SM (the batch kernel's tile and threads per transform).

Every schedule it may choose is checked for correctness against the oracle
(the two-pass bins' first radix shifted by -2..+2), and a tuning run in a
fresh process writes its choice to the tune cache, which a second process
reads back without tuning again; both give the oracle's results.
"""
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import assert_fp64_close, rel_l2

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def env():
    pytest.importorskip("torch")
    import numrs_gb300 as nr
    from numrs_gb300 import _lib as L
    from numrs_gb300 import build
    build.build()
    lib = L.load()
    yield nr, L, lib
    lib.gbfft_debug_set(L.DEBUG_BATCH_FIRST_RADIX_DELTA, 0)


SIZES = [1 << 13, 1 << 14, 1 << 16, 1 << 20, 1 << 17, 256, 1 << 15, 64, 1 << 13, 1 << 19]


@pytest.mark.parametrize("delta", [-2, -1, 1, 2])
@pytest.mark.parametrize("form", ["fp64", "fp32"])
def test_every_tuner_split_is_correct(env, delta, form):
    import torch
    import oracle as O
    from numrs_gb300 import workloads as W
    nr, L, lib = env
    host = [W.normal(7000 + i, 2 * n) for i, n in enumerate(SIZES)]
    refs = [a.copy() for a in host]
    O.fft_batch(refs, 1)
    assert lib.gbfft_debug_set(L.DEBUG_BATCH_FIRST_RADIX_DELTA, delta) == L.OK
    try:
        dev = [torch.from_numpy(a).cuda() for a in host]
        nr.FFTBatch(dev, form=form).run(1)
        torch.cuda.synchronize()
    finally:
        lib.gbfft_debug_set(L.DEBUG_BATCH_FIRST_RADIX_DELTA, 0)
    for t, ref, n in zip(dev, refs, SIZES):
        if form == "fp64":
            assert_fp64_close(t.cpu().numpy(), ref, int(np.log2(n)), "delta %d nn %d" % (delta, n))
        else:
            assert rel_l2(t.cpu().numpy(), ref) <= 1e-6


_CHILD = r'''
import sys, numpy as np
sys.path.insert(0, %r)
import numrs_gb300 as nr, oracle as O
from numrs_gb300 import workloads as W
sizes, u = W.batch_c3(count=2000)
host = W.batch_c3_data(sizes, u)
refs = [a.copy() for a in host]
O.fft_batch(refs, 1)
arrs = [a.copy() for a in host]
nr.FFTBatch(arrs, form=%r).run(1)
err = max(float(np.linalg.norm(a - r) / np.linalg.norm(r)) for a, r in zip(arrs, refs))
print("MAXERR", err)
'''


@pytest.mark.parametrize("form", ["fp64", "tc32"])
def test_tune_cache_across_processes(env, tmp_path, form):
    cache = tmp_path / "tune.txt"
    envv = dict(os.environ, GBFFT_AUTOTUNE="1", GBFFT_TUNE_CACHE=str(cache), GBFFT_TUNE_VERBOSE="1")
    code = _CHILD % (ROOT, form)
    r1 = subprocess.run([sys.executable, "-c", code], env=envv, capture_output=True, text=True,
                        timeout=600)
    assert r1.returncode == 0, r1.stderr[-2000:]
    lines = [ln for ln in cache.read_text().splitlines() if ln.startswith("batch ")]
    assert len(lines) == 1, cache.read_text()
    assert "gbfft batch tune" in r1.stderr  # the candidates were timed
    r2 = subprocess.run([sys.executable, "-c", code], env=envv, capture_output=True, text=True,
                        timeout=600)
    assert r2.returncode == 0, r2.stderr[-2000:]
    assert "gbfft batch tune" not in r2.stderr  # read back, not tuned again
    bar = 1e-12 if form == "fp64" else 1e-6
    for r in (r1, r2):
        err = float([ln for ln in r.stdout.splitlines() if ln.startswith("MAXERR")][0].split()[1])
        assert err <= bar, err
