import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libgbfft.so")


def rel_l2(got, ref):
    import numpy as np
    got = np.asarray(got)
    ref = np.asarray(ref)
    den = np.linalg.norm(ref)
    return float(np.linalg.norm(got - ref) / (den if den > 0 else 1.0))


def assert_fp64_close(got, ref, log2n, what=""):
    """FP64 bar: rel-L2 <= 1e-12 and max-abs <= 1e-12 * ||ref||_inf * log2 N."""
    import numpy as np
    got = np.asarray(got, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    e = rel_l2(got, ref)
    assert e <= 1e-12, "%s rel-L2 %.3e > 1e-12" % (what, e)
    bound = 1e-12 * max(np.abs(ref).max(), 1e-300) * max(log2n, 1)
    ma = float(np.abs(got - ref).max()) if got.size else 0.0
    assert ma <= bound, "%s max-abs %.3e > %.3e" % (what, ma, bound)
