"""CPU check of the integer-pipe float/double conversions (csrc/conv.cuh)
against the compiler's own conversions: d2f and f2d bit for bit, the
double-float split and join within their stated bounds."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_conversions_match_ieee(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    exe = str(tmp_path / "conv_check")
    subprocess.run([gxx, "-O2", "-std=c++17", "-ffp-contract=off",
                    "-I", os.path.join(ROOT, "numrs_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "conv_check.cpp"), "-o", exe], check=True)
    out = subprocess.run([exe, "1000000"], capture_output=True, text=True)
    assert out.returncode == 0 and out.stdout.strip() == "ok", out.stdout
