"""Host check of the double <-> double-float conversions the kernels use
(ig_arith.cuh compiled with g++): accuracy across the per-line scale window
and outside it, double subnormals, signed zeros, infinities and NaN."""
import os
import shutil
import subprocess
import tempfile

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_conversions_across_scales():
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "arith_check")
        subprocess.run([gxx, "-O2", "-std=c++17", "-o", exe, os.path.join(HERE, "arith_check.cpp")], check=True)
        out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    rows = [ln.split() for ln in out.splitlines() if ln.strip()]
    assert len(rows) == 11 + 1 + 7 + 1
    for name, err, limit in rows:
        assert float(err) <= float(limit), (name, err, limit)
