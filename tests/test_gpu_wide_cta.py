"""GPU parity of 8-element cores longer than 4096 points: CTAs of more than
512 threads (up to 672; 4097-5376-point lines, one double-buffered line per
CTA).  Such plans come only from tuning, so a child process loads a tune
table that forces 8 elements a thread on cores of 4160 (radix 13, the full
class), 4200, 5000, 5145 and 5376 points, in FP64 (double-float) and FP32,
and transforms complex lines (both directions), even real lines (halfcomplex,
core 5000 of length 10000) and odd real lines (5145, two lines per complex
line); the parent checks every result against the FP64 oracle."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CORES = [4160, 4200, 5000, 5145, 5376]

CHILD = r"""
import json, sys
import numpy as np
sys.path.insert(0, sys.argv[1])
from impulse_gb300 import _lib as L
from impulse_gb300 import fft as F
tmp = sys.argv[2]
F.autotune(96, L.IG_F64, 0)
F.autotune(96, L.IG_F32, 1)
F.autotune_save(tmp + "/seed.tsv")
rows = [r.split("\t") for r in open(tmp + "/seed.tsv").read().strip().splitlines()]
name = rows[0][0]
arith = sorted({r[1] for r in rows})
lines = [f"{name}\t{a}\t{m}\t0\t8\t0\t0\t0\t1.0" for a in arith for m in json.loads(sys.argv[3])]
open(tmp + "/force.tsv", "w").write("\n".join(lines) + "\n")
F.autotune_load(tmp + "/force.tsv")
out = {}
for n in json.loads(sys.argv[3]):
    rng = np.random.default_rng(n)
    x = rng.standard_normal((3, n)) + 1j * rng.standard_normal((3, n))
    for dt, cdt in (("f64", np.complex128), ("f32", np.complex64)):
        for fwd in (True, False):
            y = F.cfft_batch(x.astype(cdt), forward=fwd, fct=0.5)
            np.save(f"{tmp}/c{n}{dt}{int(fwd)}.npy", y)
for n in (10000, 5145):
    x = np.random.default_rng(n).standard_normal((4, n))
    for dt, rdt in (("f64", np.float64), ("f32", np.float32)):
        np.save(f"{tmp}/r{n}{dt}.npy", F.rfft_batch(x.astype(rdt), True, 1.0))
print("ok")
"""


def test_wide_e8_cores_match_oracle(engine, oracle_lib, tmp_path):
    r = subprocess.run([sys.executable, "-c", CHILD, ROOT, str(tmp_path), json.dumps(CORES)], capture_output=True,
                       text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-3000:]
    for n in CORES:
        x = np.random.default_rng(n)
        x = x.standard_normal((3, n)) + 1j * x.standard_normal((3, n))
        for dt in ("f64", "f32"):
            tol = 1e-12 if dt == "f64" else 2e-6 * np.log2(n)
            for fwd in (True, False):
                got = np.load(tmp_path / f"c{n}{dt}{int(fwd)}.npy")
                src = x if dt == "f64" else x.astype(np.complex64).astype(np.complex128)
                want = oracle_lib.cfft(src, forward=fwd, fct=0.5)
                assert oracle_lib.rel_l2(got, want) < tol, (n, dt, fwd)
    for n in (10000, 5145):
        x = np.random.default_rng(n).standard_normal((4, n))
        for dt in ("f64", "f32"):
            tol = 1e-12 if dt == "f64" else 2e-6 * np.log2(n)
            src = x if dt == "f64" else x.astype(np.float32).astype(np.float64)
            got = np.load(tmp_path / f"r{n}{dt}.npy")
            assert oracle_lib.rel_l2(got, oracle_lib.rfft_hc(src, True, 1.0)) < tol, (n, dt)
