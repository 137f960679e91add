"""GPU parity of the row-convolution mode of the shared-memory kernel: the
convolution of Rader and Bluestein over a multi-pass core runs as three
passes over a four-step core (columns forward with the twiddle; per row the
forward FFT, the table product, the inverse FFT and the inverse twiddle;
columns inverse) or as one launch over a one-CTA core.  Prime lengths whose
M - 1 is smooth (Rader: 8191, 12289, 65521) and lengths with a large prime
factor (Bluestein: 10007 = prime with 10006 not smooth, 2 x 10007 real),
complex and real lines, both directions, FP64 (double-float) and FP32, are
checked against the FP64 oracle, and against the same calls with the mode off
(IG_NO_ROWCONV=1 in a child process)."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def tol(dtype, n):
    return 1e-12 if dtype in (np.complex128, np.float64) else 2e-6 * max(1.0, np.log2(n))


@pytest.mark.parametrize("n", [8191, 10007, 12289, 65521])
@pytest.mark.parametrize("dtype", [np.complex128, np.complex64])
def test_rowconv_c2c(engine, oracle_lib, n, dtype):
    from impulse_gb300 import fft as F
    rng = np.random.default_rng(n + 1)
    x = (rng.standard_normal((3, n)) + 1j * rng.standard_normal((3, n))).astype(dtype)
    for fwd in (True, False):
        got = F.cfft_batch(x, forward=fwd, fct=0.5)
        want = oracle_lib.cfft(x.astype(np.complex128), forward=fwd, fct=0.5)
        assert oracle_lib.rel_l2(got, want) < tol(dtype, n), (n, fwd, oracle_lib.rel_l2(got, want))


@pytest.mark.parametrize("length", [8191, 16382, 10007, 20014, 65521])
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_rowconv_real(engine, oracle_lib, length, dtype):
    from impulse_gb300 import fft as F
    rng = np.random.default_rng(length)
    x = rng.standard_normal((4, length)).astype(dtype)
    hc = F.rfft_batch(x, forward=True, fct=1.0)
    want = oracle_lib.rfft_hc(x.astype(np.float64), forward=True)
    assert oracle_lib.rel_l2(hc, want) < tol(dtype, length)
    back = F.rfft_batch(hc, forward=False, fct=1.0 / length)
    assert oracle_lib.rel_l2(back, x.astype(np.float64)) < 2 * tol(dtype, length)


CHILD = r"""
import json, sys
import numpy as np
sys.path.insert(0, sys.argv[1])
from impulse_gb300 import fft as F
out = {}
for n in (8191, 10007, 65521):
    rng = np.random.default_rng(n)
    x = rng.standard_normal((2, n)) + 1j * rng.standard_normal((2, n))
    y = F.cfft_batch(x, forward=True, fct=1.0)
    out[str(n)] = [y.real[:, ::61].tolist(), y.imag[:, ::61].tolist()]
print(json.dumps(out))
"""


def test_rowconv_matches_four_passes(engine):
    outs = []
    for extra in ({}, {"IG_NO_ROWCONV": "1"}):
        env = dict(os.environ)
        env.pop("IG_NO_ROWCONV", None)
        env.update(extra)
        r = subprocess.run([sys.executable, "-c", CHILD, ROOT], capture_output=True, text=True, env=env, timeout=600)
        assert r.returncode == 0, r.stderr[-2000:]
        outs.append(json.loads(r.stdout.strip().splitlines()[-1]))
    for n in outs[0]:
        a = np.asarray(outs[0][n][0]) + 1j * np.asarray(outs[0][n][1])
        b = np.asarray(outs[1][n][0]) + 1j * np.asarray(outs[1][n][1])
        assert np.linalg.norm(a - b) / np.linalg.norm(b) < 1e-13, n


@pytest.mark.parametrize("shape,axes,dtype", [((8191, 3), [0], np.complex128), ((3, 8191), [1], np.complex128),
                                              ((10007, 2), [0], np.complex64), ((2, 65521), [1], np.complex64),
                                              ((65521, 2), [0], np.complex128)])
def test_rowconv_nd_axes(engine, oracle_lib, shape, axes, dtype):
    """The row-convolution plans through the N-d interface: prime axes along
    the strided and the contiguous dimension, both directions."""
    from impulse_gb300 import fft as F
    rng = np.random.default_rng(sum(shape))
    x = (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(dtype)
    for fwd in (True, False):
        got = F.c2c(x, axes, forward=fwd, fct=0.5)
        want = oracle_lib.c2c(x.astype(np.complex128), axes, forward=fwd, fct=0.5)
        assert oracle_lib.rel_l2(got, want) < tol(dtype, max(shape)), (shape, axes, fwd)


@pytest.mark.parametrize("shape,dtype", [((4, 8191), np.float64), ((3, 65521), np.float32), ((2, 2 * 10007), np.float64)])
def test_rowconv_r2c_c2r(engine, oracle_lib, shape, dtype):
    """r2c / c2r with a prime (or twice a prime) last axis: the half spectrum
    through Rader / Bluestein over multi-pass cores, and back."""
    from impulse_gb300 import fft as F
    rng = np.random.default_rng(shape[-1])
    x = rng.standard_normal(shape).astype(dtype)
    spec = F.r2c(x, [1], forward=True)
    want = oracle_lib.r2c(x.astype(np.float64), [1], forward=True)
    assert oracle_lib.rel_l2(spec, want) < tol(dtype, shape[-1])
    back = F.c2r(spec, shape, [1], forward=False, fct=1.0 / shape[-1])
    assert oracle_lib.rel_l2(back, x.astype(np.float64)) < 2 * tol(dtype, shape[-1])
