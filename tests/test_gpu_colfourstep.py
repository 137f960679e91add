"""GPU parity of the strided-axis four-step (FP32 columns of 2048+ points: two
passes with the columns as the fastest line index, scratch laid out column
by column) against the FP64 oracle: axis 0 of 2-D arrays with 32+ columns
(even and odd counts), a strided axis inside a 3-D array (a second batch
dimension), reversed views, forward and backward with a scale, r2c / c2r over
both axes (the half-spectrum columns), and the same calls with the path off
(IG_NO_COL_FOURSTEP=1 in a child process) giving results within the same
bound."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rand(rng, shape):
    return (rng.uniform(-1, 1, shape) + 1j * rng.uniform(-1, 1, shape)).astype(np.complex64)


def tol(n):
    return 2e-6 * max(1.0, np.log2(n))


@pytest.mark.parametrize("shape,axes", [((4096, 64), [0]), ((2048, 33), [0]), ((4096, 40), [0, 1]),
                                        ((3, 4096, 48), [1]), ((3, 2048, 36), [1, 2]), ((6144, 32), [0])])
@pytest.mark.parametrize("fwd", [True, False])
def test_col_fourstep_c2c(engine, oracle_lib, shape, axes, fwd):
    from impulse_gb300 import fft as F
    rng = np.random.default_rng(sum(shape) + len(axes))
    x = _rand(rng, shape)
    got = F.c2c(x, axes, forward=fwd, fct=0.5)
    want = oracle_lib.c2c(x.astype(np.complex128), axes, forward=fwd, fct=0.5)
    assert oracle_lib.rel_l2(got, want) < tol(max(shape)), (shape, axes, fwd)


def test_col_fourstep_reversed(engine, oracle_lib):
    from impulse_gb300 import fft as F
    rng = np.random.default_rng(5)
    x = _rand(rng, (4096, 34))[::-1, ::-1]
    got = F.c2c(x, [0], forward=True)
    assert oracle_lib.rel_l2(got, oracle_lib.c2c(x.astype(np.complex128), [0])) < tol(4096)


def test_col_fourstep_r2c_c2r(engine, oracle_lib):
    from impulse_gb300 import fft as F
    rng = np.random.default_rng(6)
    x = rng.standard_normal((4096, 128)).astype(np.float32)
    spec = F.r2c(x, [0, 1], forward=True)
    want = oracle_lib.r2c(x.astype(np.float64), [0, 1], forward=True)
    assert oracle_lib.rel_l2(spec, want) < tol(4096)
    back = F.c2r(spec, x.shape, [0, 1], forward=False, fct=1.0 / x.size)
    assert oracle_lib.rel_l2(back, x) < tol(4096)


CHILD = r"""
import json, sys
import numpy as np
sys.path.insert(0, sys.argv[1])
from impulse_gb300 import fft as F
rng = np.random.default_rng(9)
x = (rng.uniform(-1, 1, (4096, 64)) + 1j * rng.uniform(-1, 1, (4096, 64))).astype(np.complex64)
y = F.c2c(x, [0], forward=True)
print(json.dumps({"re": y.real.ravel()[::97].tolist(), "im": y.imag.ravel()[::97].tolist()}))
"""


def test_col_fourstep_matches_single_pass(engine):
    outs = []
    for extra in ({}, {"IG_NO_COL_FOURSTEP": "1"}):
        env = dict(os.environ)
        env.pop("IG_NO_COL_FOURSTEP", None)
        env.update(extra)
        r = subprocess.run([sys.executable, "-c", CHILD, ROOT], capture_output=True, text=True, env=env, timeout=600)
        assert r.returncode == 0, r.stderr[-2000:]
        d = json.loads(r.stdout.strip().splitlines()[-1])
        outs.append(np.asarray(d["re"]) + 1j * np.asarray(d["im"]))
    a, b = outs
    assert np.linalg.norm(a - b) / np.linalg.norm(b) < tol(4096)
