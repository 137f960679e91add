"""GPU parity: N-d strided complex transforms (pocketfft::c2c via FFTDesc.apply) vs the oracle."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

F64_TOL = 1e-12


def _rand(rng, shape, dtype=np.complex128):
    return (rng.uniform(-1, 1, shape) + 1j * rng.uniform(-1, 1, shape)).astype(dtype)


@pytest.mark.parametrize("shape,axes", [((16,), [0]), ((8, 12), [0]), ((8, 12), [1]), ((8, 12), [0, 1]),
                                        ((8, 12), [1, 0]), ((5, 6, 7), [0, 1, 2]), ((5, 6, 7), [2, 0]),
                                        ((3, 4, 5, 6), [1, 3]), ((2, 3, 4, 5, 6), [0, 2, 4]),
                                        ((64, 48), [0, 1]), ((256, 32), [0])])
@pytest.mark.parametrize("dtype", [np.complex128, np.complex64])
def test_c2c_nd(engine, oracle_lib, shape, axes, dtype):
    from impulse_gb300 import fft as F
    rng = np.random.default_rng(len(shape) * 7 + sum(shape))
    x = _rand(rng, shape, dtype)
    tol = F64_TOL if dtype == np.complex128 else 1e-6 * np.log2(max(shape) * len(axes) + 2) * 2
    for fwd in (True, False):
        got = F.c2c(x, axes, forward=fwd, fct=0.125)
        want = oracle_lib.c2c(x.astype(np.complex128), axes, forward=fwd, fct=0.125)
        assert oracle_lib.rel_l2(got, want) < tol, (shape, axes, fwd)


def test_c2c_strided_views(engine, oracle_lib):
    """Non-contiguous input and output views; in place with equal strides."""
    from impulse_gb300 import fft as F
    rng = np.random.default_rng(11)
    big = _rand(rng, (20, 30))
    x = big[::2, 1::3]            # strided input view
    out_big = np.zeros((40, 20), np.complex128)
    out = out_big[::4, ::2]       # strided output view with gaps
    F.c2c(x, [0, 1], True, 1.0, out=out)
    assert oracle_lib.rel_l2(out, oracle_lib.c2c(x, [0, 1])) < F64_TOL
    # gaps untouched
    mask = np.ones_like(out_big, bool)
    mask[::4, ::2] = False
    assert np.all(out_big[mask] == 0)
    y = big.copy()
    F.c2c(y, [1], False, 2.0, out=y)  # in place
    assert oracle_lib.rel_l2(y, oracle_lib.c2c(big, [1], False, 2.0)) < F64_TOL


def test_c2c_negative_strides(engine, oracle_lib):
    from impulse_gb300 import fft as F
    rng = np.random.default_rng(12)
    x = _rand(rng, (12, 10))[::-1, ::-1]
    got = F.c2c(x, [0, 1], True)
    assert oracle_lib.rel_l2(got, oracle_lib.c2c(x, [0, 1])) < F64_TOL


def test_config1_shapes(engine, oracle_lib):
    """c128 N=4096 along a strided axis ([4096, 64], axes=[0]) and a contiguous one ([64, 4096], axes=[1])."""
    from impulse_gb300 import fft as F
    rng = np.random.default_rng(1)
    a = _rand(rng, (4096, 64))
    assert oracle_lib.rel_l2(F.c2c(a, [0]), oracle_lib.c2c(a, [0])) < F64_TOL
    b = _rand(rng, (64, 4096))
    assert oracle_lib.rel_l2(F.c2c(b, [1]), oracle_lib.c2c(b, [1])) < F64_TOL
