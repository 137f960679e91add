"""GPU parity: complex transforms (pocketfft cfft_forward/backward, pocketfft::c2c) vs the oracle."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

F64_TOL = 1e-12   # relative L2, FP64 path (double-float butterflies)


def f32_tol(n):
    return 1e-6 * max(1.0, np.log2(max(n, 2)))


def _rand(rng, shape, dtype=np.complex128):
    x = rng.uniform(-1, 1, shape) + 1j * rng.uniform(-1, 1, shape)
    return x.astype(dtype)


SMALL = list(range(1, 70)) + [77, 96, 100, 121, 125, 127, 128, 243, 256, 343, 500, 512, 625, 720, 1000,
                               1009, 1024, 1331, 2025, 2048, 2310, 4096, 4913, 8191, 8192]


@pytest.mark.parametrize("n", SMALL)
def test_cfft_f64_matches_oracle(engine, oracle_lib, n):
    from impulse_gb300 import fft as F
    rng = np.random.default_rng(n)
    x = _rand(rng, (3, n))
    for fwd in (True, False):
        got = F.cfft_batch(x, forward=fwd, fct=0.5)
        want = oracle_lib.cfft(x, forward=fwd, fct=0.5)
        assert oracle_lib.rel_l2(got, want) < F64_TOL, (n, fwd, oracle_lib.rel_l2(got, want))


@pytest.mark.parametrize("n", [1, 2, 3, 5, 7, 11, 16, 60, 64, 97, 256, 1000, 1009, 4096, 8192])
def test_cfft_f32_matches_oracle(engine, oracle_lib, n):
    from impulse_gb300 import fft as F
    rng = np.random.default_rng(100 + n)
    x = _rand(rng, (5, n), np.complex64)
    for fwd in (True, False):
        got = F.cfft_batch(x, forward=fwd)
        want = oracle_lib.cfft(x.astype(np.complex128), forward=fwd)
        assert oracle_lib.rel_l2(got, want) < f32_tol(n), (n, fwd)


def test_cfft_single_plan_api(engine, oracle_lib):
    """ig_cfft_forward / ig_cfft_backward on one host line (pocketfft.h:22-23)."""
    from impulse_gb300 import fft as F
    rng = np.random.default_rng(7)
    for n in (1, 4, 5, 48, 4096):
        x = _rand(rng, n)
        y = x.copy()
        F.fft_impl(y, n, True)
        assert oracle_lib.rel_l2(y, oracle_lib.cfft(x)) < F64_TOL
        F.fft_impl(y, n, False)  # nkBackward: 1/n on the inverse
        assert oracle_lib.rel_l2(y, x) < F64_TOL


def test_known_answer_arange4(engine):
    """tests/test_fft2.nim:7-15 (complex and real input)."""
    from impulse_gb300 import fft as F
    expected = np.array([6, -2 + 2j, -2, -2 - 2j])
    assert np.allclose(F.tensor_fft(np.arange(4.0).astype(np.complex128)), expected, rtol=0, atol=1e-15)
    assert np.allclose(F.tensor_fft(np.arange(4.0)), expected, rtol=0, atol=1e-15)
    r = F.tensor_ifft(F.tensor_fft(np.arange(4.0)))
    assert np.allclose(r.real, np.arange(4.0), atol=1e-15) and np.allclose(r.imag, 0, atol=1e-15)
    assert np.allclose(F.tensor_fft(np.arange(4.0), normalize=F.nkForward), expected / 4, atol=1e-15)
    assert np.allclose(F.tensor_fft(np.arange(4.0), normalize=F.nkOrtho), expected / 2, atol=1e-15)
    assert np.allclose(F.tensor_ifft(np.arange(4.0)), F.tensor_fft(np.arange(4.0), forward=False), atol=1e-15)


def test_roundtrip_config1_small(engine):
    """c128 N=4096 forward then backward with 1/N returns the input within 1e-10."""
    from impulse_gb300 import fft as F
    rng = np.random.default_rng(1)
    x = _rand(rng, (64, 4096))
    y = F.cfft_batch(F.cfft_batch(x, True), False, 1.0 / 4096)
    assert np.max(np.abs(y - x)) < 1e-10


def test_f64_range_scaling(engine, oracle_lib):
    """FP64 lines far outside the float range keep FP64-level accuracy (per-line power-of-two scaling)."""
    from impulse_gb300 import fft as F
    rng = np.random.default_rng(3)
    for scale in (1e-300, 1e-200, 1e-30, 1e30, 1e200, 1e300):
        x = _rand(rng, (2, 256)) * scale
        got = F.cfft_batch(x, True)
        want = oracle_lib.cfft(x, True)
        assert oracle_lib.rel_l2(got, want) < F64_TOL, scale
