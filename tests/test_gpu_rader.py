"""GPU parity of prime lengths computed with Rader's algorithm: in one CTA
(M - 1 fits the shared-memory kernel) and over a multi-pass core of length
M - 1; complex lines, even real lines of length 2M, paired odd real lines,
both directions, several lines per CTA, magnitudes far from 1."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

F64_TOL = 1e-12


def f32_tol(n):
    return 2e-6 * max(1.0, np.log2(max(n, 2)))


PRIMES_ONE_CTA = [17, 19, 23, 29, 31, 61, 101, 211, 421, 1009, 2003, 4049]
PRIMES_MULTI = [8191, 12289, 65521, 100003]


@pytest.mark.parametrize("n", PRIMES_ONE_CTA + PRIMES_MULTI)
@pytest.mark.parametrize("dtype", [np.complex128, np.complex64])
def test_rader_c2c(engine, oracle_lib, n, dtype):
    from impulse_gb300 import fft as F
    rng = np.random.default_rng(n)
    b = 5 if n < 5000 else 2
    x = (rng.standard_normal((b, n)) + 1j * rng.standard_normal((b, n))).astype(dtype)
    tol = F64_TOL if dtype == np.complex128 else f32_tol(n)
    for fwd in (True, False):
        got = F.cfft_batch(x, forward=fwd, fct=0.75)
        want = oracle_lib.cfft(x.astype(np.complex128), forward=fwd, fct=0.75)
        assert oracle_lib.rel_l2(got, want) < tol, (n, fwd, oracle_lib.rel_l2(got, want))


@pytest.mark.parametrize("n", PRIMES_ONE_CTA + PRIMES_MULTI)
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_rader_real_paired_and_even(engine, oracle_lib, n, dtype):
    from impulse_gb300 import fft as F
    rng = np.random.default_rng(n + 7)
    tol = F64_TOL if dtype == np.float64 else f32_tol(n)
    for length in (n, 2 * n):  # odd prime: paired lines; 2p: even split over a prime core
        x = rng.standard_normal((3, length)).astype(dtype)
        hc = F.rfft_batch(x, forward=True, fct=1.0)
        want = oracle_lib.rfft_hc(x.astype(np.float64), forward=True)
        assert oracle_lib.rel_l2(hc, want) < tol, (length, oracle_lib.rel_l2(hc, want))
        back = F.rfft_batch(hc, forward=False, fct=1.0 / length)
        assert oracle_lib.rel_l2(back, x.astype(np.float64)) < 2 * tol, length


@pytest.mark.parametrize("n", [101, 8191])
def test_rader_range_scaling(engine, oracle_lib, n):
    from impulse_gb300 import fft as F
    rng = np.random.default_rng(3)
    for scale in (1e-250, 1e250):
        x = (rng.standard_normal((2, n)) + 1j * rng.standard_normal((2, n))) * scale
        got = F.cfft_batch(x, forward=True, fct=1.0)
        want = oracle_lib.cfft(x, forward=True, fct=1.0)
        assert oracle_lib.rel_l2(got, want) < F64_TOL, (n, scale)


def test_rader_nd_prime_axis(engine, oracle_lib):
    from impulse_gb300 import fft as F
    rng = np.random.default_rng(11)
    x = rng.standard_normal((6, 1009)) + 1j * rng.standard_normal((6, 1009))
    for axes in ([1], [0, 1]):
        got = F.c2c(x, axes, forward=True)
        want = oracle_lib.c2c(x, axes, forward=True)
        assert oracle_lib.rel_l2(got, want) < F64_TOL, axes
    y = rng.standard_normal((8191, 3))
    got = F.r2c(y, [0], forward=True)
    want = oracle_lib.r2c(y, [0], forward=True)
    assert oracle_lib.rel_l2(got, want) < F64_TOL


def test_noalloc_rejects_multipass_rader(engine):
    torch = pytest.importorskip("torch")
    from impulse_gb300 import _lib as L
    lib = L.load()
    plan = lib.ig_make_cfft_plan(65521, L.IG_F64)
    try:
        x = torch.zeros((1, 65521), dtype=torch.complex128, device="cuda")
        rc = lib.ig_cfft_exec_device_noalloc(plan, x.data_ptr(), x.data_ptr(), 1, 65521, 65521, 1, 1.0, None)
        assert rc == L.IG_EINVAL
        assert b"multi-pass" in lib.ig_last_error_string()
    finally:
        lib.ig_destroy_cfft_plan(plan)
