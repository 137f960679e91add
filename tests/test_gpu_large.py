"""GPU parity for lengths beyond one CTA's shared memory: four-step cores and
Bluestein over a four-step core (lengths with a large prime factor)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

F64_TOL = 1e-12


def _dtype_code(dtype):
    from impulse_gb300 import _lib as L
    return L.IG_F64 if dtype == np.float64 else L.IG_F32


def f32_tol(n):
    return 1e-6 * max(1.0, np.log2(max(n, 2)))


@pytest.mark.parametrize("n", [8191, 9973, 10000, 12288, 16384, 32768, 65521, 65536, 131072, 1 << 20])
@pytest.mark.parametrize("dtype", [np.complex128, np.complex64])
def test_cfft_large(engine, oracle_lib, n, dtype):
    from impulse_gb300 import fft as F
    rng = np.random.default_rng(n)
    b = 2 if n <= 131072 else 1
    x = (rng.uniform(-1, 1, (b, n)) + 1j * rng.uniform(-1, 1, (b, n))).astype(dtype)
    tol = F64_TOL if dtype == np.complex128 else f32_tol(n) * 2
    for fwd in (True, False):
        got = F.cfft_batch(x, forward=fwd, fct=0.5)
        want = oracle_lib.cfft(x.astype(np.complex128), forward=fwd, fct=0.5)
        assert oracle_lib.rel_l2(got, want) < tol, (n, fwd, oracle_lib.rel_l2(got, want))


@pytest.mark.parametrize("n", [16382, 16386, 19998, 20000, 32768, 40960, 65521, 65536, 8191 * 3])
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_rfft_halfcomplex_large(engine, oracle_lib, n, dtype):
    from impulse_gb300 import fft as F
    rng = np.random.default_rng(n + 1)
    x = rng.standard_normal((2, n)).astype(dtype)
    tol = F64_TOL if dtype == np.float64 else f32_tol(n) * 2
    hc = F.rfft_batch(x, forward=True, fct=1.0)
    want = oracle_lib.rfft_hc(x.astype(np.float64), forward=True)
    assert oracle_lib.rel_l2(hc, want) < tol, (n, oracle_lib.rel_l2(hc, want))
    back = F.rfft_batch(hc, forward=False, fct=1.0 / n)
    assert oracle_lib.rel_l2(back, x.astype(np.float64)) < 2 * tol, n


@pytest.mark.parametrize("shape,axes", [((3, 40000), [1]), ((2, 3, 65521), [2]), ((20000, 3), [0]),
                                        ((4, 16384), [0, 1])])
def test_r2c_c2r_large(engine, oracle_lib, shape, axes):
    from impulse_gb300 import fft as F
    rng = np.random.default_rng(sum(shape))
    x = rng.uniform(-1, 1, shape)
    for fwd in (True, False):
        got = F.r2c(x, axes, forward=fwd)
        want = oracle_lib.r2c(x, axes, forward=fwd)
        assert oracle_lib.rel_l2(got, want) < F64_TOL, (shape, axes, fwd)
        back = F.c2r(got, shape, axes, forward=fwd, fct=0.5)
        want_b = oracle_lib.c2r(want, shape, axes, forward=fwd, fct=0.5)
        assert oracle_lib.rel_l2(back, want_b) < F64_TOL, (shape, axes, fwd)


def test_c2c_large_strided_axis(engine, oracle_lib):
    from impulse_gb300 import fft as F
    rng = np.random.default_rng(5)
    x = rng.uniform(-1, 1, (32768, 4)) + 1j * rng.uniform(-1, 1, (32768, 4))
    got = F.c2c(x, [0], True, 1.0)
    assert oracle_lib.rel_l2(got, oracle_lib.c2c(x, [0])) < F64_TOL


@pytest.mark.parametrize("n,dist", [(18144, 18144 + 8), (30800, 30800 + 7), (20000, 20000)])
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_halfcomplex_fourstep_gaps(engine, oracle_lib, n, dist, dtype):
    """Even four-step lengths whose real split is fused into the row pass,
    written as halfcomplex into lines `dist` apart (gaps left untouched)."""
    from impulse_gb300 import _lib as L
    from impulse_gb300 import fft as F
    rng = np.random.default_rng(n + dist)
    batch = 5
    x = rng.standard_normal((batch, dist)).astype(dtype)
    h = x.copy()
    plan = F.FFTPlanReal(n, _dtype_code(dtype))
    L.check(L.load().ig_rfft_exec_batch(plan.pocket, h.ctypes.data, batch, dist, 1, 0.5))
    tol = F64_TOL if dtype == np.float64 else f32_tol(n) * 2
    want = oracle_lib.rfft_hc(x[:, :n].astype(np.float64), True, 0.5)
    assert oracle_lib.rel_l2(h[:, :n], want) < tol, (n, dist, oracle_lib.rel_l2(h[:, :n], want))
    assert np.array_equal(h[:, n:], x[:, n:])


@pytest.mark.parametrize("n", [4096, 2205, 18144, 29403])
def test_halfcomplex_range_scaling(engine, oracle_lib, n):
    """Real lines far outside the float range, with different magnitudes in one
    batch (and in one pair of lines for odd lengths): single-CTA, paired,
    fused four-step split and paired four-step paths keep FP64 accuracy."""
    from impulse_gb300 import fft as F
    rng = np.random.default_rng(n + 7)
    scales = np.array([1e300, 1e-300, 1.0, 1e-200, 1e250, 3.0])[:, None]
    x = rng.standard_normal((6, n)) * scales
    hc = F.rfft_batch(x, True, 1.0)
    want = oracle_lib.rfft_hc(x, True, 1.0)
    for r in range(6):
        assert oracle_lib.rel_l2(hc[r], want[r]) < F64_TOL, (n, r)
    back = F.rfft_batch(hc, False, 1.0 / n)
    for r in range(6):
        assert oracle_lib.rel_l2(back[r], x[r]) < 2 * F64_TOL, (n, r)


@pytest.mark.parametrize("n", [65521, 8191, 29403, 4096, 2205, 18144])
def test_halfcomplex_range_scaling_rader_and_odd_multipass(engine, oracle_lib, n):
    """Rader lines (65521 over a multi-pass core, 8191) and an odd four-step
    length, with rows at 1e300, 1e-300 and double-subnormal 1e-310 paired in
    one batch, in both directions: the paired-line gather rescales each line by
    its own exponent, including the negated second line of the backward Rader
    direction and its kept x[0]."""
    from impulse_gb300 import fft as F
    rng = np.random.default_rng(n + 11)
    scales = np.array([1e300, 1e-300, 1e-310, 1.0, 1e-310, 1e300, 1e-300])[:, None]
    x = rng.standard_normal((7, n)) * scales

    def scaled_oracle(a, forward, fct):
        # the oracle on each row brought to unit magnitude by an exact power of
        # two, its result scaled back with one rounding (FP64 arithmetic on
        # subnormal rows would lose the oracle's own accuracy)
        out = np.empty_like(a)
        for r in range(a.shape[0]):
            e = -int(np.floor(np.log2(np.max(np.abs(a[r])))))
            out[r] = np.ldexp(oracle_lib.rfft_hc(np.ldexp(a[r], e), forward, fct), -e)
        return out

    hc = F.rfft_batch(x, True, 1.0)
    want = scaled_oracle(x, True, 1.0)
    for r in range(7):
        assert oracle_lib.rel_l2(hc[r], want[r]) < F64_TOL, (n, r, "forward")
    spec = want.copy()
    back = F.rfft_batch(spec, False, 1.0 / n)
    want_b = scaled_oracle(spec, False, 1.0 / n)
    for r in range(7):
        assert oracle_lib.rel_l2(back[r], want_b[r]) < F64_TOL, (n, r, "backward")


@pytest.mark.parametrize("n", [4096, 1000, 2048, 65536])
def test_complex_range_scaling_subnormal_rows(engine, oracle_lib, n):
    """Complex lines of double subnormals (and huge ones) next to unit lines:
    every line keeps FP64 accuracy (single-CTA line kernel and four-step)."""
    from impulse_gb300 import fft as F
    rng = np.random.default_rng(n + 5)
    scales = np.array([1e-310, 1.0, 1e300, 1e-309, 3e-308])[:, None]
    z = (rng.standard_normal((5, n)) + 1j * rng.standard_normal((5, n))) * scales
    for fwd in (True, False):
        got = F.cfft_batch(z, fwd, 1.0)
        for r in range(5):
            e = -int(np.floor(np.log2(np.max(np.abs(z[r])))))
            want = oracle_lib.cfft(np.ldexp(z[r].real, e) + 1j * np.ldexp(z[r].imag, e), fwd, 1.0)
            want = np.ldexp(want.real, -e) + 1j * np.ldexp(want.imag, -e)
            assert oracle_lib.rel_l2(got[r], want) < F64_TOL, (n, r, fwd)
