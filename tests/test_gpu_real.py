"""GPU parity: real transforms -- halfcomplex rfft_forward/backward (C backend) and
pocketfft::r2c / c2r (C++ backend) -- vs the oracle."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

F64_TOL = 1e-12


def f32_tol(n):
    return 1e-6 * max(1.0, np.log2(max(n, 2)))


LENGTHS = list(range(1, 130)) + [160, 192, 243, 250, 256, 343, 384, 500, 512, 625, 999, 1000, 1009, 1024,
                                  1210, 2048, 2310, 4050, 4096, 6561, 8192, 9240, 16384]


@pytest.mark.parametrize("n", LENGTHS)
def test_rfft_halfcomplex_f64(engine, oracle_lib, n):
    from impulse_gb300 import fft as F
    rng = np.random.default_rng(n)
    x = rng.standard_normal((3, n))
    hc = F.rfft_batch(x, forward=True, fct=1.0)
    want = oracle_lib.rfft_hc(x, forward=True)
    assert oracle_lib.rel_l2(hc, want) < F64_TOL, n
    back = F.rfft_batch(hc, forward=False, fct=1.0 / n)
    want_b = oracle_lib.rfft_hc(want, forward=False, fct=1.0 / n)
    assert oracle_lib.rel_l2(back, want_b) < F64_TOL, n
    assert oracle_lib.rel_l2(back, x) < F64_TOL, n


@pytest.mark.parametrize("n", [1, 2, 3, 4, 5, 6, 7, 8, 9, 15, 16, 17, 64, 100, 101, 1009, 4096, 8192])
def test_rfft_halfcomplex_f32(engine, oracle_lib, n):
    from impulse_gb300 import fft as F
    rng = np.random.default_rng(1000 + n)
    x = rng.standard_normal((4, n)).astype(np.float32)
    hc = F.rfft_batch(x, forward=True)
    want = oracle_lib.rfft_hc(x.astype(np.float64), forward=True)
    assert oracle_lib.rel_l2(hc, want) < f32_tol(n), n
    back = F.rfft_batch(hc, forward=False, fct=1.0 / n)
    assert oracle_lib.rel_l2(back, x.astype(np.float64)) < 2 * f32_tol(n), n


def test_readme_halfcomplex_n5(engine):
    """README.md:41 -- rfft_forward of [1, 2, 1, -1, 1.5]."""
    from impulse_gb300 import fft as F
    x = np.array([1.0, 2.0, 1.0, -1.0, 1.5])
    got = F.rfft_packed(x)
    want = np.array([4.5, 2.081559480312316, -1.651098762732523, -1.831559480312316, 1.608220406444071])
    assert np.allclose(got, want, rtol=0, atol=1e-14)
    full = F.fft(x)
    assert np.allclose(full[:3], [4.5, 2.081559480312316 - 1.651098762732523j,
                                  -1.831559480312316 + 1.608220406444071j], atol=1e-14)
    assert np.allclose(full[3:], np.conj(full[1:3][::-1]), atol=0)
    assert np.allclose(F.fft(full, forward=False), x, atol=1e-14)


@pytest.mark.parametrize("shape,axes", [((5,), [0]), ((8, 6), [1]), ((8, 6), [0]), ((8, 6), [0, 1]),
                                        ((8, 6), [1, 0]), ((6, 10, 7), [2]), ((6, 10, 7), [0, 2]),
                                        ((6, 10, 7), [0, 1, 2]), ((4, 9, 5), [1]), ((32, 64), [0, 1])])
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_r2c_c2r_nd(engine, oracle_lib, shape, axes, dtype):
    from impulse_gb300 import fft as F
    rng = np.random.default_rng(sum(shape))
    x = rng.uniform(-1, 1, shape).astype(dtype)
    tol = F64_TOL if dtype == np.float64 else f32_tol(max(shape)) * 2
    for fwd in (True, False):
        got = F.r2c(x, axes, forward=fwd, fct=0.5)
        want = oracle_lib.r2c(x.astype(np.float64), axes, forward=fwd, fct=0.5)
        assert oracle_lib.rel_l2(got, want) < tol, (shape, axes, fwd)
        back = F.c2r(got, shape, axes, forward=fwd, fct=0.25)
        want_b = oracle_lib.c2r(want, shape, axes, forward=fwd, fct=0.25)
        assert oracle_lib.rel_l2(back, want_b) < tol, (shape, axes, fwd)


def test_cpp_readme_r2c(engine):
    """README.md:79-98 / pocketfft.nim:300-320: apply() r2c of [1, 2, 1, -1, 1.5] into a length-5 buffer."""
    from impulse_gb300 import fft as F
    dIn = np.array([1.0, 2.0, 1.0, -1.0, 1.5])
    dOut = np.zeros(5, np.complex128)
    F.apply(F.FFTDesc([0], True), F.DataDesc(dOut, [5]), F.DataDesc(dIn, [5]))
    want = [4.5, 2.081559480312316 - 1.651098762732523j, -1.831559480312316 + 1.608220406444071j, 0, 0]
    assert np.allclose(dOut, want, atol=1e-14)


@pytest.mark.parametrize("n", [5, 101, 1009, 2205, 6075, 8191, 29403, 65521])
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_odd_lengths_paired_lines_keep_own_accuracy(engine, oracle_lib, n, dtype):
    """Odd real lengths run two lines per complex transform; each line keeps its
    own relative accuracy even when the two lines differ by many orders."""
    from impulse_gb300 import fft as F
    rng = np.random.default_rng(n)
    scales = np.array([1.0, 1e-9, 1e6, 1e-30 if dtype == np.float32 else 1e-250, 3.0])[:, None]
    x = (rng.standard_normal((5, n)) * scales).astype(dtype)
    tol = 1e-12 if dtype == np.float64 else 1e-6 * np.log2(n) * 2
    hc = F.rfft_batch(x, forward=True)
    back = F.rfft_batch(hc, forward=False, fct=1.0 / n)
    for i in range(5):
        want = oracle_lib.rfft_hc(x[i].astype(np.float64), True)
        assert oracle_lib.rel_l2(hc[i], want) < tol, (n, i)
        assert oracle_lib.rel_l2(back[i], x[i].astype(np.float64)) < 2 * tol, (n, i)
    # N-d r2c / c2r over an odd last axis pairs lines too
    y = rng.uniform(-1, 1, (7, n)).astype(dtype)
    got = F.r2c(y, [1], forward=False)
    want = oracle_lib.r2c(y.astype(np.float64), [1], forward=False)
    assert oracle_lib.rel_l2(got, want) < tol
    back2 = F.c2r(got, (7, n), [1], forward=True, fct=1.0 / n)
    want2 = oracle_lib.c2r(want, (7, n), [1], forward=True, fct=1.0 / n)
    assert oracle_lib.rel_l2(back2, want2) < 2 * tol
