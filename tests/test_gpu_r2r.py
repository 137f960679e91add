"""GPU parity of the real-to-real transforms against the oracle (pinned to the
reference's dct / dst / r2r_fftpack / Hartley golden vectors): DCT / DST types
1-4 with and without ortho, every r2r_fftpack direction pair, separable and
genuine Hartley, host and device entry points, N-d strided views, errors."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LENGTHS = [2, 3, 4, 5, 8, 9, 16, 31, 100, 101, 1009, 4096, 6000]


def tol(dtype, n):
    return 1e-12 if dtype == np.float64 else 3e-6 * max(1.0, np.log2(n))


@pytest.mark.parametrize("sine", [False, True])
@pytest.mark.parametrize("t", [1, 2, 3, 4])
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_dct_dst_lines(engine, oracle_lib, sine, t, dtype):
    from impulse_gb300 import fft as F
    rng = np.random.default_rng(10 * t + sine)
    for n in LENGTHS:
        x = rng.standard_normal((3, n)).astype(dtype)
        for ortho in (False, True):
            f = F.dst if sine else F.dct
            got = f(x, [1], t, 0.5, ortho)
            want = oracle_lib.dct(x.astype(np.float64), [1], t, 0.5, ortho, sine=sine)
            assert oracle_lib.rel_l2(got, want) < tol(dtype, n), (n, ortho, oracle_lib.rel_l2(got, want))


def test_dct_nd_strided_and_inplace(engine, oracle_lib):
    from impulse_gb300 import fft as F
    rng = np.random.default_rng(3)
    base = rng.standard_normal((12, 40, 18))
    x = base[::2, :, 1:17]  # strided view
    for t in (1, 2, 3, 4):
        got = F.dct(x, [0, 2], t, 1.0, True)
        want = oracle_lib.dct(np.ascontiguousarray(x), [0, 2], t, 1.0, True)
        assert oracle_lib.rel_l2(got, want) < 1e-12, t
    y = np.ascontiguousarray(base)
    want = oracle_lib.dct(y, [1, 0], 2, 2.0, False, sine=True)
    F.dst(y, [1, 0], 2, 2.0, False, out=y)  # in place
    assert oracle_lib.rel_l2(y, want) < 1e-12


def test_dct_desc_apply(engine, oracle_lib):
    from impulse_gb300 import fft as F
    rng = np.random.default_rng(4)
    x = rng.standard_normal((16, 24))
    out = np.empty_like(x)
    F.apply(F.DCTDesc([0, 1], dctType=3, ortho=True, scalingFactor=0.25), F.DataDesc(out, out.shape), F.DataDesc(x, x.shape))
    assert oracle_lib.rel_l2(out, oracle_lib.dct(x, [0, 1], 3, 0.25, True)) < 1e-12


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_r2r_fftpack_and_hartley(engine, oracle_lib, dtype):
    from impulse_gb300 import fft as F
    rng = np.random.default_rng(5)
    x = rng.standard_normal((6, 30, 17)).astype(dtype)
    xd = x.astype(np.float64)
    for h in (False, True):
        for fwd in (False, True):
            got = F.r2r_fftpack(x, [1, 2], h, fwd, 0.5)
            want = oracle_lib.r2r_fftpack(xd, [1, 2], h, fwd, 0.5)
            assert oracle_lib.rel_l2(got, want) < tol(dtype, 30), (h, fwd)
    for axes in ([2], [1, 2], [0, 1, 2]):
        for genuine in (False, True):
            got = F.hartley(x, axes, 0.5, genuine)
            want = oracle_lib.hartley(xd, axes, 0.5, genuine)
            assert oracle_lib.rel_l2(got, want) < tol(dtype, 30), (axes, genuine)


def test_r2r_device_entry_points(engine, oracle_lib):
    torch = pytest.importorskip("torch")
    import ctypes as C
    from impulse_gb300 import _lib as L
    from impulse_gb300 import fft as F
    lib = L.load()
    rng = np.random.default_rng(6)
    x = rng.standard_normal((64, 4096))
    X = torch.from_numpy(x).cuda()
    Y = torch.empty_like(X)
    head = F._nd_head(L.IG_F64, x.shape, (8 * 4096, 8), (8 * 4096, 8), [1])
    L.check(lib.ig_dct_device(*head, 2, X.data_ptr(), Y.data_ptr(), 1.0, 0, None))
    torch.cuda.synchronize()
    assert oracle_lib.rel_l2(Y.cpu().numpy(), oracle_lib.dct(x, [1], 2)) < 1e-12
    L.check(lib.ig_r2r_hartley_device(*head, 1, X.data_ptr(), Y.data_ptr(), 1.0, None))
    torch.cuda.synchronize()
    assert oracle_lib.rel_l2(Y.cpu().numpy(), oracle_lib.hartley(x, [1])) < 1e-12


def test_r2r_errors(engine):
    from impulse_gb300 import _lib as L
    from impulse_gb300 import fft as F
    x = np.zeros((3, 1))
    with pytest.raises(L.FFTError, match="zero-length FFT requested"):
        F.dct(x, [1], 1)
    with pytest.raises(L.FFTError, match="invalid DCT type"):
        F.dct(np.zeros((2, 4)), [1], 5)
    with pytest.raises(L.FFTError, match="invalid DST type"):
        F.dst(np.zeros((2, 4)), [1], 0)
    with pytest.raises(L.FFTError, match="bad axis number"):
        F.hartley(np.zeros((2, 4)), [2])
