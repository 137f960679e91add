"""GPU parity of upfirdn (impulse signal.nim:545-594) and the explicit-filter
resample against the oracle's direct sums (pinned to the known answers of the
reference's upfirdn documentation, tests/test_oracle.py)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("n,nh,up,down", [(1, 1, 1, 1), (5, 3, 1, 1), (100, 31, 3, 2), (1000, 64, 1, 4),
                                          (4096, 257, 2, 3), (20000, 1001, 5, 7), (3, 7, 4, 1)])
def test_upfirdn_matches_oracle(engine, oracle_lib, dtype, n, nh, up, down):
    from impulse_gb300 import signal as S
    rng = np.random.default_rng(n + nh)
    t = rng.standard_normal((4, n)).astype(dtype)
    h = rng.standard_normal(nh).astype(dtype)
    got = S.upfirdn(t, h, up, down)
    want = oracle_lib.upfirdn(t.astype(np.float64), h.astype(np.float64), up, down)
    tol = 1e-12 if dtype == np.float64 else 2e-6 * np.log2(n * up + nh + 2)
    assert got.shape == want.shape
    assert oracle_lib.rel_l2(got, want) < tol, oracle_lib.rel_l2(got, want)


def test_upfirdn_known_answers(engine):
    from impulse_gb300 import signal as S
    np.testing.assert_allclose(S.upfirdn(np.array([1.0, 1, 1]), [1.0, 1, 1]), [1, 2, 3, 2, 1], atol=1e-12)
    np.testing.assert_allclose(S.upfirdn(np.arange(10.0), [0.5, 1.0, 0.5], 2, 3), [0, 1, 2.5, 4, 5.5, 7, 8.5],
                               atol=1e-12)


def test_resample_with_filter(engine, oracle_lib):
    from impulse_gb300 import signal as S
    rng = np.random.default_rng(1)
    t = rng.standard_normal(1000)
    h = rng.standard_normal(61)
    up, down = S.reduce_resampling_rates(6, 4)
    got = S.resample(t, h, up, down)
    hh, delay = S.adjust_filter_position(h, t.size, int(np.ceil(t.size * up / down)), up, down)
    want = oracle_lib.upfirdn(t, hh, up, down)[0][delay:delay + got.size]
    assert got.size == int(np.ceil(t.size * up / down))
    assert oracle_lib.rel_l2(got, want) < 1e-12


def test_upfirdn_device_and_errors(engine, oracle_lib):
    torch = pytest.importorskip("torch")
    import ctypes as C
    from impulse_gb300 import _lib as L
    lib = L.load()
    rng = np.random.default_rng(2)
    x = rng.standard_normal((3, 500))
    h = rng.standard_normal(40)
    ny = C.c_size_t()
    L.check(lib.ig_upfirdn_length(500, 40, 2, 3, C.byref(ny)))
    X, Hd = torch.from_numpy(x).cuda(), torch.from_numpy(h).cuda()
    Y = torch.empty((3, ny.value), dtype=torch.float64, device="cuda")
    L.check(lib.ig_upfirdn_device(L.IG_F64, 3, 500, X.data_ptr(), 500, 40, Hd.data_ptr(), 2, 3, Y.data_ptr(),
                                  ny.value, None))
    torch.cuda.synchronize()
    assert oracle_lib.rel_l2(Y.cpu().numpy(), oracle_lib.upfirdn(x, h, 2, 3)) < 1e-12
    assert lib.ig_upfirdn_length(10, 3, 0, 1, C.byref(ny)) == L.IG_EINVAL
