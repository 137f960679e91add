"""GPU tests of the native-FP64 arithmetic mode (ig_set_f64_arith(1)).

The default FP64 arithmetic is double-float (pairs of FP32 values, about
2^-48 per operation): it meets the 1e-12 relative-L2 bar of the parity tests
but not impulse's own acceptance bar.  impulse's tests/test_fft.nim:29-52
(test_real, after PocketFFT's ffttest.c:40-73) runs, for every real length
1..8191, rfft_forward then rfft_backward with fct = 1/length on uniform
[-0.5, 0.5] data and requires a round-trip relative L2 error of at most
2e-15.  The native-FP64 mode is the drop-in for that bar; these tests run the
same loop through the C ABI on the GPU.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

EPS_REF = 2e-15   # tests/test_fft.nim:32
MAXLEN = 8192     # tests/test_fft.nim:7


@pytest.fixture()
def native_f64(engine):
    lib = engine
    assert lib.ig_set_f64_arith(1) == 0
    try:
        yield lib
    finally:
        lib.ig_set_f64_arith(0)
        lib.ig_release_caches()


def _errcalc(data, odata):
    """tests/test_fft.nim:14-22: sqrt(sum (d - o)^2 / sum o^2)."""
    d = np.asarray(data, np.float64)
    o = np.asarray(odata, np.float64)
    return float(np.sqrt(np.sum((d - o) ** 2) / np.sum(o * o)))


def test_native_f64_real_round_trip_every_length(native_f64):
    """test_real: make_rfft_plan / rfft_forward / rfft_backward(1/length) / destroy for length 1..8191."""
    lib = native_f64
    rng = np.random.default_rng(20240)
    odata = rng.uniform(-0.5, 0.5, MAXLEN)
    odata[0] = 0.340188
    bad = []
    worst = 0.0
    for length in range(1, MAXLEN):
        data = odata[:length].copy()
        plan = lib.ig_make_rfft_plan(length, 0)
        assert plan, lib.ig_last_error_string()
        p = data.ctypes.data_as(C.c_void_p)
        assert lib.ig_rfft_forward(plan, p, 1.0) == 0
        assert lib.ig_rfft_backward(plan, p, 1.0 / length) == 0
        lib.ig_destroy_rfft_plan(plan)
        err = _errcalc(data, odata[:length])
        worst = max(worst, err)
        if err > EPS_REF:
            bad.append((length, err))
        if length % 1024 == 0:
            lib.ig_release_caches()
    assert not bad, f"{len(bad)} lengths above 2e-15, worst {worst:.3e}: {bad[:20]}"


def test_native_f64_openarray_round_trip(native_f64):
    """test_real_hl: fft(openArray, forward) then fft(openArray, backward) -- the
    openArray overload drops normalize, so the backward call scales by 1/length."""
    from impulse_gb300 import fft as F
    rng = np.random.default_rng(20241)
    odata = rng.uniform(-0.5, 0.5, MAXLEN)
    bad = []
    for length in list(range(1, 300)) + list(range(300, MAXLEN, 37)) + [4096, 8191]:
        data = odata[:length].copy()
        F.fft_inplace(data, True)
        F.fft_inplace(data, False)
        err = _errcalc(data, odata[:length])
        if err > EPS_REF:
            bad.append((length, err))
    assert not bad, bad[:20]


@pytest.mark.parametrize("n", [1, 2, 7, 16, 97, 1000, 1009, 4096, 8191, 65521, 100003, 1 << 20])
def test_native_f64_matches_oracle(native_f64, oracle_lib, n):
    """Forward and backward, complex and halfcomplex, against the FP64 oracle."""
    from impulse_gb300 import fft as F
    rng = np.random.default_rng(n)
    x = rng.standard_normal((2, n))
    got = F.rfft_batch(x, True)
    assert oracle_lib.rel_l2(got, oracle_lib.rfft_hc(x, True)) < 1e-14, n
    z = x + 1j * rng.standard_normal((2, n))
    got = F.cfft_batch(z, False, 0.5)
    assert oracle_lib.rel_l2(got, oracle_lib.cfft(z, False, 0.5)) < 1e-14, n


def test_native_f64_nd(native_f64, oracle_lib):
    from impulse_gb300 import fft as F
    rng = np.random.default_rng(5)
    x = rng.uniform(-1, 1, (64, 96)) + 1j * rng.uniform(-1, 1, (64, 96))
    assert oracle_lib.rel_l2(F.c2c(x, [0, 1]), oracle_lib.c2c(x, [0, 1])) < 1e-14
    r = rng.uniform(-1, 1, (30, 50))
    got = F.r2c(r, [0, 1])
    assert oracle_lib.rel_l2(got, oracle_lib.r2c(r, [0, 1])) < 1e-14
    back = F.c2r(got, (30, 50), [0, 1], forward=False, fct=1.0 / 1500)
    assert oracle_lib.rel_l2(back, r) < 1e-14
