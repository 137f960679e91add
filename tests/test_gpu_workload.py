"""GPU parity of the timed workloads, at the sizes the benchmark times them.

* every length of the halfcomplex benchmark (rfft_forward layout,
  pocketfft.c:2184), FP64 and FP32, after autotuning (the tuned plans are the
  ones the benchmark times), through the entry point the benchmark calls
  (ig_rfft_exec_device, out of place), at the benchmark's full batch of about
  2^24 reals per length;
* 1-D complex transforms of length 4096 x 1024 lines (c128) along a strided
  axis (shape [4096, 1024], axes=[0]) and along a contiguous one
  ([1024, 4096], axes=[1]) through pocketfft::c2c's mirror
  (pocketfft_hdronly.h:3272): forward, then backward with fct = 1/4096, round
  trip within 1e-10 and each direction within 1e-12 of the oracle;
* multi-axis transforms: 4096 x 4096 c128 and c64 over axes [0, 1],
  256^3 c64 over axes [0, 1, 2], and the 4096 x 4096 f32 r2c over axes
  [0, 1] with its c2r (pocketfft_hdronly.h:3334, 3366).

Tolerances: FP64 1e-12 relative L2 against the FP64 oracle; FP32
1e-6 * log2(N) with N the product of the transformed lengths.
"""
import ctypes as C
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

F64_TOL = 1e-12


def f32_tol(n):
    return 1e-6 * max(1.0, math.log2(max(n, 2)))


def _uniform_c(rng, shape, dtype=np.complex128):
    return (rng.uniform(-1, 1, shape) + 1j * rng.uniform(-1, 1, shape)).astype(dtype)


def _bench():
    import bench
    return bench


@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_halfcomplex_workload_lengths_autotuned(engine, oracle_lib, dtype):
    """All benchmark lengths, tuned first, at the benchmark's batch, against the oracle."""
    import torch
    from impulse_gb300 import _lib as L
    from impulse_gb300 import fft as F
    B = _bench()
    code = L.IG_F64 if dtype == "f64" else L.IG_F32
    tdt = torch.float64 if dtype == "f64" else torch.float32
    lib = engine
    s = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    failures = []
    for n in B.workload_lengths():
        F.autotune(n, code, 1)
        b = B.batch_for(n)
        rng = np.random.default_rng(n)
        x = rng.standard_normal((b, n))
        xd = torch.from_numpy(x).to("cuda", dtype=tdt)
        yd = torch.empty_like(xd)
        plan = lib.ig_make_rfft_plan(n, code)
        assert plan, lib.ig_last_error_string()
        try:
            rc = lib.ig_rfft_exec_device(plan, xd.data_ptr(), yd.data_ptr(), b, n, n, 1, 1.0, s)
            assert rc == 0, lib.ig_last_error_string()
            torch.cuda.synchronize()
        finally:
            lib.ig_destroy_rfft_plan(plan)
        got = yd.double().cpu().numpy()
        want = oracle_lib.rfft_hc(xd.double().cpu().numpy(), True)
        err = oracle_lib.rel_l2(got, want)
        tol = F64_TOL if dtype == "f64" else f32_tol(n)
        if not err < tol:
            failures.append((n, err))
        del xd, yd
    assert not failures, failures


@pytest.mark.parametrize("layout", ["strided", "contiguous"])
def test_config1_full_size_round_trip(engine, oracle_lib, layout):
    """c128, N = 4096, 1024 lines; forward, then backward with fct = 1/4096."""
    from impulse_gb300 import fft as F
    rng = np.random.default_rng(1)
    if layout == "strided":
        x, axes = _uniform_c(rng, (4096, 1024)), [0]
    else:
        x, axes = _uniform_c(rng, (1024, 4096)), [1]
    # through the DataDesc / FFTDesc / apply mirror, as impulse's C++ backend calls it
    y = np.empty_like(x)
    F.apply(F.FFTDesc(axes, True), F.DataDesc(y, list(y.shape)), F.DataDesc(x, list(x.shape)))
    want = oracle_lib.c2c(x, axes, True)
    assert oracle_lib.rel_l2(y, want) < F64_TOL
    z = np.empty_like(x)
    F.apply(F.FFTDesc(axes, False, 1.0 / 4096), F.DataDesc(z, list(z.shape)), F.DataDesc(y, list(y.shape)))
    assert oracle_lib.rel_l2(z, oracle_lib.c2c(y, axes, False, 1.0 / 4096)) < F64_TOL
    assert oracle_lib.rel_l2(z, x) < 1e-10


@pytest.mark.parametrize("shape,axes,dtype", [
    ((4096, 4096), [0, 1], np.complex128),
    ((4096, 4096), [0, 1], np.complex64),
    ((256, 256, 256), [0, 1, 2], np.complex64),
])
def test_config3_c2c_full_size(engine, oracle_lib, shape, axes, dtype):
    from impulse_gb300 import fft as F
    rng = np.random.default_rng(3)
    x = _uniform_c(rng, shape, dtype)
    n = int(np.prod([shape[a] for a in axes]))
    tol = F64_TOL if dtype == np.complex128 else f32_tol(n)
    for fwd in (True, False):
        got = F.c2c(x, axes, forward=fwd)
        want = oracle_lib.c2c(x.astype(np.complex128), axes, forward=fwd)
        assert oracle_lib.rel_l2(got, want) < tol, fwd


def test_config3_r2c_c2r_full_size(engine, oracle_lib):
    """4096 x 4096 f32 r2c over axes [0, 1] (output 4096 x 2049 c64), then c2r back."""
    from impulse_gb300 import fft as F
    rng = np.random.default_rng(3)
    x = rng.uniform(-1, 1, (4096, 4096)).astype(np.float32)
    n = 4096 * 4096
    got = F.r2c(x, [0, 1], forward=True)
    assert got.shape == (4096, 2049) and got.dtype == np.complex64
    want = oracle_lib.r2c(x.astype(np.float64), [0, 1], forward=True)
    assert oracle_lib.rel_l2(got, want) < f32_tol(n)
    back = F.c2r(got, (4096, 4096), [0, 1], forward=False, fct=1.0 / n)
    want_b = oracle_lib.c2r(got.astype(np.complex128), (4096, 4096), [0, 1], forward=False, fct=1.0 / n)
    assert oracle_lib.rel_l2(back, want_b) < f32_tol(n)
    assert oracle_lib.rel_l2(back, x.astype(np.float64)) < 2 * f32_tol(n)
