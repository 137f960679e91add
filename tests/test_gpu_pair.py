"""GPU parity of the FP32 paired-lane line kernel (k_fft_pair: two butterflies
per thread in the lanes of the f32x2 instructions), the default FP32 path for
complex lines and even real lines (halfcomplex out) of 512 points and more
whose plan starts with an even radix.  Cases cover both last-stage kinds, the
real split's pair edges (M divisible by 4 and M = 2 mod 4), the 7/11 radix
class, line distances longer than the line, output starts that are not
16-byte aligned (the engine then takes k_fft_line) and a backward complex
transform; every result is checked against the FP64 oracle at 1e-6 log2 N."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def tol(n):
    return 1e-6 * max(1.0, np.log2(n))


@pytest.mark.parametrize("n", [1024, 1100, 1200, 1232, 1280, 1680, 4096, 6144, 8192, 10000, 16384])
@pytest.mark.parametrize("dist_pad", [0, 6])
def test_pair_halfcomplex(engine, oracle_lib, n, dist_pad):
    import ctypes as C
    import torch
    from impulse_gb300 import _lib as L
    b = 23
    dist = n + dist_pad
    rng = np.random.default_rng(n + dist_pad)
    host = rng.standard_normal((b, dist)).astype(np.float32)
    x = torch.from_numpy(host).cuda()
    y = torch.zeros_like(x)
    plan = engine.ig_make_rfft_plan(n, L.IG_F32)
    s = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    L.check(engine.ig_rfft_exec_device(plan, x.data_ptr(), y.data_ptr(), b, dist, dist, 1, 0.25, s))
    torch.cuda.synchronize()
    engine.ig_destroy_rfft_plan(plan)
    got = y.cpu().numpy()[:, :n].astype(np.float64)
    want = oracle_lib.rfft_hc(host[:, :n].astype(np.float64), forward=True, fct=0.25)
    assert oracle_lib.rel_l2(got, want) < tol(n), n


@pytest.mark.parametrize("n", [512, 1000, 1024, 2048, 4096, 5040, 8192])
@pytest.mark.parametrize("fwd", [1, 0])
@pytest.mark.parametrize("out_off", [0, 1])
def test_pair_complex(engine, oracle_lib, n, fwd, out_off):
    import ctypes as C
    import torch
    from impulse_gb300 import _lib as L
    b = 9
    rng = np.random.default_rng(7 * n + fwd)
    host = (rng.standard_normal((b, n)) + 1j * rng.standard_normal((b, n))).astype(np.complex64)
    x = torch.from_numpy(host).cuda()
    # out_off = 1: output lines start 8 bytes past a 16-byte boundary
    ybuf = torch.zeros(b * n + 1, dtype=torch.complex64, device="cuda")
    y = ybuf[out_off:out_off + b * n]
    plan = engine.ig_make_cfft_plan(n, L.IG_F32)
    s = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    L.check(engine.ig_cfft_exec_device(plan, x.data_ptr(), y.data_ptr(), b, n, n, fwd, 0.5, s))
    torch.cuda.synchronize()
    engine.ig_destroy_cfft_plan(plan)
    got = y.cpu().numpy().reshape(b, n)
    want = oracle_lib.cfft(host.astype(np.complex128), bool(fwd), 0.5)
    assert oracle_lib.rel_l2(got, want) < tol(n), n


@pytest.mark.parametrize("shape,axes", [((33, 4096), [1]), ((7, 1000), [1]), ((5, 96), [1]), ((3, 6144), [1]),
                                        ((4, 5, 2048), [2]), ((64, 512), [0, 1]), ((2, 40, 256), [1, 2])])
@pytest.mark.parametrize("fwd", [True, False])
def test_r2c_half_spectrum_f32(engine, oracle_lib, shape, axes, fwd):
    """pocketfft::r2c FP32 with an even contiguous last axis: the half-spectrum
    split of the paired-lane kernel (last axes of 1024+ points) or of the line
    kernel (shorter ones); DC and Nyquist imaginary parts 0, conjugated for a
    backward transform."""
    from impulse_gb300 import fft as F
    rng = np.random.default_rng(sum(shape) + fwd)
    x = rng.standard_normal(shape).astype(np.float32)
    got = F.r2c(x, axes, forward=fwd, fct=0.5)
    want = oracle_lib.r2c(x.astype(np.float64), axes, forward=fwd, fct=0.5)
    assert oracle_lib.rel_l2(got, want) < tol(max(shape)) * 2, (shape, axes, fwd)
    last = got.reshape(-1, got.shape[-1]) if axes[-1] == len(shape) - 1 else None
    if last is not None and len(axes) == 1:
        assert np.all(last[:, 0].imag == 0) and np.all(last[:, -1].imag == 0)


@pytest.mark.parametrize("shape,axes", [((33, 4096), [1]), ((7, 1000), [1]), ((5, 96), [1]), ((3, 6144), [1]),
                                        ((4, 5, 2048), [2]), ((64, 512), [0, 1]), ((2, 40, 256), [1, 2])])
@pytest.mark.parametrize("fwd", [True, False])
def test_c2r_half_spectrum_f32(engine, oracle_lib, shape, axes, fwd):
    """pocketfft::c2r FP32 with an even contiguous last axis: the line kernel
    with the Hermitian pre-step read straight from HBM (DC and Nyquist
    imaginary parts ignored, input conjugated for a forward c2r)."""
    from impulse_gb300 import fft as F
    rng = np.random.default_rng(sum(shape) + 3 * fwd)
    hs = list(shape)
    hs[axes[-1]] = shape[axes[-1]] // 2 + 1
    x = (rng.standard_normal(hs) + 1j * rng.standard_normal(hs)).astype(np.complex64)
    got = F.c2r(x, shape, axes, forward=fwd, fct=0.25)
    want = oracle_lib.c2r(x.astype(np.complex128), shape, axes, forward=fwd, fct=0.25)
    assert oracle_lib.rel_l2(got, want) < tol(max(shape)) * 2, (shape, axes, fwd)
