"""GPU parity of the device-resident API (impulse_gb300.device): the Nim
interface's DataDesc / apply and Tensor overloads over CUDA tensors, on a
caller's stream, against the oracle."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

F64_TOL = 1e-12


def _cuda(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def test_apply_c2c_r2c_c2r_on_a_stream(engine, oracle_lib):
    from impulse_gb300 import device as D
    rng = np.random.default_rng(11)
    x = rng.uniform(-1, 1, (6, 10, 7)) + 1j * rng.uniform(-1, 1, (6, 10, 7))
    s = torch.cuda.Stream()
    xi = _cuda(x)
    xo = torch.empty_like(xi)
    D.apply(D.FFTDesc([0, 2], True, 0.5), D.DataDesc(xo, x.shape), D.DataDesc(xi, x.shape), stream=s)
    s.synchronize()
    want = oracle_lib.c2c(x, [0, 2], True, 0.5)
    assert oracle_lib.rel_l2(xo.cpu().numpy(), want) < F64_TOL

    r = rng.uniform(-1, 1, (8, 6, 5))
    ri = _cuda(r)
    co = torch.empty((8, 6, 3), dtype=torch.complex128, device="cuda")
    D.apply(D.FFTDesc([0, 2], True, 1.0), D.DataDesc(co, co.shape), D.DataDesc(ri, r.shape), stream=s)
    s.synchronize()
    assert oracle_lib.rel_l2(co.cpu().numpy(), oracle_lib.r2c(r, [0, 2], True, 1.0)) < F64_TOL
    # c2r takes the descriptors' shapes as the reference's apply passes them (descIn.shape)
    back = torch.empty((8, 6, 5), dtype=torch.float64, device="cuda")
    desc_in = D.DataDesc(co, (8, 6, 5), [18, 3, 1])
    D.apply(D.FFTDesc([0, 2], False, 1.0 / 40), D.DataDesc(back, back.shape), desc_in, stream=s)
    s.synchronize()
    assert oracle_lib.rel_l2(back.cpu().numpy(), r) < 1e-12


def test_apply_strided_views_and_dct(engine, oracle_lib):
    from impulse_gb300 import device as D
    rng = np.random.default_rng(12)
    big = rng.uniform(-1, 1, (16, 24)) + 1j * rng.uniform(-1, 1, (16, 24))
    g = _cuda(big)
    view = g[::2, 1::3]  # (8, 8) view, strides (48, 3) elements
    out = torch.zeros((8, 8), dtype=torch.complex128, device="cuda")
    D.apply(D.FFTDesc([0, 1], False, 1.0), D.DataDesc.of(out), D.DataDesc.of(view))
    torch.cuda.synchronize()
    want = oracle_lib.c2c(big[::2, 1::3], [0, 1], False, 1.0)
    assert oracle_lib.rel_l2(out.cpu().numpy(), want) < F64_TOL
    xr = rng.standard_normal((4, 6, 5))
    xi = _cuda(xr)
    yo = torch.empty_like(xi)
    D.apply(D.DCTDesc([0, 2], 2, True), D.DataDesc(yo, xr.shape), D.DataDesc(xi, xr.shape))
    torch.cuda.synchronize()
    assert oracle_lib.rel_l2(yo.cpu().numpy(), oracle_lib.dct(xr, [0, 2], 2, 1.0, True)) < F64_TOL


@pytest.mark.parametrize("n", [4, 5, 96, 1009, 4096, 18144])
def test_tensor_overloads(engine, oracle_lib, n):
    """pocketfft_arraymancer.nim:25-94 on CUDA tensors: normalize honoured."""
    from impulse_gb300 import device as D
    from impulse_gb300 import fft as F
    rng = np.random.default_rng(n)
    x = rng.standard_normal(n)
    t = _cuda(x)
    s = torch.cuda.Stream()
    for kind in (F.nkBackward, F.nkOrtho, F.nkForward):
        fct = oracle_lib.init_normalize(int(kind), True, 0.0, n)
        want_hc = oracle_lib.rfft_hc(x, True, fct)
        hc = D.tensor_rfft_packed(t, True, kind, stream=s)
        s.synchronize()
        assert oracle_lib.rel_l2(hc.cpu().numpy(), want_hc) < F64_TOL
        u = D.tensor_rfft(t, True, kind, stream=s)
        s.synchronize()
        assert oracle_lib.rel_l2(u.cpu().numpy(), oracle_lib.unpack_fft(want_hc)) < F64_TOL
        full = D.tensor_fft(t, True, kind, stream=s)
        s.synchronize()
        assert oracle_lib.rel_l2(full.cpu().numpy(), oracle_lib.symmetrize(want_hc)) < F64_TOL
    z = x + 1j * rng.standard_normal(n)
    tz = _cuda(z)
    back = D.tensor_ifft(D.tensor_fft(tz, True), True)
    torch.cuda.synchronize()
    assert oracle_lib.rel_l2(back.cpu().numpy(), z) < F64_TOL
    # the Hermitian half of a complex half spectrum (symmTargetSize reads the last element)
    u = oracle_lib.unpack_fft(oracle_lib.rfft_hc(x, True, 1.0))
    assert oracle_lib.rel_l2(D.symmetrize(_cuda(u)).cpu().numpy(), oracle_lib.symmetrize(u)) < F64_TOL


def test_rows_with_gaps_f32(engine, oracle_lib):
    from impulse_gb300 import device as D
    rng = np.random.default_rng(13)
    n, rows, dist = 2205, 9, 2205 + 11
    x = rng.standard_normal((rows, dist)).astype(np.float32)
    t = _cuda(x)
    D.rfft_rows(t[:, :n], True, 1.0)
    torch.cuda.synchronize()
    y = t.cpu().numpy()
    want = oracle_lib.rfft_hc(x[:, :n].astype(np.float64), True, 1.0)
    assert oracle_lib.rel_l2(y[:, :n], want) < 2e-6 * np.log2(n)
    assert np.array_equal(y[:, n:], x[:, n:])

