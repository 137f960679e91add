"""GPU parity of the differentiable FFT convolution and the real-transform adjoints.

Forward against direct convolution (scipy) and against the same FFT pipeline
built from the oracle's PocketFFT restatement; gradients against the analytic
correlation form, against the oracle-built FFT gradient, and against FP64
central finite differences at 64x64 with 7x7 filters."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
signal = pytest.importorskip("scipy.signal")


def _oracle_conv(O, x, k, P):
    """FFT convolution through the oracle's r2c / c2r (the reference's algorithm)."""
    B, H, W = x.shape
    K = k.shape[-1]
    c = (K - 1) // 2
    xp = np.zeros((B, P[0], P[1]))
    xp[:, :H, :W] = x
    kp = np.zeros((k.shape[0], P[0], P[1]))
    kp[:, :K, :K] = k
    Z = O.r2c(xp, [1, 2]) * O.r2c(kp, [1, 2])
    z = O.c2r(Z, (B, P[0], P[1]), [1, 2], False, 1.0 / (P[0] * P[1]))
    return z[:, c:c + H, c:c + W]


@pytest.mark.parametrize("nf", [1, 3])
def test_conv_forward_f64(engine, oracle_lib, nf):
    from impulse_gb300.fftconv import FFTConv2d
    rng = np.random.default_rng(5)
    x = rng.uniform(0, 1, (3, 64, 64))
    k = rng.standard_normal((nf, 7, 7))
    k /= np.abs(k).sum(axis=(1, 2), keepdims=True)
    op = FFTConv2d(3, 64, 64, 7, nf, torch.float64)
    y = op.forward(torch.from_numpy(x).cuda(), torch.from_numpy(k).cuda()).cpu().numpy()
    direct = np.stack([signal.convolve2d(x[b], k[b % nf], mode="same") for b in range(3)])
    assert oracle_lib.rel_l2(y, direct) < 1e-12
    assert oracle_lib.rel_l2(y, _oracle_conv(oracle_lib, x, k if nf == 3 else np.repeat(k, 3, 0), op.padded)) < 1e-12


@pytest.mark.parametrize("nf", [1, 3])
@pytest.mark.parametrize("recompute", [True, False])
def test_conv_gradients_f64(engine, oracle_lib, nf, recompute):
    from impulse_gb300.fftconv import FFTConv2d
    rng = np.random.default_rng(6)
    x = rng.uniform(0, 1, (3, 64, 64))
    k = rng.standard_normal((nf, 7, 7))
    g = rng.standard_normal((3, 64, 64))
    op = FFTConv2d(3, 64, 64, 7, nf, torch.float64, recompute=recompute)
    X, Kt, G = (torch.from_numpy(a).cuda() for a in (x, k, g))
    op.forward(X, Kt)
    gx, gk = op.backward(G)
    gx, gk = gx.cpu().numpy(), gk.cpu().numpy()
    # analytic: gx = correlate(g, k) 'same'; gk[p, q] = sum_ij g[i, j] x[i + c - p, j + c - q]
    gx_ref = np.stack([signal.correlate2d(g[b], k[b % nf], mode="same") for b in range(3)])
    assert oracle_lib.rel_l2(gx, gx_ref) < 1e-12
    c = 3
    xpad = np.pad(x, ((0, 0), (c, c), (c, c)))
    gk_b = np.stack([signal.correlate2d(xpad[b], g[b], mode="valid")[::-1, ::-1] for b in range(3)])
    gk_ref = gk_b.sum(0, keepdims=True) if nf == 1 else gk_b
    assert oracle_lib.rel_l2(gk, gk_ref) < 1e-12
    # central finite differences in FP64 along random directions
    def loss(xx, kk):
        o = FFTConv2d(3, 64, 64, 7, nf, torch.float64)
        return float((o.forward(torch.from_numpy(xx).cuda(), torch.from_numpy(kk).cuda()).cpu().numpy() * g).sum())
    eps = 1e-4
    vx = rng.standard_normal(x.shape)
    vk = rng.standard_normal(k.shape)
    fd_x = (loss(x + eps * vx, k) - loss(x - eps * vx, k)) / (2 * eps)
    fd_k = (loss(x, k + eps * vk) - loss(x, k - eps * vk)) / (2 * eps)
    assert abs(fd_x - (gx * vx).sum()) <= 1e-8 * abs(fd_x) + 1e-9
    assert abs(fd_k - (gk * vk).sum()) <= 1e-8 * abs(fd_k) + 1e-9


def test_conv_autograd_and_f32(engine):
    from impulse_gb300.fftconv import fftconv2d
    rng = np.random.default_rng(7)
    x64 = torch.from_numpy(rng.uniform(0, 1, (2, 256, 256))).cuda().requires_grad_(True)
    k64 = torch.from_numpy(rng.standard_normal((1, 31, 31))).cuda().requires_grad_(True)
    y64 = fftconv2d(x64, k64)
    (y64 * y64).sum().backward()
    x32 = x64.detach().float().requires_grad_(True)
    k32 = k64.detach().float().requires_grad_(True)
    y32 = fftconv2d(x32, k32)
    (y32 * y32).sum().backward()
    rel = lambda a, b: float(torch.linalg.vector_norm(a.detach().double() - b.detach()) / torch.linalg.vector_norm(b.detach()))
    tol = 1e-6 * np.log2(512) * 4
    assert rel(y32, y64.detach()) < tol
    assert rel(x32.grad, x64.grad) < tol
    assert rel(k32.grad, k64.grad) < tol


@pytest.mark.parametrize("shape,axes", [((16,), [0]), ((6, 10), [1]), ((6, 10), [0, 1]), ((4, 5, 9), [0, 2])])
@pytest.mark.parametrize("forward", [True, False])
def test_real_transform_adjoints(engine, shape, axes, forward):
    """<r2c(x), G>_R = <x, r2c_adj(G)> and <c2r(Y), y> = <Y, c2r_adj(y)>_R (dot-product tests)."""
    from impulse_gb300 import fft as F
    from impulse_gb300.fftconv import c2r_adjoint, r2c_adjoint
    rng = np.random.default_rng(len(shape) + sum(shape))
    x = rng.standard_normal(shape)
    hshape = list(shape)
    hshape[axes[-1]] = hshape[axes[-1]] // 2 + 1
    G = rng.standard_normal(hshape) + 1j * rng.standard_normal(hshape)
    lhs = np.sum((F.r2c(x, axes, forward) * np.conj(G)).real)
    xa = r2c_adjoint(torch.from_numpy(G).cuda(), shape, axes, forward).cpu().numpy()
    rhs = np.sum(x * xa)
    assert abs(lhs - rhs) <= 1e-12 * max(1.0, abs(lhs))
    y = rng.standard_normal(shape)
    # c2r output y_c = c2r(G): <c2r(G), y> = <G, c2r_adj(y)>_R
    lhs2 = np.sum(F.c2r(G, shape, axes, forward) * y)
    Ga = c2r_adjoint(torch.from_numpy(y).cuda(), axes, forward).cpu().numpy()
    rhs2 = np.sum((G * np.conj(Ga)).real)
    assert abs(lhs2 - rhs2) <= 1e-11 * max(1.0, abs(lhs2))


@pytest.mark.parametrize("shape,axes", [((16,), [0]), ((6, 10), [1]), ((6, 10), [0, 1]), ((4, 5, 9), [0, 2]),
                                        ((3, 4096), [1]), ((97, 5), [0])])
@pytest.mark.parametrize("forward", [True, False])
def test_c2c_adjoint(engine, shape, axes, forward):
    """<c2c(x), G>_R = <x, c2c_adj(G)>_R (dot-product test), FP64 and FP32."""
    from impulse_gb300 import fft as F
    from impulse_gb300.fftconv import c2c_adjoint
    rng = np.random.default_rng(len(shape) + sum(shape) + int(forward))
    x = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    G = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    fct = 0.25
    lhs = np.sum((F.c2c(x, axes, forward, fct) * np.conj(G)).real)
    xa = c2c_adjoint(torch.from_numpy(G).cuda(), axes, forward, fct).cpu().numpy()
    rhs = np.sum((x * np.conj(xa)).real)
    assert abs(lhs - rhs) <= 1e-12 * max(1.0, abs(lhs))
    xa32 = c2c_adjoint(torch.from_numpy(G.astype(np.complex64)).cuda(), axes, forward, fct).cpu().numpy()
    n = int(np.prod([shape[a] for a in axes]))
    assert np.linalg.norm(xa32 - xa) / np.linalg.norm(xa) < 1e-6 * max(1.0, np.log2(n))
