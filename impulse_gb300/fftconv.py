"""Differentiable FFT convolution and real-transform adjoints over the GPU engine.

``FFTConv2d`` is a forward/backward object shaped like an autograd Function:
``forward(x, k)`` returns the 'same' 2-D convolution of a batch of images with
odd-sized filters (zero padded, r2c -> spectrum product -> c2r), and
``backward(gy)`` returns the gradients with respect to the images and the
filters, recomputing the spectra instead of storing them when
``recompute=True``.  ``fftconv2d`` wraps it as a ``torch.autograd.Function``.
All arithmetic runs in libimpulse_gpu.so (``ig_fftconv_*``); tensors are CUDA
tensors.  The reference has no counterpart (impulse's signal module convolves
directly, impulse/signal.nim:594); this is the FFT-domain form of that
operation with hand-written adjoints.
"""
from __future__ import annotations

import ctypes as C

import torch

from . import _lib as L


def _code(dt):
    if dt in (torch.float64, torch.complex128):
        return L.IG_F64
    if dt in (torch.float32, torch.complex64):
        return L.IG_F32
    raise TypeError(f"unsupported dtype {dt}")


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


class FFTConv2d:
    def __init__(self, batch, height, width, ksize, nfilters=1, dtype=torch.float32, recompute=True, pad=None):
        lib = L.load()
        self.shape = (batch, height, width)
        self.kshape = (nfilters, ksize, ksize)
        self.dtype = dtype
        pr, pc = pad if pad else (0, 0)
        self.h = lib.ig_fftconv_create(_code(dtype), batch, height, width, nfilters, ksize, pr, pc, int(recompute))
        if not self.h:
            raise L.FFTError(L.IG_EINVAL, lib.ig_last_error_string().decode())
        r, c = C.c_size_t(), C.c_size_t()
        L.check(lib.ig_fftconv_padded_size(self.h, C.byref(r), C.byref(c)))
        self.padded = (r.value, c.value)
        self.saved = None

    def __del__(self):
        if getattr(self, "h", None):
            L.load().ig_fftconv_destroy(self.h)
            self.h = None

    def forward(self, x, k):
        x = x.contiguous()
        k = k.contiguous()
        assert tuple(x.shape) == self.shape and tuple(k.shape) == self.kshape
        y = torch.empty_like(x)
        L.check(L.load().ig_fftconv_forward(self.h, x.data_ptr(), k.data_ptr(), y.data_ptr(), _stream()))
        self.saved = (x, k)
        return y

    def backward(self, gy, need_x=True, need_k=True):
        x, k = self.saved
        gy = gy.contiguous()
        gx = torch.empty_like(x) if need_x else None
        gk = torch.empty_like(k) if need_k else None
        L.check(L.load().ig_fftconv_backward(self.h, x.data_ptr(), k.data_ptr(), gy.data_ptr(),
                                             gx.data_ptr() if gx is not None else None,
                                             gk.data_ptr() if gk is not None else None, _stream()))
        return gx, gk


class _Fn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, k, op):
        ctx.op = op
        return op.forward(x.detach(), k.detach())

    @staticmethod
    def backward(ctx, gy):
        gx, gk = ctx.op.backward(gy, ctx.needs_input_grad[0], ctx.needs_input_grad[1])
        return gx, gk, None


def fftconv2d(x, k, recompute=True, pad=None):
    """'same' convolution of x [B, H, W] with k [1 or B, K, K], differentiable through torch.autograd."""
    op = FFTConv2d(x.shape[0], x.shape[1], x.shape[2], k.shape[-1], k.shape[0], x.dtype, recompute, pad)
    return _Fn.apply(x, k, op)


def _nd_args(x_shape, a, b, axes):
    return (len(x_shape), L.arr(C.c_size_t, x_shape), L.arr(C.c_ssize_t, [s * a.element_size() for s in a.stride()]),
            L.arr(C.c_ssize_t, [s * b.element_size() for s in b.stride()]), len(axes), L.arr(C.c_size_t, axes))


def c2c_adjoint(g, axes, forward=True, fct=1.0):
    """Adjoint of c2c(axes, forward, fct): x_bar from the complex gradient g (same shape)."""
    x = torch.empty_like(g)
    n, sh, sg, sx, na, ax = _nd_args(list(g.shape), g, x, list(axes))
    L.check(L.load().ig_c2c_adjoint_device(_code(g.dtype), n, sh, sg, sx, na, ax, int(forward), g.data_ptr(),
                                           x.data_ptr(), float(fct), _stream()))
    return x


def r2c_adjoint(g, shape_in, axes, forward=True, fct=1.0):
    """Adjoint of r2c(axes, forward): real x_bar of shape shape_in from the half-spectrum gradient g."""
    rdt = torch.float64 if g.dtype == torch.complex128 else torch.float32
    x = torch.empty(shape_in, dtype=rdt, device=g.device)
    n, sh, sg, sx, na, ax = _nd_args(list(shape_in), g, x, list(axes))
    L.check(L.load().ig_r2c_adjoint_device(_code(rdt), n, sh, sg, sx, na, ax, int(forward), g.data_ptr(),
                                           x.data_ptr(), float(fct), _stream()))
    return x


def c2r_adjoint(y, axes, forward=False, fct=1.0):
    """Adjoint of c2r(axes, forward): half-spectrum gradient from the real gradient y."""
    cdt = torch.complex128 if y.dtype == torch.float64 else torch.complex64
    shp = list(y.shape)
    shp[axes[-1]] = shp[axes[-1]] // 2 + 1
    g = torch.empty(shp, dtype=cdt, device=y.device)
    n, sh, sy, sg, na, ax = _nd_args(list(y.shape), y, g, list(axes))
    L.check(L.load().ig_c2r_adjoint_device(_code(y.dtype), n, sh, sy, sg, na, ax, int(forward), y.data_ptr(),
                                           g.data_ptr(), float(fct), _stream()))
    return g
