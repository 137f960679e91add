"""Device-resident mirror of impulse's FFT interface: data in GPU memory
(torch CUDA tensors), every call enqueued on a CUDA stream.

The names and argument meanings are those of ``impulse_gb300.fft`` (the
restatement of impulse's Nim API, impulse/fft/c_pocketfft/pocketfft.nim,
pocketfft_arraymancer.nim and cpp_pocketfft/pocketfft.nim); only the memory
space differs, and each call takes an optional ``stream`` (a
``torch.cuda.Stream``, a raw ``cudaStream_t`` as int, or None for torch's
current stream).  No host copy is made: the transforms go through the
``*_device`` entry points of libimpulse_gpu.so, and the O(N) glue of the Nim
layer (``unpackFFT``, ``symmetrize``) runs as device gathers.

* ``DataDesc`` / ``apply`` -- cpp_pocketfft/pocketfft.nim:137-295 over device
  buffers (c2c, r2c, c2r with the reference's c2r shape quirk, and DCTDesc).
* ``tensor_fft_inplace``, ``tensor_rfft_packed``, ``tensor_rfft``,
  ``tensor_fft``, ``tensor_ifft`` -- pocketfft_arraymancer.nim:25-94
  (normalize honoured) on 1-d CUDA tensors.
* ``rfft_rows`` / ``cfft_rows`` -- every row of a 2-d CUDA tensor in one call
  (the batched form of the same 1-d transforms).
"""
from __future__ import annotations

import ctypes as C
import math

from . import _lib as L
from .fft import DCTDesc, FFTDesc, NormalizeKind, initNormalize, nkBackward  # noqa: F401

__all__ = ["DataDesc", "FFTDesc", "DCTDesc", "apply", "tensor_fft_inplace", "tensor_rfft_packed", "tensor_rfft",
           "tensor_fft", "tensor_ifft", "unpackFFT", "symmetrize", "symmTargetSize", "rfft_rows", "cfft_rows"]


def _torch():
    import torch
    return torch


def _check_cuda(*ts):
    for t in ts:
        if not (hasattr(t, "is_cuda") and t.is_cuda):
            raise TypeError("device API: buffers must be CUDA tensors (use impulse_gb300.fft for host arrays)")


def _dtype_code(t) -> int:
    torch = _torch()
    if t.dtype in (torch.float64, torch.complex128):
        return L.IG_F64
    if t.dtype in (torch.float32, torch.complex64):
        return L.IG_F32
    raise TypeError(f"unsupported dtype {t.dtype}")


def _stream_ptr(stream):
    torch = _torch()
    if stream is None:
        return C.c_void_p(torch.cuda.current_stream().cuda_stream)
    if isinstance(stream, int):
        return C.c_void_p(stream)
    return C.c_void_p(stream.cuda_stream)


def _on(stream):
    """Make `stream` torch's current stream for the duration (the device
    gathers of the glue and the transforms then run in stream order)."""
    import contextlib
    torch = _torch()
    if stream is None:
        return contextlib.nullcontext()
    if isinstance(stream, int):
        stream = torch.cuda.ExternalStream(stream)
    return torch.cuda.stream(stream)


class DataDesc:
    """DataDesc (pocketfft.nim:137-199) over a CUDA tensor: shape and BYTE strides.

    ``DataDesc(buf, shape)`` is the row-major constructor (pocketfft.nim:178);
    ``DataDesc(buf, shape, stride)`` takes element strides (pocketfft.nim:158-176).
    Offsets start at ``buf.data_ptr()``."""

    def __init__(self, buf, shape, stride=None):
        _check_cuda(buf)
        self.buf = buf
        self.shape = [int(s) for s in shape]
        isz = buf.element_size()
        if stride is None:
            st = [0] * len(self.shape)
            acc = isz
            for i in range(len(self.shape) - 1, -1, -1):
                st[i] = acc
                acc *= self.shape[i]
            self.stride = st
        else:
            assert len(stride) == len(self.shape)
            self.stride = [int(s) * isz for s in stride]

    @classmethod
    def of(cls, t):
        """The descriptor of a tensor view as it is (its own shape and strides)."""
        return cls(t, list(t.shape), list(t.stride()))

    @property
    def complex(self):
        return self.buf.is_complex()


def _nd_head(dtype, shape, sin, sout, axes):
    return [dtype, len(shape), L.arr(C.c_size_t, list(shape)), L.arr(C.c_ssize_t, list(sin)),
            L.arr(C.c_ssize_t, list(sout)), len(axes), L.arr(C.c_size_t, list(axes))]


def apply(fft, descOut: DataDesc, descIn: DataDesc, stream=None):
    """apply (pocketfft.nim:235-295) on device buffers, enqueued on `stream`."""
    _check_cuda(descIn.buf, descOut.buf)
    lib = L.load()
    s = _stream_ptr(stream)
    dt = _dtype_code(descIn.buf)
    pin, pout = descIn.buf.data_ptr(), descOut.buf.data_ptr()
    if isinstance(fft, DCTDesc):
        head = _nd_head(dt, descIn.shape, descIn.stride, descOut.stride, fft.axes)
        L.check(lib.ig_dct_device(*head, fft.dctType, pin, pout, fft.scalingFactor, int(fft.ortho), s))
        return
    head = _nd_head(dt, descIn.shape, descIn.stride, descOut.stride, fft.axes)
    if descIn.complex and descOut.complex:
        fn = lib.ig_c2c_device
    elif descOut.complex:
        fn = lib.ig_r2c_device
    elif descIn.complex:
        # descIn.shape where pocketfft::c2r expects the real output's shape (pocketfft.nim:266)
        fn = lib.ig_c2r_device
    else:
        raise TypeError("Not implemented")
    L.check(fn(*head, int(fft.forward), pin, pout, float(fft.scalingFactor), s))


# ---- 1-d Tensor overloads (pocketfft_arraymancer.nim: normalize honoured) ----

class _Plan:
    def __init__(self, real, n, dtype):
        lib = L.load()
        self.real = real
        self.p = (lib.ig_make_rfft_plan if real else lib.ig_make_cfft_plan)(n, dtype)
        if not self.p:
            raise L.FFTError(L.IG_EZERO_LEN if n == 0 else L.IG_EINVAL, lib.ig_last_error_string().decode())

    def __del__(self):
        if getattr(self, "p", None):
            lib = L.load()
            (lib.ig_destroy_rfft_plan if self.real else lib.ig_destroy_cfft_plan)(self.p)
            self.p = None


def _exec_rows(t, forward, fct, stream, out=None):
    """Every row of a 2-d (or the one row of a 1-d) CUDA tensor; rows may be `dist` apart."""
    _check_cuda(t)
    out = t if out is None else out
    real = not t.is_complex()
    n = t.shape[-1]
    if t.stride(-1) != 1 or out.stride(-1) != 1:
        raise ValueError("rows must be contiguous along the transform axis")
    rows = 1 if t.dim() == 1 else t.shape[0]
    dist_in = n if t.dim() == 1 else t.stride(0)
    dist_out = n if out.dim() == 1 else out.stride(0)
    plan = _Plan(real, n, _dtype_code(t))
    lib = L.load()
    fn = lib.ig_rfft_exec_device if real else lib.ig_cfft_exec_device
    rc = fn(plan.p, t.data_ptr(), out.data_ptr(), rows, dist_in, dist_out, int(forward), float(fct),
            _stream_ptr(stream))
    if rc != 0:
        raise Exception(("Forward" if forward else "Backward") + " FFT calculation failed.")
    return out


def rfft_rows(t, forward=True, fct=1.0, stream=None, out=None):
    """Halfcomplex transform of every row of a real 2-d CUDA tensor (in place unless `out`)."""
    return _exec_rows(t, forward, fct, stream, out)


def cfft_rows(t, forward=True, fct=1.0, stream=None, out=None):
    """Complex transform of every row of a complex 2-d CUDA tensor (in place unless `out`)."""
    return _exec_rows(t, forward, fct, stream, out)


def tensor_fft_inplace(data, forward: bool = True, normalize=nkBackward, normValue=math.inf, stream=None):
    """pocketfft_arraymancer.nim:33-37 on a contiguous 1-d CUDA tensor."""
    _check_cuda(data)
    flat = data.view(-1)
    norm = initNormalize(normalize, forward, normValue, flat.numel())
    _exec_rows(flat, forward, norm, stream)


def tensor_rfft_packed(data, forward: bool = True, normalize=nkBackward, normValue=math.inf, stream=None):
    """pocketfft_arraymancer.nim:39-46"""
    with _on(stream):
        res = data.clone().view(-1)
        tensor_fft_inplace(res, forward, normalize, normValue)
    return res


def unpackFFT(data):
    """pocketfft.nim:126-158 on the device: halfcomplex -> N/2+1 (even) / (N+1)/2 (odd) complex."""
    torch = _torch()
    _check_cuda(data)
    d = data.view(-1)
    n = d.numel()
    zero = d.new_zeros(1)
    re = torch.cat([d[0:1], d[1::2]])
    im = torch.cat([zero, d[2::2]] + ([zero] if n % 2 == 0 else []))
    return torch.complex(re, im)


def symmTargetSize(data) -> int:
    """pocketfft.nim:173-183 (reads the last element for complex input, as the reference does)."""
    d = data.view(-1)
    if not d.is_complex():
        return d.numel()
    return d.numel() * 2 - (2 if float(d[-1].imag.item()) == 0.0 else 1)


def symmetrize(data):
    """pocketfft.nim:160-171, 185-187 on the device: recover the Hermitian half."""
    torch = _torch()
    _check_cuda(data)
    d = data.view(-1)
    out_len = symmTargetSize(d)
    cdt = torch.complex128 if d.dtype in (torch.float64, torch.complex128) else torch.complex64
    u = d if d.is_complex() else unpackFFT(d)
    res = torch.empty(out_len, dtype=cdt, device=d.device)
    res[: u.numel()] = u
    i = torch.arange(1, (out_len + 1) // 2, device=d.device)
    res[out_len - i] = torch.conj(res[i])
    return res


def tensor_rfft(data, forward: bool = True, normalize=nkBackward, normValue=math.inf, stream=None):
    """pocketfft_arraymancer.nim:48-60"""
    with _on(stream):
        return unpackFFT(tensor_rfft_packed(data, forward, normalize, normValue))


def tensor_fft(data, forward: bool = True, normalize=nkBackward, normValue=math.inf, stream=None):
    """pocketfft_arraymancer.nim:69-82"""
    with _on(stream):
        if not data.is_complex():
            return symmetrize(tensor_rfft_packed(data, forward, normalize, normValue))
        res = data.clone().view(-1)
        tensor_fft_inplace(res, forward, normalize, normValue)
        return res


def tensor_ifft(data, backward: bool = True, normalize=nkBackward, normValue=math.inf, stream=None):
    """pocketfft_arraymancer.nim:84-94"""
    return tensor_fft(data, not backward, normalize, normValue, stream)
