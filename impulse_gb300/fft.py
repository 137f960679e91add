"""Host-side mirror of impulse's Nim FFT interface over the GPU engine.

Nim is not available on this machine, so the layer above the C ABI is
restated here in Python, name for name, with the reference's argument meaning
and quirks; the arithmetic all happens in libimpulse_gpu.so.  A Nim user binds
the same C ABI with ``{.importc, dynlib.}`` (the module nim/impulse_gpu_fft.nim).

C backend (impulse/fft/c_pocketfft/pocketfft.nim, pocketfft_arraymancer.nim):

* ``fft_inplace(data, forward)`` -- ``fft*(var openArray[T], forward)``
  (pocketfft.nim:305): in place; real data gives the packed halfcomplex
  layout; the normalisation arguments are dropped, so ``nkBackward`` always
  applies (pocketfft.nim:310).
* ``rfft_packed``, ``rfft``, ``fft``, ``ifft`` -- the value-returning
  openArray / seq overloads (pocketfft.nim:312-360); they drop
  ``normalize`` as the reference does (pocketfft.nim:319, 331, 347).
* ``tensor_*`` -- the Arraymancer Tensor overloads
  (pocketfft_arraymancer.nim:25-94), which honour ``normalize``.
* ``unpackFFT``, ``symmetrize``, ``symmTargetSize``, ``initNormalize``
  (pocketfft.nim:126-204).

C++ backend (impulse/fft/cpp_pocketfft/pocketfft.nim):

* ``DataDesc``, ``FFTDesc``, ``apply`` (pocketfft.nim:137-277), including the
  c2r call that passes the complex input's shape as the output shape
  (pocketfft.nim:266).

Arrays are numpy arrays in host memory (float64/complex128 or
float32/complex64).
"""
from __future__ import annotations

import ctypes as C
import enum
import math

import numpy as np

from . import _lib as L


class NormalizeKind(enum.IntEnum):
    """pocketfft.nim:189-193"""
    nkBackward = 0
    nkOrtho = 1
    nkForward = 2
    nkCustom = 3


nkBackward = NormalizeKind.nkBackward
nkOrtho = NormalizeKind.nkOrtho
nkForward = NormalizeKind.nkForward
nkCustom = NormalizeKind.nkCustom


def initNormalize(kind, forward, value, length):
    """pocketfft.nim:199-204"""
    kind = NormalizeKind(kind)
    if kind == nkBackward:
        return 1.0 if forward else 1.0 / float(length)
    if kind == nkForward:
        return 1.0 / float(length) if forward else 1.0
    if kind == nkOrtho:
        return 1.0 / math.sqrt(float(length))
    return float(value)


def _dtype_code(a: np.ndarray) -> int:
    if a.dtype in (np.float64, np.complex128):
        return L.IG_F64
    if a.dtype in (np.float32, np.complex64):
        return L.IG_F32
    raise TypeError(f"unsupported dtype {a.dtype}")


class FFTPlanReal:
    """Plan wrapper of pocketfft.nim:84-114 (plan made per call, freed on drop)."""

    def __init__(self, length: int, dtype=L.IG_F64):
        lib = L.load()
        self.length = length
        self.pocket = lib.ig_make_rfft_plan(length, dtype)
        if not self.pocket:
            raise L.FFTError(L.IG_EZERO_LEN if length == 0 else L.IG_EINVAL,
                             lib.ig_last_error_string().decode())

    def __del__(self):
        if getattr(self, "pocket", None):
            L.load().ig_destroy_rfft_plan(self.pocket)
            self.pocket = None


class FFTPlanComplex:
    def __init__(self, length: int, dtype=L.IG_F64):
        lib = L.load()
        self.length = length
        self.pocket = lib.ig_make_cfft_plan(length, dtype)
        if not self.pocket:
            raise L.FFTError(L.IG_EZERO_LEN if length == 0 else L.IG_EINVAL,
                             lib.ig_last_error_string().decode())

    def __del__(self):
        if getattr(self, "pocket", None):
            L.load().ig_destroy_cfft_plan(self.pocket)
            self.pocket = None


def _call(plan, real, data, forward, fct):
    """callFFT (pocketfft.nim:206-214): a non-zero status raises."""
    lib = L.load()
    ptr = data.ctypes.data
    if real:
        rc = (lib.ig_rfft_forward if forward else lib.ig_rfft_backward)(plan.pocket, ptr, fct)
    else:
        rc = (lib.ig_cfft_forward if forward else lib.ig_cfft_backward)(plan.pocket, ptr, fct)
    if rc != 0:
        raise Exception(("Forward" if forward else "Backward") + " FFT calculation failed.")


def fft_impl(data: np.ndarray, length: int, forward: bool, normalize=nkBackward, normValue=math.inf):
    """pocketfft.nim:290-303 -- in place on a contiguous 1-d array."""
    assert data.flags.c_contiguous and data.ndim == 1
    norm = initNormalize(normalize, forward, normValue, length)
    real = not np.iscomplexobj(data)
    plan = (FFTPlanReal if real else FFTPlanComplex)(length, _dtype_code(data))
    _call(plan, real, data, forward, norm)


def rfft_inplace(data: np.ndarray, length: int, forward: bool, normalize=nkBackward, normValue=math.inf):
    """rfft (pocketfft.nim:216-288): in-place halfcomplex real transform."""
    norm = initNormalize(normalize, forward, normValue, length)
    plan = FFTPlanReal(length, _dtype_code(data))
    _call(plan, True, data, forward, norm)


# ---- openArray / seq overloads (normalize dropped, as in the reference) ----

def fft_inplace(data: np.ndarray, forward: bool = True, normalize=nkBackward, normValue=math.inf):
    """fft*(var openArray[T]) (pocketfft.nim:305-310): normalize is not forwarded."""
    fft_impl(data, data.size, forward)


def rfft_packed(data, forward: bool = True, normalize=nkBackward, normValue=math.inf):
    """pocketfft.nim:312-319: copy, in-place rfft; normalize is not forwarded."""
    res = np.array(data, dtype=np.asarray(data).dtype, copy=True)
    rfft_inplace(res, res.size, forward)
    return res


def unpackFFT(data):
    """pocketfft.nim:126-158: halfcomplex -> N/2+1 (even) / (N+1)/2 (odd) complex."""
    data = np.asarray(data)
    n = data.size
    out_len = (n + 1) // 2 if n % 2 else (n + 2) // 2
    cdt = np.complex128 if data.dtype == np.float64 else np.complex64
    out = np.empty(out_len, cdt)
    out[0] = complex(data[0], 0.0)
    k = 1
    re = data[0]
    for i in range(1, n):
        if i & 1:
            re = data[i]
        else:
            out[k] = complex(re, data[i])
            k += 1
    if n % 2 == 0:
        out[k] = complex(re, 0.0)
    return out


def symmTargetSize(data) -> int:
    """pocketfft.nim:173-183"""
    data = np.asarray(data)
    if not np.iscomplexobj(data):
        return data.size
    return data.size * 2 - (2 if data[-1].imag == 0.0 else 1)


def symmetrize(data):
    """pocketfft.nim:160-171, 185-187: recover the Hermitian half."""
    data = np.asarray(data)
    out_len = symmTargetSize(data)
    cdt = np.complex128 if data.dtype in (np.float64, np.complex128) else np.complex64
    res = np.empty(out_len, cdt)
    if np.iscomplexobj(data):
        res[: data.size] = data
    else:
        u = unpackFFT(data)
        res[: u.size] = u
    k = out_len - 1
    for i in range(1, (out_len + 1) // 2):
        res[k] = np.conj(res[i])
        k -= 1
    return res


def rfft(data, forward: bool = True, normalize=nkBackward, normValue=math.inf):
    """pocketfft.nim:321-332: N/2+1 complex terms; normalize is not forwarded."""
    res = np.array(data, copy=True)
    fft_inplace(res, forward)
    return unpackFFT(res)


def fft(data, forward: bool = True, normalize=nkBackward, normValue=math.inf):
    """pocketfft.nim:334-348: value-returning FFT (N complex terms)."""
    data = np.asarray(data)
    if not np.iscomplexobj(data):
        return symmetrize(rfft_packed(data, forward, normalize, normValue))
    res = np.array(data, copy=True)
    fft_inplace(res, forward, normalize, normValue)
    return res


def ifft(data, backward: bool = True, normalize=nkBackward, normValue=math.inf):
    """pocketfft.nim:350-360"""
    return fft(data, not backward, normalize, normValue)


# ---- Tensor overloads (pocketfft_arraymancer.nim: normalize honoured) ----

def tensor_fft_inplace(data, forward: bool = True, normalize=nkBackward, normValue=math.inf):
    """pocketfft_arraymancer.nim:33-37"""
    fft_impl(data, data.size, forward, normalize, normValue)


def tensor_rfft_packed(data, forward: bool = True, normalize=nkBackward, normValue=math.inf):
    """pocketfft_arraymancer.nim:39-46"""
    res = np.array(data, copy=True)
    rfft_inplace(res, res.size, forward, normalize, normValue)
    return res


def tensor_rfft(data, forward: bool = True, normalize=nkBackward, normValue=math.inf):
    """pocketfft_arraymancer.nim:48-60"""
    res = np.array(data, copy=True)
    tensor_fft_inplace(res, forward, normalize, normValue)
    return unpackFFT(res)


def tensor_fft(data, forward: bool = True, normalize=nkBackward, normValue=math.inf):
    """pocketfft_arraymancer.nim:69-82"""
    data = np.asarray(data)
    if not np.iscomplexobj(data):
        return symmetrize(tensor_rfft_packed(data, forward, normalize, normValue))
    res = np.array(data, copy=True)
    tensor_fft_inplace(res, forward, normalize, normValue)
    return res


def tensor_ifft(data, backward: bool = True, normalize=nkBackward, normValue=math.inf):
    """pocketfft_arraymancer.nim:84-94"""
    return tensor_fft(data, not backward, normalize, normValue)


# ---- C++ backend: DataDesc / FFTDesc / apply (cpp_pocketfft/pocketfft.nim) ----

class DataDesc:
    """pocketfft.nim:137-199: shape, BYTE strides and a buffer.

    ``DataDesc(buf, shape)`` is the row-major constructor (pocketfft.nim:178);
    ``DataDesc(buf, shape, stride)`` takes element strides and multiplies them
    by the element size (pocketfft.nim:158-176)."""

    def __init__(self, buf: np.ndarray, shape, stride=None):
        assert buf is not None
        self.buf = buf
        self.shape = [int(s) for s in shape]
        isz = buf.dtype.itemsize
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

    @property
    def complex(self):
        return np.iscomplexobj(self.buf)


class FFTDesc:
    """pocketfft.nim:144-149, 201-215"""

    def __init__(self, axes, forward: bool, scalingFactor: float = 1.0, nthreads: int = 1):
        self.axes = [int(a) for a in axes]
        self.forward = bool(forward)
        self.scalingFactor = float(scalingFactor)
        self.nthreads = int(nthreads)


def _nd_call(fn, dtype, shape, sin, sout, axes, forward, pin, pout, fct, nthreads):
    rc = fn(dtype, len(shape), L.arr(C.c_size_t, shape), L.arr(C.c_ssize_t, sin), L.arr(C.c_ssize_t, sout),
            len(axes), L.arr(C.c_size_t, axes), int(forward), pin, pout, float(fct), nthreads)
    L.check(rc)


def apply(fft, descOut: DataDesc, descIn: DataDesc):
    """pocketfft.nim:235-277: compile-time dispatch to c2c / r2c / c2r; the
    DCTDesc overload (pocketfft.nim:279-295) goes to pocketfft::dct."""
    if isinstance(fft, DCTDesc):
        return apply_dct(fft, descOut, descIn)
    lib = L.load()
    dt = _dtype_code(descIn.buf)
    if descIn.complex and descOut.complex:
        _nd_call(lib.ig_c2c, dt, descIn.shape, descIn.stride, descOut.stride, fft.axes, fft.forward,
                 descIn.buf.ctypes.data, descOut.buf.ctypes.data, fft.scalingFactor, fft.nthreads)
    elif descOut.complex:
        _nd_call(lib.ig_r2c, dt, descIn.shape, descIn.stride, descOut.stride, fft.axes, fft.forward,
                 descIn.buf.ctypes.data, descOut.buf.ctypes.data, fft.scalingFactor, fft.nthreads)
    elif descIn.complex:
        # the reference passes descIn.shape where pocketfft::c2r expects the
        # real output's shape (pocketfft.nim:266); kept as is
        _nd_call(lib.ig_c2r, dt, descIn.shape, descIn.stride, descOut.stride, fft.axes, fft.forward,
                 descIn.buf.ctypes.data, descOut.buf.ctypes.data, fft.scalingFactor, fft.nthreads)
    else:
        raise TypeError("Not implemented")


# ---- raw C-ABI helpers on numpy arrays (used by tests and the benchmark) ----

class DCTDesc:
    """pocketfft.nim:151-156, 217-233: axes, DCT type (default 2), ortho, scalingFactor, nthreads."""

    def __init__(self, axes, dctType: int = 2, ortho: bool = False, scalingFactor: float = 1.0, nthreads: int = 1):
        self.axes = [int(a) for a in axes]
        if not 1 <= int(dctType) <= 4:
            raise ValueError("dctType must be in 1..4")
        self.dctType = int(dctType)
        self.ortho = bool(ortho)
        self.scalingFactor = float(scalingFactor)
        self.nthreads = int(nthreads)


def apply_dct(dct: DCTDesc, descOut: DataDesc, descIn: DataDesc):
    """The DCTDesc overload of apply (pocketfft.nim:279-295): pocketfft::dct over dct.axes."""
    head = _nd_head(_dtype_code(descIn.buf), descIn.shape, descIn.stride, descOut.stride, dct.axes)
    L.check(L.load().ig_dct(*head, dct.dctType, descIn.buf.ctypes.data, descOut.buf.ctypes.data,
                            dct.scalingFactor, int(dct.ortho), dct.nthreads))


def _nd_head(dtype, shape, sin, sout, axes):
    return [dtype, len(shape), L.arr(C.c_size_t, list(shape)), L.arr(C.c_ssize_t, list(sin)),
            L.arr(C.c_ssize_t, list(sout)), len(axes), L.arr(C.c_size_t, list(axes))]


def dct(x: np.ndarray, axes, type=2, fct=1.0, ortho=False, out=None):
    """pocketfft::dct (pocketfft_hdronly.h:3284-3300) on host arrays."""
    out = np.empty_like(x) if out is None else out
    L.check(L.load().ig_dct(*_nd_head(_dtype_code(x), x.shape, x.strides, out.strides, axes), int(type),
                            x.ctypes.data, out.ctypes.data, float(fct), int(ortho), 1))
    return out


def dst(x: np.ndarray, axes, type=2, fct=1.0, ortho=False, out=None):
    """pocketfft::dst (pocketfft_hdronly.h:3302-3318) on host arrays."""
    out = np.empty_like(x) if out is None else out
    L.check(L.load().ig_dst(*_nd_head(_dtype_code(x), x.shape, x.strides, out.strides, axes), int(type),
                            x.ctypes.data, out.ctypes.data, float(fct), int(ortho), 1))
    return out


def r2r_fftpack(x: np.ndarray, axes, real2hermitian=True, forward=True, fct=1.0, out=None):
    """pocketfft::r2r_fftpack (pocketfft_hdronly.h:3392-3403), bound at pocketfft.nim:71-81."""
    out = np.empty_like(x) if out is None else out
    L.check(L.load().ig_r2r_fftpack(*_nd_head(_dtype_code(x), x.shape, x.strides, out.strides, axes),
                                    int(real2hermitian), int(forward), x.ctypes.data, out.ctypes.data, float(fct), 1))
    return out


def hartley(x: np.ndarray, axes, fct=1.0, genuine=False, out=None):
    """r2r_separable_hartley / r2r_genuine_hartley (pocketfft_hdronly.h:3405-3445)."""
    out = np.empty_like(x) if out is None else out
    fn = L.load().ig_r2r_genuine_hartley if genuine else L.load().ig_r2r_separable_hartley
    L.check(fn(*_nd_head(_dtype_code(x), x.shape, x.strides, out.strides, axes), x.ctypes.data, out.ctypes.data,
               float(fct), 1))
    return out


def c2c(x: np.ndarray, axes, forward=True, fct=1.0, out=None):
    out = np.empty_like(x) if out is None else out
    _nd_call(L.load().ig_c2c, _dtype_code(x), x.shape, x.strides, out.strides, list(axes), forward,
             x.ctypes.data, out.ctypes.data, fct, 1)
    return out


def r2c(x: np.ndarray, axes, forward=True, fct=1.0):
    shp = list(x.shape)
    shp[axes[-1]] = shp[axes[-1]] // 2 + 1
    out = np.empty(shp, np.complex128 if x.dtype == np.float64 else np.complex64)
    _nd_call(L.load().ig_r2c, _dtype_code(x), x.shape, x.strides, out.strides, list(axes), forward,
             x.ctypes.data, out.ctypes.data, fct, 1)
    return out


def c2r(x: np.ndarray, shape_out, axes, forward=False, fct=1.0):
    out = np.empty(shape_out, np.float64 if x.dtype == np.complex128 else np.float32)
    _nd_call(L.load().ig_c2r, _dtype_code(x), list(shape_out), x.strides, out.strides, list(axes), forward,
             x.ctypes.data, out.ctypes.data, fct, 1)
    return out


def rfft_batch(x: np.ndarray, forward=True, fct=1.0):
    """Halfcomplex transform of every row of a C-contiguous 2-d array, in one launch."""
    x = np.ascontiguousarray(x).copy()
    n = x.shape[-1]
    plan = FFTPlanReal(n, _dtype_code(x))
    L.check(L.load().ig_rfft_exec_batch(plan.pocket, x.ctypes.data, x.size // n, n, int(forward), fct))
    return x


def cfft_batch(x: np.ndarray, forward=True, fct=1.0):
    x = np.ascontiguousarray(x).copy()
    n = x.shape[-1]
    plan = FFTPlanComplex(n, _dtype_code(x))
    L.check(L.load().ig_cfft_exec_batch(plan.pocket, x.ctypes.data, x.size // n, n, int(forward), fct))
    return x


def autotune(n, dtype=L.IG_F64, kind=1):
    """Autotune the length-n transform (kind 0 complex, 1 real halfcomplex); returns ms per call."""
    ms = C.c_double()
    L.check(L.load().ig_autotune(dtype, n, kind, C.byref(ms)))
    return ms.value


def autotune_save(path=None):
    """Write the tuned table (one line per length, keyed by GPU name); None uses IG_AUTOTUNE_CACHE."""
    L.check(L.load().ig_autotune_save(path.encode() if path else None))


def autotune_load(path=None):
    """Read a table written by autotune_save; entries for other GPU models are skipped."""
    L.check(L.load().ig_autotune_load(path.encode() if path else None))
