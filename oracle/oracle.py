"""ctypes bindings for the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Two libraries are bound:

* ``libimpulse_oracle.so`` -- this repository's own FP64 C restatement of the
  reference algorithms (impulse_oracle.c).  It exists wherever the repository
  is built, including the GPU host, and is the checker used by the GPU tests.
* ``_ref/libpocketfft_ref.so`` -- impulse's vendored PocketFFT compiled in
  place from the reference checkout (Makefile target ``ref``).  It exists only
  where the reference sources are present; it pins the restatement and makes
  the golden fixtures under ``tests/golden``.

Only tests, the smoke check and the benchmark's CPU-baseline leg use this.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "libimpulse_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libpocketfft_ref.so")
REF_SCALAR_SO = os.path.join(HERE, "_ref", "libpocketfft_ref_scalar.so")

_sz = C.c_size_t
_pd = C.c_ssize_t
_dp = C.POINTER(C.c_double)


def build(ref: bool | None = None) -> None:
    """Compile the oracle; with ``ref`` (or, when ``ref`` is None, whenever
    IMPULSE_REF names an impulse checkout) also the reference shim.

    The reference's location comes only from the IMPULSE_REF environment
    variable; asking for the shim without it is an error."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    refdir = os.environ.get("IMPULSE_REF", "")
    present = bool(refdir) and os.path.isdir(os.path.join(refdir, "impulse", "fft"))
    if ref is None:
        ref = present
    if ref:
        if not present:
            raise RuntimeError("IMPULSE_REF must name an impulse checkout (with impulse/fft) to build the "
                               f"reference PocketFFT; got {refdir!r}")
        subprocess.run(["make", "-s", "-C", HERE, "ref", "ref-scalar", f"IMPULSE_REF={refdir}"], check=True)


_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_SO):
            build(ref=False)
        L = C.CDLL(ORACLE_SO)
        L.io_cfft.argtypes = [_sz, _dp, C.c_int, C.c_double]
        L.io_rfft.argtypes = [_sz, _dp, C.c_int, C.c_double]
        L.io_cfft_batch.argtypes = [_sz, _sz, _dp, _sz, C.c_int, C.c_double, C.c_int]
        L.io_rfft_batch.argtypes = [_sz, _sz, _dp, _sz, C.c_int, C.c_double, C.c_int]
        for nm in ("io_c2c", "io_r2c", "io_c2r"):
            getattr(L, nm).argtypes = [_sz, C.POINTER(_sz), C.POINTER(_pd), C.POINTER(_pd), _sz,
                                       C.POINTER(_sz), C.c_int, C.c_void_p, C.c_void_p, C.c_double, C.c_int]
        nd_head = [_sz, C.POINTER(_sz), C.POINTER(_pd), C.POINTER(_pd), _sz, C.POINTER(_sz)]
        for nm in ("io_dct", "io_dst"):
            getattr(L, nm).argtypes = nd_head + [C.c_int, C.c_void_p, C.c_void_p, C.c_double, C.c_int, C.c_int]
        L.io_r2r_fftpack.argtypes = nd_head + [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_double, C.c_int]
        for nm in ("io_r2r_separable_hartley", "io_r2r_genuine_hartley"):
            getattr(L, nm).argtypes = nd_head + [C.c_void_p, C.c_void_p, C.c_double, C.c_int]
        L.io_upfirdn_length.argtypes = [_sz, _sz, C.c_int, C.c_int]
        L.io_upfirdn_length.restype = _sz
        L.io_upfirdn.argtypes = [_sz, _sz, _dp, _sz, _sz, _dp, C.c_int, C.c_int, _dp, _sz]
        L.io_largest_prime_factor.argtypes = [_sz]
        L.io_largest_prime_factor.restype = _sz
        L.io_good_size.argtypes = [_sz]
        L.io_good_size.restype = _sz
        L.io_cost_guess.argtypes = [_sz]
        L.io_cost_guess.restype = C.c_double
        L.io_use_bluestein.argtypes = [_sz, C.c_int]
        L.io_unpack_fft.argtypes = [_dp, _dp, _sz]
        L.io_symmetrize.argtypes = [_dp, C.c_int, _sz, _dp, _sz]
        L.io_symm_target_size_complex.argtypes = [C.c_double, _sz]
        L.io_symm_target_size_complex.restype = _sz
        L.io_init_normalize.argtypes = [C.c_int, C.c_int, C.c_double, _sz]
        L.io_init_normalize.restype = C.c_double
        _lib = L
    return _lib


def ref_available() -> bool:
    return os.path.exists(REF_SO)


_ref_scalar = None


def ref_scalar():
    """The reference built without PocketFFT's SIMD (as on aarch64): r2r_fftpack
    and the C backend's rfft_forward / rfft_backward line loop."""
    global _ref_scalar
    if _ref_scalar is None:
        L = C.CDLL(REF_SCALAR_SO)
        L.ref_rfft_batch.argtypes = [_sz, _sz, _dp, C.c_int, C.c_double]
        L.ref_r2r_fftpack_f64.argtypes = [_sz, C.POINTER(_sz), C.POINTER(_pd), C.POINTER(_pd), _sz,
                                          C.POINTER(_sz), C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_double, _sz]
        _ref_scalar = L
    return _ref_scalar


def ref():
    """The reference's own PocketFFT (C and C++ backends), compiled in place."""
    global _ref
    if _ref is None:
        L = C.CDLL(REF_SO)
        L.make_cfft_plan.argtypes = [_sz]
        L.make_cfft_plan.restype = C.c_void_p
        L.make_rfft_plan.argtypes = [_sz]
        L.make_rfft_plan.restype = C.c_void_p
        for nm in ("cfft_forward", "cfft_backward", "rfft_forward", "rfft_backward"):
            getattr(L, nm).argtypes = [C.c_void_p, _dp, C.c_double]
            getattr(L, nm).restype = C.c_int
        L.destroy_cfft_plan.argtypes = [C.c_void_p]
        L.destroy_rfft_plan.argtypes = [C.c_void_p]
        for sfx in ("f64", "f32"):
            for nm in ("ref_c2c", "ref_r2c", "ref_c2r"):
                getattr(L, f"{nm}_{sfx}").argtypes = [_sz, C.POINTER(_sz), C.POINTER(_pd), C.POINTER(_pd), _sz,
                                                      C.POINTER(_sz), C.c_int, C.c_void_p, C.c_void_p,
                                                      C.c_double, _sz]
            getattr(L, f"ref_r2r_fftpack_{sfx}").argtypes = [_sz, C.POINTER(_sz), C.POINTER(_pd), C.POINTER(_pd),
                                                           _sz, C.POINTER(_sz), C.c_int, C.c_int, C.c_void_p,
                                                           C.c_void_p, C.c_double, _sz]
            nd_head = [_sz, C.POINTER(_sz), C.POINTER(_pd), C.POINTER(_pd), _sz, C.POINTER(_sz)]
            for nm in ("ref_dct", "ref_dst"):
                getattr(L, f"{nm}_{sfx}").argtypes = nd_head + [C.c_int, C.c_void_p, C.c_void_p, C.c_double,
                                                                C.c_int, _sz]
            getattr(L, f"ref_hartley_{sfx}").argtypes = nd_head + [C.c_int, C.c_void_p, C.c_void_p, C.c_double, _sz]
        L.ref_last_error.restype = C.c_char_p
        _ref = L
    return _ref


def _p(a):
    return a.ctypes.data_as(_dp)


def _arr(t, vals):
    return (t * max(1, len(vals)))(*vals)


# ---------------------------------------------------------------------------
# restatement (libimpulse_oracle)
# ---------------------------------------------------------------------------

def cfft(x, forward=True, fct=1.0):
    """In-place-style complex FFT of the last axis (batched over leading axes)."""
    a = np.ascontiguousarray(x, dtype=np.complex128).copy()
    n = a.shape[-1]
    b = a.size // n if n else 0
    rc = lib().io_cfft_batch(n, b, _p(a.view(np.float64)), n, int(forward), fct, os.cpu_count() or 1)
    assert rc == 0
    return a


def rfft_hc(x, forward=True, fct=1.0, nthreads=None):
    """Halfcomplex real FFT of the last axis (pocketfft rfft_forward/backward)."""
    a = np.ascontiguousarray(x, dtype=np.float64).copy()
    n = a.shape[-1]
    b = a.size // n if n else 0
    rc = lib().io_rfft_batch(n, b, _p(a), n, int(forward), fct, nthreads or os.cpu_count() or 1)
    assert rc == 0
    return a


def _nd(fn, shape, xin, xout, axes, forward, fct, nthreads):
    nd = len(shape)
    sin = [s for s in xin.strides]
    sout = [s for s in xout.strides]
    return fn(nd, _arr(_sz, shape), _arr(_pd, sin), _arr(_pd, sout), len(axes), _arr(_sz, list(axes)),
              int(forward), xin.ctypes.data, xout.ctypes.data, float(fct), nthreads)


def c2c(x, axes, forward=True, fct=1.0, out=None, nthreads=None):
    x = np.asarray(x, dtype=np.complex128)
    if out is None:
        out = np.empty(x.shape, np.complex128)
    rc = _nd(lib().io_c2c, x.shape, x, out, axes, forward, fct, nthreads or os.cpu_count() or 1)
    if rc:
        raise ValueError(f"oracle c2c status {rc}")
    return out


def r2c(x, axes, forward=True, fct=1.0, nthreads=None):
    x = np.asarray(x, dtype=np.float64)
    shp = list(x.shape)
    shp[axes[-1]] = shp[axes[-1]] // 2 + 1
    out = np.empty(shp, np.complex128)
    rc = _nd(lib().io_r2c, x.shape, x, out, axes, forward, fct, nthreads or os.cpu_count() or 1)
    if rc:
        raise ValueError(f"oracle r2c status {rc}")
    return out


def c2r(x, shape_out, axes, forward=False, fct=1.0, nthreads=None):
    x = np.asarray(x, dtype=np.complex128)
    out = np.empty(shape_out, np.float64)
    rc = _nd(lib().io_c2r, tuple(shape_out), x, out, axes, forward, fct, nthreads or os.cpu_count() or 1)
    if rc:
        raise ValueError(f"oracle c2r status {rc}")
    return out


def _nd_head(shape, xin, xout, axes):
    return [len(shape), _arr(_sz, shape), _arr(_pd, list(xin.strides)), _arr(_pd, list(xout.strides)), len(axes),
            _arr(_sz, list(axes))]


def dct(x, axes, type=2, fct=1.0, ortho=False, nthreads=None, sine=False):
    """pocketfft::dct / dst (pocketfft_hdronly.h:3284-3318) by the defining sums."""
    x = np.asarray(x, dtype=np.float64)
    out = np.empty(x.shape, np.float64)
    fn = lib().io_dst if sine else lib().io_dct
    rc = fn(*_nd_head(x.shape, x, out, axes), int(type), x.ctypes.data, out.ctypes.data, float(fct), int(ortho),
            nthreads or os.cpu_count() or 1)
    if rc:
        raise ValueError(f"oracle dct/dst status {rc}")
    return out


def dst(x, axes, type=2, fct=1.0, ortho=False, nthreads=None):
    return dct(x, axes, type, fct, ortho, nthreads, sine=True)


def r2r_fftpack(x, axes, real2hermitian=True, forward=True, fct=1.0, nthreads=None):
    x = np.asarray(x, dtype=np.float64)
    out = np.empty(x.shape, np.float64)
    rc = lib().io_r2r_fftpack(*_nd_head(x.shape, x, out, axes), int(real2hermitian), int(forward), x.ctypes.data,
                              out.ctypes.data, float(fct), nthreads or os.cpu_count() or 1)
    if rc:
        raise ValueError(f"oracle r2r_fftpack status {rc}")
    return out


def hartley(x, axes, fct=1.0, genuine=False, nthreads=None):
    x = np.asarray(x, dtype=np.float64)
    out = np.empty(x.shape, np.float64)
    fn = lib().io_r2r_genuine_hartley if genuine else lib().io_r2r_separable_hartley
    rc = fn(*_nd_head(x.shape, x, out, axes), x.ctypes.data, out.ctypes.data, float(fct), nthreads or os.cpu_count() or 1)
    if rc:
        raise ValueError(f"oracle hartley status {rc}")
    return out


def upfirdn(t, h, up=1, down=1):
    """impulse signal.nim:545-594 by direct sums; t 1-d or rows of a 2-d array."""
    t = np.ascontiguousarray(np.atleast_2d(np.asarray(t, dtype=np.float64)))
    h = np.ascontiguousarray(np.asarray(h, dtype=np.float64).ravel())
    b, n = t.shape
    ny = lib().io_upfirdn_length(n, h.size, up, down)
    y = np.empty((b, ny))
    assert lib().io_upfirdn(b, n, _p(t), n, h.size, _p(h), up, down, _p(y), ny) == 0
    return y


def unpack_fft(hc):
    hc = np.ascontiguousarray(hc, dtype=np.float64)
    n = hc.size
    m = (n + 1) // 2 if n % 2 else (n + 2) // 2
    out = np.empty(m, np.complex128)
    lib().io_unpack_fft(_p(hc), _p(out.view(np.float64)), n)
    return out


def symmetrize(data):
    data = np.ascontiguousarray(data)
    if data.dtype == np.float64:
        n_out = data.size
        out = np.empty(n_out, np.complex128)
        lib().io_symmetrize(_p(data), 1, data.size, _p(out.view(np.float64)), n_out)
    else:
        data = data.astype(np.complex128)
        n_out = lib().io_symm_target_size_complex(float(data[-1].imag), data.size)
        out = np.empty(n_out, np.complex128)
        lib().io_symmetrize(_p(data.view(np.float64)), 0, data.size, _p(out.view(np.float64)), n_out)
    return out


def init_normalize(kind, forward, value, length):
    return lib().io_init_normalize(int(kind), int(forward), float(value), int(length))


def uses_bluestein(n, real=False):
    return bool(lib().io_use_bluestein(n, int(real)))


def good_size(n):
    return int(lib().io_good_size(n))


# ---------------------------------------------------------------------------
# reference (compiled in place)
# ---------------------------------------------------------------------------

def ref_cfft(x, forward=True, fct=1.0):
    L = ref()
    a = np.ascontiguousarray(x, dtype=np.complex128).copy()
    n = a.shape[-1]
    p = L.make_cfft_plan(n)
    flat = a.reshape(-1, n)
    for row in flat:
        f = L.cfft_forward if forward else L.cfft_backward
        assert f(p, row.view(np.float64).ctypes.data_as(_dp), fct) == 0
    L.destroy_cfft_plan(p)
    return a


def ref_rfft_hc(x, forward=True, fct=1.0):
    L = ref()
    a = np.ascontiguousarray(x, dtype=np.float64).copy()
    n = a.shape[-1]
    p = L.make_rfft_plan(n)
    flat = a.reshape(-1, n)
    for row in flat:
        f = L.rfft_forward if forward else L.rfft_backward
        assert f(p, row.ctypes.data_as(_dp), fct) == 0
    L.destroy_rfft_plan(p)
    return a


def _ref_nd(name, dtype, shape, xin, xout, axes, forward, fct, nthreads, extra=None):
    L = ref()
    sfx = "f64" if dtype in (np.float64, np.complex128) else "f32"
    fn = getattr(L, f"{name}_{sfx}")
    nd = len(shape)
    args = [nd, _arr(_sz, shape), _arr(_pd, list(xin.strides)), _arr(_pd, list(xout.strides)), len(axes),
            _arr(_sz, list(axes))]
    if extra is not None:
        args.append(extra)
    args += [int(forward), xin.ctypes.data, xout.ctypes.data, float(fct), nthreads]
    rc = fn(*args)
    if rc:
        raise ValueError(L.ref_last_error().decode())
    return xout


def ref_c2c(x, axes, forward=True, fct=1.0, nthreads=1):
    out = np.empty(x.shape, x.dtype)
    return _ref_nd("ref_c2c", x.dtype, x.shape, x, out, axes, forward, fct, nthreads)


def ref_r2c(x, axes, forward=True, fct=1.0, nthreads=1):
    shp = list(x.shape)
    shp[axes[-1]] = shp[axes[-1]] // 2 + 1
    out = np.empty(shp, np.complex128 if x.dtype == np.float64 else np.complex64)
    return _ref_nd("ref_r2c", x.dtype, x.shape, x, out, axes, forward, fct, nthreads)


def ref_c2r(x, shape_out, axes, forward=False, fct=1.0, nthreads=1):
    out = np.empty(shape_out, np.float64 if x.dtype == np.complex128 else np.float32)
    return _ref_nd("ref_c2r", x.dtype, tuple(shape_out), x, out, axes, forward, fct, nthreads)


def ref_r2r_fftpack(x, axes, real2hermitian=True, forward=True, fct=1.0, nthreads=1):
    out = np.empty(x.shape, x.dtype)
    return _ref_nd("ref_r2r_fftpack", x.dtype, x.shape, x, out, axes, forward, fct, nthreads,
                   extra=int(real2hermitian))


def ref_dct(x, axes, type=2, fct=1.0, ortho=False, nthreads=1, sine=False):
    out = np.empty(x.shape, x.dtype)
    L = ref()
    sfx = "f64" if x.dtype == np.float64 else "f32"
    fn = getattr(L, f"ref_{'dst' if sine else 'dct'}_{sfx}")
    rc = fn(*_nd_head(x.shape, x, out, axes), int(type), x.ctypes.data, out.ctypes.data, float(fct), int(ortho),
            nthreads)
    if rc:
        raise ValueError(L.ref_last_error().decode())
    return out


def ref_hartley(x, axes, fct=1.0, genuine=False, nthreads=1):
    out = np.empty(x.shape, x.dtype)
    L = ref()
    fn = getattr(L, f"ref_hartley_{'f64' if x.dtype == np.float64 else 'f32'}")
    rc = fn(*_nd_head(x.shape, x, out, axes), int(genuine), x.ctypes.data, out.ctypes.data, float(fct), nthreads)
    if rc:
        raise ValueError(L.ref_last_error().decode())
    return out


def rel_l2(a, b):
    """||a - b||_2 / ||b||_2, scaled first so that huge or tiny values do not overflow."""
    a = np.asarray(a).astype(np.complex128 if np.iscomplexobj(a) or np.iscomplexobj(b) else np.float64)
    b = np.asarray(b).astype(a.dtype)
    s = float(np.max(np.abs(b))) if b.size else 0.0
    if not np.isfinite(s):
        return float("nan")
    if s == 0.0:
        return float(np.linalg.norm((a - b).ravel()))
    den = np.linalg.norm((b / s).ravel())
    num = np.linalg.norm(((a - b) / s).ravel())
    return float(num / den)
