"""GPU versions of impulse's FFT-friendly signal routines (impulse/signal.nim).

* ``upfirdn(t, h, up, down)`` -- signal.nim:545-594: upsample by ``up`` (zeros
  between samples), full convolution with the FIR filter ``h``, every
  ``down``-th sample.  Computed on the GPU by FFT (``ig_upfirdn``); ``t`` may be
  one signal or the rows of a 2-d array (one filter for all rows).
* ``reduce_resampling_rates`` -- signal.nim:596-610.
* ``resample(t, h, up, down)`` -- the explicit-filter overload (signal.nim:690-744):
  the filter is padded by ``adjust_filter_position`` (signal.nim:638-688) so that
  the decimation takes the filter's middle point, then ``upfirdn`` and a crop to
  ``ceil(len * up / down)`` samples.

The filter-designing overload of ``resample`` (firls + Kaiser window, signal.nim:
746-809) designs its filter on the host and is not part of the GPU path.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _lib as L


def _code(a: np.ndarray) -> int:
    if a.dtype == np.float64:
        return L.IG_F64
    if a.dtype == np.float32:
        return L.IG_F32
    raise TypeError(f"unsupported dtype {a.dtype}")


def upfirdn(t, h, up: int = 1, down: int = 1) -> np.ndarray:
    t = np.asarray(t)
    if t.dtype not in (np.float32, np.float64):
        t = t.astype(np.float64)
    h = np.ascontiguousarray(np.asarray(h, dtype=t.dtype).ravel())
    x = np.ascontiguousarray(np.atleast_2d(t))
    b, n = x.shape
    ny = C.c_size_t()
    lib = L.load()
    L.check(lib.ig_upfirdn_length(n, h.size, int(up), int(down), C.byref(ny)))
    y = np.empty((b, ny.value), dtype=x.dtype)
    L.check(lib.ig_upfirdn(_code(x), b, n, x.ctypes.data, n, h.size, h.ctypes.data, int(up), int(down),
                           y.ctypes.data, ny.value))
    return y[0] if t.ndim == 1 else y


def reduce_resampling_rates(up: int, down: int):
    g = math.gcd(up, down)
    return up // g, down // g


def adjust_filter_position(h: np.ndarray, input_len: int, result_len: int, up: int, down: int):
    """signal.nim:638-688: leading zeros so that decimation takes the filter's
    middle point, trailing zeros so that the output reaches result_len; returns
    (padded filter, total delay after decimation)."""
    middle = (h.size - 1) / 2.0
    lead = int(math.floor(down - math.fmod(middle, down) if middle >= 0 else down - (middle % down)))
    hh = np.concatenate([np.zeros(lead, h.dtype), h])
    middle += lead
    total_delay = int(math.floor(math.ceil(middle) / down))
    filt_len = (input_len - 1) * up + hh.size
    trail = 0
    while total_delay + result_len >= math.ceil((filt_len + trail) / down):
        trail += 1
    return np.concatenate([hh, np.zeros(trail, h.dtype)]), total_delay


def resample(t, h, up: int = 1, down: int = 1) -> np.ndarray:
    """signal.nim:690-744 (explicit filter)."""
    t = np.asarray(t)
    if up == 1 and down == 1:
        return t.copy()
    h = np.squeeze(np.asarray(h, dtype=t.dtype if t.dtype in (np.float32, np.float64) else np.float64))
    if h.ndim != 1:
        raise ValueError(f"Squeezed filter rank ({h.ndim}) must be 1")
    n = t.shape[-1]
    result_len = int(math.ceil(n * up / down))
    h, delay = adjust_filter_position(h, n, result_len, up, down)
    y = upfirdn(t, h, up, down)
    return y[..., delay:delay + result_len]
