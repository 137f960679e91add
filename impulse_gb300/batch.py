"""Batched complex transforms of uneven lengths (ig_multi_plan) and the
seeded uneven-length workload: `count` lengths log-uniform over [lo, hi],
90 % rounded to the nearest 2^a 3^b 5^c 7^d, 10 % to the nearest prime,
rescaled so that their sum is about `total` elements."""
from __future__ import annotations

import bisect
import ctypes as C
import math

import numpy as np

from . import _lib as L


def _smooth7(limit):
    out = []
    a = 1
    while a <= limit:
        b = a
        while b <= limit:
            c = b
            while c <= limit:
                d = c
                while d <= limit:
                    out.append(d)
                    d *= 7
                c *= 5
            b *= 3
        a *= 2
    return sorted(out)


def _is_prime(n):
    if n < 2:
        return False
    if n % 2 == 0:
        return n == 2
    f = 3
    while f * f <= n:
        if n % f == 0:
            return False
        f += 2
    return True


def _nearest_prime(n):
    d = 0
    while True:
        for c in (n - d, n + d):
            if c >= 2 and _is_prime(c):
                return c
        d += 1


def uneven_lengths(count=20000, total=1 << 28, lo=16, hi=1 << 20, seed=4):
    rng = np.random.default_rng(seed)
    raw = np.exp(rng.uniform(math.log(lo), math.log(hi), count))
    raw *= total / raw.sum()
    raw = np.maximum(raw, 2.0)
    prime = rng.uniform(0, 1, count) < 0.1
    sm = _smooth7(int(raw.max() * 2) + 16)
    out = []
    for v, p in zip(raw, prime):
        n = int(round(v))
        if p:
            out.append(_nearest_prime(max(n, 2)))
        else:
            i = bisect.bisect_left(sm, n)
            cands = [sm[j] for j in (i - 1, i) if 0 <= j < len(sm)]
            out.append(min(cands, key=lambda s: abs(math.log(s) - math.log(max(n, 1)))))
    return out


class MultiFFT:
    """Plan for many complex transforms of different lengths in one buffer."""

    def __init__(self, lengths, dtype=L.IG_F32, forward=True, fct=1.0, offsets=None):
        lib = L.load()
        self.lengths = list(int(n) for n in lengths)
        n = len(self.lengths)
        offs = L.arr(C.c_size_t, offsets) if offsets is not None else None
        self.h = lib.ig_make_multi_plan(dtype, n, L.arr(C.c_size_t, self.lengths), offs, int(forward), float(fct))
        if not self.h:
            raise L.FFTError(L.IG_EINVAL, lib.ig_last_error_string().decode())
        a, b, c = C.c_size_t(), C.c_size_t(), C.c_size_t()
        L.check(lib.ig_multi_info(self.h, C.byref(a), C.byref(b), C.byref(c)))
        self.info = {"worklist": a.value, "fourstep": b.value, "general": c.value}

    def __del__(self):
        if getattr(self, "h", None):
            L.load().ig_destroy_multi_plan(self.h)
            self.h = None

    def run_part(self, x_ptr, y_ptr, parts, stream=None):
        """One part of the sequence: mask of 1 (work-list phase 0), 2 (phase 1), 4 (general path)."""
        L.check(L.load().ig_multi_exec_part(self.h, x_ptr, y_ptr, int(parts), stream))

    def run(self, x_ptr, y_ptr, stream=None, mode="worklist"):
        lib = L.load()
        fn = {"worklist": lib.ig_multi_exec_device, "graph": lib.ig_multi_exec_graph,
              "loop": lib.ig_multi_exec_loop_device}[mode]
        L.check(fn(self.h, x_ptr, y_ptr, stream))
