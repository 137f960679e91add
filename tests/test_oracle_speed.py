"""Speed of the oracle port against the reference's own PocketFFT (CPU).

The benchmark's CPU baseline and its reference arm time this repository's
FP64 restatement of PocketFFT (oracle/impulse_oracle.c), because the
reference's compiled PocketFFT cannot run on the GPU host.  For those numbers
to stand for impulse's CPU path, the port must run about as fast as the
reference on the same work.  This test times, single-threaded and on a
bounded sample of the halfcomplex benchmark workload (every length, 1/512 of
its batch), the port's batched transform against the reference compiled in
place without SIMD (as PocketFFT builds on aarch64 hosts):
pocketfft::r2r_fftpack (pocketfft_hdronly.h:3392-3445, the C++ backend) and
the C backend's rfft_forward line loop (pocketfft.c:2184, as impulse's
fft(var openArray[float]) calls it), and requires the port to be within 1.5x
of the faster of the two.  It runs where the reference checkout was built
(oracle/_ref); elsewhere it is skipped.
"""
import ctypes as C
import os
import time

import numpy as np
import pytest


def _best(fn, reps=3):
    best = float("inf")
    for _ in range(reps):
        t0 = time.perf_counter()
        fn()
        best = min(best, time.perf_counter() - t0)
    return best


def test_port_within_1p5x_of_pocketfft():
    from oracle import oracle as O
    if not os.path.exists(O.REF_SCALAR_SO):
        pytest.skip("reference PocketFFT not built here (needs IMPULSE_REF at build time)")
    import bench
    L = O.lib()
    R = O.ref_scalar()
    dp = C.POINTER(C.c_double)
    arr = lambda t, v: (t * len(v))(*v)
    rng = np.random.default_rng(2)
    t_port = t_hdr = t_pfc = 0.0
    for n in bench.workload_lengths():
        b = max(2, bench.batch_for(n) // 512)
        x = rng.standard_normal((b, n))
        a = x.copy()
        t_port += _best(lambda: L.io_rfft_batch(n, b, a.ctypes.data_as(dp), n, 1, 1.0, 1))
        y = np.empty_like(x)
        shp, st = arr(C.c_size_t, [b, n]), arr(C.c_ssize_t, [8 * n, 8])
        t_hdr += _best(lambda: R.ref_r2r_fftpack_f64(2, shp, st, st, 1, arr(C.c_size_t, [1]), 1, 1,
                                                     x.ctypes.data, y.ctypes.data, 1.0, 1))
        c = x.copy()
        t_pfc += _best(lambda: R.ref_rfft_batch(n, b, c.ctypes.data_as(dp), 1, 1.0))
    ratio = t_port / min(t_hdr, t_pfc)
    print(f"port {t_port:.3f} s, r2r_fftpack {t_hdr:.3f} s, rfft_forward loop {t_pfc:.3f} s, ratio {ratio:.2f}")
    assert ratio <= 1.5, (t_port, t_hdr, t_pfc)
