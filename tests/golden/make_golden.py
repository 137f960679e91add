"""Generates tests/golden/pocketfft_ref.npz from impulse's own PocketFFT.

The reference's C backend (impulse/fft/c_pocketfft/pocketfft.c) and C++
backend (impulse/fft/cpp_pocketfft/pocketfft_hdronly.h) are compiled in place
by ``make -C oracle ref`` (IMPULSE_REF points at the impulse checkout) and
called through ctypes; inputs are seeded numpy draws saved beside the
outputs.  Run from the repository root:

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle import oracle as O  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "pocketfft_ref.npz")

CFFT_LENGTHS = list(range(1, 33)) + [48, 64, 97, 100, 128, 360, 1009, 2025, 4096]
RFFT_LENGTHS = list(range(1, 41)) + [64, 100, 101, 1009, 4096, 8191]


def main():
    O.build(ref=True)
    assert O.ref_available(), "reference PocketFFT not built (set IMPULSE_REF)"
    rng = np.random.default_rng(20240601)
    d = {}
    for n in CFFT_LENGTHS:
        x = rng.uniform(-1, 1, n) + 1j * rng.uniform(-1, 1, n)
        d[f"cfft_in_{n}"] = x
        d[f"cfft_fwd_{n}"] = O.ref_cfft(x, True, 1.0)
        d[f"cfft_bwd_{n}"] = O.ref_cfft(x, False, 1.0 / n)
    for n in RFFT_LENGTHS:
        x = rng.standard_normal(n)
        d[f"rfft_in_{n}"] = x
        hc = O.ref_rfft_hc(x, True, 1.0)
        d[f"rfft_fwd_{n}"] = hc
        d[f"rfft_bwd_{n}"] = O.ref_rfft_hc(hc, False, 1.0 / n)
    # N-d through the C++ backend's templates
    x = rng.uniform(-1, 1, (6, 10, 7)) + 1j * rng.uniform(-1, 1, (6, 10, 7))
    d["c2c_in"] = x
    d["c2c_fwd_axes02"] = O.ref_c2c(x, [0, 2], True, 0.5)
    d["c2c_bwd_axes210"] = O.ref_c2c(x, [2, 1, 0], False, 1.0)
    r = rng.uniform(-1, 1, (8, 6, 5))
    d["r2c_in"] = r
    d["r2c_fwd_axes01"] = O.ref_r2c(r, [0, 1], True, 1.0)
    d["r2c_bwd_axes2"] = O.ref_r2c(r, [2], False, 0.25)
    d["c2r_out_axes01"] = O.ref_c2r(d["r2c_fwd_axes01"], (8, 6, 5), [0, 1], False, 1.0 / 48)
    xf = (rng.uniform(-1, 1, (5, 12)) + 1j * rng.uniform(-1, 1, (5, 12))).astype(np.complex64)
    d["c2c32_in"] = xf
    d["c2c32_fwd_axes1"] = O.ref_c2c(xf, [1], True, 1.0)
    # halfcomplex layout of the C backend equals r2r_fftpack(real2hermitian, forward) of the C++ backend
    rr = rng.standard_normal((4, 30))
    d["r2r_in"] = rr
    d["r2r_fftpack"] = O.ref_r2r_fftpack(rr, [1], True, True, 1.0)
    # real-to-real transforms of the C++ backend (DCTDesc.apply -> pocketfft::dct, and the
    # bound dst / r2r_fftpack / Hartley templates)
    for sine in (False, True):
        nm = "dst" if sine else "dct"
        for t in (1, 2, 3, 4):
            for n in (2, 3, 8, 9, 16, 31):
                x = rng.standard_normal((2, n))
                d[f"{nm}{t}_in_{n}"] = x
                d[f"{nm}{t}_{n}"] = O.ref_dct(x, [1], t, 0.5, False, sine=sine)
                d[f"{nm}{t}_ortho_{n}"] = O.ref_dct(x, [1], t, 1.0, True, sine=sine)
    xr = rng.standard_normal((4, 6, 5))
    d["r2r3_in"] = xr
    for h in (0, 1):
        for f in (0, 1):
            d[f"r2r_fftpack_{h}{f}"] = O.ref_r2r_fftpack(xr, [1, 2], bool(h), bool(f), 0.5)
    d["dct2_axes02"] = O.ref_dct(xr, [0, 2], 2, 1.0, True)
    d["hartley_sep_axes12"] = O.ref_hartley(xr, [1, 2], 0.5, genuine=False)
    d["hartley_gen_axes012"] = O.ref_hartley(xr, [0, 1, 2], 0.5, genuine=True)
    np.savez_compressed(OUT, **d)
    print(OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
