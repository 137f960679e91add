"""CPU tests: the oracle (FP64 C restatement of PocketFFT + impulse's Nim glue)
pinned against golden vectors produced by the reference's own PocketFFT and
against the known answers of impulse's tests and README."""
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(__file__), "golden", "pocketfft_ref.npz")
TOL = 1e-14


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLD)


def test_cfft_vs_reference(oracle_lib, gold):
    for k in gold.files:
        if not k.startswith("cfft_in_"):
            continue
        n = int(k.split("_")[-1])
        x = gold[k]
        assert oracle_lib.rel_l2(oracle_lib.cfft(x, True, 1.0), gold[f"cfft_fwd_{n}"]) < TOL, n
        assert oracle_lib.rel_l2(oracle_lib.cfft(x, False, 1.0 / n), gold[f"cfft_bwd_{n}"]) < TOL, n


def test_rfft_halfcomplex_vs_reference(oracle_lib, gold):
    for k in gold.files:
        if not k.startswith("rfft_in_"):
            continue
        n = int(k.split("_")[-1])
        hc = oracle_lib.rfft_hc(gold[k], True, 1.0)
        assert oracle_lib.rel_l2(hc, gold[f"rfft_fwd_{n}"]) < TOL, n
        assert oracle_lib.rel_l2(oracle_lib.rfft_hc(gold[f"rfft_fwd_{n}"], False, 1.0 / n),
                                 gold[f"rfft_bwd_{n}"]) < TOL, n


def test_nd_vs_reference(oracle_lib, gold):
    x = gold["c2c_in"]
    assert oracle_lib.rel_l2(oracle_lib.c2c(x, [0, 2], True, 0.5), gold["c2c_fwd_axes02"]) < TOL
    assert oracle_lib.rel_l2(oracle_lib.c2c(x, [2, 1, 0], False, 1.0), gold["c2c_bwd_axes210"]) < TOL
    r = gold["r2c_in"]
    assert oracle_lib.rel_l2(oracle_lib.r2c(r, [0, 1], True, 1.0), gold["r2c_fwd_axes01"]) < TOL
    assert oracle_lib.rel_l2(oracle_lib.r2c(r, [2], False, 0.25), gold["r2c_bwd_axes2"]) < TOL
    c2r = oracle_lib.c2r(gold["r2c_fwd_axes01"], (8, 6, 5), [0, 1], False, 1.0 / 48)
    assert oracle_lib.rel_l2(c2r, gold["c2r_out_axes01"]) < TOL
    assert oracle_lib.rel_l2(c2r, r) < TOL  # round trip
    xf = gold["c2c32_in"].astype(np.complex128)
    assert oracle_lib.rel_l2(oracle_lib.c2c(xf, [1]), gold["c2c32_fwd_axes1"]) < 1e-6


def test_halfcomplex_equals_r2r_fftpack(oracle_lib, gold):
    """C rfft_forward layout == C++ r2r_fftpack(real2hermitian, forward)."""
    assert oracle_lib.rel_l2(oracle_lib.rfft_hc(gold["r2r_in"]), gold["r2r_fftpack"]) < TOL


def test_dct_dst_vs_reference(oracle_lib, gold):
    for k in gold.files:
        if "_in_" not in k or not (k.startswith("dct") or k.startswith("dst")):
            continue
        nm, n = k.split("_in_")
        n = int(n)
        t, sine = int(nm[3]), nm.startswith("dst")
        x = gold[k]
        got = oracle_lib.dct(x, [1], t, 0.5, False, sine=sine)
        assert oracle_lib.rel_l2(got, gold[f"{nm}_{n}"]) < TOL, (nm, n)
        got = oracle_lib.dct(x, [1], t, 1.0, True, sine=sine)
        assert oracle_lib.rel_l2(got, gold[f"{nm}_ortho_{n}"]) < TOL, (nm, n, "ortho")
    xr = gold["r2r3_in"]
    assert oracle_lib.rel_l2(oracle_lib.dct(xr, [0, 2], 2, 1.0, True), gold["dct2_axes02"]) < TOL


def test_r2r_and_hartley_vs_reference(oracle_lib, gold):
    xr = gold["r2r3_in"]
    for h in (0, 1):
        for f in (0, 1):
            got = oracle_lib.r2r_fftpack(xr, [1, 2], bool(h), bool(f), 0.5)
            assert oracle_lib.rel_l2(got, gold[f"r2r_fftpack_{h}{f}"]) < TOL, (h, f)
    assert oracle_lib.rel_l2(oracle_lib.hartley(xr, [1, 2], 0.5), gold["hartley_sep_axes12"]) < TOL
    assert oracle_lib.rel_l2(oracle_lib.hartley(xr, [0, 1, 2], 0.5, genuine=True), gold["hartley_gen_axes012"]) < TOL


def test_upfirdn_known_answers(oracle_lib):
    """The examples of upfirdn's documentation, impulse/signal.nim:560-592."""
    cases = [(([1, 1, 1], [1, 1, 1], 1, 1), [1, 2, 3, 2, 1]),
             (([1, 2, 3], [1], 3, 1), [1, 0, 0, 2, 0, 0, 3]),
             (([1, 2, 3], [1, 1, 1], 3, 1), [1, 1, 1, 2, 2, 2, 3, 3, 3]),
             (([1.0, 1.0, 1.0], [0.5, 1.0, 0.5], 2, 1), [0.5, 1, 1, 1, 1, 1, 0.5]),
             ((np.arange(10.0), [1.0], 1, 3), [0, 3, 6, 9]),
             ((np.arange(10.0), [0.5, 1.0, 0.5], 2, 3), [0, 1, 2.5, 4, 5.5, 7, 8.5])]
    for (t, h, up, down), want in cases:
        np.testing.assert_allclose(oracle_lib.upfirdn(t, h, up, down)[0], want, atol=1e-14)


def test_known_answers(oracle_lib):
    """tests/test_fft2.nim:7-15 and README.md:41,68,98."""
    x = np.arange(4.0)
    want = np.array([6, -2 + 2j, -2, -2 - 2j])
    assert np.allclose(oracle_lib.cfft(x.astype(complex)), want, atol=1e-15)
    assert np.allclose(oracle_lib.symmetrize(oracle_lib.rfft_hc(x)), want, atol=1e-15)
    d5 = np.array([1.0, 2.0, 1.0, -1.0, 1.5])
    hc5 = [4.5, 2.081559480312316, -1.651098762732523, -1.831559480312316, 1.608220406444071]
    assert np.allclose(oracle_lib.rfft_hc(d5), hc5, atol=1e-14)
    full = oracle_lib.symmetrize(oracle_lib.rfft_hc(d5))
    assert np.allclose(full, [4.5, 2.081559480312316 - 1.651098762732523j, -1.831559480312316 + 1.608220406444071j,
                              -1.831559480312316 - 1.608220406444071j, 2.081559480312316 + 1.651098762732523j],
                       atol=1e-14)
    r2c = oracle_lib.r2c(d5, [0])
    assert np.allclose(r2c, full[:3], atol=1e-14)


def test_roundtrip_like_test_fft_nim(oracle_lib):
    """tests/test_fft.nim:29-52: rfft_forward then rfft_backward(1/n) within 2e-15, lengths 1..600."""
    rng = np.random.default_rng(0)
    odata = rng.uniform(-0.5, 0.5, 600)
    odata[0] = 0.340188
    for n in range(1, 600):
        d = oracle_lib.rfft_hc(odata[:n], True, 1.0)
        d = oracle_lib.rfft_hc(d, False, 1.0 / n)
        assert oracle_lib.rel_l2(d, odata[:n]) < 2e-15, n


def test_plan_heuristics(oracle_lib):
    """pocketfft.c:205-260, 2066-2153: Bluestein for 1009, 8191, 65521 with n2 = 2025, 16384, 131072."""
    for n, n2 in ((1009, 2025), (8191, 16384), (65521, 131072)):
        assert oracle_lib.uses_bluestein(n, False)
        assert oracle_lib.uses_bluestein(n, True)
        assert oracle_lib.good_size(2 * n - 1) == n2
    for n in (64, 4096, 9240, 49, 97 * 2):
        assert not oracle_lib.uses_bluestein(n, False)


def test_nim_glue_mirror_matches_oracle(oracle_lib):
    """impulse_gb300.fft restates pocketfft.nim's unpackFFT / symmetrize / initNormalize (host code, no GPU)."""
    from impulse_gb300 import fft as F
    rng = np.random.default_rng(4)
    for n in (1, 2, 3, 4, 5, 8, 9, 64, 65):
        hc = rng.standard_normal(n)
        assert np.array_equal(F.unpackFFT(hc), oracle_lib.unpack_fft(hc))
        assert np.array_equal(F.symmetrize(hc), oracle_lib.symmetrize(hc))
        c = rng.standard_normal(n // 2 + 1) + 1j * rng.standard_normal(n // 2 + 1)
        assert np.array_equal(F.symmetrize(c), oracle_lib.symmetrize(c))
    for kind in range(4):
        for fwd in (True, False):
            assert F.initNormalize(kind, fwd, 0.3, 16) == oracle_lib.init_normalize(kind, fwd, 0.3, 16)


def test_oracle_error_codes(oracle_lib):
    x = np.zeros((3, 4), complex)
    with pytest.raises(ValueError, match="-2"):
        oracle_lib.c2c(x, [2])
    with pytest.raises(ValueError, match="-3"):
        oracle_lib.c2c(x, [1, 1])
