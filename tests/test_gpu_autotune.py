"""GPU parity of autotuned plans: every tuned configuration must give the oracle's results."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,kind,dtype", [
    (4096, 1, "f64"),     # single-CTA core: radix order x E x lines per CTA
    (1000, 0, "f32"),
    (2205, 1, "f64"),     # odd real length, paired lines
    (52272, 1, "f64"),    # four-step split
    (65521, 1, "f32"),    # Bluestein over a four-step core
])
def test_tuned_plan_matches_oracle(engine, oracle_lib, n, kind, dtype):
    from impulse_gb300 import _lib as L
    from impulse_gb300 import fft as F
    code = L.IG_F32 if dtype == "f32" else L.IG_F64
    ms = F.autotune(n, code, kind)
    assert ms > 0
    rng = np.random.default_rng(n)
    tol = 1e-12 if dtype == "f64" else 2e-6 * max(1.0, np.log2(n))
    if kind == 1:
        x = rng.standard_normal((6, n))
        got = F.rfft_batch(x.astype(np.float32) if dtype == "f32" else x, True, 1.0)
        for r in range(6):
            want = oracle_lib.rfft_hc(x[r], True, 1.0)
            assert oracle_lib.rel_l2(got[r], want) < tol
    else:
        x = rng.standard_normal((6, n)) + 1j * rng.standard_normal((6, n))
        got = F.cfft_batch(x.astype(np.complex64) if dtype == "f32" else x, True, 1.0)
        for r in range(6):
            want = oracle_lib.cfft(x[r], True, 1.0)
            assert oracle_lib.rel_l2(got[r], want) < tol


def test_tune_table_round_trip(engine, oracle_lib, tmp_path):
    from impulse_gb300 import _lib as L
    from impulse_gb300 import fft as F
    F.autotune(3000, L.IG_F64, 0)
    path = tmp_path / "tune.tsv"
    F.autotune_save(str(path))
    rows = path.read_text().strip().splitlines()
    assert any(r.split("\t")[2] == "3000" for r in rows)
    F.autotune_load(str(path))
    x = np.random.default_rng(2).standard_normal((3, 3000)) + 0j
    got = F.cfft_batch(x, False, 0.25)
    for r in range(3):
        assert oracle_lib.rel_l2(got[r], oracle_lib.cfft(x[r], False, 0.25)) < 1e-12
    with pytest.raises(L.FFTError):
        F.autotune_load(str(tmp_path / "missing.tsv"))
