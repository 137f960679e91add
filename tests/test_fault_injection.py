"""Allocation-failure handling, injected on the host (no GPU fault is made).

impulse's callFFT (impulse/fft/c_pocketfft/pocketfft.nim:206-214) raises
"Forward FFT calculation failed." / "Backward FFT calculation failed." when
the C call returns non-zero; PocketFFT returns -1 when its scratch malloc
fails (pocketfft.c:878).  The engine returns IG_ENOMEM (-1) when a device
allocation fails; IG_FAIL_MALLOC makes every engine allocation fail, so the
whole error path runs without exhausting memory.

* CPU: the Python mirror of callFFT turns a failing status of a fake engine
  into the reference's exception texts.
* GPU: with IG_FAIL_MALLOC set, a host-memory transform that needs a fresh
  workspace returns IG_ENOMEM with the injected message, the mirror raises
  the reference's text, and the engine works again once the variable is gone.
"""
import ctypes as C
import os

import numpy as np
import pytest


class _FakeEngine:
    """Stands in for libimpulse_gpu.so: plans are handles, executions fail with IG_ENOMEM."""

    def __init__(self):
        self.destroyed = 0

    def ig_make_rfft_plan(self, n, dtype):
        return 1234

    def ig_make_cfft_plan(self, n, dtype):
        return 1234

    def ig_destroy_rfft_plan(self, p):
        self.destroyed += 1

    def ig_destroy_cfft_plan(self, p):
        self.destroyed += 1

    def _fail(self, *a):
        return -1

    ig_rfft_forward = ig_rfft_backward = ig_cfft_forward = ig_cfft_backward = _fail

    def ig_last_error_string(self):
        return b"cudaMalloc: injected failure (IG_FAIL_MALLOC)"


@pytest.mark.parametrize("real", [True, False])
def test_callfft_raises_reference_texts(monkeypatch, real):
    from impulse_gb300 import _lib as L
    from impulse_gb300 import fft as F
    fake = _FakeEngine()
    monkeypatch.setattr(L, "load", lambda: fake)
    data = np.zeros(8) if real else np.zeros(8, np.complex128)
    with pytest.raises(Exception, match=r"^Forward FFT calculation failed\.$"):
        F.fft_inplace(data, True)
    with pytest.raises(Exception, match=r"^Backward FFT calculation failed\.$"):
        F.fft_inplace(data, False)
    assert fake.destroyed >= 1


@pytest.mark.gpu
def test_injected_device_malloc_failure(engine, oracle_lib, monkeypatch):
    from impulse_gb300 import _lib as L
    from impulse_gb300 import fft as F
    lib = engine
    n = 3000
    lib.ig_release_caches()  # the next host-memory call has to allocate its workspace
    plan = F.FFTPlanReal(n)
    x = np.random.default_rng(9).standard_normal(n)
    data = x.copy()
    monkeypatch.setenv("IG_FAIL_MALLOC", "1")
    rc = lib.ig_rfft_forward(plan.pocket, data.ctypes.data_as(C.c_void_p), 1.0)
    assert rc == L.IG_ENOMEM
    assert b"injected failure" in lib.ig_last_error_string()
    with pytest.raises(Exception, match=r"^Forward FFT calculation failed\.$"):
        F._call(plan, True, data, True, 1.0)
    with pytest.raises(Exception, match=r"^Backward FFT calculation failed\.$"):
        F._call(plan, True, data, False, 1.0)
    # a new plan cannot be built either (pocketfft's make_rfft_plan returns NULL)
    with pytest.raises(L.FFTError):
        F.FFTPlanReal(3001)
    monkeypatch.delenv("IG_FAIL_MALLOC")
    assert "IG_FAIL_MALLOC" not in os.environ
    data = x.copy()
    F._call(plan, True, data, True, 1.0)
    assert oracle_lib.rel_l2(data, oracle_lib.rfft_hc(x, True)) < 1e-12
