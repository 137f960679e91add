"""GPU test of ig_cfft_exec_device_noalloc, the allocation-free entry point.

Callers that cannot allocate device memory while they run -- a process whose
device-memory budget is reserved up front in a pool that must not grow, or a
latency-bound loop where cudaMalloc / cudaFree are not allowed -- use this
call; its scratch is a static device array instead of the engine's cached
workspace.  The test calls it through the C ABI and compares it with
ig_cfft_exec_device and with the FP64 oracle on the same inputs, twice in a
row (the array keeps the previous call's contents), for a single-CTA length
and for four-step lengths, and checks the size limit.  This file is collected
last so that a first-failure run has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = {np.complex128: 1e-12, np.complex64: 2e-6}


def _run(lib, fn, plan, x, fwd, fct):
    import torch
    dt = torch.complex128 if x.dtype == np.complex128 else torch.complex64
    d_in = torch.from_numpy(x).to("cuda", dtype=dt)
    d_out = torch.empty_like(d_in)
    b, n = x.shape
    s = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = fn(plan, d_in.data_ptr(), d_out.data_ptr(), b, n, n, int(fwd), fct, s)
    torch.cuda.synchronize()
    return rc, d_out.cpu().numpy()


@pytest.mark.parametrize("n,b", [(4096, 8), (32768, 4), (65536, 3), (1 << 20, 2)])
@pytest.mark.parametrize("dtype", [np.complex128, np.complex64])
def test_noalloc_matches_exec_device(engine, oracle_lib, n, b, dtype):
    from impulse_gb300 import _lib as L
    lib = engine
    code = L.IG_F64 if dtype == np.complex128 else L.IG_F32
    plan = lib.ig_make_cfft_plan(n, code)
    assert plan, lib.ig_last_error_string()
    try:
        rng = np.random.default_rng(n + b)
        for call in range(2):  # two calls in a row on the shared static scratch
            x = (rng.uniform(-1, 1, (b, n)) + 1j * rng.uniform(-1, 1, (b, n))).astype(dtype)
            fwd = call == 0
            rc0, want = _run(lib, lib.ig_cfft_exec_device, plan, x, fwd, 0.5)
            assert rc0 == 0, lib.ig_last_error_string()
            rc1, got = _run(lib, lib.ig_cfft_exec_device_noalloc, plan, x, fwd, 0.5)
            assert rc1 == 0, lib.ig_last_error_string()
            err = np.linalg.norm(got - want) / np.linalg.norm(want)
            assert err <= TOL[dtype], (n, b, call, err)
            # and against the FP64 oracle on the same input
            ref = oracle_lib.cfft(x.astype(np.complex128), fwd, 0.5)
            tol = 1e-12 if dtype == np.complex128 else 1e-6 * np.log2(n)
            err_o = oracle_lib.rel_l2(got, ref)
            assert err_o <= tol, (n, b, call, err_o)
    finally:
        lib.ig_destroy_cfft_plan(plan)


def test_noalloc_rejects_oversize(engine):
    from impulse_gb300 import _lib as L
    lib = engine
    n = 1 << 20
    plan = lib.ig_make_cfft_plan(n, L.IG_F64)
    try:
        import torch
        x = torch.zeros((5, n), dtype=torch.complex128, device="cuda")  # 80 MiB > 64 MiB
        rc = lib.ig_cfft_exec_device_noalloc(plan, x.data_ptr(), x.data_ptr(), 5, n, n, 1, 1.0, None)
        assert rc == L.IG_ETOOLARGE
        assert b"64 MiB" in lib.ig_last_error_string()
    finally:
        lib.ig_destroy_cfft_plan(plan)
