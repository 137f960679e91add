"""GPU parity of host-memory batches larger than one pipeline chunk (16 MiB):
page-locked and pageable buffers, line gaps, lines off a 16-byte boundary."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("pinned", [True, False])
@pytest.mark.parametrize("n,dist", [(4096, 4096), (3000, 3007), (8191, 8191)])
def test_rfft_exec_batch_pipelined(engine, oracle_lib, pinned, n, dist):
    torch = pytest.importorskip("torch")
    from impulse_gb300 import _lib as L
    from impulse_gb300 import fft as F
    lib = L.load()
    batch = (160 << 20) // (8 * dist)  # ~160 MiB: several chunks
    rng = np.random.default_rng(n)
    x = rng.standard_normal((batch, dist))
    if pinned:
        h = torch.from_numpy(x.copy()).pin_memory()
        ptr = h.data_ptr()
    else:
        h = x.copy()
        ptr = h.ctypes.data
    plan = F.FFTPlanReal(n, L.IG_F64)
    L.check(lib.ig_rfft_exec_batch(plan.pocket, ptr, batch, dist, 1, 1.0))
    y = h.numpy() if pinned else h
    for r in (0, 1, batch // 2, batch - 1):
        want = oracle_lib.rfft_hc(x[r, :n], True, 1.0)
        assert oracle_lib.rel_l2(y[r, :n], want) < 1e-12, r
        assert np.array_equal(y[r, n:], x[r, n:])  # gaps untouched
    # back again
    L.check(lib.ig_rfft_exec_batch(plan.pocket, ptr, batch, dist, 0, 1.0 / n))
    y = h.numpy() if pinned else h
    assert oracle_lib.rel_l2(y[:, :n], x[:, :n]) < 1e-12


def test_device_pointers_offset_by_one_real(engine, oracle_lib):
    """Lines that start 8 bytes past a 16-byte boundary: the kernels read the
    two halves of each complex value separately instead of as one pair."""
    torch = pytest.importorskip("torch")
    from impulse_gb300 import _lib as L
    lib = L.load()
    n, b = 4096, 64
    rng = np.random.default_rng(1)
    x = rng.standard_normal(b * n)
    buf = torch.zeros(b * n + 1, dtype=torch.float64, device="cuda")
    buf[1:] = torch.from_numpy(x).cuda()
    out = torch.zeros(b * n + 1, dtype=torch.float64, device="cuda")
    plan = lib.ig_make_rfft_plan(n, L.IG_F64)
    try:
        L.check(lib.ig_rfft_exec_device(plan, buf.data_ptr() + 8, out.data_ptr() + 8, b, n, n, 1, 1.0, None))
        torch.cuda.synchronize()
        y = out[1:].cpu().numpy().reshape(b, n)
        for r in (0, b - 1):
            assert oracle_lib.rel_l2(y[r], oracle_lib.rfft_hc(x.reshape(b, n)[r], True, 1.0)) < 1e-12
    finally:
        lib.ig_destroy_rfft_plan(plan)
    # complex lines at an 8-byte offset
    cplan = lib.ig_make_cfft_plan(1000, L.IG_F64)
    try:
        z = rng.standard_normal((3, 1000)) + 1j * rng.standard_normal((3, 1000))
        zb = torch.zeros(2 * 3000 + 1, dtype=torch.float64, device="cuda")
        zb[1:] = torch.from_numpy(z.view(np.float64).ravel()).cuda()
        L.check(lib.ig_cfft_exec_device(cplan, zb.data_ptr() + 8, zb.data_ptr() + 8, 3, 1000, 1000, 1, 1.0, None))
        torch.cuda.synchronize()
        got = zb[1:].cpu().numpy().view(np.complex128).reshape(3, 1000)
        for r in range(3):
            assert oracle_lib.rel_l2(got[r], oracle_lib.cfft(z[r], True, 1.0)) < 1e-12
        # the no-allocation entry refuses such pointers instead of faulting
        rc = lib.ig_cfft_exec_device_noalloc(cplan, zb.data_ptr() + 8, zb.data_ptr() + 8, 3, 1000, 1000, 1, 1.0, None)
        assert rc == L.IG_EINVAL
    finally:
        lib.ig_destroy_cfft_plan(cplan)
