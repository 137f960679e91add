"""GPU parity of host-memory batches larger than one pipeline chunk (16 MiB):
page-locked and pageable buffers, line gaps, lines off a 16-byte boundary.
Pageable buffers on a GPU that walks the host page tables are copied by SM
copy kernels (16-, 8- and 4-byte units by alignment); IG_PAGEABLE_CE=1 in a
child process keeps the copy engines and must give identical bytes."""
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


@pytest.mark.parametrize("n,dist", [(4096, 4096), (1000, 1003)])
def test_pageable_f32_lines_off_8_bytes(engine, oracle_lib, n, dist):
    """FP32 real lines in pageable memory starting 4 bytes past an 8-byte
    boundary: the copy kernels move 4-byte units; the words before and between
    the lines stay untouched."""
    from impulse_gb300 import _lib as L
    lib = L.load()
    batch = (40 << 20) // (4 * dist)
    rng = np.random.default_rng(dist)
    buf = rng.standard_normal(batch * dist + 2).astype(np.float32)
    x = buf.copy()
    off = 1 if buf.ctypes.data % 8 == 0 else 2  # start at 4 mod 8
    ptr = buf.ctypes.data + 4 * off
    assert ptr % 8 == 4
    plan = lib.ig_make_rfft_plan(n, L.IG_F32)
    try:
        L.check(lib.ig_rfft_exec_batch(plan, ptr, batch, dist, 1, 1.0))
    finally:
        lib.ig_destroy_rfft_plan(plan)
    y = buf[off:off + batch * dist].reshape(batch, dist)
    xs = x[off:off + batch * dist].reshape(batch, dist)
    assert np.array_equal(buf[:off], x[:off]) and np.array_equal(buf[off + batch * dist:], x[off + batch * dist:])
    assert np.array_equal(y[:, n:], xs[:, n:])
    rows = [0, 1, batch // 3, batch - 1]
    want = oracle_lib.rfft_hc(xs[rows, :n].astype(np.float64), forward=True, fct=1.0)
    assert oracle_lib.rel_l2(y[rows, :n].astype(np.float64), want) < 1e-6 * np.log2(n)


CHILD = r"""
import ctypes as C, hashlib, sys
import numpy as np
sys.path.insert(0, sys.argv[1])
from impulse_gb300 import _lib as L
lib = L.load()
n = 4096
x = np.random.default_rng(3).standard_normal((5000, n))
plan = lib.ig_make_rfft_plan(n, L.IG_F64)
L.check(lib.ig_rfft_exec_batch(plan, x.ctypes.data, 5000, n, 1, 1.0))
print(hashlib.sha256(x.tobytes()).hexdigest())
"""


def test_pageable_sm_copies_match_copy_engines(engine):
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    outs = []
    for extra in ({}, {"IG_PAGEABLE_CE": "1"}):
        env = dict(os.environ)
        env.pop("IG_PAGEABLE_CE", None)
        env.update(extra)
        r = subprocess.run([sys.executable, "-c", CHILD, root], capture_output=True, text=True, env=env, timeout=600)
        assert r.returncode == 0, r.stderr[-2000:]
        outs.append(r.stdout.strip().splitlines()[-1])
    assert outs[0] == outs[1]


@pytest.mark.parametrize("dtype", [np.complex128, np.complex64])
@pytest.mark.parametrize("n,dist", [(4096, 4096), (1000, 1001)])
def test_cfft_exec_batch_pageable(engine, oracle_lib, dtype, n, dist):
    """Complex lines in pageable memory, several pipeline chunks, line gaps:
    the SM copy kernels in both directions, checked against the oracle and the
    gaps left untouched."""
    from impulse_gb300 import _lib as L
    lib = L.load()
    es = np.dtype(dtype).itemsize
    batch = (48 << 20) // (es * dist)
    rng = np.random.default_rng(n + es)
    x = (rng.standard_normal((batch, dist)) + 1j * rng.standard_normal((batch, dist))).astype(dtype)
    h = x.copy()
    code = L.IG_F64 if dtype == np.complex128 else L.IG_F32
    plan = lib.ig_make_cfft_plan(n, code)
    try:
        L.check(lib.ig_cfft_exec_batch(plan, h.ctypes.data, batch, dist, 1, 0.5))
    finally:
        lib.ig_destroy_cfft_plan(plan)
    assert np.array_equal(h[:, n:], x[:, n:])
    tol = 1e-12 if dtype == np.complex128 else 2e-6 * np.log2(n)
    rows = [0, batch // 2, batch - 1]
    want = oracle_lib.cfft(x[rows, :n].astype(np.complex128), True, 0.5)
    assert oracle_lib.rel_l2(h[rows, :n], want) < tol
