"""GPU parity of the pipelined FP32 line kernel (k_fft_line_pipe: input lines
staged into shared memory by bulk copies, persistent CTAs).  The kernel is off
by default and selected with IG_PIPE=1 at process start, so each case runs in
a child process with and without it: the outputs must be bit-identical (the
same butterflies in the same order), match the FP64 oracle within the FP32
bound, and no bounded wait may have given up."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import ctypes as C, json, sys
import numpy as np, torch
sys.path.insert(0, sys.argv[1])
from impulse_gb300 import _lib as L
lib = L.load()
s = C.c_void_p(torch.cuda.current_stream().cuda_stream)
out = {}
for kind, n, b, fwd in json.loads(sys.argv[2]):
    rng = np.random.default_rng(n * 7 + b)
    if kind == "r":
        x = torch.from_numpy(rng.standard_normal((b, n)).astype(np.float32)).cuda()
        plan = lib.ig_make_rfft_plan(n, L.IG_F32); fn = lib.ig_rfft_exec_device; des = lib.ig_destroy_rfft_plan
    else:
        x = torch.from_numpy((rng.standard_normal((b, n)) + 1j * rng.standard_normal((b, n))).astype(np.complex64)).cuda()
        plan = lib.ig_make_cfft_plan(n, L.IG_F32); fn = lib.ig_cfft_exec_device; des = lib.ig_destroy_cfft_plan
    y = torch.empty_like(x)
    L.check(fn(plan, x.data_ptr(), y.data_ptr(), b, n, n, fwd, 0.5, s))
    torch.cuda.synchronize()
    des(plan)
    out[f"{kind}{n}x{b}f{fwd}"] = y.cpu().numpy().tolist() if kind == "r" else [y.real.cpu().numpy().tolist(), y.imag.cpu().numpy().tolist()]
cnt = C.c_uint(0)
L.check(lib.ig_device_faults(C.byref(cnt)))
print(json.dumps({"faults": cnt.value, "out": out}))
"""

# (kind, length, lines, forward): every first / last radix class the line
# kernel compiles, one-line and many-line tiles, a partial last tile
CASES = [("r", 256, 301, 1), ("r", 4096, 37, 1), ("r", 132, 77, 1), ("r", 180, 50, 1), ("r", 7840, 5, 1),
         ("r", 1200, 9, 1), ("r", 96, 130, 1), ("c", 4096, 19, 1), ("c", 4096, 19, 0), ("c", 256, 65, 0),
         ("c", 1000, 7, 1), ("c", 8192, 3, 1)]


def _run(env_extra):
    env = dict(os.environ)
    env.pop("IG_PIPE", None)
    env.pop("IG_NO_PAIR", None)
    env.update(env_extra)
    r = subprocess.run([sys.executable, "-c", CHILD, ROOT, json.dumps(CASES)], capture_output=True, text=True,
                       env=env, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    return json.loads(r.stdout.strip().splitlines()[-1])


def test_pipelined_lines_match_default_and_oracle(engine, oracle_lib):
    # the default FP32 path for these lines is the paired-lane kernel; the
    # bit-for-bit reference of the pipelined kernel is k_fft_line
    piped = _run({"IG_PIPE": "1"})
    plain = _run({"IG_NO_PAIR": "1"})
    assert piped["faults"] == 0
    for kind, n, b, fwd in CASES:
        key = f"{kind}{n}x{b}f{fwd}"
        a = np.asarray(piped["out"][key], dtype=np.float64)
        assert np.array_equal(a, np.asarray(plain["out"][key], dtype=np.float64)), key
        rng = np.random.default_rng(n * 7 + b)
        tol = 1e-6 * max(1.0, np.log2(n))
        if kind == "r":
            x = rng.standard_normal((b, n)).astype(np.float32).astype(np.float64)
            want = oracle_lib.rfft_hc(x, forward=True, fct=0.5)
            assert oracle_lib.rel_l2(a, want) < tol, key
        else:
            x = (rng.standard_normal((b, n)) + 1j * rng.standard_normal((b, n))).astype(np.complex64)
            want = oracle_lib.cfft(x.astype(np.complex128), bool(fwd), 0.5)
            got = a[0] + 1j * a[1]
            assert oracle_lib.rel_l2(got, want) < tol, key
