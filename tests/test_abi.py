"""CPU tests of the C ABI: the library builds for sm_103a, loads, exports every
function include/impulse_gpu.h declares, and reports argument errors with the
reference's error model before touching the GPU."""
import ctypes as C
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "impulse_gpu.h")


def header_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(ig_[a-z0-9_]+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    from impulse_gb300 import _lib, build
    if not os.path.exists(_lib.LIB_PATH):
        build.build()
    return _lib.load()


def test_exports_every_declared_symbol(lib):
    from impulse_gb300 import _lib
    names = header_functions()
    assert len(names) >= 28
    for n in names:
        assert hasattr(lib, n), n
        assert n in _lib.SIGNATURES, n


def test_only_c_abi_exported(lib):
    import subprocess
    from impulse_gb300 import _lib
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB_PATH], capture_output=True, text=True).stdout
    syms = [ln.split()[-1] for ln in out.splitlines() if " T " in ln]
    assert syms and all(s.startswith("ig_") for s in syms), syms


def test_version_and_error_string(lib):
    assert lib.ig_version() >= 100
    assert isinstance(lib.ig_last_error_string(), bytes)


def _nd(lib, fn, shape, axes, inplace=False, sout=None):
    from impulse_gb300 import _lib as L
    x = np.zeros(shape, np.complex128)
    y = x if inplace else np.zeros(shape, np.complex128)
    si = list(x.strides)
    so = list(sout if sout is not None else y.strides)
    return fn(L.IG_F64, len(shape), L.arr(C.c_size_t, shape), L.arr(C.c_ssize_t, si), L.arr(C.c_ssize_t, so),
              len(axes), L.arr(C.c_size_t, axes), 1, x.ctypes.data, y.ctypes.data, 1.0, 1)


def test_error_model(lib):
    """pocketfft_hdronly.h:446-477 exceptions become status codes, with the same messages."""
    from impulse_gb300 import _lib as L
    assert _nd(lib, lib.ig_c2c, (4, 5), [2]) == L.IG_EINVAL_AXIS
    assert lib.ig_last_error_string() == b"bad axis number"
    assert _nd(lib, lib.ig_c2c, (4, 5), [1, 1]) == L.IG_EREPEAT_AXIS
    assert lib.ig_last_error_string() == b"axis specified repeatedly"
    assert _nd(lib, lib.ig_c2c, (4, 5), [0], inplace=True, sout=[16, 64]) == L.IG_ESTRIDE_INPLACE
    assert lib.ig_last_error_string() == b"stride mismatch"
    assert _nd(lib, lib.ig_c2c, (0, 5), [0]) == L.IG_OK      # empty shape: early return
    assert _nd(lib, lib.ig_r2c, (4, 5), [3]) == L.IG_EINVAL_AXIS
    assert _nd(lib, lib.ig_c2r, (4, 5), [0, 0]) == L.IG_EREPEAT_AXIS
    assert lib.ig_make_cfft_plan(0, L.IG_F64) is None       # make_cfft_plan(0) -> NULL
    assert lib.ig_last_error_string() == b"zero-length FFT requested"
    assert lib.ig_make_rfft_plan(0, L.IG_F32) is None
    assert lib.ig_set_f64_arith(7) == L.IG_EINVAL
    assert lib.ig_cfft_forward(None, None, 1.0) == L.IG_EINVAL


def test_api_mirror_raises_like_reference(lib):
    """callFFT (pocketfft.nim:206-214): a failing plan raises; zero length fails at plan time."""
    from impulse_gb300 import fft as F
    from impulse_gb300 import _lib as L
    with pytest.raises(L.FFTError):
        F.FFTPlanComplex(0)


def test_device_api_rejects_host_tensors(lib):
    """The device-resident mirror takes CUDA tensors only; host data goes through impulse_gb300.fft."""
    torch = pytest.importorskip("torch")
    from impulse_gb300 import device as D
    x = torch.zeros(8, dtype=torch.float64)
    with pytest.raises(TypeError):
        D.tensor_rfft_packed(x)
    with pytest.raises(TypeError):
        D.DataDesc(x, (8,))
