"""ctypes binding of libimpulse_gpu.so (the C ABI in include/impulse_gpu.h).

The library is loaded from this package directory only.  There is no
fallback: if it is missing or does not load, importing raises, so a missing
extension fails loudly instead of silently running something else.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libimpulse_gpu.so")

IG_OK = 0
IG_ENOMEM = -1
IG_EINVAL_AXIS = -2
IG_EREPEAT_AXIS = -3
IG_ESTRIDE_INPLACE = -4
IG_EZERO_LEN = -5
IG_ECUDA = -6
IG_ENDIM = -7
IG_EINVAL = -8
IG_ETIMEOUT = -9
IG_ETOOLARGE = -10
IG_F64 = 0
IG_F32 = 1

_sz = C.c_size_t
_pd = C.c_ssize_t
_vp = C.c_void_p
# dtype, ndim, shape, stride_in, stride_out, naxes, axes
_ND_HEAD = [C.c_int, _sz, C.POINTER(_sz), C.POINTER(_pd), C.POINTER(_pd), _sz, C.POINTER(_sz)]

# name -> (restype, argtypes)
SIGNATURES = {
    "ig_last_error_string": (C.c_char_p, []),
    "ig_version": (C.c_int, []),
    "ig_make_cfft_plan": (_vp, [_sz, C.c_int]),
    "ig_destroy_cfft_plan": (None, [_vp]),
    "ig_cfft_backward": (C.c_int, [_vp, _vp, C.c_double]),
    "ig_cfft_forward": (C.c_int, [_vp, _vp, C.c_double]),
    "ig_cfft_length": (_sz, [_vp]),
    "ig_make_rfft_plan": (_vp, [_sz, C.c_int]),
    "ig_destroy_rfft_plan": (None, [_vp]),
    "ig_rfft_backward": (C.c_int, [_vp, _vp, C.c_double]),
    "ig_rfft_forward": (C.c_int, [_vp, _vp, C.c_double]),
    "ig_rfft_length": (_sz, [_vp]),
    "ig_cfft_exec_batch": (C.c_int, [_vp, _vp, _sz, _sz, C.c_int, C.c_double]),
    "ig_rfft_exec_batch": (C.c_int, [_vp, _vp, _sz, _sz, C.c_int, C.c_double]),
    "ig_cfft_exec_device": (C.c_int, [_vp, _vp, _vp, _sz, _sz, _sz, C.c_int, C.c_double, _vp]),
    "ig_rfft_exec_device": (C.c_int, [_vp, _vp, _vp, _sz, _sz, _sz, C.c_int, C.c_double, _vp]),
    "ig_cfft_exec_device_noalloc": (C.c_int, [_vp, _vp, _vp, _sz, _sz, _sz, C.c_int, C.c_double, _vp]),
    "ig_cfft_uses_bluestein": (C.c_int, [_vp, C.POINTER(_sz)]),
    "ig_rfft_uses_bluestein": (C.c_int, [_vp, C.POINTER(_sz)]),
    "ig_c2c": (C.c_int, [C.c_int, _sz, C.POINTER(_sz), C.POINTER(_pd), C.POINTER(_pd), _sz, C.POINTER(_sz),
                         C.c_int, _vp, _vp, C.c_double, _sz]),
    "ig_r2c": (C.c_int, [C.c_int, _sz, C.POINTER(_sz), C.POINTER(_pd), C.POINTER(_pd), _sz, C.POINTER(_sz),
                         C.c_int, _vp, _vp, C.c_double, _sz]),
    "ig_c2r": (C.c_int, [C.c_int, _sz, C.POINTER(_sz), C.POINTER(_pd), C.POINTER(_pd), _sz, C.POINTER(_sz),
                         C.c_int, _vp, _vp, C.c_double, _sz]),
    "ig_c2c_device": (C.c_int, [C.c_int, _sz, C.POINTER(_sz), C.POINTER(_pd), C.POINTER(_pd), _sz,
                                C.POINTER(_sz), C.c_int, _vp, _vp, C.c_double, _vp]),
    "ig_r2c_device": (C.c_int, [C.c_int, _sz, C.POINTER(_sz), C.POINTER(_pd), C.POINTER(_pd), _sz,
                                C.POINTER(_sz), C.c_int, _vp, _vp, C.c_double, _vp]),
    "ig_c2r_device": (C.c_int, [C.c_int, _sz, C.POINTER(_sz), C.POINTER(_pd), C.POINTER(_pd), _sz,
                                C.POINTER(_sz), C.c_int, _vp, _vp, C.c_double, _vp]),
    "ig_c2c_adjoint_device": (C.c_int, [C.c_int, _sz, C.POINTER(_sz), C.POINTER(_pd), C.POINTER(_pd), _sz,
                                        C.POINTER(_sz), C.c_int, _vp, _vp, C.c_double, _vp]),
    "ig_r2c_adjoint_device": (C.c_int, [C.c_int, _sz, C.POINTER(_sz), C.POINTER(_pd), C.POINTER(_pd), _sz,
                                        C.POINTER(_sz), C.c_int, _vp, _vp, C.c_double, _vp]),
    "ig_c2r_adjoint_device": (C.c_int, [C.c_int, _sz, C.POINTER(_sz), C.POINTER(_pd), C.POINTER(_pd), _sz,
                                        C.POINTER(_sz), C.c_int, _vp, _vp, C.c_double, _vp]),
    "ig_fftconv_create": (_vp, [C.c_int, _sz, _sz, _sz, _sz, _sz, _sz, _sz, C.c_int]),
    "ig_fftconv_destroy": (None, [_vp]),
    "ig_fftconv_padded_size": (C.c_int, [_vp, C.POINTER(_sz), C.POINTER(_sz)]),
    "ig_fftconv_forward": (C.c_int, [_vp, _vp, _vp, _vp, _vp]),
    "ig_fftconv_backward": (C.c_int, [_vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "ig_make_multi_plan": (_vp, [C.c_int, _sz, C.POINTER(_sz), C.POINTER(_sz), C.c_int, C.c_double]),
    "ig_destroy_multi_plan": (None, [_vp]),
    "ig_multi_info": (C.c_int, [_vp, C.POINTER(_sz), C.POINTER(_sz), C.POINTER(_sz)]),
    "ig_multi_exec_device": (C.c_int, [_vp, _vp, _vp, _vp]),
    "ig_multi_exec_graph": (C.c_int, [_vp, _vp, _vp, _vp]),
    "ig_multi_exec_loop_device": (C.c_int, [_vp, _vp, _vp, _vp]),
    "ig_multi_exec_part": (C.c_int, [_vp, _vp, _vp, C.c_int, _vp]),
    "ig_dct": (C.c_int, _ND_HEAD + [C.c_int, _vp, _vp, C.c_double, C.c_int, _sz]),
    "ig_dst": (C.c_int, _ND_HEAD + [C.c_int, _vp, _vp, C.c_double, C.c_int, _sz]),
    "ig_r2r_fftpack": (C.c_int, _ND_HEAD + [C.c_int, C.c_int, _vp, _vp, C.c_double, _sz]),
    "ig_r2r_separable_hartley": (C.c_int, _ND_HEAD + [_vp, _vp, C.c_double, _sz]),
    "ig_r2r_genuine_hartley": (C.c_int, _ND_HEAD + [_vp, _vp, C.c_double, _sz]),
    "ig_dct_device": (C.c_int, _ND_HEAD + [C.c_int, _vp, _vp, C.c_double, C.c_int, _vp]),
    "ig_dst_device": (C.c_int, _ND_HEAD + [C.c_int, _vp, _vp, C.c_double, C.c_int, _vp]),
    "ig_r2r_fftpack_device": (C.c_int, _ND_HEAD + [C.c_int, C.c_int, _vp, _vp, C.c_double, _vp]),
    "ig_r2r_hartley_device": (C.c_int, _ND_HEAD + [C.c_int, _vp, _vp, C.c_double, _vp]),
    "ig_upfirdn_length": (C.c_int, [_sz, _sz, C.c_int, C.c_int, C.POINTER(_sz)]),
    "ig_upfirdn": (C.c_int, [C.c_int, _sz, _sz, _vp, _sz, _sz, _vp, C.c_int, C.c_int, _vp, _sz]),
    "ig_upfirdn_device": (C.c_int, [C.c_int, _sz, _sz, _vp, _sz, _sz, _vp, C.c_int, C.c_int, _vp, _sz, _vp]),
    "ig_autotune": (C.c_int, [C.c_int, _sz, C.c_int, C.POINTER(C.c_double)]),
    "ig_autotune_save": (C.c_int, [C.c_char_p]),
    "ig_autotune_load": (C.c_int, [C.c_char_p]),
    "ig_set_f64_arith": (C.c_int, [C.c_int]),
    "ig_release_caches": (None, []),
    "ig_launch_count": (C.c_ulonglong, [C.c_int]),
    "ig_device_faults": (C.c_int, [C.POINTER(C.c_uint)]),
}

_lib = None


def load(path: str = LIB_PATH):
    """Load libimpulse_gpu.so; raises OSError if it is missing (no fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(path):
            raise OSError(f"libimpulse_gpu.so not built at {path}: run `python -m impulse_gb300.build`")
        L = C.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


class FFTError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{msg} (status {code})")
        self.code = code


def check(rc: int) -> None:
    if rc != IG_OK:
        raise FFTError(rc, load().ig_last_error_string().decode())


def arr(t, vals):
    vals = list(vals)
    return (t * max(1, len(vals)))(*vals)
