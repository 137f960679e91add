"""impulse_gb300 -- GB300-native FFT engine behind impulse's FFT API.

The product is ``libimpulse_gpu.so`` (hand-written sm_103a CUDA kernels behind
the C ABI of ``include/impulse_gpu.h``).  This package holds its sources
(``csrc/``), the in-tree build (``build.py``), a ctypes binding of the C ABI
(``_lib.py``) and a host-side mirror of impulse's Nim FFT interface
(``fft.py``: the C backend's fft/rfft/ifft/unpackFFT/symmetrize and the C++
backend's DataDesc/FFTDesc/apply).
"""
from . import _lib  # noqa: F401
