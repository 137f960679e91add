## impulse_gpu_fft -- drop-in Nim binding of the GB300 FFT engine for impulse.
##
## NOT COMPILED HERE: there is no Nim toolchain on the machines this engine is
## built and tested on.  The module restates, as Nim source, the bindings that
## the C ABI (include/impulse_gpu.h) is designed for; the same calls are
## exercised from Python through ctypes (impulse_gb300/_lib.py, fft.py,
## device.py) by the test-suite.
##
## How impulse uses it:
##
## * C backend (impulse/fft/c_pocketfft/pocketfft.nim): replace the
##   `{.importc, header.}` block at pocketfft.nim:71-81 and the compile of
##   pocketfft.c (pocketfft.nim:14) with `import impulse_gpu_fft`.  The procs
##   below keep the names and argument meaning of pocketfft.h (pocketfft.h:18-32),
##   so FFTPlanReal / FFTPlanComplex, callFFT, rfft, fft_impl, fft, unpackFFT,
##   symmetrize and the Arraymancer overloads (pocketfft_arraymancer.nim)
##   compile unchanged.  A failing call returns non-zero, and callFFT raises
##   "Forward FFT calculation failed." / "Backward FFT calculation failed."
##   (pocketfft.nim:206-214) as before.
## * C++ backend (impulse/fft/cpp_pocketfft/pocketfft.nim): replace the
##   `{.importcpp: "pocketfft::c2c(@)".}` imports at pocketfft.nim:35-69 by the
##   c2c / r2c / c2r procs below; DataDesc, FFTDesc and apply
##   (pocketfft.nim:137-277) stay, including apply's c2r call with
##   descIn.shape (pocketfft.nim:266).
## * Data already on the GPU: DeviceDataDesc and the apply overload taking a
##   stream bind the *_device entry points (no host copies).

import std/complex

const igLib* {.strdefine.} = "libimpulse_gpu.so"

const
  IG_F64* = 0.cint
  IG_F32* = 1.cint

type
  cfft_plan* = pointer
  rfft_plan* = pointer
  CudaStream* = pointer  ## cudaStream_t; nil = the default stream

# ---- the C ABI (include/impulse_gpu.h) ---------------------------------------

proc ig_last_error_string*(): cstring {.importc, dynlib: igLib.}
proc ig_make_cfft_plan(length: csize_t, dtype: cint): cfft_plan {.importc, dynlib: igLib.}
proc ig_destroy_cfft_plan(plan: cfft_plan) {.importc, dynlib: igLib.}
proc ig_cfft_forward(plan: cfft_plan; c: pointer; fct: cdouble): cint {.importc, dynlib: igLib.}
proc ig_cfft_backward(plan: cfft_plan; c: pointer; fct: cdouble): cint {.importc, dynlib: igLib.}
proc ig_cfft_length(plan: cfft_plan): csize_t {.importc, dynlib: igLib.}
proc ig_make_rfft_plan(length: csize_t, dtype: cint): rfft_plan {.importc, dynlib: igLib.}
proc ig_destroy_rfft_plan(plan: rfft_plan) {.importc, dynlib: igLib.}
proc ig_rfft_forward(plan: rfft_plan; c: pointer; fct: cdouble): cint {.importc, dynlib: igLib.}
proc ig_rfft_backward(plan: rfft_plan; c: pointer; fct: cdouble): cint {.importc, dynlib: igLib.}
proc ig_rfft_length(plan: rfft_plan): csize_t {.importc, dynlib: igLib.}
proc ig_cfft_exec_batch*(plan: cfft_plan; c: pointer; batch, dist: csize_t; forward: cint;
                         fct: cdouble): cint {.importc, dynlib: igLib.}
proc ig_rfft_exec_batch*(plan: rfft_plan; c: pointer; batch, dist: csize_t; forward: cint;
                         fct: cdouble): cint {.importc, dynlib: igLib.}
proc ig_cfft_exec_device*(plan: cfft_plan; dataIn, dataOut: pointer; batch, distIn, distOut: csize_t;
                          forward: cint; fct: cdouble; stream: CudaStream): cint {.importc, dynlib: igLib.}
proc ig_rfft_exec_device*(plan: rfft_plan; dataIn, dataOut: pointer; batch, distIn, distOut: csize_t;
                          forward: cint; fct: cdouble; stream: CudaStream): cint {.importc, dynlib: igLib.}
proc ig_c2c(dtype: cint; ndim: csize_t; shape: ptr csize_t; strideIn, strideOut: ptr int;
            naxes: csize_t; axes: ptr csize_t; forward: cint; dataIn, dataOut: pointer;
            fct: cdouble; nthreads: csize_t): cint {.importc, dynlib: igLib.}
proc ig_r2c(dtype: cint; ndim: csize_t; shapeIn: ptr csize_t; strideIn, strideOut: ptr int;
            naxes: csize_t; axes: ptr csize_t; forward: cint; dataIn, dataOut: pointer;
            fct: cdouble; nthreads: csize_t): cint {.importc, dynlib: igLib.}
proc ig_c2r(dtype: cint; ndim: csize_t; shapeOut: ptr csize_t; strideIn, strideOut: ptr int;
            naxes: csize_t; axes: ptr csize_t; forward: cint; dataIn, dataOut: pointer;
            fct: cdouble; nthreads: csize_t): cint {.importc, dynlib: igLib.}
proc ig_c2c_device(dtype: cint; ndim: csize_t; shape: ptr csize_t; strideIn, strideOut: ptr int;
                   naxes: csize_t; axes: ptr csize_t; forward: cint; dataIn, dataOut: pointer;
                   fct: cdouble; stream: CudaStream): cint {.importc, dynlib: igLib.}
proc ig_r2c_device(dtype: cint; ndim: csize_t; shapeIn: ptr csize_t; strideIn, strideOut: ptr int;
                   naxes: csize_t; axes: ptr csize_t; forward: cint; dataIn, dataOut: pointer;
                   fct: cdouble; stream: CudaStream): cint {.importc, dynlib: igLib.}
proc ig_c2r_device(dtype: cint; ndim: csize_t; shapeOut: ptr csize_t; strideIn, strideOut: ptr int;
                   naxes: csize_t; axes: ptr csize_t; forward: cint; dataIn, dataOut: pointer;
                   fct: cdouble; stream: CudaStream): cint {.importc, dynlib: igLib.}
proc ig_dct(dtype: cint; ndim: csize_t; shape: ptr csize_t; strideIn, strideOut: ptr int;
            naxes: csize_t; axes: ptr csize_t; dctType: cint; dataIn, dataOut: pointer;
            fct: cdouble; ortho: cint; nthreads: csize_t): cint {.importc, dynlib: igLib.}
proc ig_autotune*(dtype: cint; length: csize_t; kind: cint; ms: ptr cdouble): cint {.importc, dynlib: igLib.}
proc ig_autotune_load*(path: cstring): cint {.importc, dynlib: igLib.}
proc ig_autotune_save*(path: cstring): cint {.importc, dynlib: igLib.}
proc ig_set_f64_arith*(mode: cint): cint {.importc, dynlib: igLib.}

# ---- C backend: the pocketfft.h names (pocketfft.h:18-32) --------------------
# Float64 data, as impulse's C backend handles (pocketfft.nim:18-20: Complex64
# is binary-compatible with the interleaved (re, im) doubles).

proc make_cfft_plan*(length: csize_t): cfft_plan = ig_make_cfft_plan(length, IG_F64)
proc destroy_cfft_plan*(plan: cfft_plan) = ig_destroy_cfft_plan(plan)
proc cfft_forward*(plan: cfft_plan; c: ptr Complex64; fct: cdouble): cint = ig_cfft_forward(plan, c, fct)
proc cfft_backward*(plan: cfft_plan; c: ptr Complex64; fct: cdouble): cint = ig_cfft_backward(plan, c, fct)
proc cfft_length*(plan: cfft_plan): csize_t = ig_cfft_length(plan)
proc make_rfft_plan*(length: csize_t): rfft_plan = ig_make_rfft_plan(length, IG_F64)
proc destroy_rfft_plan*(plan: rfft_plan) = ig_destroy_rfft_plan(plan)
proc rfft_forward*(plan: rfft_plan; c: ptr cdouble; fct: cdouble): cint = ig_rfft_forward(plan, c, fct)
proc rfft_backward*(plan: rfft_plan; c: ptr cdouble; fct: cdouble): cint = ig_rfft_backward(plan, c, fct)
proc rfft_length*(plan: rfft_plan): csize_t = ig_rfft_length(plan)

# ---- C++ backend: pocketfft::c2c / r2c / c2r (pocketfft_hdronly.h:3272, 3334, 3366)
# Same arguments as the imported templates: shapes, BYTE strides, axes,
# forward, scale factor, thread count (accepted, unused: the GPU grid
# replaces the host threads).  Errors raise ValueError with pocketfft's own
# message texts ("bad axis number", "axis specified repeatedly", "stride
# mismatch", "zero-length FFT requested").

type
  Shape* = seq[uint]
  Stride* = seq[int]

template dtypeOf(T: typedesc): cint =
  (when T is float32: IG_F32 else: IG_F64)

proc check(rc: cint) =
  if rc != 0: raise newException(ValueError, $ig_last_error_string())

proc c2c*[T: SomeFloat](shape: Shape; strideIn, strideOut: Stride; axes: Shape; forward: bool;
                        dataIn, dataOut: pointer; fct: T; nthreads: uint = 1) =
  check ig_c2c(dtypeOf(T), shape.len.csize_t, cast[ptr csize_t](shape[0].unsafeAddr),
               strideIn[0].unsafeAddr, strideOut[0].unsafeAddr, axes.len.csize_t,
               cast[ptr csize_t](axes[0].unsafeAddr), forward.cint, dataIn, dataOut, fct.cdouble,
               nthreads.csize_t)

proc r2c*[T: SomeFloat](shapeIn: Shape; strideIn, strideOut: Stride; axes: Shape; forward: bool;
                        dataIn, dataOut: pointer; fct: T; nthreads: uint = 1) =
  check ig_r2c(dtypeOf(T), shapeIn.len.csize_t, cast[ptr csize_t](shapeIn[0].unsafeAddr),
               strideIn[0].unsafeAddr, strideOut[0].unsafeAddr, axes.len.csize_t,
               cast[ptr csize_t](axes[0].unsafeAddr), forward.cint, dataIn, dataOut, fct.cdouble,
               nthreads.csize_t)

proc c2r*[T: SomeFloat](shapeOut: Shape; strideIn, strideOut: Stride; axes: Shape; forward: bool;
                        dataIn, dataOut: pointer; fct: T; nthreads: uint = 1) =
  check ig_c2r(dtypeOf(T), shapeOut.len.csize_t, cast[ptr csize_t](shapeOut[0].unsafeAddr),
               strideIn[0].unsafeAddr, strideOut[0].unsafeAddr, axes.len.csize_t,
               cast[ptr csize_t](axes[0].unsafeAddr), forward.cint, dataIn, dataOut, fct.cdouble,
               nthreads.csize_t)

proc dct*[T: SomeFloat](shape: Shape; strideIn, strideOut: Stride; axes: Shape; dctType: int;
                        dataIn, dataOut: pointer; fct: T; ortho: bool; nthreads: uint = 1) =
  check ig_dct(dtypeOf(T), shape.len.csize_t, cast[ptr csize_t](shape[0].unsafeAddr),
               strideIn[0].unsafeAddr, strideOut[0].unsafeAddr, axes.len.csize_t,
               cast[ptr csize_t](axes[0].unsafeAddr), dctType.cint, dataIn, dataOut, fct.cdouble,
               ortho.cint, nthreads.csize_t)

# ---- data in GPU memory ---------------------------------------------------------

type DeviceDataDesc*[T] = object
  ## DataDesc (pocketfft.nim:137-199) over a device buffer: shape, BYTE
  ## strides, device pointer.
  shape*: Shape
  stride*: Stride
  buf*: pointer

proc initDeviceDataDesc*[T](buf: pointer; shape: openArray[int]): DeviceDataDesc[T] =
  ## Row-major byte strides, as DataDesc.init (pocketfft.nim:178-199).
  result.buf = buf
  result.shape = newSeq[uint](shape.len)
  result.stride = newSeq[int](shape.len)
  var acc = sizeof(T)
  for i in countdown(shape.len - 1, 0):
    result.shape[i] = shape[i].uint
    result.stride[i] = acc
    acc *= shape[i]

proc applyDevice*[In, Out](axes: Shape; forward: bool; scalingFactor: float;
                           descOut: var DeviceDataDesc[Out]; descIn: DeviceDataDesc[In];
                           stream: CudaStream = nil) =
  ## apply (pocketfft.nim:235-277) on device buffers, asynchronous on `stream`.
  let dt = (when In is float32 or In is Complex32: IG_F32 else: IG_F64)
  template call(f: untyped) =
    check f(dt, descIn.shape.len.csize_t, cast[ptr csize_t](descIn.shape[0].unsafeAddr),
            descIn.stride[0].unsafeAddr, descOut.stride[0].unsafeAddr, axes.len.csize_t,
            cast[ptr csize_t](axes[0].unsafeAddr), forward.cint, descIn.buf, descOut.buf,
            scalingFactor.cdouble, stream)
  when In is Complex and Out is Complex: call(ig_c2c_device)
  elif Out is Complex: call(ig_r2c_device)
  else: call(ig_c2r_device)  # descIn.shape, as pocketfft.nim:266 passes it
