/*
 * impulse_gpu.h -- C ABI of the GB300 FFT engine behind impulse's FFT API.
 *
 * The engine replaces the native numerics under impulse's Nim FFT module:
 *
 *   C backend   impulse/fft/c_pocketfft/pocketfft.nim binds pocketfft.h
 *               (impulse/fft/c_pocketfft/pocketfft.h:18-32) with
 *               {.importc, header.} at pocketfft.nim:71-81;
 *   C++ backend impulse/fft/cpp_pocketfft/pocketfft.nim binds the
 *               templates pocketfft::c2c / r2c / c2r
 *               (impulse/fft/cpp_pocketfft/pocketfft_hdronly.h:3272, 3334,
 *               3366) with {.importcpp.} at pocketfft.nim:35-69.
 *
 * Every function here is a plain C entry point (no exceptions, no C++ or
 * torch types) that a Nim module binds with {.importc, dynlib.}.
 * Data pointers of the pocketfft-shaped entry points are HOST pointers, as in
 * the reference; the engine copies to the GPU, runs hand-written sm_103a
 * kernels and copies back.  The *_device entry points take device pointers
 * and a CUDA stream and do no host copies.
 *
 * dtype: IG_F64 (double / complex128 data) or IG_F32 (float / complex64).
 * Complex data is interleaved (re, im), binary-compatible with Nim's
 * Complex64 / Complex32 and std::complex.
 */
#ifndef IMPULSE_GPU_H
#define IMPULSE_GPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif
#if defined(__GNUC__)
#pragma GCC visibility push(default)
#endif

/* ---- status codes ------------------------------------------------------ */
#define IG_OK 0
#define IG_ENOMEM (-1)          /* allocation failed: pocketfft's -1 (pocketfft.c:878) */
#define IG_EINVAL_AXIS (-2)     /* "bad axis number" (pocketfft_hdronly.h:466) */
#define IG_EREPEAT_AXIS (-3)    /* "axis specified repeatedly" (pocketfft_hdronly.h:467) */
#define IG_ESTRIDE_INPLACE (-4) /* "stride mismatch" (pocketfft_hdronly.h:453) */
#define IG_EZERO_LEN (-5)       /* "zero-length FFT requested" (pocketfft_hdronly.h:2360) */
#define IG_ECUDA (-6)           /* CUDA runtime error */
#define IG_ENDIM (-7)           /* "ndim must be >= 1" / "stride dimension mismatch" (pocketfft_hdronly.h:450-452) */
#define IG_EINVAL (-8)          /* other invalid argument (null pointer, bad dtype, ...) */
#define IG_ETIMEOUT (-9)        /* a bounded device-side wait expired */
#define IG_ETOOLARGE (-10)      /* size beyond a documented limit */

#define IG_F64 0
#define IG_F32 1

/* Message of the last failing call on this thread ("" after success). */
const char *ig_last_error_string(void);
/* ABI version (major * 10000 + minor * 100 + patch). */
int ig_version(void);

/* ---- 1-D plans: mirror of pocketfft.h (pocketfft.h:18-32) ---------------
 * A plan is a host handle to device-resident twiddle / chirp tables, built on
 * the GPU.  Plans are read-only after construction and may be shared between
 * threads, as the reference's plans are (c_pocketfft/README.md:32-36).
 * make_* returns NULL for length 0 or on failure (reason in
 * ig_last_error_string), like make_cfft_plan (pocketfft.c:2068).        */
typedef struct ig_cfft_plan_i *ig_cfft_plan;
typedef struct ig_rfft_plan_i *ig_rfft_plan;

/* replaces make_cfft_plan (pocketfft.h:20) */
ig_cfft_plan ig_make_cfft_plan(size_t length, int dtype);
/* replaces destroy_cfft_plan (pocketfft.h:21) */
void ig_destroy_cfft_plan(ig_cfft_plan plan);
/* replaces cfft_backward (pocketfft.h:22): in place on `length` complex values
 * at host pointer c, c[k] = fct * sum_m c[m] exp(+2 pi i m k / n) */
int ig_cfft_backward(ig_cfft_plan plan, void *c, double fct);
/* replaces cfft_forward (pocketfft.h:23): exp(-2 pi i m k / n) */
int ig_cfft_forward(ig_cfft_plan plan, void *c, double fct);
/* replaces cfft_length (pocketfft.h:24) */
size_t ig_cfft_length(ig_cfft_plan plan);

/* replaces make_rfft_plan (pocketfft.h:28) */
ig_rfft_plan ig_make_rfft_plan(size_t length, int dtype);
/* replaces destroy_rfft_plan (pocketfft.h:29) */
void ig_destroy_rfft_plan(ig_rfft_plan plan);
/* replaces rfft_backward (pocketfft.h:30): halfcomplex
 * [r0, r1, i1, ..., (r_{n/2})] -> n reals, in place */
int ig_rfft_backward(ig_rfft_plan plan, void *c, double fct);
/* replaces rfft_forward (pocketfft.h:31): n reals -> halfcomplex, in place */
int ig_rfft_forward(ig_rfft_plan plan, void *c, double fct);
/* replaces rfft_length (pocketfft.h:32) */
size_t ig_rfft_length(ig_rfft_plan plan);

/* Batched host-memory variants: `batch` lines, line b starting `dist`
 * elements (complex for cfft, real for rfft) after line b-1.  The reference
 * loops over lines in Nim (one pocketfft call each); these move the loop
 * into one GPU launch. */
int ig_cfft_exec_batch(ig_cfft_plan plan, void *c, size_t batch, size_t dist, int forward, double fct);
int ig_rfft_exec_batch(ig_rfft_plan plan, void *c, size_t batch, size_t dist, int forward, double fct);

/* Device-memory variants (no host copies; `in` may equal `out`).  Line b of
 * the input starts dist_in elements after line b-1, likewise the output. */
int ig_cfft_exec_device(ig_cfft_plan plan, const void *in, void *out, size_t batch, size_t dist_in,
                        size_t dist_out, int forward, double fct, void *stream);
int ig_rfft_exec_device(ig_rfft_plan plan, const void *in, void *out, size_t batch, size_t dist_in,
                        size_t dist_out, int forward, double fct, void *stream);

/* Allocation-free variant of ig_cfft_exec_device.  No counterpart in the
 * reference (PocketFFT mallocs its scratch on every call).  For callers that
 * cannot allocate device memory while they run: a process that reserves its
 * whole device-memory budget up front in a pool that must not grow, or a
 * latency-bound loop where cudaMalloc / cudaFree (which can synchronise the
 * device and take unbounded time) are not allowed.  Transforms longer than
 * one CTA take their scratch from a static device array of 64 MiB (held by
 * every GPU that loads the library) instead of the engine's cached
 * workspace.  Limit: batch * length * complex element size <= 64 MiB for
 * plans longer than one CTA (IG_ETOOLARGE beyond); plans running Bluestein or
 * Rader over a multi-pass core are rejected (IG_EINVAL), and so are pointers
 * not aligned to the complex element size.  The first call on each device
 * looks the array up there; make that first call before any stream capture.
 * Calls share the array; calls that overlap on the GPU race. */
int ig_cfft_exec_device_noalloc(ig_cfft_plan plan, const void *in, void *out, size_t batch, size_t dist_in,
                                size_t dist_out, int forward, double fct, void *stream);

/* Plan introspection: 1 when the plan runs Bluestein; the padded length.
 * (Prime lengths whose predecessor is 13-smooth run Rader's algorithm and
 * report 0.) */
int ig_cfft_uses_bluestein(ig_cfft_plan plan, size_t *n2);
int ig_rfft_uses_bluestein(ig_rfft_plan plan, size_t *n2);

/* ---- N-d strided transforms: mirror of pocketfft::c2c / r2c / c2r --------
 * shape, strides (in BYTES, may be negative), axes and fct as in
 * pocketfft_hdronly.h:3272 (c2c), 3334 (r2c: shape is the real input's
 * shape, the output has shape[axes.back()]/2+1 there), 3366 (c2r: shape is
 * the real OUTPUT's shape).  `nthreads` is accepted for signature parity and
 * ignored: the GPU grid replaces the host thread pool.  Host pointers. */
int ig_c2c(int dtype, size_t ndim, const size_t *shape, const ptrdiff_t *stride_in, const ptrdiff_t *stride_out,
           size_t naxes, const size_t *axes, int forward, const void *data_in, void *data_out, double fct,
           size_t nthreads);
int ig_r2c(int dtype, size_t ndim, const size_t *shape_in, const ptrdiff_t *stride_in,
           const ptrdiff_t *stride_out, size_t naxes, const size_t *axes, int forward, const void *data_in,
           void *data_out, double fct, size_t nthreads);
int ig_c2r(int dtype, size_t ndim, const size_t *shape_out, const ptrdiff_t *stride_in,
           const ptrdiff_t *stride_out, size_t naxes, const size_t *axes, int forward, const void *data_in,
           void *data_out, double fct, size_t nthreads);

/* Device-pointer variants of the three above, on `stream` (cudaStream_t;
 * NULL = the default stream). */
int ig_c2c_device(int dtype, size_t ndim, const size_t *shape, const ptrdiff_t *stride_in,
                  const ptrdiff_t *stride_out, size_t naxes, const size_t *axes, int forward, const void *data_in,
                  void *data_out, double fct, void *stream);
int ig_r2c_device(int dtype, size_t ndim, const size_t *shape_in, const ptrdiff_t *stride_in,
                  const ptrdiff_t *stride_out, size_t naxes, const size_t *axes, int forward,
                  const void *data_in, void *data_out, double fct, void *stream);
int ig_c2r_device(int dtype, size_t ndim, const size_t *shape_out, const ptrdiff_t *stride_in,
                  const ptrdiff_t *stride_out, size_t naxes, const size_t *axes, int forward,
                  const void *data_in, void *data_out, double fct, void *stream);

/* ---- batched complex transforms of uneven lengths ---------------------------
 * `count` complex transforms, transform i of lengths[i] at element offset
 * offsets[i] (NULL = packed back to back) of the same layout in `in` and
 * `out` (device pointers; may be equal).  The plan groups equal lengths that
 * fit one CTA and runs them, with the column passes of longer four-step
 * lengths, through one persistent work-list launch; a second launch runs the
 * row passes; lengths needing Bluestein or Rader over a multi-pass core use
 * the general path, on up to sixteen side streams forked from and joined back
 * into the caller's stream.  ig_multi_exec_graph captures that sequence into a CUDA graph
 * on its first call for given pointers and replays it afterwards;
 * ig_multi_exec_loop_device is the one-call-per-transform pattern, for
 * comparison.  The reference transforms one line per call
 * (pocketfft.nim:290-303). */
typedef struct ig_multi_plan_i *ig_multi_plan;
ig_multi_plan ig_make_multi_plan(int dtype, size_t count, const size_t *lengths, const size_t *offsets, int forward,
                                 double fct);
void ig_destroy_multi_plan(ig_multi_plan plan);
int ig_multi_info(ig_multi_plan plan, size_t *n_worklist, size_t *n_fourstep, size_t *n_general);
int ig_multi_exec_device(ig_multi_plan plan, const void *in, void *out, void *stream);
int ig_multi_exec_graph(ig_multi_plan plan, const void *in, void *out, void *stream);
int ig_multi_exec_loop_device(ig_multi_plan plan, const void *in, void *out, void *stream);
/* One part of ig_multi_exec_device's sequence, for timing the paths apart:
 * parts is a mask of 1 (work-list phase 0: single-CTA lengths and four-step
 * column passes), 2 (phase 1: four-step row passes, after phase 0) and 4
 * (lengths on the general path, on the plan's side streams joined back into
 * `stream`).  No counterpart in the reference. */
int ig_multi_exec_part(ig_multi_plan plan, const void *in, void *out, int parts, void *stream);

/* ---- adjoints ----------------------------------------------------------------
 * Gradients of a real loss through c2c / r2c / c2r (device pointers).  With g
 * the gradient with respect to (Re X, Im X) packed as complex:
 *   adjoint of c2c(axes, forward, fct): x_bar = c2c(axes, !forward, fct) of g
 *     (the DFT matrix is symmetric, so its adjoint is its conjugate);
 *   adjoint of r2c(axes, forward): x_bar = c2r(axes, !forward) of g with the
 *     inner bins of the last axis halved;
 *   adjoint of c2r(axes, forward): g_bar = r2c(axes, !forward) of y_bar with
 *     the inner bins of the last axis doubled (the Hermitian 2x weighting).
 * No counterpart in the reference (PocketFFT has no adjoints); shapes and
 * byte strides follow pocketfft::c2c / r2c / c2r (pocketfft_hdronly.h:3272,
 * 3334, 3366). */
int ig_c2c_adjoint_device(int dtype, size_t ndim, const size_t *shape, const ptrdiff_t *stride_g,
                          const ptrdiff_t *stride_x, size_t naxes, const size_t *axes, int forward, const void *g,
                          void *x, double fct, void *stream);
int ig_r2c_adjoint_device(int dtype, size_t ndim, const size_t *shape_in, const ptrdiff_t *stride_g,
                          const ptrdiff_t *stride_x, size_t naxes, const size_t *axes, int forward, const void *g,
                          void *x, double fct, void *stream);
int ig_c2r_adjoint_device(int dtype, size_t ndim, const size_t *shape_out, const ptrdiff_t *stride_y,
                          const ptrdiff_t *stride_g, size_t naxes, const size_t *axes, int forward, const void *y,
                          void *g, double fct, void *stream);

/* ---- differentiable FFT convolution -----------------------------------------
 * 'same' 2-D convolution of `batch` real H x W images with odd K x K filters
 * (one shared filter or one per image), zero padded to pad_rows x pad_cols
 * (0 = smallest 2^a3^b5^c7^d11^e >= size + K - 1) and computed as
 * c2r(r2c(x) * r2c(k)).  forward(x, k) -> y; backward(x, k, gy) -> gx, gk
 * (either may be NULL).  With recompute = 1 the backward recomputes the
 * spectra of x and k instead of keeping them from the forward.  Contiguous
 * row-major device arrays: x, y, gy, gx [batch][H][W]; k, gk [nfilters][K][K].
 * No counterpart in the reference (impulse convolves directly, signal.nim:594). */
typedef struct ig_fftconv_i *ig_fftconv;
ig_fftconv ig_fftconv_create(int dtype, size_t batch, size_t height, size_t width, size_t nfilters, size_t ksize,
                             size_t pad_rows, size_t pad_cols, int recompute);
void ig_fftconv_destroy(ig_fftconv conv);
int ig_fftconv_padded_size(ig_fftconv conv, size_t *rows, size_t *cols);
int ig_fftconv_forward(ig_fftconv conv, const void *x, const void *k, void *y, void *stream);
int ig_fftconv_backward(ig_fftconv conv, const void *x, const void *k, const void *gy, void *gx, void *gk,
                        void *stream);

/* ---- real-to-real transforms ------------------------------------------------
 * pocketfft::dct / dst (pocketfft_hdronly.h:3284-3318; DCTDesc.apply at
 * cpp_pocketfft/pocketfft.nim:279-295), r2r_fftpack, r2r_separable_hartley and
 * r2r_genuine_hartley (pocketfft_hdronly.h:3392-3445, bound at
 * cpp_pocketfft/pocketfft.nim:71-106).  Same arguments: shape, byte strides,
 * axes (transformed in order; fct on the first), DCT/DST type 1-4 and the
 * ortho flag with the reference's scaling steps, real2hermitian / forward
 * with the reference's sign conventions.  Real arrays of dtype IG_F64 or
 * IG_F32, in host memory (nthreads ignored) or, for the _device forms, in
 * device memory on `stream`.  Errors: "invalid DCT type" / "invalid DST
 * type" (IG_EINVAL), "zero-length FFT requested" for DCT-I along an axis of
 * length 1, and the axis / stride errors of ig_c2c. */
int ig_dct(int dtype, size_t ndim, const size_t *shape, const ptrdiff_t *stride_in, const ptrdiff_t *stride_out,
           size_t naxes, const size_t *axes, int type, const void *data_in, void *data_out, double fct, int ortho,
           size_t nthreads);
int ig_dst(int dtype, size_t ndim, const size_t *shape, const ptrdiff_t *stride_in, const ptrdiff_t *stride_out,
           size_t naxes, const size_t *axes, int type, const void *data_in, void *data_out, double fct, int ortho,
           size_t nthreads);
int ig_r2r_fftpack(int dtype, size_t ndim, const size_t *shape, const ptrdiff_t *stride_in,
                   const ptrdiff_t *stride_out, size_t naxes, const size_t *axes, int real2hermitian, int forward,
                   const void *data_in, void *data_out, double fct, size_t nthreads);
int ig_r2r_separable_hartley(int dtype, size_t ndim, const size_t *shape, const ptrdiff_t *stride_in,
                             const ptrdiff_t *stride_out, size_t naxes, const size_t *axes, const void *data_in,
                             void *data_out, double fct, size_t nthreads);
int ig_r2r_genuine_hartley(int dtype, size_t ndim, const size_t *shape, const ptrdiff_t *stride_in,
                           const ptrdiff_t *stride_out, size_t naxes, const size_t *axes, const void *data_in,
                           void *data_out, double fct, size_t nthreads);
int ig_dct_device(int dtype, size_t ndim, const size_t *shape, const ptrdiff_t *stride_in, const ptrdiff_t *stride_out,
                  size_t naxes, const size_t *axes, int type, const void *data_in, void *data_out, double fct,
                  int ortho, void *stream);
int ig_dst_device(int dtype, size_t ndim, const size_t *shape, const ptrdiff_t *stride_in, const ptrdiff_t *stride_out,
                  size_t naxes, const size_t *axes, int type, const void *data_in, void *data_out, double fct,
                  int ortho, void *stream);
int ig_r2r_fftpack_device(int dtype, size_t ndim, const size_t *shape, const ptrdiff_t *stride_in,
                          const ptrdiff_t *stride_out, size_t naxes, const size_t *axes, int real2hermitian,
                          int forward, const void *data_in, void *data_out, double fct, void *stream);
int ig_r2r_hartley_device(int dtype, size_t ndim, const size_t *shape, const ptrdiff_t *stride_in,
                          const ptrdiff_t *stride_out, size_t naxes, const size_t *axes, int genuine,
                          const void *data_in, void *data_out, double fct, void *stream);

/* ---- upfirdn (impulse signal.nim:545-594) -----------------------------------
 * upfirdn(t, h, up, down) = t upsampled by `up` (up - 1 zeros between
 * samples), fully convolved with the FIR filter h, every `down`-th sample
 * kept; computed by FFT.  `batch` signals of n reals, signal b at
 * x + b * dist_x; one filter of nh reals; output rows of length
 * ig_upfirdn_length(n, nh, up, down) = ceil(((n - 1) up + nh) / down) at
 * y + b * dist_y.  Host memory, or device memory on `stream` for _device. */
int ig_upfirdn_length(size_t n, size_t nh, int up, int down, size_t *out_len);
int ig_upfirdn(int dtype, size_t batch, size_t n, const void *x, size_t dist_x, size_t nh, const void *h, int up,
               int down, void *y, size_t dist_y);
int ig_upfirdn_device(int dtype, size_t batch, size_t n, const void *x, size_t dist_x, size_t nh, const void *h,
                      int up, int down, void *y, size_t dist_y, void *stream);

/* ---- autotuner -----------------------------------------------------------------
 * ig_autotune times every candidate configuration of one transform (kind 0:
 * complex, 1: real halfcomplex forward) -- radix order, elements per thread
 * and lines (transforms) per CTA for single-CTA lengths, the split N1 x N2
 * for four-step lengths -- on a ~64 MiB synthetic batch with CUDA events,
 * keeps the fastest for plans made afterwards and returns its time per call.
 * ig_autotune_save / _load write / read the table (one line per entry, keyed
 * by GPU name); path NULL means the IG_AUTOTUNE_CACHE environment variable.
 * No counterpart in the reference (PocketFFT's planner is fixed). */
int ig_autotune(int dtype, size_t length, int kind, double *best_ms);
int ig_autotune_save(const char *path);
int ig_autotune_load(const char *path);

/* ---- engine control ------------------------------------------------------ */
/* Select the arithmetic used for IG_F64 data: 0 = double-float (default;
 * FP32-pair butterflies, ~48-bit significand, for GB300's narrow FP64
 * pipe), 1 = native FP64 butterflies.  Applies to plans made afterwards. */
int ig_set_f64_arith(int mode);
/* Release cached plans and workspace memory. */
void ig_release_caches(void);
/* Number of kernel launches the engine issued since the last reset. */
unsigned long long ig_launch_count(int reset);
/* Synchronise the current device and report in *count how many waits of the
 * engine's pipelined kernels gave up since the last call (each wait on a bulk
 * copy is bounded; a CTA that gives up abandons its remaining lines).  0 in
 * normal operation; the counters are cleared.  No counterpart in the
 * reference (CPU code has no device waits). */
int ig_device_faults(unsigned *count);

#if defined(__GNUC__)
#pragma GCC visibility pop
#endif
#ifdef __cplusplus
}
#endif
#endif /* IMPULSE_GPU_H */
