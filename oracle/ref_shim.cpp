// ref_shim.cpp -- TEST INFRASTRUCTURE ONLY.
//
// extern "C" entry points around impulse's vendored C++ PocketFFT header so
// that the test-suite can call the reference's own code through ctypes.  The
// header is included from the reference checkout at build time (see
// oracle/Makefile); nothing of it is copied here.  Built into
// oracle/_ref/libpocketfft_ref.so together with the reference's C backend
// (impulse/fft/c_pocketfft/pocketfft.c), whose pocketfft.h functions are
// exported unchanged.
//
// Each wrapper mirrors one template the Nim C++ backend binds
// (impulse/fft/cpp_pocketfft/pocketfft.nim:35-106).  Exceptions do not cross
// the C boundary: they become negative status codes and the message is kept
// for ref_last_error().
#include <complex>
#include <cstring>
#include <stdexcept>
#include <string>
#include "pocketfft_hdronly.h"
extern "C" {
#include "pocketfft.h"  // the reference's C backend (impulse/fft/c_pocketfft/pocketfft.h)
}

static thread_local std::string g_err;

template <class F>
static int guard(F &&f)
{
  try { f(); g_err.clear(); return 0; }
  catch (const std::invalid_argument &e) { g_err = e.what(); return -2; }
  catch (const std::runtime_error &e) { g_err = e.what(); return -3; }
  catch (const std::exception &e) { g_err = e.what(); return -1; }
}

static pocketfft::shape_t mk_shape(size_t n, const size_t *p) { return pocketfft::shape_t(p, p + n); }
static pocketfft::stride_t mk_stride(size_t n, const ptrdiff_t *p) { return pocketfft::stride_t(p, p + n); }

extern "C" {

const char *ref_last_error(void) { return g_err.c_str(); }

#define REF_WRAP(T, SFX)                                                                          \
  int ref_c2c_##SFX(size_t ndim, const size_t *shape, const ptrdiff_t *sin, const ptrdiff_t *sout, \
                    size_t naxes, const size_t *axes, int forward, const void *in, void *out,      \
                    double fct, size_t nthreads)                                                   \
  {                                                                                                \
    return guard([&] {                                                                             \
      pocketfft::c2c<T>(mk_shape(ndim, shape), mk_stride(ndim, sin), mk_stride(ndim, sout),        \
                        mk_shape(naxes, axes), forward != 0, (const std::complex<T> *)in,          \
                        (std::complex<T> *)out, (T)fct, nthreads);                                 \
    });                                                                                            \
  }                                                                                                \
  int ref_r2c_##SFX(size_t ndim, const size_t *shape_in, const ptrdiff_t *sin,                     \
                    const ptrdiff_t *sout, size_t naxes, const size_t *axes, int forward,          \
                    const void *in, void *out, double fct, size_t nthreads)                        \
  {                                                                                                \
    return guard([&] {                                                                             \
      pocketfft::r2c<T>(mk_shape(ndim, shape_in), mk_stride(ndim, sin), mk_stride(ndim, sout),     \
                        mk_shape(naxes, axes), forward != 0, (const T *)in,                        \
                        (std::complex<T> *)out, (T)fct, nthreads);                                 \
    });                                                                                            \
  }                                                                                                \
  int ref_c2r_##SFX(size_t ndim, const size_t *shape_out, const ptrdiff_t *sin,                    \
                    const ptrdiff_t *sout, size_t naxes, const size_t *axes, int forward,          \
                    const void *in, void *out, double fct, size_t nthreads)                        \
  {                                                                                                \
    return guard([&] {                                                                             \
      pocketfft::c2r<T>(mk_shape(ndim, shape_out), mk_stride(ndim, sin), mk_stride(ndim, sout),    \
                        mk_shape(naxes, axes), forward != 0, (const std::complex<T> *)in,          \
                        (T *)out, (T)fct, nthreads);                                               \
    });                                                                                            \
  }                                                                                                \
  int ref_r2r_fftpack_##SFX(size_t ndim, const size_t *shape, const ptrdiff_t *sin,                \
                            const ptrdiff_t *sout, size_t naxes, const size_t *axes,               \
                            int real2hermitian, int forward, const void *in, void *out,            \
                            double fct, size_t nthreads)                                           \
  {                                                                                                \
    return guard([&] {                                                                             \
      pocketfft::r2r_fftpack<T>(mk_shape(ndim, shape), mk_stride(ndim, sin),                       \
                                mk_stride(ndim, sout), mk_shape(naxes, axes),                      \
                                real2hermitian != 0, forward != 0, (const T *)in, (T *)out,        \
                                (T)fct, nthreads);                                                 \
    });                                                                                            \
  }

#define REF_WRAP2(T, SFX)                                                                         \
  int ref_dct_##SFX(size_t ndim, const size_t *shape, const ptrdiff_t *sin, const ptrdiff_t *sout,   \
                    size_t naxes, const size_t *axes, int type, const void *in, void *out, double fct, \
                    int ortho, size_t nthreads)                                                    \
  {                                                                                                \
    return guard([&] {                                                                             \
      pocketfft::dct<T>(mk_shape(ndim, shape), mk_stride(ndim, sin), mk_stride(ndim, sout),        \
                        mk_shape(naxes, axes), type, (const T *)in, (T *)out, (T)fct, ortho != 0,  \
                        nthreads);                                                                 \
    });                                                                                            \
  }                                                                                                \
  int ref_dst_##SFX(size_t ndim, const size_t *shape, const ptrdiff_t *sin, const ptrdiff_t *sout,   \
                    size_t naxes, const size_t *axes, int type, const void *in, void *out, double fct, \
                    int ortho, size_t nthreads)                                                    \
  {                                                                                                \
    return guard([&] {                                                                             \
      pocketfft::dst<T>(mk_shape(ndim, shape), mk_stride(ndim, sin), mk_stride(ndim, sout),        \
                        mk_shape(naxes, axes), type, (const T *)in, (T *)out, (T)fct, ortho != 0,  \
                        nthreads);                                                                 \
    });                                                                                            \
  }                                                                                                \
  int ref_hartley_##SFX(size_t ndim, const size_t *shape, const ptrdiff_t *sin,                    \
                        const ptrdiff_t *sout, size_t naxes, const size_t *axes, int genuine,      \
                        const void *in, void *out, double fct, size_t nthreads)                    \
  {                                                                                                \
    return guard([&] {                                                                             \
      if (genuine)                                                                                 \
        pocketfft::r2r_genuine_hartley<T>(mk_shape(ndim, shape), mk_stride(ndim, sin),             \
                                          mk_stride(ndim, sout), mk_shape(naxes, axes),            \
                                          (const T *)in, (T *)out, (T)fct, nthreads);              \
      else                                                                                         \
        pocketfft::r2r_separable_hartley<T>(mk_shape(ndim, shape), mk_stride(ndim, sin),           \
                                            mk_stride(ndim, sout), mk_shape(naxes, axes),          \
                                            (const T *)in, (T *)out, (T)fct, nthreads);            \
    });                                                                                            \
  }

// The C backend's per-line loop as impulse's fft(var openArray[float]) runs
// it (pocketfft.nim:290-303 over rfft_forward / rfft_backward), for `batch`
// contiguous lines of n reals, one plan for all of them.
int ref_rfft_batch(size_t n, size_t batch, double *c, int forward, double fct)
{
  rfft_plan plan = make_rfft_plan(n);
  if (!plan) return -1;
  int rc = 0;
  for (size_t b = 0; b < batch && rc == 0; ++b)
    rc = forward ? rfft_forward(plan, c + b * n, fct) : rfft_backward(plan, c + b * n, fct);
  destroy_rfft_plan(plan);
  return rc;
}

REF_WRAP(double, f64)
REF_WRAP(float, f32)
REF_WRAP2(double, f64)
REF_WRAP2(float, f32)

}  // extern "C"
