// ig_arith.cuh -- scalar and complex arithmetic of the GPU FFT engine.
//
// Three arithmetics share one set of FFT kernels through templates:
//
//   float  : FP32 data, FP32 butterflies (the batched FP32 path).
//   df     : FP64 data, double-float butterflies.  A value is the unevaluated
//            sum h + l of two floats; addition uses Knuth's TwoSum and
//            Dekker's Fast2Sum, multiplication uses the FMA-based exact
//            product (Dekker 1971; Knuth, TAOCP vol. 2, 4.2.2).  The result
//            carries about 48 significant bits.  GB300's FP64 pipe is ~70x
//            slower than its FP32 pipe, so FP64 data is computed this way.
//   double : native FP64 butterflies (kept for comparison and for building
//            tables; not a fast path on this GPU).
//
// The double <-> df conversions are done with integer and FP32 instructions
// only, because GB300 executes FP64 conversions on its slow FP64 pipe.
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define IGD __host__ __device__ __forceinline__
#else
#define IGD inline
#endif

#if defined(__CUDA_ARCH__)
#define IG_FADD(a, b) __fadd_rn((a), (b))
#define IG_FSUB(a, b) __fsub_rn((a), (b))
#define IG_FMUL(a, b) __fmul_rn((a), (b))
#define IG_FMA(a, b, c) __fmaf_rn((a), (b), (c))
#else
#include <math.h>
#include <string.h>
// host builds of this header are compiled with -ffp-contract=off
#define IG_FADD(a, b) ((a) + (b))
#define IG_FSUB(a, b) ((a) - (b))
#define IG_FMUL(a, b) ((a) * (b))
#define IG_FMA(a, b, c) fmaf((a), (b), (c))
#endif

namespace ig {

IGD uint32_t f2u(float f)
{
#if defined(__CUDA_ARCH__)
    return __float_as_uint(f);
#else
    uint32_t u; memcpy(&u, &f, 4); return u;
#endif
}
IGD float u2f(uint32_t u)
{
#if defined(__CUDA_ARCH__)
    return __uint_as_float(u);
#else
    float f; memcpy(&f, &u, 4); return f;
#endif
}
IGD uint64_t d2u(double d)
{
#if defined(__CUDA_ARCH__)
    return (uint64_t)__double_as_longlong(d);
#else
    uint64_t u; memcpy(&u, &d, 8); return u;
#endif
}
IGD double u2d(uint64_t u)
{
#if defined(__CUDA_ARCH__)
    return __longlong_as_double((long long)u);
#else
    double d; memcpy(&d, &u, 8); return d;
#endif
}
IGD int clz64(uint64_t x)
{
#if defined(__CUDA_ARCH__)
    return __clzll((long long)x);
#else
    return x ? __builtin_clzll(x) : 64;
#endif
}

// ---------------------------------------------------------------------------
// double-float
// ---------------------------------------------------------------------------
struct df {
    float h, l;
};

// compile-time split of a double constant into a double-float
constexpr df df_const(double c) { return df{(float)c, (float)(c - (double)(float)c)}; }

// Knuth TwoSum of the high parts, low parts added in float ("sloppy"
// double-float add: the error bound is relative to |a| + |b|, which is what a
// normwise FFT error analysis needs).  The result is left unnormalised (the
// low part may reach a few ulps of the high part); butterflies renormalise
// their outputs once with df_renorm.  Products accept unnormalised inputs.
IGD df operator+(df a, df b)
{
    float s = IG_FADD(a.h, b.h);
    float bb = IG_FSUB(s, a.h);
    float e = IG_FADD(IG_FSUB(a.h, IG_FSUB(s, bb)), IG_FSUB(b.h, bb));
    return df{s, IG_FADD(e, IG_FADD(a.l, b.l))};
}
// Dekker's Fast2Sum: |l| is a few ulps of h at most, or h == 0
IGD df df_renorm(df a)
{
    float h = IG_FADD(a.h, a.l);
    return df{h, IG_FSUB(a.l, IG_FSUB(h, a.h))};
}
IGD df operator-(df a) { return df{-a.h, -a.l}; }
IGD df operator-(df a, df b) { return a + df{-b.h, -b.l}; }
// exact product of the high parts by FMA, cross terms folded in
IGD df operator*(df a, df b)
{
    float p = IG_FMUL(a.h, b.h);
    float e = IG_FMA(a.h, b.h, -p);
    e = IG_FMA(a.h, b.l, e);
    e = IG_FMA(a.l, b.h, e);
    float h = IG_FADD(p, e);
    return df{h, IG_FSUB(e, IG_FSUB(h, p))};
}
// a*b - c*d with one rounding step for the two high products (twiddle multiply)
IGD df df_mul_sub(df a, df b, df c, df d)
{
    float p1 = IG_FMUL(a.h, b.h);
    float e1 = IG_FMA(a.h, b.h, -p1);
    float p2 = IG_FMUL(c.h, d.h);
    float e2 = IG_FMA(c.h, d.h, -p2);
    // TwoSum(p1, -p2)
    float s = IG_FSUB(p1, p2);
    float bb = IG_FSUB(s, p1);
    float e = IG_FSUB(IG_FSUB(p1, IG_FSUB(s, bb)), IG_FADD(p2, bb));
    e = IG_FADD(e, IG_FSUB(e1, e2));
    e = IG_FMA(a.h, b.l, e);
    e = IG_FMA(a.l, b.h, e);
    e = IG_FMA(-c.h, d.l, e);
    e = IG_FMA(-c.l, d.h, e);
    float h = IG_FADD(s, e);
    return df{h, IG_FSUB(e, IG_FSUB(h, s))};
}
IGD df df_mul_add(df a, df b, df c, df d) { return df_mul_sub(a, b, df{-c.h, -c.l}, d); }
IGD df df_scale2(df a, float p2) { return df{IG_FMUL(a.h, p2), IG_FMUL(a.l, p2)}; }

// double -> double-float with integer and FP32 instructions only.  `escale`
// multiplies by 2^escale exactly (per-line range scaling).  High part: the
// sign, the rebiased exponent and the top 23 fraction bits (truncated); low
// part: the remaining 29 fraction bits rounded to 23, placed under a power of
// two with one exact FP32 subtraction.  Relative error <= 2^-47.  Double
// subnormals are normalised first (an exact product by 2^64); values below
// the float range of the scaled high part flush to zero; infinities and NaNs
// map to float infinities and NaNs.
//
// the fast formula for a normal double (words hw, lw) whose scaled high part
// has the float biased exponent ef in [24, 254]
IGD df df_from_fields(uint32_t hw, uint32_t lw, int ef)
{
    const uint32_t sign = hw & 0x80000000u;
    const uint32_t f23 = ((hw << 3) | (lw >> 29)) & 0x7fffffu;
    const uint32_t eb = (uint32_t)ef << 23;
    const float h = u2f(sign | eb | f23);
    // (1 + m / 2^23) 2^(ef-23-127) - 2^(ef-23-127) = m 2^(ef-173), m = fraction bits
    // 28..0 / 2^6 rounded (m = 2^23 carries into the exponent, which is exact too)
    const uint32_t lb = eb - (23u << 23);
    const float l = IG_FSUB(u2f(lb + (((lw & 0x1fffffffu) + 32u) >> 6)), u2f(lb));
    return df{h, u2f(f2u(l) | sign)};
}
IGD df df_from_double(double x, int escale = 0)
{
    uint64_t b = d2u(x);
    uint32_t hw = (uint32_t)(b >> 32), lw = (uint32_t)b;
    int e = (int)((hw >> 20) & 0x7ffu);
    int ef = e + escale - 896;  // float biased exponent of the high part
    // for escale in [-896, 919] (a per-line test the loops hoist) ef in
    // [24, 254] already excludes zero and subnormal (e = 0) and non-finite
    // (e = 0x7ff) x; outside that window e is tested as well
    if ((unsigned)(ef - 24) < 231u && ((unsigned)(escale + 896) <= 1815u || (unsigned)(e - 1) < 2046u))
        return df_from_fields(hw, lw, ef);
    const uint32_t sign = hw & 0x80000000u;
    if (e == 0x7ff) {  // inf / nan
        const uint32_t frac = ((hw & 0xfffffu) | lw) ? 0x400000u : 0u;
        return df{u2f(sign | 0x7f800000u | frac), 0.0f};
    }
    if (e == 0) {
        if (((hw & 0x7fffffffu) | lw) == 0u) return df{u2f(sign), 0.0f};
        // subnormal double: normalised by an exact product with 2^64
        b = d2u(x * 18446744073709551616.0);
        hw = (uint32_t)(b >> 32);
        lw = (uint32_t)b;
        e = (int)((hw >> 20) & 0x7ffu);
        ef = e + escale - 64 - 896;
        if ((unsigned)(ef - 24) < 231u) return df_from_fields(hw, lw, ef);
    }
    if (ef >= 255) return df{u2f(sign | 0x7f800000u), 0.0f};
    if (ef <= 0) return df{u2f(sign), 0.0f};
    // 0 < ef < 24: high part only (the low part would be a float subnormal)
    const uint32_t f23 = ((hw << 3) | (lw >> 29)) & 0x7fffffu;
    return df{u2f(sign | ((uint32_t)ef << 23) | f23), 0.0f};
}

// float -> exact double via bit manipulation (normal floats; others special-cased)
IGD double f2d_bits(float f)
{
    uint32_t u = f2u(f);
    uint64_t sign = (uint64_t)(u & 0x80000000u) << 32;
    uint32_t ef = (u >> 23) & 0xff;
    uint32_t fr = u & 0x7fffffu;
    if (ef == 0xff) return u2d(sign | 0x7ff0000000000000ull | ((uint64_t)fr << 29));
    if (ef == 0) return u2d(sign);  // zero / float subnormal flushed
    return u2d(sign | ((uint64_t)(ef - 127 + 1023) << 52) | ((uint64_t)fr << 29));
}

// double-float -> double, general case: the two significands are aligned
// into one 64-bit integer (the larger part's units, 37 bits below its last
// bit, plus a sticky bit for any discarded low bits), normalised and rounded
// once to nearest with ties to even, and the double is assembled with integer
// instructions.
IGD double df_to_double_slow(df v, int escale)
{
    uint32_t uh = f2u(v.h), ul = f2u(v.l);
    int eh = (int)((uh >> 23) & 0xff);
    int el = (int)((ul >> 23) & 0xff);
    if (eh == 0xff) return f2d_bits(v.h);
    if (el == 0xff) return f2d_bits(v.l);
    // the sum is symmetric: align to the part with the larger exponent
    if (el > eh) {
        const uint32_t tu = uh; uh = ul; ul = tu;
        const int te = eh; eh = el; el = te;
    }
    if (eh == 0) return f2d_bits(v.h);  // zeros and float subnormals
    int64_t H = (int64_t)((uh & 0x7fffffu) | 0x800000u);
    if (uh & 0x80000000u) H = -H;
    int64_t K = H * ((int64_t)1 << 37);  // units of 2^(eh-127-23-37)
    int stk = 0;
    if (el != 0) {
        int64_t L = (int64_t)((ul & 0x7fffffu) | 0x800000u);
        if (ul & 0x80000000u) L = -L;
        const int sh = 37 - (eh - el);  // align L to K's units (sh <= 37)
        if (sh >= 0) {
            K += L * ((int64_t)1 << sh);
        } else if (sh > -62) {
            const int64_t q = L >> (-sh);  // floor; the remainder is >= 0
            stk = (L - q * ((int64_t)1 << (-sh))) != 0;
            K += q;
        } else {
            stk = 1;
            K += L < 0 ? -1 : 0;
        }
    }
    // one more bit: K2 = 2 K + sticky lies strictly inside the interval that
    // holds the exact sum whenever bits were discarded (units 2^(eh-127-61))
    K = 2 * K + stk;
    if (K == 0) return 0.0;
    uint64_t sgn = K < 0 ? 0x8000000000000000ull : 0;
    const uint64_t M0 = (uint64_t)(K < 0 ? -K : K);
    int lz = clz64(M0);
    int shift = 11 - lz;  // bring the leading one to bit 52
    // exponent of the result: value = M0 * 2^(eh - 127 - 61), M0 >> shift in [2^52, 2^53)
    int ed = eh - 127 - 9 + 1023 + shift - escale;
    // subnormal result: F 2^-1074 with F = M0 >> (shift + 1 - ed), one rounding
    // from the exact sum (a carry into bit 52 gives the smallest normal, encoded
    // the same way)
    const bool sub = ed <= 0;
    const int s = sub ? shift + 1 - ed : shift;
    uint64_t M;
    if (s <= 0) {
        M = M0 << (-s);
    } else if (s < 64) {
        // round to nearest, ties to even
        const uint64_t q = M0 >> s, rem = M0 & (((uint64_t)1 << s) - 1), half = (uint64_t)1 << (s - 1);
        M = q + ((rem > half || (rem == half && (q & 1))) ? 1 : 0);
    } else {
        M = (s == 64 && M0 > ((uint64_t)1 << 63)) ? 1 : 0;
    }
    if (sub) return u2d(sgn | M);
    if (M >> 53) { M >>= 1; ++ed; }
    if (ed >= 0x7ff) return u2d(sgn | 0x7ff0000000000000ull);
    return u2d(sgn | ((uint64_t)ed << 52) | (M & 0xfffffffffffffull));
}

// double-float -> double: both parts are rebuilt exactly as doubles from
// their bit fields (scaled by 2^-escale through the exponent) and added
// with one correctly rounded FP64 addition.  Zero, special and
// out-of-range parts take the general path.
IGD double df_to_double(df v, int escale = 0)
{
    const uint32_t uh = f2u(v.h), ul = f2u(v.l);
    const int eh = (int)((uh >> 23) & 0xffu), el = (int)((ul >> 23) & 0xffu);
    // a normal float part (biased exponent 1..254) rebiased by 896 - escale is a
    // normal double whenever |escale| <= 896 (a per-line test the loops hoist)
    if ((unsigned)(escale + 896) <= 1792u && (unsigned)(eh - 1) < 254u && (el == 0 || (unsigned)(el - 1) < 254u)) {
        const uint32_t rebias = (uint32_t)(896 - escale) << 20;
        const double dh = u2d(((uint64_t)((uh & 0x80000000u) | (((uh & 0x7fffffffu) >> 3) + rebias)) << 32) |
                              (uint64_t)(uh << 29));
        // a zero (or float subnormal) low part adds nothing
        const uint32_t lhi = el ? (ul & 0x80000000u) | (((ul & 0x7fffffffu) >> 3) + rebias) : 0u;
        const double dl = u2d(((uint64_t)lhi << 32) | (uint64_t)(el ? ul << 29 : 0u));
        return dh + dl;
    }
    return df_to_double_slow(v, escale);
}

// sign flip of a double through its bit pattern (no FP64 instruction)
IGD double dneg(double x) { return u2d(d2u(x) ^ 0x8000000000000000ull); }

// x 2^es exactly, by an add to the exponent field when x and the result are
// normal doubles; zeros, subnormals, specials and out-of-range results go
// through the double-float conversions
IGD double pow2_scale(double x, int es)
{
    const uint64_t b = d2u(x);
    const int e = (int)((b >> 52) & 0x7ffu);
    if ((unsigned)(e - 1) < 2046u && (unsigned)(e + es - 1) < 2046u)
        return u2d(b + ((uint64_t)(int64_t)es << 52));
    return df_to_double(df_from_double(x, es), 0);
}

// ---------------------------------------------------------------------------
// generic real helpers: constants, scale by power of two
// ---------------------------------------------------------------------------
template <class R> struct RealOps;
template <> struct RealOps<float> {
    static constexpr float k(double c) { return (float)c; }
};
template <> struct RealOps<double> {
    static constexpr double k(double c) { return c; }
};
template <> struct RealOps<df> {
    static constexpr df k(double c) { return df_const(c); }
};

// ---------------------------------------------------------------------------
// complex
// ---------------------------------------------------------------------------
template <class R> struct cx {
    R r, i;
};
template <class R> IGD cx<R> operator+(cx<R> a, cx<R> b) { return cx<R>{a.r + b.r, a.i + b.i}; }
template <class R> IGD cx<R> operator-(cx<R> a, cx<R> b) { return cx<R>{a.r - b.r, a.i - b.i}; }
// a * w
template <class R> IGD cx<R> cmul(cx<R> a, cx<R> w) { return cx<R>{a.r * w.r - a.i * w.i, a.r * w.i + a.i * w.r}; }
// a * conj(w)
template <class R> IGD cx<R> cmulc(cx<R> a, cx<R> w) { return cx<R>{a.r * w.r + a.i * w.i, a.i * w.r - a.r * w.i}; }
template <> IGD cx<df> cmul<df>(cx<df> a, cx<df> w)
{
    return cx<df>{df_mul_sub(a.r, w.r, a.i, w.i), df_mul_add(a.r, w.i, a.i, w.r)};
}
template <> IGD cx<df> cmulc<df>(cx<df> a, cx<df> w)
{
    return cx<df>{df_mul_add(a.r, w.r, a.i, w.i), df_mul_sub(a.i, w.r, a.r, w.i)};
}
// a * w or a * conj(w)
template <bool FWD, class R> IGD cx<R> twmul(cx<R> a, cx<R> w) { return FWD ? cmul(a, w) : cmulc(a, w); }
// multiply by -i (forward) / +i (backward)
template <bool FWD, class R> IGD cx<R> rot(cx<R> a)
{
    if (FWD) return cx<R>{a.i, -a.r};
    return cx<R>{-a.i, a.r};
}
template <class R> IGD cx<R> cscale(cx<R> a, R s) { return cx<R>{a.r * s, a.i * s}; }
// exact halving
IGD cx<float> chalf(cx<float> a) { return cx<float>{a.r * 0.5f, a.i * 0.5f}; }
IGD cx<double> chalf(cx<double> a) { return cx<double>{a.r * 0.5, a.i * 0.5}; }
IGD cx<df> chalf(cx<df> a) { return cx<df>{df_scale2(a.r, 0.5f), df_scale2(a.i, 0.5f)}; }
// times 2^d, d <= 0 (exact; below the float range the value flushes to zero)
IGD cx<float> cscale_pow2(cx<float> a, int d)
{
    if (!d) return a;
    if (d < -126) return cx<float>{0.0f, 0.0f};
    const float f = u2f((uint32_t)(127 + d) << 23);
    return cx<float>{IG_FMUL(a.r, f), IG_FMUL(a.i, f)};
}
IGD cx<double> cscale_pow2(cx<double> a, int) { return a; }
IGD cx<df> cscale_pow2(cx<df> a, int d)
{
    if (!d) return a;
    if (d < -126) return cx<df>{df{0.0f, 0.0f}, df{0.0f, 0.0f}};
    const float f = u2f((uint32_t)(127 + d) << 23);
    return cx<df>{df_scale2(a.r, f), df_scale2(a.i, f)};
}
// renormalise a double-float complex (no-op for float / double)
IGD cx<float> crenorm(cx<float> a) { return a; }
IGD cx<double> crenorm(cx<double> a) { return a; }
IGD cx<df> crenorm(cx<df> a) { return cx<df>{df_renorm(a.r), df_renorm(a.i)}; }
template <class R> IGD cx<R> conjx(cx<R> a) { return cx<R>{a.r, -a.i}; }

// ---------------------------------------------------------------------------
// storage <-> arithmetic
// ---------------------------------------------------------------------------
template <class R> struct Store;
template <> struct Store<float> {
    using real = float;
    // x * 2^es (exact; es is clamped to the normal exponent range)
    IGD static float in(float x, int es)
    {
        if (!es) return x;
        int e = es < -126 ? -126 : (es > 127 ? 127 : es);
        return IG_FMUL(x, u2f((uint32_t)(127 + e) << 23));
    }
    IGD static float out(float x, int) { return x; }
};
template <> struct Store<double> {
    using real = double;
    IGD static double in(double x, int) { return x; }
    IGD static double out(double x, int) { return x; }
};
template <> struct Store<df> {
    using real = double;
    IGD static df in(double x, int es) { return df_from_double(x, es); }
    IGD static double out(df x, int es) { return df_to_double(x, es); }
};

}  // namespace ig
