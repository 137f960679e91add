// ig_kernels.cuh -- device kernels of the GPU FFT engine (templates).
//
// k_fft_smem is the workhorse: one CTA owns `lpc` whole lines, stages them
// from HBM into shared memory, runs a Stockham autosort FFT of length L in
// shared memory with register-resident radix-R butterflies, and writes the
// result back.  Around the core it fuses the layout work of impulse's FFT
// path:
//   - complex lines (pocketfft::c2c, pocketfft_hdronly.h:3272);
//   - real input packed as N/2 complex values with the split step that
//     writes FFTPACK halfcomplex order directly (rfft_forward,
//     impulse/fft/c_pocketfft/pocketfft.c:2184) or the N/2+1 half spectrum
//     (general_r2c, pocketfft_hdronly.h:3125);
//   - the inverse of both (rfft_backward pocketfft.c:2176, general_c2r
//     pocketfft_hdronly.h:3180);
//   - Bluestein for lengths with large prime factors (fftblue_fft,
//     pocketfft.c:1945): chirp premultiply, zero padding, forward FFT,
//     pointwise product with the transformed chirp, backward FFT and chirp
//     postmultiply, all in shared memory;
//   - the inter-pass twiddle of the four-step decomposition used for lines
//     longer than shared memory.
// FP64 lines computed in double-float are range-scaled per line by a power
// of two (exact), so any finite input magnitude keeps ~48-bit accuracy.
#pragma once
#include <cuda_runtime.h>
#include <type_traits>
#include "ig_dft.cuh"
#include "ig_pdf.cuh"
#include "ig_types.h"

namespace ig {

template <class T> struct Traits;
template <> struct Traits<float> {
    using S = float;
    using S2 = float2;
    static constexpr bool kRaw = false;
};
template <> struct Traits<double> {
    using S = double;
    using S2 = double2;
    static constexpr bool kRaw = false;
};
template <> struct Traits<df> {
    using S = double;
    using S2 = double2;
    static constexpr bool kRaw = true;  // prologue stages raw doubles, first reader converts
};

__device__ __forceinline__ unsigned fdiv(unsigned n, FastDiv f)
{
    return (unsigned)(((unsigned long long)n * f.m) >> f.s);
}

// n / d for element indices: 32-bit fast division below 2^31, else 64-bit
__device__ __forceinline__ long long qdiv(long long n, long long d, FastDiv f)
{
    return n < 0x7fffffffLL ? (long long)fdiv((unsigned)n, f) : n / d;
}

// streaming global accesses of line data: each element is read and written
// once, so it goes through L1 evict-first and leaves the cache to the
// twiddle tables
template <class V> __device__ __forceinline__ V ldg_s(const char *p) { return __ldcs(reinterpret_cast<const V *>(p)); }
template <class V> __device__ __forceinline__ void stg_s(char *p, V v) { __stcs(reinterpret_cast<V *>(p), v); }

// POST_SPLIT4 row order: slot j of a transform's N1 rows holds row
// r = j / 2 + 1 (j even) or N1 - r (j odd) while r < N1 / 2, then row 0 twice
// and, for even N1, row N1 / 2 twice
__device__ __forceinline__ int split_row(int j, int N1)
{
    const int h2 = ((N1 - 1) >> 1) << 1;
    if (j < h2) {
        const int r = (j >> 1) + 1;
        return (j & 1) ? N1 - r : r;
    }
    return ((j - h2) >> 1) ? (N1 >> 1) : 0;
}

// byte offset of line l: from the offset tables when present, else
// l -> (l mod bn0, (l / bn0) mod bn1, l / (bn0 bn1)) over the batch dims
// (on the input side of POST_SPLIT4 the first index is a row slot)
__device__ __forceinline__ long long line_off(const IODesc &io, long long l, bool out)
{
    if (out ? io.loff_out != nullptr : io.loff_in != nullptr) return out ? io.loff_out[l] : io.loff_in[l];
    const unsigned lu = (unsigned)l;
    const unsigned q0 = fdiv(lu, io.fb0);
    unsigned i0 = lu - q0 * (unsigned)io.bn[0];
    const unsigned q1 = fdiv(q0, io.fb1);
    const unsigned i1 = q0 - q1 * (unsigned)io.bn[1];
    if (!out && io.split_N1) i0 = (unsigned)split_row((int)i0, io.split_N1);
    return out ? (long long)i0 * io.bso[0] + (long long)i1 * io.bso[1] + (long long)q1 * io.bso[2]
               : (long long)i0 * io.bsi[0] + (long long)i1 * io.bsi[1] + (long long)q1 * io.bsi[2];
}
__device__ __forceinline__ int line_i0(const IODesc &io, long long l)
{
    const unsigned lu = (unsigned)l;
    return (int)(lu - fdiv(lu, io.fb0) * (unsigned)io.bn[0]);
}
// index of line l along batch dim 1
__device__ __forceinline__ int line_i1(const IODesc &io, long long l)
{
    const unsigned q0 = fdiv((unsigned)l, io.fb0);
    return (int)(q0 - fdiv(q0, io.fb1) * (unsigned)io.bn[1]);
}

__device__ __forceinline__ int dexp(double x) { return (int)((__double_as_longlong(x) >> 52) & 0x7ff); }

// Line-scale keys.  A line's elements are reduced to the largest magnitude
// word (dmag: the high 32 bits of |x| for doubles, fmag: |x| for floats,
// whose unsigned order is the order of |x|; two integer operations per
// element), and that maximum to a key once: the biased exponent as if the
// value were normal (double subnormals get their true exponent below the
// normal range, down to -19 from the high word -- values under 2^-1042 count
// as zero; float subnormals down to -22), plus kKeyOff, so that 0 stays "no
// value" (zeros; infinities and NaN dominate the maximum and also give 0, no
// rescaling).  A line's exact power-of-two scale is (bias + kKeyOff) - key.
constexpr int kKeyOff = 64;
__device__ __forceinline__ unsigned dmag(double x) { return (unsigned)(__double_as_longlong(x) >> 32) & 0x7fffffffu; }
__device__ __forceinline__ unsigned fmag(float x) { return __float_as_uint(x) & 0x7fffffffu; }
__device__ __forceinline__ int dkey_mag(unsigned m)
{
    const int e = (int)(m >> 20);
    if (e == 0x7ff || m == 0) return 0;
    if (e) return e + kKeyOff;
    return (31 - __clz((int)m)) - 19 + kKeyOff;
}
__device__ __forceinline__ int fkey_mag(unsigned m)
{
    const int e = (int)(m >> 23);
    if (e == 0xff || m == 0) return 0;
    if (e) return e + kKeyOff;
    return (31 - __clz((int)m)) - 22 + kKeyOff;
}

// slot read with optional raw-double conversion
template <class T, bool RAW> __device__ __forceinline__ cx<T> sload(const cx<T> *p, int esc)
{
    if constexpr (RAW) {
        double2 d = *reinterpret_cast<const double2 *>(p);
        return cx<T>{Store<T>::in(d.x, esc), Store<T>::in(d.y, esc)};
    } else {
        return *p;
    }
}

// shared-memory slot access: double-float complexes are stored as
// (re.h, im.h, re.l, im.l) for the packed butterflies
template <class T> __device__ __forceinline__ cx<T> sget(const cx<T> *p) { return *p; }
template <class T> __device__ __forceinline__ void sput(cx<T> *p, cx<T> v) { *p = v; }
template <> __device__ __forceinline__ cx<df> sget<df>(const cx<df> *p) { return from_p(pld(p)); }
template <> __device__ __forceinline__ void sput<df>(cx<df> *p, cx<df> v) { pst(p, to_p(v)); }

// padded shared-memory slot of element i
__device__ __forceinline__ int sp(int i, int pad) { return i + (i >> pad); }

// Butterfly arithmetic of the stages: plain complexes for float / double,
// packed pairs (ig_pdf.cuh) for double-float, whose stage twiddle table
// holds (wr.h, wi.h, wr.l, wi.l), 16 bytes an entry, paired in registers.
template <class T> struct Bfly {
    using V = cx<T>;
    using W = cx<T>;
    static __device__ __forceinline__ V ld(const cx<T> *p) { return *p; }
    static __device__ __forceinline__ void st(cx<T> *p, V v) { *p = crenorm(v); }
    static __device__ __forceinline__ V tw(V a, const W *w, const CoreDesc &) { return cmul(a, *w); }
    template <int R> static __device__ __forceinline__ void dft(V *v) { ig::dft<R, true>(v); }
};
template <> struct Bfly<df> {
    using V = pcx;
    using W = ptw;
    static __device__ __forceinline__ V ld(const cx<df> *p) { return pld(p); }
    static __device__ __forceinline__ void st(cx<df> *p, V v) { pst(p, prenorm(v)); }
    // the stage butterflies add twiddled inputs lazily: products stay unrenormalised
    static __device__ __forceinline__ V tw(V a, const W *w, const CoreDesc &P) { return pmulw<false>(a, w, P.neg1); }
    template <int R> static __device__ __forceinline__ void dft(V *v) { pdft<R>(v); }
};

// z * w (forward) or z * conj(w) with w in the stage-twiddle format
template <class T>
__device__ __forceinline__ cx<T> tw_apply(cx<T> z, const typename Bfly<T>::W *w, int fwd, const CoreDesc &P)
{
    if constexpr (std::is_same<T, df>::value) {
        pcx a = to_p(z);
        if (!fwd) a = pconj(a);
        a = pmulw(a, w, P.neg1);
        if (!fwd) a = pconj(a);
        return from_p(a);
    } else {
        (void)P;
        return fwd ? cmul(z, *w) : cmulc(z, *w);
    }
}

// One Stockham stage of radix R in shared memory, in place through
// registers.  Butterfly j (j < L/R) of a line reads x[j + m L/R], twiddles
// input m by w^(m k) (k = j mod ns, w = exp(-+2 pi i/(ns R))), runs a radix-R
// DFT and writes y[(j / ns) ns R + k + m ns].  All reads of a stage precede
// the barrier and all writes follow it.
template <class T, int E, int R>
__device__ __forceinline__ void stage(cx<T> *sm, const CoreDesc &P, int si, int nl, int tpl, int g, int t, int LSl)
{
    using B = Bfly<T>;
    using V = typename B::V;
    constexpr int NB = (E + R - 1) / R;
    const int nr = P.L / R, ns = P.st[si].ns, pad = P.pad;
    const FastDiv fns = P.st[si].fns;
    const typename B::W *tw = reinterpret_cast<const typename B::W *>(P.tw) + P.st[si].tw;
    cx<T> *line = sm + (size_t)g * LSl;
    V v[NB][R];
    int jj[NB];
#pragma unroll
    for (int i = 0; i < NB; ++i) {
        int j = t + i * tpl;
        jj[i] = (g < nl && j < nr) ? j : -1;
        if (jj[i] >= 0) {
#pragma unroll
            for (int m = 0; m < R; ++m) v[i][m] = B::ld(line + sp(j + m * nr, pad));
        }
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < NB; ++i) {
        if (jj[i] >= 0) {
            const int j = jj[i];
            const int q = (int)fdiv((unsigned)j, fns), k = j - q * ns;
            if (k) {
                const typename B::W *twk = tw + k * (R - 1) - 1;
#pragma unroll
                for (int m = 1; m < R; ++m) v[i][m] = B::tw(v[i][m], twk + m, P);
            }
            B::template dft<R>(v[i]);
            const int base = q * ns * R + k;
#pragma unroll
            for (int m = 0; m < R; ++m) B::st(line + sp(base + m * ns, pad), v[i][m]);
        }
        // keep the next butterfly's twiddle loads below this one's stores, so
        // that only one butterfly's twiddles are live at a time
        asm volatile("" ::: "memory");
    }
    __syncthreads();
}

// The same stage between two buffers (double-buffered Stockham): each
// butterfly reads src and writes dst, so no barrier separates its reads from
// its writes and only one butterfly is live in registers at a time; one
// barrier per stage.  Line g's buffers are src/dst + g * LS2.
template <class T, int E, int R>
__device__ __forceinline__ void stage_db(const cx<T> *src, cx<T> *dst, int LS2, const CoreDesc &P, int si, int nl,
                                         int tpl, int g, int t)
{
    using B = Bfly<T>;
    using V = typename B::V;
    constexpr int NB = (E + R - 1) / R;
    const int nr = P.L / R, ns = P.st[si].ns, pad = P.pad;
    const FastDiv fns = P.st[si].fns;
    const typename B::W *tw = reinterpret_cast<const typename B::W *>(P.tw) + P.st[si].tw;
    if (g >= nl) return;
    const cx<T> *in = src + (size_t)g * LS2;
    cx<T> *out = dst + (size_t)g * LS2;
    // when the element step (nr for the reads, ns for the writes) is a multiple
    // of the padding period, sp(x + m step) = sp(x) + m sp(step): one add per
    // element instead of the shift-and-add of each padded index
    const int pmask = pad >= 31 ? 0 : (1 << pad) - 1;
    const bool lin_ld = (nr & pmask) == 0, lin_st = (ns & pmask) == 0;
    const int nrp = sp(nr, pad), nsp = sp(ns, pad);
#pragma unroll
    for (int i = 0; i < NB; ++i) {
        const int j = t + i * tpl;
        if (j < nr) {
            V v[R];
            if (lin_ld) {
                const cx<T> *p0 = in + sp(j, pad);
#pragma unroll
                for (int m = 0; m < R; ++m) v[m] = B::ld(p0 + m * nrp);
            } else {
#pragma unroll
                for (int m = 0; m < R; ++m) v[m] = B::ld(in + sp(j + m * nr, pad));
            }
            const int q = (int)fdiv((unsigned)j, fns), k = j - q * ns;
            if (k) {
                const typename B::W *twk = tw + k * (R - 1) - 1;
#pragma unroll
                for (int m = 1; m < R; ++m) v[m] = B::tw(v[m], twk + m, P);
            }
            B::template dft<R>(v);
            const int base = q * ns * R + k;
            if (lin_st) {
                cx<T> *p0 = out + sp(base, pad);
#pragma unroll
                for (int m = 0; m < R; ++m) B::st(p0 + m * nsp, v[m]);
            } else {
#pragma unroll
                for (int m = 0; m < R; ++m) B::st(out + sp(base + m * ns, pad), v[m]);
            }
        }
        asm volatile("" ::: "memory");
    }
}

// Radix classes: a kernel instantiation compiles only the radix cases of its
// class, which keeps the register allocation of the whole kernel small
// (the union of all radix cases spills).
// radix 16 only in the 16-elements-per-thread variants (the planner caps
// 8-element cores at radix 8)
template <int E, int RS> __host__ __device__ constexpr bool rs_has(int R)
{
    return (R == 2 || R == 4 || R == 8) || (R == 16 && E == 16) || (RS >= RS_P235 && (R == 3 || R == 5 || R == 9)) ||
           (RS >= RS_ALL && (R == 7 || R == 11)) || (RS == RS_FULL && R == 13);
}

// Forward stages only: a backward transform runs them on conjugated data
// (IFFT(x) = conj(FFT(conj(x)))), with the conjugations folded into the
// prologue, the epilogue and the Bluestein steps.
template <class T, int E, int RS>
__device__ __forceinline__ void run_stages(cx<T> *sm, const CoreDesc &P, int nl, int tpl, int g, int t, int LSl)
{
    for (int s = 0; s < P.nst; ++s) {
        switch (P.st[s].R) {
        case 2: stage<T, E, 2>(sm, P, s, nl, tpl, g, t, LSl); break;
        case 4: stage<T, E, 4>(sm, P, s, nl, tpl, g, t, LSl); break;
        case 8: stage<T, E, 8>(sm, P, s, nl, tpl, g, t, LSl); break;
        case 16: if constexpr (rs_has<E, RS>(16)) stage<T, E, 16>(sm, P, s, nl, tpl, g, t, LSl); break;
        case 3: if constexpr (rs_has<E, RS>(3)) stage<T, E, 3>(sm, P, s, nl, tpl, g, t, LSl); break;
        case 5: if constexpr (rs_has<E, RS>(5)) stage<T, E, 5>(sm, P, s, nl, tpl, g, t, LSl); break;
        case 9: if constexpr (rs_has<E, RS>(9)) stage<T, E, 9>(sm, P, s, nl, tpl, g, t, LSl); break;
        case 7: if constexpr (rs_has<E, RS>(7)) stage<T, E, 7>(sm, P, s, nl, tpl, g, t, LSl); break;
        case 11: if constexpr (rs_has<E, RS>(11)) stage<T, E, 11>(sm, P, s, nl, tpl, g, t, LSl); break;
        case 13: if constexpr (rs_has<E, RS>(13)) stage<T, E, 13>(sm, P, s, nl, tpl, g, t, LSl); break;
        default: break;
        }
    }
}

// double-buffered core: buffers A = sm, B = sm + LS (line stride LS2 = 2 LS);
// returns the offset (0 or LS) of the buffer that holds the result
template <class T, int E, int RS>
__device__ __forceinline__ int run_stages_db(cx<T> *sm, int cur, const CoreDesc &P, int nl, int tpl, int g, int t,
                                             int LS2)
{
    const int LS = P.LS;
    for (int s = 0; s < P.nst; ++s) {
        const cx<T> *src = sm + cur;
        cx<T> *dst = sm + (LS - cur);
        switch (P.st[s].R) {
        case 2: stage_db<T, E, 2>(src, dst, LS2, P, s, nl, tpl, g, t); break;
        case 4: stage_db<T, E, 4>(src, dst, LS2, P, s, nl, tpl, g, t); break;
        case 8: stage_db<T, E, 8>(src, dst, LS2, P, s, nl, tpl, g, t); break;
        case 16: if constexpr (rs_has<E, RS>(16)) stage_db<T, E, 16>(src, dst, LS2, P, s, nl, tpl, g, t); break;
        case 3: if constexpr (rs_has<E, RS>(3)) stage_db<T, E, 3>(src, dst, LS2, P, s, nl, tpl, g, t); break;
        case 5: if constexpr (rs_has<E, RS>(5)) stage_db<T, E, 5>(src, dst, LS2, P, s, nl, tpl, g, t); break;
        case 9: if constexpr (rs_has<E, RS>(9)) stage_db<T, E, 9>(src, dst, LS2, P, s, nl, tpl, g, t); break;
        case 7: if constexpr (rs_has<E, RS>(7)) stage_db<T, E, 7>(src, dst, LS2, P, s, nl, tpl, g, t); break;
        case 11: if constexpr (rs_has<E, RS>(11)) stage_db<T, E, 11>(src, dst, LS2, P, s, nl, tpl, g, t); break;
        case 13: if constexpr (rs_has<E, RS>(13)) stage_db<T, E, 13>(src, dst, LS2, P, s, nl, tpl, g, t); break;
        default: break;
        }
        cur = LS - cur;
        __syncthreads();
    }
    return cur;
}

// scale helper: multiply by fct and store with the per-line exponent
template <class T> struct OutScale;
__device__ __forceinline__ float fpow2(int e)  // 2^e, e in [-126, 127]
{
    return __uint_as_float((unsigned)(127 + max(-126, min(127, e))) << 23);
}
__device__ __forceinline__ int fexp(float x) { return (int)((__float_as_uint(x) >> 23) & 0xff); }
template <> struct OutScale<float> {
    float f;
    __device__ void init(const IODesc &io) { f = io.fct_f; }
    __device__ float apply(float v, int esc) const { return esc ? v * (f * fpow2(-esc)) : v * f; }
};
template <> struct OutScale<double> {
    double f;
    __device__ void init(const IODesc &io) { f = io.fct; }
    __device__ double apply(double v, int) const { return v * f; }
};
template <> struct OutScale<df> {
    df m;
    int e;
    bool pow2;
    __device__ void init(const IODesc &io)
    {
        // fct = m * 2^e with m in [1, 2) (split on the host): the exponent is
        // folded into the output conversion; a power of two (m = 1) costs nothing
        m = df{io.fct_h, io.fct_l};
        e = io.fct_e;
        pow2 = io.fct_h == 1.0f && io.fct_l == 0.0f;
    }
    __device__ double apply(df v, int esc) const { return df_to_double(pow2 ? v : v * m, esc - e); }
};

// load one storage unit of an input line (kinds of IODesc), as raw storage values
template <class S, class S2>
__device__ __forceinline__ void load_unit(const IODesc &io, const char *base, int u, S &re, S &im)
{
    if (io.in_kind == IN_C) {
        S2 z = ldg_s<S2>(base + (long long)u * io.is);
        re = z.x;
        im = z.y;
    } else if (io.in_kind == IN_R) {
        re = ldg_s<S>(base + (long long)u * io.is);
        im = S(0);
    } else if (io.in_kind == IN_P) {
        const char *p = base + (long long)u * io.is;
        re = ldg_s<S>(p);
        im = ldg_s<S>(p + io.ps_in);
    } else {  // IN_HC: unit 0 = (r0, 0); unit k = (r_{2k-1}, r_{2k}); even N: last = (r_{N-1}, 0)
        if (u == 0) {
            re = ldg_s<S>(base);
            im = S(0);
        } else {
            re = ldg_s<S>(base + (2 * (long long)u - 1) * io.is);
            im = (2 * (long long)u < io.nreal) ? ldg_s<S>(base + (2 * (long long)u) * io.is) : S(0);
        }
    }
}
__device__ __forceinline__ float negs(float x) { return -x; }
__device__ __forceinline__ double negs(double x) { return dneg(x); }

// write unit u of an output line (kinds of IODesc) with the output scale
template <class T, class S, class S2>
__device__ __forceinline__ void store_unit(const IODesc &io, char *base, int u, cx<T> z, const OutScale<T> &sc, int esc)
{
    if (io.out_kind == OUT_C) {
        S2 o;
        o.x = sc.apply(z.r, esc);
        o.y = sc.apply(z.i, esc);
        stg_s<S2>(base + (long long)u * io.os, o);
    } else if (io.out_kind == OUT_R) {
        stg_s<S>(base + (long long)u * io.os, sc.apply(z.r, esc));
    } else if (io.out_kind == OUT_P) {
        char *p = base + (long long)u * io.os;
        stg_s<S>(p, sc.apply(z.r, esc));
        stg_s<S>(p + io.ps_out, sc.apply(z.i, esc));
    } else {  // OUT_HC
        if (u == 0) stg_s<S>(base, sc.apply(z.r, esc));
        else {
            stg_s<S>(base + (2 * (long long)u - 1) * io.os, sc.apply(z.r, esc));
            if (2 * (long long)u < io.nreal) stg_s<S>(base + (2 * (long long)u) * io.os, sc.apply(z.i, esc));
        }
    }
}

// One block of lines: lines [blk * lpc, blk * lpc + lpc) of (P, io), with the
// input / output base pointers given explicitly (the persistent work-list
// kernel keeps its groups' pointers relative to per-launch bases).  Threads
// beyond lpc * tpl take part only in the barriers.
// Rader permutations of one line through registers (reads, barrier, writes,
// barrier).  A thread covers u = t + k tpl, k <= E, which reaches M because
// E tpl >= L = M - 1.
//  gather (out = false): line[q] = line[idx[q]] for q < L, x[0] saved at *x0s;
//  scatter (out = true): line[0] = x0 + A0 (A0 saved at *a0s), and
//  line[u] = x0 + conj(line[idx[u]]) for 0 < u < M.
template <class T, int E>
__device__ __forceinline__ void rader_permute(cx<T> *line, const int *__restrict__ idx, int L, int tpl, int t,
                                              int pad, bool act, cx<T> *x0s, cx<T> *a0s, bool out)
{
    constexpr int K = E + 1;
    const int n = out ? L + 1 : L;
    cx<T> v[K];
    cx<T> x0{};
    if (act) {
        x0 = out ? sget(x0s) : sget(line);
        const cx<T> a0 = out ? sget(a0s) : cx<T>{};
#pragma unroll
        for (int k = 0; k < K; ++k) {
            const int u = t + k * tpl;
            if (u < n) {
                if (!out) v[k] = sget(line + sp(idx[u], pad));
                else v[k] = u == 0 ? a0 : conjx(sget(line + sp(idx[u], pad)));
            }
        }
    }
    __syncthreads();
    if (act) {
#pragma unroll
        for (int k = 0; k < K; ++k) {
            const int u = t + k * tpl;
            if (u < n) sput(line + sp(u, pad), out ? crenorm(x0 + v[k]) : v[k]);
        }
        if (!out && t == 0) sput(x0s, x0);
    }
    __syncthreads();
}

// RC: the row-convolution mode (IODesc::rowconv) compiled in (layout class
// LAY_RC: the twiddle / table variant plus the mode, kept apart so that the
// plain twiddle variant keeps its registers)
template <class T, int E, int RS, int LAY, bool DB = (E == 8), bool RC = (LAY == LAY_RC)>
__device__ __forceinline__ void fft_block(const CoreDesc &P, const IODesc &io, long long blk, const char *in_base,
                                          char *out_base)
{
    using S = typename Traits<T>::S;
    using S2 = typename Traits<T>::S2;
    constexpr bool RAW = Traits<T>::kRaw;  // double-float: per-line range check and scaling
    extern __shared__ __align__(16) unsigned char smraw[];
    cx<T> *sm = reinterpret_cast<cx<T> *>(smraw);
    __shared__ int s_esc[2 * kMaxLinesPerCta];   // per real sub-line: 2 g (+1 for line b of a pair)
    __shared__ int s_emax[2 * kMaxLinesPerCta];
    __shared__ int s_rescale;

    // DB: double-buffered stages (2 LS slots per line)
    // per-line stride of the CTA's line buffers: odd (in slots), so that the
    // column-mapped prologue and epilogue (consecutive threads on consecutive
    // lines) hit distinct banks
    const int LSt = DB ? 2 * P.LS + 1 : (P.LS | 1);
    const int lpc = io.lpc, tpl = io.tpl, pad = P.pad;
    const long long line0 = blk * lpc;
    const int nl = (int)min((long long)lpc, io.nlines - line0);
    const int M = P.M;
    // backward Stockham cores run the forward stages on conjugated data
    // (Rader cores compute the forward DFT like Stockham ones)
    const bool cc = !io.fwd && P.blue != 1;
    // core mapping: line g, lane t of the line
    const int g = threadIdx.x / tpl, t = threadIdx.x - g * tpl;
    cx<T> *const line_a = sm + (size_t)(g < nl ? g : 0) * LSt;
    int cur = 0;  // offset of the buffer holding the line (double-buffered stages)
    cx<T> *myline = line_a;

    // range scaling: double-float lines always, FP32 lines when two real lines share one complex line
    const bool paired = LAY == LAY_PR2HC || (LAY == LAY_GEN && io.pair != 0);
    const bool scaled = RAW || paired;
    if (scaled) {
        for (int i = threadIdx.x; i < 2 * lpc; i += blockDim.x) { s_esc[i] = 0; s_emax[i] = 0; }
        if (threadIdx.x == 0) s_rescale = 0;
        __syncthreads();
    }

    // ---- prologue: HBM -> shared memory, converting to the arithmetic type.
    // Lines whose largest element lies far from 1 (double-float), or the two
    // real lines of a pair whose magnitudes differ (so that each keeps its own
    // relative accuracy), are loaded a second time with exact power-of-two
    // scales, one per real line.
    {
        int gi, ti;
        if (io.cols_in) { gi = threadIdx.x % lpc; ti = threadIdx.x / lpc; }
        else { gi = g; ti = t; }
        const bool act = gi < nl && ti < tpl;
        const char *base = act ? in_base + line_off(io, line0 + gi, false) : nullptr;
        const bool has_b = act && paired && (2LL * line_i0(io, line0 + gi) + 1 < io.pair_n0);
        const char *base_b = base + io.pair_in;
        cx<T> *line = sm + (size_t)(act ? gi : 0) * LSt;
        for (int attempt = 0; attempt < (scaled ? 2 : 1); ++attempt) {
            const int esc = (scaled && act) ? s_esc[2 * gi] : 0;
            const int escb = (scaled && act) ? s_esc[2 * gi + 1] : 0;
            unsigned emax = 0, emaxb = 0;  // largest magnitude words (dmag / fmag)
            if (act && (LAY == LAY_C2C || LAY == LAY_R2HC || LAY == LAY_TW || LAY == LAY_RC)) {
                // complex units, no conjugation / Hermitian steps / pairs
                // loads in flight per thread before the first is used: the prologue is
                // latency-bound on global loads; FP32 units are small enough for eight
                constexpr int CH = RAW ? 4 : 8;
                const int cnt = io.cnt_in;
                const long long is = io.is;
                for (int u0 = ti; u0 < cnt; u0 += CH * tpl) {
                    S2 v[CH];
#pragma unroll
                    for (int c = 0; c < CH; ++c) {
                        const int u = u0 + c * tpl;
                        if (u < cnt) v[c] = ldg_s<S2>(base + (long long)u * is);
                    }
#pragma unroll
                    for (int c = 0; c < CH; ++c) {
                        const int u = u0 + c * tpl;
                        if (u >= cnt) break;
                        if constexpr (RAW) {
                            emax = max(emax, max(dmag(v[c].x), dmag(v[c].y)));
                        }
                        cx<T> z{Store<T>::in(v[c].x, esc), Store<T>::in(v[c].y, esc)};
                        sput(line + sp(u, pad), cc ? conjx(z) : z);
                    }
                }
            } else if (act && LAY == LAY_PR2HC) {
                // two real lines -> (a, b)
                // loads in flight per thread before the first is used: the prologue is
                // latency-bound on global loads; FP32 units are small enough for eight
                constexpr int CH = RAW ? 4 : 8;
                const int cnt = io.cnt_in;
                const long long is = io.is;
                for (int u0 = ti; u0 < cnt; u0 += CH * tpl) {
                    S va[CH], vb[CH];
#pragma unroll
                    for (int c = 0; c < CH; ++c) {
                        const int u = u0 + c * tpl;
                        va[c] = vb[c] = S(0);
                        if (u < cnt) {
                            va[c] = ldg_s<S>(base + (long long)u * is);
                            if (has_b) vb[c] = ldg_s<S>(base_b + (long long)u * is);
                        }
                    }
#pragma unroll
                    for (int c = 0; c < CH; ++c) {
                        const int u = u0 + c * tpl;
                        if (u >= cnt) break;
                        if constexpr (RAW) {
                            emax = max(emax, dmag(va[c]));
                            emaxb = max(emaxb, dmag(vb[c]));
                        } else {
                            emax = max(emax, fmag(va[c]));
                            emaxb = max(emaxb, fmag(vb[c]));
                        }
                        sput(line + sp(u, pad), cx<T>{Store<T>::in(va[c], esc), Store<T>::in(vb[c], escb)});
                    }
                }
            } else if (act) {
                // chunks of 4 units: all loads of a chunk are issued before any is used
                constexpr int CH = 4;
                for (int u0 = ti; u0 < io.cnt_in; u0 += CH * tpl) {
                S cre[CH], cim[CH], crb[CH], cib[CH];
#pragma unroll
                for (int c = 0; c < CH; ++c) {
                    const int u = u0 + c * tpl;
                    cre[c] = cim[c] = crb[c] = cib[c] = S(0);
                    if (u < io.cnt_in) {
                        load_unit<S, S2>(io, base, u, cre[c], cim[c]);
                        if (has_b) load_unit<S, S2>(io, base_b, u, crb[c], cib[c]);
                    }
                }
#pragma unroll
                for (int c = 0; c < CH; ++c) {
                    const int u = u0 + c * tpl;
                    if (u >= io.cnt_in) break;
                    S re = cre[c], im = cim[c], rb = crb[c], ib = cib[c];
                    if (io.conj_in) { im = negs(im); ib = negs(ib); }
                    // general_c2r reads only the real part of the DC and Nyquist bins
                    if (io.pre != PRE_NONE && (u == 0 || (io.pre == PRE_HERM_EVEN && u == M))) { im = S(0); ib = S(0); }
                    if (scaled) {
                        if constexpr (RAW) {
                            emax = max(emax, max(dmag(re), dmag(im)));
                            emaxb = max(emaxb, max(dmag(rb), dmag(ib)));
                        } else {
                            emax = max(emax, max(fmag((float)re), fmag((float)im)));
                            emaxb = max(emaxb, max(fmag((float)rb), fmag((float)ib)));
                        }
                    }
                    if (!paired) {
                        cx<T> z{Store<T>::in(re, esc), Store<T>::in(im, esc)};
                        const bool cz = cc && io.pre != PRE_HERM_EVEN;
                        sput(line + sp(u, pad), cz ? conjx(z) : z);
                        if (io.pre == PRE_HERM_ODD && u > 0) sput(line + sp(M - u, pad), cz ? z : conjx(z));
                    } else {
                        // Z = A + i B: real lines -> (a, b); half spectra -> Z[u] = A + iB,
                        // Z[M-u] = conj(A) + i conj(B)
                        cx<T> A{Store<T>::in(re, esc), Store<T>::in(im, esc)};
                        cx<T> B{Store<T>::in(rb, escb), Store<T>::in(ib, escb)};
                        cx<T> z = cx<T>{A.r - B.i, A.i + B.r};
                        sput(line + sp(u, pad), cc ? conjx(z) : z);
                        if (io.in_kind != IN_R && u > 0) {
                            cx<T> zm = cx<T>{A.r + B.i, B.r - A.i};
                            sput(line + sp(M - u, pad), cc ? conjx(zm) : zm);
                        }
                    }
                }
                }
            }
            if (!scaled || attempt == 1) break;
            {
                const int ka = RAW ? dkey_mag(emax) : fkey_mag(emax), kb = RAW ? dkey_mag(emaxb) : fkey_mag(emaxb);
                if (act && ka > 0) atomicMax(&s_emax[2 * gi], ka);
                if (act && kb > 0) atomicMax(&s_emax[2 * gi + 1], kb);
            }
            __syncthreads();
            for (int l = threadIdx.x; l < nl; l += blockDim.x) {
                const int ea = s_emax[2 * l], eb = s_emax[2 * l + 1];  // line-scale keys
                if (RAW) {
                    // safe window: largest element within 2^+-40 (all-zero lines are safe)
                    constexpr int c = 1023 + kKeyOff;
                    if (ea != 0 && (ea > c + 40 || ea < c - 40)) { s_esc[2 * l] = c - ea; s_rescale = 1; }
                    if (paired && eb != 0 && (eb > c + 40 || eb < c - 40)) { s_esc[2 * l + 1] = c - eb; s_rescale = 1; }
                    if (paired && ea != 0 && eb != 0 && abs(ea - eb) > 8) {
                        s_esc[2 * l] = c - ea;
                        s_esc[2 * l + 1] = c - eb;
                        s_rescale = 1;
                    }
                } else if (paired && ea != 0 && eb != 0) {
                    constexpr int c = 127 + kKeyOff;
                    if (abs(ea - eb) > 8 || abs(ea - c) > 40 || abs(eb - c) > 40) {
                        s_esc[2 * l] = c - ea;
                        s_esc[2 * l + 1] = c - eb;
                        s_rescale = 1;
                    }
                }
            }
            __syncthreads();
            if (!s_rescale) break;
        }
    }
    __syncthreads();

    // ---- pre-processing: Hermitian half spectrum -> packed complex input ----
    if (LAY == LAY_GEN && io.pre == PRE_HERM_EVEN && g < nl) {
        // X[0..M] (X[M] Nyquist) -> Z[k] = (X[k] + conj(X[M-k])) + i e^{+2 pi i k/2M} (X[k] - conj(X[M-k])).
        // Each thread owns the slot pair (k, M-k): no barrier between its reads and writes.
        const cx<T> *rtw = reinterpret_cast<const cx<T> *>(P.rtw);
        for (int k = t; k <= M / 2; k += tpl) {
            const int k2 = M - k;
            cx<T> a = sget(myline + sp(k, pad)), b = sget(myline + sp(k2, pad));
            {
                cx<T> xb = conjx(b);
                cx<T> A = a + xb, Bv = a - xb;
                cx<T> tB = cmulc(Bv, rtw[k]);
                cx<T> z{A.r - tB.i, A.i + tB.r};
                sput(myline + sp(k, pad), cc ? conjx(z) : z);  // conjugated for a backward Stockham core
            }
            if (k > 0 && k2 != k) {
                cx<T> xb = conjx(a);
                cx<T> A = b + xb, Bv = b - xb;
                cx<T> tB = cmulc(Bv, rtw[k2]);
                cx<T> z{A.r - tB.i, A.i + tB.r};
                sput(myline + sp(k2, pad), cc ? conjx(z) : z);
            }
        }
    }
    if (LAY == LAY_GEN && io.pre == PRE_HERM_EVEN) __syncthreads();

    // ---- core ---------------------------------------------------------------
    // Stockham: one pass in the transform's direction.  Bluestein (fftblue_fft,
    // pocketfft.c:1945): a = x * chirp(-+), zero pad to L, FFT_L, multiply by
    // chirpf (conjugated for the backward transform), IFFT_L, multiply by chirp(-+).
    // Rader (prime M, L = M - 1; forward): a[q] = x[g^-q], A = FFT_L(a),
    // C = A * B with B = FFT_L(w^(g^m)) / L, c = IFFT_L(C) as conj(FFT_L(conj C)),
    // X[0] = x[0] + A[0], X[g^p] = x[0] + c[p].
    // Row convolution (io.rowconv; the rows of a four-step core L = N1 N2, or
    // whole lines when N1 = 1): Y = FFT_N2(row k1), C = Y * tab[k1 mul_a + u
    // mul_b] (the product of a convolution in the natural spectrum order
    // k1 + N1 k2), the inverse FFT_N2 as conj(FFT_N2(conj C)); the epilogue
    // applies the final conjugation and the inverse four-step twiddle.
    {
        const cx<T> *ch = reinterpret_cast<const cx<T> *>(P.chirp);
        const cx<T> *chf = reinterpret_cast<const cx<T> *>(P.chirpf);
        const int L = P.L;
        constexpr bool kRader = RS == RS_FULL || RS == RS_ALLR;  // Rader steps: these two classes only
        const bool blue = P.blue == 1, rader = kRader && P.blue == 2;
        const bool rowconv = RC && io.rowconv;
        const int npass = (P.blue || rowconv) ? 2 : 1;
        for (int pass = 0; pass < npass; ++pass) {
            if (blue && g < nl) {
                if (pass == 0) {
                    for (int u = t; u < L; u += tpl) {
                        cx<T> z = cx<T>{RealOps<T>::k(0.0), RealOps<T>::k(0.0)};
                        if (u < M) z = io.fwd ? cmulc(sget(myline + sp(u, pad)), ch[u]) : cmul(sget(myline + sp(u, pad)), ch[u]);
                        sput(myline + sp(u, pad), z);
                    }
                } else {
                    // backward FFT_L as conj(FFT_L(conj(.)))
                    for (int u = t; u < L; u += tpl) {
                        cx<T> z = io.fwd ? cmul(sget(myline + sp(u, pad)), chf[u]) : cmulc(sget(myline + sp(u, pad)), chf[u]);
                        sput(myline + sp(u, pad), conjx(z));
                    }
                }
            }
            if constexpr (kRader) if (rader) {
                if (pass == 0) {
                    // gather a[q] = x[rin[q]] through registers; x[0] kept at slot L + 1
                    rader_permute<T, E>(myline, P.rin, L, tpl, t, pad, g < nl, line_a + sp(L + 1, pad), nullptr, false);
                } else {
                    // A[0] to slot L; C = A B, stored conjugated
                    cx<T> a0{};
                    if (g < nl) a0 = sget(myline);
                    __syncthreads();
                    if (g < nl) {
                        if (t == 0) sput(line_a + sp(L, pad), a0);
                        if constexpr (std::is_same<T, df>::value) {
                            for (int u = t; u < L; u += tpl) {
                                cx<df> *p = myline + sp(u, pad);
                                pst(p, pconj(prenorm(pmulw_cx<false>(pld(p), chf + u, P.neg1))));
                            }
                        } else {
                            for (int u = t; u < L; u += tpl) sput(myline + sp(u, pad), conjx(cmul(sget(myline + sp(u, pad)), chf[u])));
                        }
                    }
                }
            }
            if constexpr (RC) if (rowconv && pass == 1 && g < nl) {
                const long long l = line0 + g;
                const int k1 = line_i0(io, l);
                const cx<T> *tb = reinterpret_cast<const cx<T> *>(io.mul) + (long long)k1 * io.mul_a;
                const long long mb = io.mul_b;
                // unit 0 of row 0 before the product (Rader's A[0]), by the
                // thread that owns unit 0
                if (t == 0 && io.keep0 && (io.keep0_rows == 1 || k1 == 0)) {
                    OutScale<T> sc;
                    sc.init(io);
                    const int esc = scaled ? s_esc[2 * g] : 0;
                    const cx<T> z = sget(myline);
                    S2 o;
                    o.x = sc.apply(z.r, esc);
                    o.y = sc.apply(z.i, esc);
                    reinterpret_cast<S2 *>(io.keep0)[io.keep0_rows == 1 ? l : (long long)fdiv((unsigned)l, io.fb0)] = o;
                }
                bool done = false;
                if constexpr (std::is_same<T, df>::value) {
                    if (!io.mul_conj) {
                        for (int u = t; u < L; u += tpl) {
                            cx<df> *p = myline + sp(u, pad);
                            pst(p, pconj(prenorm(pmulw_cx<false>(pld(p), tb + (long long)u * mb, P.neg1))));
                        }
                        done = true;
                    }
                }
                if (!done)
                    for (int u = t; u < L; u += tpl) {
                        const cx<T> z = sget(myline + sp(u, pad)), w = tb[(long long)u * mb];
                        sput(myline + sp(u, pad), conjx(io.mul_conj ? cmulc(z, w) : cmul(z, w)));
                    }
            }
            if (P.blue || rowconv) __syncthreads();
            if constexpr (DB) {
                cur = run_stages_db<T, E, RS>(sm, cur, P, nl, tpl, g, t, LSt);
                myline = line_a + cur;
            } else {
                run_stages<T, E, RS>(sm, P, nl, tpl, g, t, LSt);
            }
        }
        if (blue) {
            if (g < nl)
                for (int u = t; u < M; u += tpl) {
                    cx<T> z = conjx(sget(myline + sp(u, pad)));
                    sput(myline + sp(u, pad), io.fwd ? cmulc(z, ch[u]) : cmul(z, ch[u]));
                }
            __syncthreads();
        }
        if constexpr (kRader)
            if (rader)
                rader_permute<T, E>(myline, P.rout, L, tpl, t, pad, g < nl, line_a + sp(L + 1, pad),
                                    line_a + sp(L, pad), true);
    }

    // ---- post-processing: real split ------------------------------------------
    const bool post_split = LAY == LAY_R2HC || (LAY == LAY_GEN && io.post == POST_SPLIT);
    const bool post_pair = LAY == LAY_PR2HC || (LAY == LAY_GEN && io.post == POST_PAIR);
    if (post_split && g < nl) {
        // Z = FFT_M(x_even + i x_odd) -> X[k] = E_k + w^k O_k, k = 0..M,
        // E_k = (Z[k] + conj(Z[M-k]))/2, O_k = -i (Z[k] - conj(Z[M-k]))/2, w = e^{-2 pi i/2M};
        // thread-owned slot pairs (k, M-k), slot M receives X[M]
        const cx<T> *rtw = reinterpret_cast<const cx<T> *>(P.rtw);
        if constexpr (std::is_same<T, df>::value) {
            // packed pairs (re, im): X = (a + conj b)/2 + w (-i) (a - conj b)/2
            const f2p half = bcast(0.5f), cj = pk(1.0f, -1.0f);
            for (int k = t; k <= M / 2; k += tpl) {
                const int k2 = M - k;
                const pcx a = pld(myline + sp(k, pad)), b = pld(myline + sp(k == 0 ? 0 : k2, pad));
                {
                    const pcx zb = plane(b, cj);
                    const pcx Ev = plane(a + zb, half), D = plane(a - zb, half);
                    pst(myline + sp(k, pad), prenorm(Ev + pmulw_cx<false>(prot<true>(D), rtw + k, P.neg1)));
                }
                if (k2 != k) {
                    const pcx za = plane(a, cj);
                    const pcx Ev = plane(b + za, half), D = plane(b - za, half);
                    pst(myline + sp(k2, pad), prenorm(Ev + pmulw_cx<false>(prot<true>(D), rtw + k2, P.neg1)));
                }
            }
        } else {
            for (int k = t; k <= M / 2; k += tpl) {
                const int k2 = M - k;
                cx<T> a = sget(myline + sp(k, pad)), b = sget(myline + sp(k == 0 ? 0 : k2, pad));
                {
                    cx<T> zb = conjx(b);
                    cx<T> Ev = chalf(a + zb), D = chalf(a - zb);
                    sput(myline + sp(k, pad), crenorm(Ev + cmul(cx<T>{D.i, -D.r}, rtw[k])));
                }
                if (k2 != k) {
                    cx<T> zb = conjx(a);
                    cx<T> Ev = chalf(b + zb), D = chalf(b - zb);
                    sput(myline + sp(k2, pad), crenorm(Ev + cmul(cx<T>{D.i, -D.r}, rtw[k2])));
                }
            }
        }
    }
    if (post_split) __syncthreads();
    if (post_pair && g < nl) {
        // Z = FFT(a + i b) -> A[k] = (Z[k] + conj(Z[M-k]))/2 at slot k,
        // B[k] = -i (Z[k] - conj(Z[M-k]))/2 at slot M-k; slot 0 keeps (A[0], B[0])
        if constexpr (std::is_same<T, df>::value) {
            const f2p half = bcast(0.5f), cj = pk(1.0f, -1.0f);
            for (int k = 1 + t; 2 * k < M + 1; k += tpl) {
                const int k2 = M - k;
                const pcx a = pld(myline + sp(k, pad)), b = plane(pld(myline + sp(k2, pad)), cj);
                pst(myline + sp(k, pad), prenorm(plane(a + b, half)));
                pst(myline + sp(k2, pad), prenorm(prot<true>(plane(a - b, half))));
            }
        } else {
            for (int k = 1 + t; 2 * k < M + 1; k += tpl) {
                const int k2 = M - k;
                cx<T> a = sget(myline + sp(k, pad)), b = conjx(sget(myline + sp(k2, pad)));
                cx<T> A = chalf(a + b), D = chalf(a - b);
                sput(myline + sp(k, pad), crenorm(A));
                sput(myline + sp(k2, pad), crenorm(cx<T>{D.i, -D.r}));
            }
        }
    }
    if (post_pair) __syncthreads();

    // ---- fused real split of a four-step second pass (POST_SPLIT4) --------------
    // pair q = lines (2q, 2q + 1) = rows (r, N1 - r) (split_row); element u of row r is
    // Z[k], k = r + N1 u, and Z[M - k] sits in the mirror row at N2 - 1 - u
    // (row 0: at N2 - u).  Both rows come to the smaller of their two range
    // scales; X[k] and X[M - k] are written as halfcomplex.
    if constexpr (LAY == LAY_GEN || LAY == LAY_C2C) {
        if (io.post == POST_SPLIT4) {
            const int N2 = io.cnt_in, N1 = io.split_N1;
            const long long Mt = (long long)N1 * N2;
            const int npairs = nl >> 1;
            const cx<T> *rtw = reinterpret_cast<const cx<T> *>(io.split_tw);
            OutScale<T> sc;
            sc.init(io);
            // element i = q + npairs u, rows fastest (consecutive outputs); the
            // walk steps (q, u) by blockDim.x without a division per element
            const int dq = (int)(blockDim.x % (unsigned)npairs), du = (int)(blockDim.x / (unsigned)npairs);
            int q = (int)(threadIdx.x % (unsigned)npairs), u = (int)(threadIdx.x / (unsigned)npairs);
            for (; u < N2;) {
                const int ga = 2 * q, gb = ga + 1;
                const long long la = line0 + ga;
                const int ja = line_i0(io, la);
                const int ra = split_row(ja, N1), rb = split_row(ja + 1, N1);
                const int u2 = ra == 0 ? (u == 0 ? 0 : N2 - u) : N2 - 1 - u;
                if (ra != rb || u <= u2) {
                    cx<T> a = sget(sm + (size_t)ga * LSt + cur + sp(u, pad));
                    cx<T> b = sget(sm + (size_t)gb * LSt + cur + sp(u2, pad));
                    int ec = 0;
                    if (scaled) {
                        const int ea = s_esc[2 * ga], eb = s_esc[2 * gb];
                        ec = min(ea, eb);
                        if (ea != ec) a = cscale_pow2(a, ec - ea);
                        if (eb != ec) b = cscale_pow2(b, ec - eb);
                    }
                    const long long k = ra + (long long)N1 * u, km = Mt - k;
                    char *base = io.out + line_off(io, la, true);
                    auto split_store = [&](cx<T> za, cx<T> zb, long long kk) {
                        cx<T> X;
                        if constexpr (std::is_same<T, df>::value) {
                            // packed pairs (re, im), as the in-CTA real split
                            const f2p half = bcast(0.5f), cj = pk(1.0f, -1.0f);
                            const pcx pa = to_p(za), pc = plane(to_p(zb), cj);
                            const pcx Ev = plane(pa + pc, half), D = plane(pa - pc, half);
                            X = from_p(prenorm(Ev + pmulw_cx<false>(prot<true>(D), rtw + kk, P.neg1)));
                        } else {
                            const cx<T> zc = conjx(zb);
                            const cx<T> Ev = chalf(za + zc), D = chalf(za - zc);
                            X = crenorm(Ev + cmul(cx<T>{D.i, -D.r}, rtw[kk]));
                        }
                        if (kk == 0) {
                            stg_s<S>(base, sc.apply(X.r, ec));
                        } else if (kk == Mt) {
                            stg_s<S>(base + (2 * Mt - 1) * io.os, sc.apply(X.r, ec));
                        } else {
                            char *p = base + (2 * kk - 1) * io.os;
                            stg_s<S>(p, sc.apply(X.r, ec));
                            stg_s<S>(p + io.os, sc.apply(X.i, ec));
                        }
                    };
                    split_store(a, b, k);
                    if (km != k) split_store(b, a, km);
                }
                q += dq;
                u += du;
                if (q >= npairs) { q -= npairs; ++u; }
            }
            return;
        }
    }

    // ---- epilogue: shared memory -> HBM ---------------------------------------
    {
        int g2, t2;
        if (io.cols_out) { g2 = threadIdx.x % lpc; t2 = threadIdx.x / lpc; }
        else { g2 = g; t2 = t; }
        if (g2 < nl && t2 < tpl) {
            OutScale<T> sc;
            sc.init(io);
            const int esc = scaled ? s_esc[2 * g2] : 0;
            const int escb = scaled ? s_esc[2 * g2 + 1] : 0;
            const long long l = line0 + g2;
            char *base = out_base + line_off(io, l, true);
            const cx<T> *line = sm + (size_t)g2 * LSt + cur;
            const int i0l = (io.tw4 || io.mul || io.keep0 || paired) ? line_i0(io, l) : 0;
            const bool has_b = paired && (2LL * i0l + 1 < io.pair_n0);
            const int n2 = io.tw4 ? (io.tw4_dim1 ? line_i1(io, l) : i0l) : 0;
            const int ml = io.mul ? (int)(i0l * io.mul_a) : 0;
            const cx<T> *whi = reinterpret_cast<const cx<T> *>(io.tw4hi);
            const cx<T> *wlo = reinterpret_cast<const cx<T> *>(io.tw4lo);
            const cx<T> *mt = reinterpret_cast<const cx<T> *>(io.mul);
            const cx<T> z0 = paired ? sget(line + 0) : cx<T>{};
            constexpr T zero = RealOps<T>::k(0.0);
            if constexpr (LAY == LAY_C2C) {
                const int cnt = io.cnt_out;
                const long long os = io.os;
                for (int u = t2; u < cnt; u += tpl) {
                    cx<T> z = sget(line + sp(u, pad));
                    if (cc) z.i = -z.i;
                    S2 o;
                    o.x = sc.apply(z.r, esc);
                    o.y = sc.apply(z.i, esc);
                    stg_s<S2>(base + (long long)u * os, o);
                }
                return;
            }
            if constexpr (LAY == LAY_R2HC) {
                const int cnt = io.cnt_out;
                const long long os = io.os, nreal = io.nreal;
                for (int u = t2; u < cnt; u += tpl) {
                    const cx<T> z = sget(line + sp(u, pad));
                    if (u == 0) {
                        stg_s<S>(base, sc.apply(z.r, esc));
                    } else {
                        char *p = base + (2 * (long long)u - 1) * os;
                        stg_s<S>(p, sc.apply(z.r, esc));
                        if (2 * (long long)u < nreal) stg_s<S>(p + os, sc.apply(z.i, esc));
                    }
                }
                return;
            }
            if constexpr (LAY == LAY_TW || LAY == LAY_RC) {
                // complex units out (the layout class guarantees it), with the
                // four-step twiddle and / or the pointwise table product; the
                // output pointer and the table rows advance by one add per unit
                const int cnt = io.cnt_out;
                const long long os = io.os, pstep = (long long)tpl * os;
                // row convolution: the product and unit 0 were taken between
                // the passes; here the final conjugation and the inverse twiddle
                const bool rc = RC && io.rowconv;
                const auto *wrow = io.tw4 && io.tw4tab
                                       ? reinterpret_cast<const typename Bfly<T>::W *>(io.tw4tab) + (size_t)n2 * cnt
                                       : nullptr;
                const cx<T> *mrow = io.mul && !rc ? mt + ml : nullptr;
                const long long mb = io.mul_b;
                const bool twf = io.fwd && !rc;
                char *p = base + (long long)t2 * os;
                for (int u = t2; u < cnt; u += tpl, p += pstep) {
                    cx<T> z = sget(line + sp(u, pad));
                    if (cc || rc) z.i = -z.i;
                    if (wrow) {
                        z = tw_apply<T>(z, wrow + u, twf, P);
                    } else if (io.tw4) {
                        const unsigned tt = (unsigned)n2 * (unsigned)u;
                        const unsigned hi = fdiv(tt, io.fdS), lo = tt - hi * (unsigned)io.tw4S;
                        const cx<T> w = cmul(whi[hi], wlo[lo]);
                        z = twf ? cmul(z, w) : cmulc(z, w);
                    }
                    if (io.keep0 && !rc && u == 0 && (io.keep0_rows == 1 || i0l == 0)) {
                        S2 o;
                        o.x = sc.apply(z.r, esc);
                        o.y = sc.apply(z.i, esc);
                        reinterpret_cast<S2 *>(io.keep0)[io.keep0_rows == 1 ? l : (long long)fdiv((unsigned)l, io.fb0)] =
                            o;
                    }
                    if (mrow) {
                        const cx<T> w = mrow[(long long)u * mb];
                        z = io.mul_conj ? cmulc(z, w) : cmul(z, w);
                    }
                    S2 o;
                    o.x = sc.apply(z.r, esc);
                    o.y = sc.apply(z.i, esc);
                    stg_s<S2>(p, o);
                }
                return;
            }
            if constexpr (LAY == LAY_PR2HC) {
                const int cnt = io.cnt_out;
                const long long os = io.os, nreal = io.nreal, po = io.pair_out;
                for (int u = t2; u < cnt; u += tpl) {
                    const cx<T> za = u == 0 ? cx<T>{z0.r, zero} : sget(line + sp(u, pad));
                    const cx<T> zb = u == 0 ? cx<T>{z0.i, zero} : sget(line + sp(M - u, pad));
                    if (u == 0) {
                        stg_s<S>(base, sc.apply(za.r, esc));
                        if (has_b) stg_s<S>(base + po, sc.apply(zb.r, escb));
                    } else {
                        char *p = base + (2 * (long long)u - 1) * os;
                        stg_s<S>(p, sc.apply(za.r, esc));
                        if (has_b) stg_s<S>(p + po, sc.apply(zb.r, escb));
                        if (2 * (long long)u < nreal) {
                            stg_s<S>(p + os, sc.apply(za.i, esc));
                            if (has_b) stg_s<S>(p + os + po, sc.apply(zb.i, escb));
                        }
                    }
                }
                return;
            }
            for (int u = t2; u < io.cnt_out; u += tpl) {
                if (paired) {
                    if (io.out_kind == OUT_R) {
                        cx<T> z = sget(line + sp(u, pad));
                        if (cc) z.i = -z.i;
                        stg_s<S>(base + (long long)u * io.os, sc.apply(z.r, esc));
                        if (has_b) stg_s<S>(base + io.pair_out + (long long)u * io.os, sc.apply(z.i, escb));
                    } else {
                        cx<T> za = u == 0 ? cx<T>{z0.r, zero} : sget(line + sp(u, pad));
                        cx<T> zb = u == 0 ? cx<T>{z0.i, zero} : sget(line + sp(M - u, pad));
                        if (io.conj_out) { za.i = -za.i; zb.i = -zb.i; }
                        store_unit<T, S, S2>(io, base, u, za, sc, esc);
                        if (has_b) store_unit<T, S, S2>(io, base + io.pair_out, u, zb, sc, escb);
                    }
                    continue;
                }
                cx<T> z = sget(line + sp(u, pad));
                if (cc) z.i = -z.i;
                if (io.tw4 && io.tw4tab) {
                    // full table, row n2: w^(n2 u)
                    const auto *w = reinterpret_cast<const typename Bfly<T>::W *>(io.tw4tab) + (size_t)n2 * io.cnt_out + u;
                    z = tw_apply<T>(z, w, io.fwd, P);
                } else if (io.tw4) {
                    // t = n2 u < M: w^t = w_hi[t / S] * w_lo[t mod S]
                    const unsigned tt = (unsigned)n2 * (unsigned)u;
                    const unsigned hi = fdiv(tt, io.fdS), lo = tt - hi * (unsigned)io.tw4S;
                    cx<T> w = cmul(whi[hi], wlo[lo]);
                    z = io.fwd ? cmul(z, w) : cmulc(z, w);
                }
                if (io.keep0 && u == 0 && (io.keep0_rows == 1 || i0l == 0)) {
                    // the transform's unit 0 before the product (Rader's A[0])
                    S2 o;
                    o.x = sc.apply(z.r, esc);
                    o.y = sc.apply(z.i, esc);
                    reinterpret_cast<S2 *>(io.keep0)[io.keep0_rows == 1 ? l : (long long)fdiv((unsigned)l, io.fb0)] = o;
                }
                if (io.mul) {
                    cx<T> w = mt[ml + (long long)u * io.mul_b];
                    z = io.mul_conj ? cmulc(z, w) : cmul(z, w);
                }
                if (io.conj_out) z.i = -z.i;
                // general_r2c stores the DC and Nyquist bins with a zero imaginary part
                if (io.real_out && (u == 0 || (io.post == POST_SPLIT && u == M))) z.i = zero;
                store_unit<T, S, S2>(io, base, u, z, sc, esc);
            }
        }
    }
}

// register caps of the shared-memory kernel: the double-buffered 8-element
// variants hold one butterfly at a time and fit without spills in fewer
// registers, which lets three 256-thread CTAs share an SM
template <class T, int E, int RS, bool DB> constexpr int fft_smem_regs()
{
    if constexpr (DB && E == 8 && std::is_same<T, df>::value) return RS == RS_FULL ? 96 : 80;
    if constexpr (DB && E == 8 && std::is_same<T, float>::value) return 80;
    // FP32 16-element double-buffered lines (4097-8192 points) fit 64 registers
    // without spills below the full class: two 512-thread CTAs per SM
    if constexpr (DB && E == 16 && std::is_same<T, float>::value) return RS == RS_FULL ? 128 : 64;
    return 128;
}

// NT: the launch bound (kMaxThreadsE8 for the wide double-float variants)
template <class T, int E, int RS, int LAY, bool DB, int NT = 512>
__global__ void __launch_bounds__(NT) __maxnreg__((fft_smem_regs<T, E, RS, DB>()))
    k_fft_smem(const __grid_constant__ CoreDesc P, const __grid_constant__ IODesc io)
{
    fft_block<T, E, RS, LAY, DB>(P, io, blockIdx.x, io.in, io.out);
}

// Persistent kernel over a device work list: item w is block (w - prefix[g])
// of group g (binary search on prefix).  Groups hold their own core and line
// descriptors; their in/out pointers are byte offsets from one of three
// bases (0: input, 1: output, 2: scratch).  Items are claimed with one
// atomic per block; the counter is reset before every launch.  One
// instantiation per shared-memory kernel variant (elements per thread,
// buffering, radix class, layout class): the host partitions the groups by
// the variant their core and layout ask for and launches each partition with
// as many CTAs as the occupancy calculator allows.
template <class T, int E, int RS, int LAY, bool DB>
__global__ void __launch_bounds__(512) __maxnreg__((fft_smem_regs<T, E, RS, DB>()))
    k_fft_worklist(const WorkGroup *__restrict__ groups, const long long *__restrict__ prefix, int ngroups,
                   unsigned long long total, unsigned long long *counter, const char *in, char *out, char *scr)
{
    __shared__ unsigned long long s_item;
    __shared__ int s_group;
    if (threadIdx.x == 0) s_group = 0;
    for (;;) {
        if (threadIdx.x == 0) {
            const unsigned long long w = atomicAdd(counter, 1ull);
            s_item = w;
            // a CTA's claims increase, so its group index only moves forward:
            // gallop from the previous group, then bisect (no full search of
            // dependent loads per item)
            if (w < total) {
                int lo = s_group, step = 1, hi = lo;
                while (hi + 1 < ngroups && (unsigned long long)prefix[hi + 1] <= w) {
                    lo = hi + 1;
                    hi = min(ngroups - 1, hi + step);
                    step <<= 1;
                }
                if ((unsigned long long)prefix[hi] > w) --hi;
                while (lo < hi) {
                    const int mid = (lo + hi + 1) >> 1;
                    if ((unsigned long long)prefix[mid] <= w) lo = mid;
                    else hi = mid - 1;
                }
                s_group = lo;
            }
        }
        __syncthreads();
        const unsigned long long w = s_item;
        const int lo = s_group;
        __syncthreads();
        if (w >= total) break;
        const WorkGroup &G = groups[lo];
        const char *ib = G.in_base == 0 ? in : G.in_base == 1 ? (const char *)out : (const char *)scr;
        char *ob = G.out_base == 1 ? out : G.out_base == 2 ? scr : (char *)in;
        fft_block<T, E, RS, LAY, DB, false>(G.P, G.io, (long long)(w - (unsigned long long)prefix[lo]),
                                     ib + (size_t)G.io.in, ob + (size_t)G.io.out);
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// elementwise line maps of the multi-pass paths
// ---------------------------------------------------------------------------

// double-float helpers with a shared power-of-two scale per small group of
// values (exact), so that elementwise steps keep ~48-bit accuracy for any
// finite magnitude without FP64 arithmetic
template <class T> struct Loc {
    int esc = 0;
    __device__ void fit(double a, double b, double c = 0.0, double d = 0.0) {}
    __device__ cx<T> in(double re, double im) const { return cx<T>{(T)re, (T)im}; }
    __device__ double out(T v) const { return (double)v; }
};
template <> struct Loc<df> {
    int esc = 0;
    __device__ void fit(double a, double b, double c = 0.0, double d = 0.0)
    {
        const int e = dkey_mag(max(max(dmag(a), dmag(b)), max(dmag(c), dmag(d))));
        esc = e > 0 ? 1023 + kKeyOff - e : 0;
    }
    __device__ cx<df> in(double re, double im) const { return cx<df>{df_from_double(re, esc), df_from_double(im, esc)}; }
    __device__ double out(df v) const { return df_to_double(v, esc); }
};

// conversions with an explicit power-of-two exponent (double-float) or plain casts
template <class T> struct Loc2 {
    __device__ static T in(double v) { return (T)v; }
    __device__ static double out(T v, int) { return (double)v; }
};
template <> struct Loc2<df> {
    __device__ static df in(double v) { return df_from_double(v, 0); }
    __device__ static double out(df v, int esc) { return df_to_double(v, esc); }
};

// read unit u of the user-facing input line at `base` (kinds of IODesc)
template <class S, class S2>
__device__ __forceinline__ void read_unit(const IODesc &io, const char *base, long long u, double &re, double &im)
{
    if (io.in_kind == IN_C) {
        S2 z = ldg_s<S2>(base + u * io.is);
        re = z.x; im = z.y;
    } else if (io.in_kind == IN_R) {
        re = ldg_s<S>(base + u * io.is);
        im = 0;
    } else if (io.in_kind == IN_P) {
        re = ldg_s<S>(base + u * io.is);
        im = ldg_s<S>(base + u * io.is + io.ps_in);
    } else {
        if (u == 0) { re = ldg_s<S>(base); im = 0; }
        else {
            re = ldg_s<S>(base + (2 * u - 1) * io.is);
            im = (2 * u < io.nreal) ? (double)ldg_s<S>(base + (2 * u) * io.is) : 0.0;
        }
    }
    if (io.conj_in) im = -im;
}

// gather: user input -> scratch lines (one thread per scratch element)
template <class T>
__global__ void k_gather(const __grid_constant__ IODesc io, const __grid_constant__ MapDesc mp)
{
    using S = typename Traits<T>::S;
    using S2 = typename Traits<T>::S2;
    const long long total = io.nlines * mp.scr_len;
    for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x) {
        long long l = qdiv(idx, mp.scr_len, mp.fsl), u = idx - l * mp.scr_len;
        const char *base = io.in + line_off(io, l, false);
        S2 *dst = reinterpret_cast<S2 *>(mp.scr) + l * mp.scr_len + u;
        double re = 0, im = 0;
        if (mp.kind == MAP_HERM_EVEN) {
            // Z[k] = (X[k] + conj(X[M-k])) + i e^{+2 pi i k/2M} (X[k] - conj(X[M-k])), k < M
            if (u >= mp.M) continue;
            double ar, ai, br, bi;
            read_unit<S, S2>(io, base, u, ar, ai);
            read_unit<S, S2>(io, base, mp.M - u, br, bi);
            if (u == 0) ai = 0;
            if (mp.M - u == mp.M || mp.M - u == 0) bi = 0;
            Loc<T> lc;
            lc.fit(ar, ai, br, bi);
            cx<T> xa = lc.in(ar, ai), xb = lc.in(br, -bi);
            cx<T> A = xa + xb, Bv = xa - xb;
            cx<T> w = conjx(reinterpret_cast<const cx<T> *>(mp.rtw)[u]);
            cx<T> tB = cmul(Bv, w);
            cx<T> z = cx<T>{A.r - tB.i, A.i + tB.r};
            S2 o;
            o.x = (S)lc.out(z.r);
            o.y = (S)lc.out(z.i);
            *dst = o;
            continue;
        }
        long long cnt = io.cnt_in;
        auto read_z = [&](long long v, double &zr, double &zi) {
            long long uu = v;
            bool cj = false;
            zr = zi = 0;
            if (io.pre == PRE_HERM_ODD && v >= cnt) { uu = mp.M - v; cj = true; }
            if (uu < cnt) {
                read_unit<S, S2>(io, base, uu, zr, zi);
                if (io.pre != PRE_NONE && uu == 0) zi = 0;
                if (cj) zi = -zi;
            }
        };
        if (mp.kind == MAP_RADER) {
            // a[q] = x[g^-q]; x[0] kept per line (conjugated for the backward direction)
            read_z(mp.ridx[u], re, im);
            if (!mp.fwd) im = -im;
            if (u == 0) {
                double r0, i0;
                read_z(0, r0, i0);
                S2 o0;
                o0.x = (S)r0;
                o0.y = (S)(mp.fwd ? i0 : -i0);
                reinterpret_cast<S2 *>(mp.x0buf)[l] = o0;
            }
        } else if (u < mp.M) {
            read_z(u, re, im);
        }
        if (mp.kind == MAP_BLUE) {
            if (u < mp.M) {
                Loc<T> lc;
                lc.fit(re, im);
                cx<T> x = lc.in(re, im);
                cx<T> c = reinterpret_cast<const cx<T> *>(mp.chirp)[u];
                x = mp.fwd ? cmulc(x, c) : cmul(x, c);
                re = lc.out(x.r);
                im = lc.out(x.i);
            } else {
                re = im = 0;
            }
        }
        S2 o;
        o.x = (S)re;
        o.y = (S)im;
        *dst = o;
    }
}

// scatter: scratch lines -> user output (one thread per output unit)
template <class T>
__global__ void k_scatter(const __grid_constant__ IODesc io, const __grid_constant__ MapDesc mp)
{
    using S = typename Traits<T>::S;
    using S2 = typename Traits<T>::S2;
    const long long cnt = io.cnt_out;
    const long long total = io.nlines * cnt;
    OutScale<T> sc;
    sc.init(io);
    for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x) {
        long long l = qdiv(idx, cnt, mp.fcnt), u = idx - l * cnt;
        char *base = io.out + line_off(io, l, true);
        const S2 *src = reinterpret_cast<const S2 *>(mp.scr) + l * mp.scr_len;
        cx<T> z;
        Loc<T> lc;
        if (mp.kind == MAP_SPLIT_EVEN) {
            // X[k] = E_k + w^k O_k from Z[k], Z[M-k] (k <= M, Z[M] = Z[0])
            long long M = mp.M;
            S2 a = src[u == M ? 0 : u], b = src[u == 0 ? 0 : M - u];
            lc.fit(a.x, a.y, b.x, b.y);
            cx<T> za = lc.in(a.x, a.y), zb = conjx(lc.in(b.x, b.y));
            cx<T> E = chalf(za + zb);
            cx<T> D = chalf(za - zb);
            cx<T> O = cx<T>{D.i, -D.r};
            z = E + cmul(O, reinterpret_cast<const cx<T> *>(mp.rtw)[u]);
        } else if (mp.kind == MAP_RADER) {
            // X[0] = x0 + A0, X[u] = x0 + c[log_g u]
            const S2 x0 = reinterpret_cast<const S2 *>(mp.x0buf)[l];
            const S2 a = u == 0 ? reinterpret_cast<const S2 *>(mp.a0buf)[l] : src[mp.ridx[u]];
            lc.fit(a.x, a.y, x0.x, x0.y);
            z = crenorm(lc.in(a.x, a.y) + lc.in(x0.x, x0.y));
            if (!mp.fwd) z = conjx(z);
        } else {
            S2 a = src[u];
            lc.fit(a.x, a.y);
            z = lc.in(a.x, a.y);
            if (mp.kind == MAP_BLUE) {
                cx<T> c = reinterpret_cast<const cx<T> *>(mp.chirp)[u];
                z = mp.fwd ? cmulc(z, c) : cmul(z, c);
            }
        }
        if (io.conj_out) z.i = -z.i;
        if (io.real_out && (u == 0 || (mp.kind == MAP_SPLIT_EVEN && u == mp.M))) z.i = RealOps<T>::k(0.0);
        // OutScale folds the group's scale back in: esc of the output conversion
        const int esc = lc.esc;
        if (io.out_kind == OUT_C) {
            S2 o;
            o.x = sc.apply(z.r, esc);
            o.y = sc.apply(z.i, esc);
            stg_s<S2>(base + u * io.os, o);
        } else if (io.out_kind == OUT_R) {
            stg_s<S>(base + u * io.os, sc.apply(z.r, esc));
        } else if (io.out_kind == OUT_P) {
            stg_s<S>(base + u * io.os, sc.apply(z.r, esc));
            stg_s<S>(base + u * io.os + io.ps_out, sc.apply(z.i, esc));
        } else {
            if (u == 0) stg_s<S>(base, sc.apply(z.r, esc));
            else {
                stg_s<S>(base + (2 * u - 1) * io.os, sc.apply(z.r, esc));
                if (2 * u < io.nreal) stg_s<S>(base + (2 * u) * io.os, sc.apply(z.i, esc));
            }
        }
    }
}

// ---------------------------------------------------------------------------
// two real lines per complex line on the multi-pass paths
// ---------------------------------------------------------------------------

// exponent scale of each real line of a pair: the largest element of every
// line is brought to [1, 2) (double-float) or near 1 (FP32) by 2^esc, so that
// both lines of a pair keep their own relative accuracy
template <class T>
__global__ void k_line_exp(const __grid_constant__ IODesc io, int *__restrict__ esc)
{
    using S = typename Traits<T>::S;
    using S2 = typename Traits<T>::S2;
    __shared__ int s_e[2];
    if (threadIdx.x < 2) s_e[threadIdx.x] = 0;
    __syncthreads();
    const long long l = blockIdx.x;
    const char *base = io.in + line_off(io, l, false);
    const bool has_b = 2LL * line_i0(io, l) + 1 < io.pair_n0;
    unsigned ma = 0, mb = 0;
    for (int u = threadIdx.x; u < io.cnt_in; u += blockDim.x) {
        S re, im, rb = S(0), ib = S(0);
        load_unit<S, S2>(io, base, u, re, im);
        if (has_b) load_unit<S, S2>(io, base + io.pair_in, u, rb, ib);
        if constexpr (sizeof(S) == 8) {
            ma = max(ma, max(dmag((double)re), dmag((double)im)));
            mb = max(mb, max(dmag((double)rb), dmag((double)ib)));
        } else {
            ma = max(ma, max(fmag((float)re), fmag((float)im)));
            mb = max(mb, max(fmag((float)rb), fmag((float)ib)));
        }
    }
    const int ea = sizeof(S) == 8 ? dkey_mag(ma) : fkey_mag(ma), eb = sizeof(S) == 8 ? dkey_mag(mb) : fkey_mag(mb);
    if (ea) atomicMax(&s_e[0], ea);
    if (eb) atomicMax(&s_e[1], eb);
    __syncthreads();
    if (threadIdx.x == 0) {
        const int c = (sizeof(S) == 8 ? 1023 : 127) + kKeyOff;
        esc[2 * l] = s_e[0] ? c - s_e[0] : 0;
        esc[2 * l + 1] = s_e[1] ? c - s_e[1] : 0;
    }
}

// gather of pairs: Z[u] = 2^ea A[u] + i 2^eb B[u] for real lines; for half
// spectra Z[u] = A + iB (u < cnt), Z[u] = conj(A[M-u]) + i conj(B[M-u]) above;
// times the chirp for MAP_BLUE; zero padded to scr_len
template <class T>
__global__ void k_gather_pair(const __grid_constant__ IODesc io, const __grid_constant__ MapDesc mp,
                              const int *__restrict__ esc)
{
    using S = typename Traits<T>::S;
    using S2 = typename Traits<T>::S2;
    const long long total = io.nlines * mp.scr_len;
    for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x) {
        const long long l = qdiv(idx, mp.scr_len, mp.fsl), u = idx - l * mp.scr_len;
        S2 *dst = reinterpret_cast<S2 *>(mp.scr) + idx;
        cx<T> z{RealOps<T>::k(0.0), RealOps<T>::k(0.0)};
        const char *base = io.in + line_off(io, l, false);
        const bool has_b = 2LL * line_i0(io, l) + 1 < io.pair_n0;
        const int ea = esc[2 * l], eb = esc[2 * l + 1];
        if constexpr (std::is_same<T, df>::value) {
            // real lines into plain or Rader order: the pair (2^ea a, 2^eb b) is an
            // exact rescale of the stored doubles (no double-float round trip)
            if (io.in_kind == IN_R && !io.conj_in && (mp.kind == MAP_RADER || mp.kind == MAP_PLAIN)) {
                const bool neg_b = mp.kind == MAP_RADER && !mp.fwd;  // conjugated for the backward direction
                auto rz = [&](long long v) {
                    const double a = ldg_s<double>(base + v * io.is);
                    const double b = has_b ? ldg_s<double>(base + io.pair_in + v * io.is) : 0.0;
                    const double sb = pow2_scale(b, eb);
                    return make_double2(pow2_scale(a, ea), neg_b ? dneg(sb) : sb);
                };
                if (mp.kind == MAP_RADER) {
                    *dst = rz(mp.ridx[u]);
                    if (u == 0) reinterpret_cast<double2 *>(mp.x0buf)[l] = rz(0);
                } else {
                    *dst = u < mp.M ? rz(u) : make_double2(0.0, 0.0);
                }
                continue;
            }
        }
        // Z at logical index v of the complex line
        auto zat = [&](long long v) {
            const bool mirror = io.in_kind != IN_R && v >= io.cnt_in;
            const int uu = (int)(mirror ? mp.M - v : v);
            S ar, ai, br = S(0), bi = S(0);
            load_unit<S, S2>(io, base, uu, ar, ai);
            if (has_b) load_unit<S, S2>(io, base + io.pair_in, uu, br, bi);
            if (io.conj_in) { ai = negs(ai); bi = negs(bi); }
            if (io.in_kind != IN_R && uu == 0) { ai = S(0); bi = S(0); }
            cx<T> A{Store<T>::in(ar, ea), Store<T>::in(ai, ea)};
            cx<T> B{Store<T>::in(br, eb), Store<T>::in(bi, eb)};
            if (io.in_kind == IN_R) return cx<T>{A.r, B.r};
            if (!mirror) return cx<T>{A.r - B.i, A.i + B.r};
            return cx<T>{A.r + B.i, B.r - A.i};
        };
        if (mp.kind == MAP_RADER) {
            z = zat(mp.ridx[u]);
            if (!mp.fwd) z = conjx(z);
            if (u == 0) {
                cx<T> z0 = zat(0);
                if (!mp.fwd) z0 = conjx(z0);
                S2 o0;
                o0.x = (S)Loc2<T>::out(crenorm(z0).r, 0);
                o0.y = (S)Loc2<T>::out(crenorm(z0).i, 0);
                reinterpret_cast<S2 *>(mp.x0buf)[l] = o0;
            }
        } else if (u < mp.M) {
            z = zat(u);
            if (mp.kind == MAP_BLUE) {
                cx<T> c = reinterpret_cast<const cx<T> *>(mp.chirp)[u];
                z = mp.fwd ? cmulc(z, c) : cmul(z, c);
            }
        }
        S2 o;
        o.x = (S)Loc2<T>::out(crenorm(z).r, 0);
        o.y = (S)Loc2<T>::out(crenorm(z).i, 0);
        *dst = o;
    }
}

// scatter of pairs: forward -> A[k] = (Z[k] + conj(Z[M-k]))/2 to line a,
// B[k] = -i (Z[k] - conj(Z[M-k]))/2 to line b; backward (OUT_R) -> Re Z to a,
// Im Z to b; chirp first for MAP_BLUE; each line unscaled by its own 2^-esc
template <class T>
__global__ void k_scatter_pair(const __grid_constant__ IODesc io, const __grid_constant__ MapDesc mp,
                               const int *__restrict__ esc)
{
    using S = typename Traits<T>::S;
    using S2 = typename Traits<T>::S2;
    const long long cnt = io.cnt_out;
    const long long total = io.nlines * cnt;
    OutScale<T> sc;
    sc.init(io);
    for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x) {
        const long long l = qdiv(idx, cnt, mp.fcnt);
        const int u = (int)(idx - l * cnt);
        char *base = io.out + line_off(io, l, true);
        const bool has_b = 2LL * line_i0(io, l) + 1 < io.pair_n0;
        const int ea = esc[2 * l], eb = esc[2 * l + 1];
        const S2 *src = reinterpret_cast<const S2 *>(mp.scr) + l * mp.scr_len;
        const cx<T> *ch = reinterpret_cast<const cx<T> *>(mp.chirp);
        auto fetch = [&](long long k) {
            if (mp.kind == MAP_RADER) {
                // X[0] = x0 + A0, X[k] = x0 + c[log_g k]
                const S2 x0 = reinterpret_cast<const S2 *>(mp.x0buf)[l];
                const S2 a = k == 0 ? reinterpret_cast<const S2 *>(mp.a0buf)[l] : src[mp.ridx[k]];
                cx<T> z = crenorm(cx<T>{Loc2<T>::in(a.x), Loc2<T>::in(a.y)} + cx<T>{Loc2<T>::in(x0.x), Loc2<T>::in(x0.y)});
                return mp.fwd ? z : conjx(z);
            }
            S2 a = src[k];
            cx<T> z{Loc2<T>::in(a.x), Loc2<T>::in(a.y)};
            if (mp.kind == MAP_BLUE) z = mp.fwd ? cmulc(z, ch[k]) : cmul(z, ch[k]);
            return z;
        };
        if (io.out_kind == OUT_R) {
            cx<T> z = fetch(u);
            stg_s<S>(base + (long long)u * io.os, sc.apply(z.r, ea));
            if (has_b) stg_s<S>(base + io.pair_out + (long long)u * io.os, sc.apply(z.i, eb));
            continue;
        }
        cx<T> za, zb;
        const cx<T> z1 = fetch(u);
        if (u == 0) {
            za = cx<T>{z1.r, RealOps<T>::k(0.0)};
            zb = cx<T>{z1.i, RealOps<T>::k(0.0)};
        } else {
            const cx<T> z2 = conjx(fetch(mp.M - u));
            cx<T> A = chalf(z1 + z2), D = chalf(z1 - z2);
            za = crenorm(A);
            zb = crenorm(cx<T>{D.i, -D.r});
        }
        if (io.conj_out) { za.i = -za.i; zb.i = -zb.i; }
        store_unit<T, S, S2>(io, base, u, za, sc, ea);
        if (has_b) store_unit<T, S, S2>(io, base + io.pair_out, u, zb, sc, eb);
    }
}

// ---------------------------------------------------------------------------
// real-to-real transforms (DCT / DST I-IV, r2r_fftpack, Hartley)
// ---------------------------------------------------------------------------
// With N the length along the axis and U the forward FFT of the scratch line:
//   DCT-I  (L2 = 2(N-1)): u = even extension of x;            y[k] = Re U[k]
//   DST-I  (L2 = 2(N+1)): u = (0, x, 0, -reversed x);          y[k] = -Im U[k+1]
//   DCT-II / DST-II (L2 = 2N): u = x, zero padded;             y[k] = 2 Re(w^k U[k]) / -2 Im(w^(k+1) U[k+1])
//   DCT-III: u[m] = c_m x[m] w^m (c_0 = 1, else 2);            y[k] = Re U[k]
//   DST-III: u[m] = c_m x[m-1] w^m, 1 <= m <= N (c_N = 1, else 2); y[k] = -Im U[k]
//   DCT-IV / DST-IV: u[m] = x[m] w^m;                          y[k] = 2 Re / -2 Im(v^(2k+1) U[k])
// with w = exp(-i pi / 2N), v = exp(-i pi / 4N), times fct; ortho scales as
// the reference's steps do (DCT-I: x[0], x[N-1] by sqrt 2 and y[0], y[N-1] by
// 1/sqrt 2; DCT-II, DST-II: y[0] by 1/sqrt 2; DCT-III, DST-III: x[0] by sqrt 2).
constexpr double kSqrt2 = 1.4142135623730950488016887;
template <class T>
__global__ void k_r2r_pre(const __grid_constant__ IODesc io, const __grid_constant__ R2RDesc d)
{
    using S = typename Traits<T>::S;
    using S2 = typename Traits<T>::S2;
    const long long total = io.nlines * d.L2, N = d.N;
    for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x) {
        const long long l = qdiv(idx, d.L2, d.fL2), m = idx - l * d.L2;
        const char *base = io.in + line_off(io, l, false);
        auto X = [&](long long j) { return (double)ldg_s<S>(base + j * io.is); };
        if (d.mode == R2R_COPY || d.mode == R2R_HARTLEY) {
            double v = X(m);
            if (d.neg_even && m >= 2 && (m & 1) == 0) v = -v;
            reinterpret_cast<S *>(d.scr)[idx] = (S)v;
            continue;
        }
        double v = 0.0, w = 1.0;
        bool tw = false;
        switch (d.mode) {
        case R2R_DCT1: {
            const long long src = m <= N - 1 ? m : d.L2 - m;
            v = X(src);
            if (d.ortho && (src == 0 || src == N - 1)) w = kSqrt2;
            break;
        }
        case R2R_DST1:
            if (m >= 1 && m <= N) v = X(m - 1);
            else if (m >= N + 2) v = -X(d.L2 - 1 - m);
            break;
        case R2R_DCT2:
        case R2R_DST2:
            if (m < N) v = X(m);
            break;
        case R2R_DCT3:
            if (m < N) {
                v = X(m);
                w = m == 0 ? (d.ortho ? kSqrt2 : 1.0) : 2.0;
                tw = true;
            }
            break;
        case R2R_DST3:
            if (m >= 1 && m <= N) {
                v = X(m - 1);
                w = m == N ? 1.0 : 2.0;
                if (d.ortho && m == 1) w *= kSqrt2;
                tw = true;
            }
            break;
        default:  // types IV
            if (m < N) {
                v = X(m);
                tw = true;
            }
            break;
        }
        v *= w;
        S2 o;
        if (!tw) {
            o.x = (S)v;
            o.y = S(0);
        } else {
            Loc<T> lc;
            lc.fit(v, 0.0);
            const cx<T> z = cmul(lc.in(v, 0.0), reinterpret_cast<const cx<T> *>(d.tw1)[m]);
            o.x = (S)lc.out(z.r);
            o.y = (S)lc.out(z.i);
        }
        reinterpret_cast<S2 *>(d.scr)[idx] = o;
    }
}

template <class T>
__global__ void k_r2r_post(const __grid_constant__ IODesc io, const __grid_constant__ R2RDesc d)
{
    using S = typename Traits<T>::S;
    using S2 = typename Traits<T>::S2;
    const long long N = d.N, total = io.nlines * N;
    for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x) {
        const long long l = qdiv(idx, N, d.fN), k = idx - l * N;
        S *dst = reinterpret_cast<S *>(io.out + line_off(io, l, true) + k * io.os);
        if (d.mode == R2R_COPY) {
            double v = reinterpret_cast<const S *>(d.scr)[l * d.L2 + k];
            if (d.neg_even && k >= 2 && (k & 1) == 0) v = -v;
            *dst = (S)v;
            continue;
        }
        if (d.mode == R2R_HARTLEY) {
            // h[0]; h[2j-1] +- h[2j] to j and N - j; h[N-1] to N/2 for even N
            const S *h = reinterpret_cast<const S *>(d.scr) + l * d.L2;
            S v;
            if (k == 0) v = h[0];
            else if (2 * k < N) v = h[2 * k - 1] + h[2 * k];
            else if (2 * k == N) v = h[N - 1];
            else v = h[2 * (N - k) - 1] - h[2 * (N - k)];
            *dst = v;
            continue;
        }
        const S2 *U = reinterpret_cast<const S2 *>(d.scr) + l * d.L2;
        double y, w = d.fct;
        const cx<T> *tw1 = reinterpret_cast<const cx<T> *>(d.tw1);
        const cx<T> *tw2 = reinterpret_cast<const cx<T> *>(d.tw2);
        auto twisted = [&](S2 a, cx<T> t, bool re) {
            Loc<T> lc;
            lc.fit(a.x, a.y);
            const cx<T> z = cmul(lc.in(a.x, a.y), t);
            return re ? lc.out(z.r) : lc.out(z.i);
        };
        switch (d.mode) {
        case R2R_DCT1:
            y = U[k].x;
            if (d.ortho && (k == 0 || k == N - 1)) w /= kSqrt2;
            break;
        case R2R_DST1: y = -(double)U[k + 1].y; break;
        case R2R_DCT2:
            y = 2.0 * twisted(U[k], tw1[k], true);
            if (d.ortho && k == 0) w /= kSqrt2;
            break;
        case R2R_DST2:
            y = -2.0 * twisted(U[k + 1], tw1[k + 1], false);
            if (d.ortho && k == 0) w /= kSqrt2;
            break;
        case R2R_DCT3: y = U[k].x; break;
        case R2R_DST3: y = -(double)U[k].y; break;
        case R2R_DCT4: y = 2.0 * twisted(U[k], tw2[k], true); break;
        default: y = -2.0 * twisted(U[k], tw2[k], false); break;
        }
        *dst = (S)(y * w);
    }
}

// genuine Hartley fold of an r2c half spectrum (contiguous, shape tshp)
template <class T>
__global__ void k_hartley_fold(const typename Traits<T>::S2 *__restrict__ X, char *out, const __grid_constant__ HartleyDesc h)
{
    using S = typename Traits<T>::S;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < h.total;
         e += (long long)gridDim.x * blockDim.x) {
        long long r = e, o = 0, ro = 0;
        for (int dd = h.ndim - 1; dd >= 0; --dd) {
            const long long i = r % h.tshp[dd];
            r /= h.tshp[dd];
            const long long ri = (h.rev[dd] && i) ? h.shape[dd] - i : i;
            o += i * h.sout[dd];
            ro += ri * h.sout[dd];
        }
        const typename Traits<T>::S2 v = X[e];
        stg_s<S>(out + o, v.x + v.y);
        stg_s<S>(out + ro, v.x - v.y);
    }
}

// ---------------------------------------------------------------------------
// upfirdn helpers (storage type S)
// ---------------------------------------------------------------------------
// U[b, m] = x[b, m / up] when m is a multiple of up and m / up < n, else 0 (m < P)
template <class S>
__global__ void k_upsample_pad(const S *__restrict__ x, long long dx, long long n, int up, S *__restrict__ U, long long P,
                               long long B)
{
    const long long total = B * P;
    for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x) {
        const long long b = idx / P, m = idx - b * P;
        const long long q = m / up;
        U[idx] = (m - q * up == 0 && q < n) ? x[b * dx + q] : S(0);
    }
}
// y[b, j] = C[b, j down], j < ny
template <class S>
__global__ void k_decimate(const S *__restrict__ C, long long P, int down, S *__restrict__ y, long long dy, long long ny,
                           long long B)
{
    const long long total = B * ny;
    for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x) {
        const long long b = idx / ny, j = idx - b * ny;
        y[b * dy + j] = C[b * P + j * (long long)down];
    }
}

// ---------------------------------------------------------------------------
// FFT-convolution helpers (elementwise; storage type S, arithmetic T)
// ---------------------------------------------------------------------------

// out[b, i, j] (P0 x P1) = in[b, i - r0, j - c0] inside the H x W source, else 0
template <class S>
__global__ void k_pad2d(const S *__restrict__ in, S *__restrict__ out, long long B, long long H, long long W,
                        long long P0, long long P1, long long r0, long long c0)
{
    // one output row per block iteration (the row's source decided once), the
    // threads over its columns: no 64-bit division per element
    const long long rows = B * P0;
    for (long long r = blockIdx.x; r < rows; r += gridDim.x) {
        const long long b = r / P0, si = r - b * P0 - r0;
        S *orow = out + r * P1;
        if (si >= 0 && si < H) {
            const S *irow = in + (b * H + si) * W;
            for (long long j = threadIdx.x; j < P1; j += blockDim.x) {
                const long long sj = j - c0;
                orow[j] = (sj >= 0 && sj < W) ? irow[sj] : S(0);
            }
        } else {
            for (long long j = threadIdx.x; j < P1; j += blockDim.x) orow[j] = S(0);
        }
    }
}

// out[b, i, j] (H x W) = in[b, i + r0, j + c0] of a P0 x P1 source
template <class S>
__global__ void k_crop2d(const S *__restrict__ in, S *__restrict__ out, long long B, long long H, long long W,
                         long long P0, long long P1, long long r0, long long c0)
{
    const long long rows = B * H;
    for (long long r = blockIdx.x; r < rows; r += gridDim.x) {
        const long long b = r / H, i = r - b * H;
        const S *irow = in + (b * P0 + i + r0) * P1 + c0;
        S *orow = out + r * W;
        for (long long j = threadIdx.x; j < W; j += blockDim.x) orow[j] = irow[j];
    }
}

// spectrum products: mode 0: out[b,e] = a[b,e] * f[b % nf, e];  mode 1: * conj(f)
// mode 2: out[e] = sum_b a[b,e] * conj(f[b,e])   (gradient of a shared filter)
template <class T>
__global__ void k_spec_mul(const typename Traits<T>::S2 *__restrict__ a, const typename Traits<T>::S2 *__restrict__ f,
                           typename Traits<T>::S2 *__restrict__ out, long long B, long long nf, long long n, int mode)
{
    using S2 = typename Traits<T>::S2;
    using S = typename Traits<T>::S;
    const long long total = mode == 2 ? n : B * n;
    for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x) {
        if (mode == 2) {
            cx<T> acc{RealOps<T>::k(0.0), RealOps<T>::k(0.0)};
            // accumulate with a common scale: the largest operand exponents of each product
            for (long long b = 0; b < B; ++b) {
                S2 x = a[b * n + idx], y = f[b * n + idx];
                Loc<T> la, lf;
                la.fit(x.x, x.y);
                lf.fit(y.x, y.y);
                cx<T> p = cmulc(la.in(x.x, x.y), lf.in(y.x, y.y));
                // bring each product back to true scale before summing
                const double qr = Loc2<T>::out(p.r, la.esc + lf.esc), qi = Loc2<T>::out(p.i, la.esc + lf.esc);
                acc = crenorm(acc + cx<T>{Loc2<T>::in(qr), Loc2<T>::in(qi)});
            }
            S2 o;
            o.x = (S)Loc2<T>::out(acc.r, 0);
            o.y = (S)Loc2<T>::out(acc.i, 0);
            out[idx] = o;
        } else {
            long long b = idx / n, e = idx - b * n;
            S2 x = a[idx], y = f[(b % nf) * n + e];
            Loc<T> la, lf;
            la.fit(x.x, x.y);
            lf.fit(y.x, y.y);
            cx<T> xx = la.in(x.x, x.y), yy = lf.in(y.x, y.y);
            cx<T> p = mode == 1 ? cmulc(xx, yy) : cmul(xx, yy);
            S2 o;
            o.x = (S)Loc2<T>::out(p.r, la.esc + lf.esc);
            o.y = (S)Loc2<T>::out(p.i, la.esc + lf.esc);
            out[idx] = o;
        }
    }
}

// Hermitian weighting of half spectra (n_half bins per line, real length nreal):
// bins 1 .. ceil(nreal/2)-1 are multiplied by w; DC (and Nyquist for even
// nreal) keep their real part and lose the imaginary part when drop_im
template <class T>
__global__ void k_half_weight(typename Traits<T>::S2 *__restrict__ x, long long lines, long long n_half,
                              long long nreal, typename Traits<T>::S w, int drop_im)
{
    using S = typename Traits<T>::S;
    const long long total = lines * n_half;
    for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x) {
        long long k = idx % n_half;
        bool edge = k == 0 || (nreal % 2 == 0 && k == nreal / 2);
        if (edge) {
            if (drop_im) x[idx].y = S(0);
        } else {
            x[idx].x *= w;  // w is 2 or 1/2: exact
            x[idx].y *= w;
        }
    }
}

// ---------------------------------------------------------------------------
// table builders (FP64, exact integer angle reduction, CUDA's sincospi)
// ---------------------------------------------------------------------------

// exp(+2 pi i t / D) for 0 <= t: reduce t/D to the first octant with integer
// arithmetic, evaluate sincospi there, and undo the reduction by symmetry.
__device__ inline double2 exp2pi_frac(unsigned long long t, unsigned long long D)
{
    t %= D;
    bool neg = false;
    if (2 * t > D) { t = D - t; neg = true; }
    double c, s;
    if (4 * t > D) {
        // angle = pi/2 + 2 pi (4t - D) / (4D)
        unsigned long long num = 4 * t - D, den = 4 * D;
        double cq, sq;
        if (8 * num > den) {
            double x = 2.0 * (double)(den - 4 * num) / (double)(4 * den);
            sincospi(x, &cq, &sq);  // cos(q) = sin(pi/2 - q)
        } else {
            double x = 2.0 * (double)num / (double)den;
            sincospi(x, &sq, &cq);
        }
        c = -sq;
        s = cq;
    } else if (8 * t > D) {
        double x = 2.0 * (double)(D - 4 * t) / (double)(4 * D);
        sincospi(x, &c, &s);  // swapped: angle = pi/2 - x pi
    } else {
        double x = 2.0 * (double)t / (double)D;
        sincospi(x, &s, &c);
    }
    return make_double2(c, neg ? -s : s);
}

template <class T> __device__ inline cx<T> to_arith(double2 v);
template <> __device__ inline cx<float> to_arith<float>(double2 v) { return cx<float>{__double2float_rn(v.x), __double2float_rn(v.y)}; }
template <> __device__ inline cx<double> to_arith<double>(double2 v) { return cx<double>{v.x, v.y}; }
template <> __device__ inline cx<df> to_arith<df>(double2 v) { return cx<df>{df_from_double(v.x), df_from_double(v.y)}; }

// stage twiddles: entry k*(R-1) + m-1 = exp(-2 pi i m k / (ns R)), k < ns, 1 <= m < R
template <class T> __global__ void k_gen_stage_tw(typename Bfly<T>::W *tw, int R, int ns)
{
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ns * (R - 1)) return;
    int k = e / (R - 1), m = e % (R - 1) + 1;
    double2 v = exp2pi_frac((unsigned long long)m * k, (unsigned long long)ns * R);
    v.y = -v.y;
    if constexpr (std::is_same<T, df>::value) {
        const cx<df> w = to_arith<df>(v);
        tw[e] = ptw{w.r.h, w.i.h, w.r.l, w.i.l};
    } else {
        tw[e] = to_arith<T>(v);
    }
}

// r2r twiddles: tw1[m] = exp(-2 pi i m / 4N) (m <= N), tw2[k] = exp(-2 pi i (2k+1) / 8N) (k < N)
template <class T> __global__ void k_gen_r2r_tw(cx<T> *tw1, cx<T> *tw2, long long N)
{
    const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (j <= N) {
        double2 v = exp2pi_frac((unsigned long long)j, 4ull * (unsigned long long)N);
        v.y = -v.y;
        tw1[j] = to_arith<T>(v);
    }
    if (j < N) {
        double2 v = exp2pi_frac(2ull * (unsigned long long)j + 1ull, 8ull * (unsigned long long)N);
        v.y = -v.y;
        tw2[j] = to_arith<T>(v);
    }
}

// four-step twiddles, in the stage-twiddle format of the arithmetic:
// tab[n2 N1 + k1] = exp(-2 pi i n2 k1 / (N1 N2))
template <class T> __global__ void k_gen_tw4(typename Bfly<T>::W *tab, long long N1, long long N2)
{
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= N1 * N2) return;
    const long long n2 = e / N1, k1 = e - n2 * N1;
    double2 v = exp2pi_frac((unsigned long long)(n2 * k1), (unsigned long long)(N1 * N2));
    v.y = -v.y;
    if constexpr (std::is_same<T, df>::value) {
        const cx<df> w = to_arith<df>(v);
        tab[e] = ptw{w.r.h, w.i.h, w.r.l, w.i.l};
    } else {
        tab[e] = to_arith<T>(v);
    }
}

// roots: out[j] = exp(-2 pi i (j * mult) / D), j < count
template <class T> __global__ void k_gen_roots(cx<T> *out, long long count, unsigned long long mult, unsigned long long D)
{
    long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= count) return;
    double2 v = exp2pi_frac(((unsigned long long)j * mult) % D, D);
    v.y = -v.y;
    out[j] = to_arith<T>(v);
}

// Bluestein chirp exp(+i pi m^2 / n) with m^2 mod 2n in exact integers
// (pocketfft.c:1907-1914 keeps the same quantity by a recurrence)
static __global__ void k_gen_chirp64(double2 *bk, long long n)
{
    long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= n) return;
    unsigned long long mm = (unsigned long long)m % (2ull * n);
    unsigned long long coeff = (mm * mm) % (2ull * n);
    bk[m] = exp2pi_frac(coeff, 2ull * n);
}

// symmetric zero padding of the chirp to length L (scaled 1/L), for its FFT
static __global__ void k_pad_chirp64(const double2 *bk, double2 *out, long long n, long long L)
{
    long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= L) return;
    double s = 1.0 / (double)L;
    double2 v = make_double2(0.0, 0.0);
    if (k < n) v = bk[k];
    else if (L - k < n) v = bk[L - k];
    out[k] = make_double2(v.x * s, v.y * s);
}

template <class T> __global__ void k_convert64(const double2 *in, cx<T> *out, long long n)
{
    long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) out[k] = to_arith<T>(in[k]);
}

}  // namespace ig
