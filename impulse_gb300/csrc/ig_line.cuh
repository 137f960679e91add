// ig_line.cuh -- k_fft_line: single-CTA Stockham transforms of whole lines
// with the HBM traffic fused into the first and last stages.
//
// k_fft_smem stages a line into shared memory in a prologue pass, runs every
// Stockham stage shared memory -> registers -> shared memory, and writes the
// line back in an epilogue pass (with one more pass for the real split).  For
// the two layouts that carry the bulk of the work -- complex lines
// (pocketfft::c2c, pocketfft_hdronly.h:3272; cfft_forward / cfft_backward,
// impulse/fft/c_pocketfft/pocketfft.c:2160-2170) and real lines of even
// length written as halfcomplex (rfft_forward, pocketfft.c:2184) -- this
// kernel:
//   * runs the first stage (ns = 1, no twiddles) on units loaded straight from
//     HBM into registers: butterfly j of a line reads units j + m L/R, so
//     consecutive threads read consecutive units;
//   * runs the last stage from shared memory straight to HBM: its outputs
//     j + m L/R are the natural order, again consecutive per warp;
//   * for the halfcomplex layout, gives each thread the mirror butterflies j
//     and L/R - j of the last stage: their outputs are the partner bins Z[k]
//     and Z[M - k] of the real split, which is computed in registers and
//     written as X[k], X[M - k] (T = w^k (-i)(Z[k] - conj Z[M-k]),
//     X[k] = Z[k] + conj Z[M-k] + T, X[M-k] = conj(Z[k] + conj Z[M-k] - T),
//     the 1/2 folded into the output scale).
// Two shared-memory round trips and two barriers per line go away; the middle
// stages are k_fft_smem's.  Double-float lines are range-checked on the
// loaded values: a line whose largest element lies outside 2^+-40 gets an
// exact power-of-two scale, as in k_fft_smem.
#pragma once
#include "ig_kernels.cuh"
#include "ig_tma.cuh"

namespace ig {

constexpr int LK_C2C = 0;   // complex units in, complex units out
constexpr int LK_R2HC = 1;  // real pairs in (as complex units), halfcomplex out
// the same for double-float: the last stage writes the spectrum Z to the
// other line buffer and a split pass reads Z[k], Z[M - k] from it (the mirror
// butterflies of LK_R2HC keep two butterflies live, which cost double-float
// lines a CTA per SM)
constexpr int LK_R2HC_S = 2;
// real pairs in, half spectrum out as complex units (pocketfft::r2c's last
// axis, general_r2c, pocketfft_hdronly.h:3125): the LK_R2HC butterflies with
// X[k] stored as unit k (DC and Nyquist imaginary parts 0, conjugated for
// a backward r2c)
constexpr int LK_R2C = 3;
// half spectrum in (complex units X[0..M]), real pairs out (pocketfft::c2r's
// last axis, general_c2r, pocketfft_hdronly.h:3180): the Hermitian pre-step
// reads X[k] and X[M - k] straight from HBM and writes Z[k], Z[M - k] to the
// line buffer, every stage then runs from shared memory and the last one
// writes the real pairs to HBM
constexpr int LK_C2R = 4;

// c2r pre-step from HBM into `line`: Z[k] = (X[k] + conj X[M-k]) + i w^-k
// (X[k] - conj X[M-k]) for the slot pairs (k, M - k) a thread owns (the DC
// and Nyquist bins' imaginary parts read as 0, the input conjugated when
// cin, the backward core's conjugation folded in when cc)
template <class T>
__device__ __forceinline__ void line_herm_pre(cx<T> *line, const char *base, long long is, const CoreDesc &P, int tpl,
                                              int t, bool act, bool cin, bool cc)
{
    using S2 = typename Traits<T>::S2;
    const int M = P.L, pad = P.pad;
    const cx<T> *rtw = reinterpret_cast<const cx<T> *>(P.rtw);
    if (!act) return;
    for (int k = t; 2 * k <= M; k += tpl) {
        const int k2 = M - k;
        const S2 ra = ldg_s<S2>(base + (long long)k * is), rb = ldg_s<S2>(base + (long long)k2 * is);
        cx<T> a{ra.x, cin ? -ra.y : ra.y}, b{rb.x, cin ? -rb.y : rb.y};
        if (k == 0) {
            a.i = T(0);
            b.i = T(0);
        }
        {
            const cx<T> xb = conjx(b), A = a + xb, Bv = a - xb;
            const cx<T> tB = cmulc(Bv, rtw[k]);
            const cx<T> z{A.r - tB.i, A.i + tB.r};
            sput(line + sp(k, pad), cc ? conjx(z) : z);
        }
        if (k > 0 && k2 != k) {
            const cx<T> xb = conjx(a), A = b + xb, Bv = b - xb;
            const cx<T> tB = cmulc(Bv, rtw[k2]);
            const cx<T> z{A.r - tB.i, A.i + tB.r};
            sput(line + sp(k2, pad), cc ? conjx(z) : z);
        }
    }
}

// First stage: load, (double-float: range check), convert, radix-R DFT, write
// the Stockham positions j R + m of buffer `line`.  Returns the line's
// exponent scale (0 for FP32).
template <class T, int E, int R>
__device__ __forceinline__ int line_first(cx<T> *line, const char *base, long long is, const CoreDesc &P, int tpl,
                                          int t, bool act, bool cc, int g, int *s_emax, int *s_flag)
{
    using S2 = typename Traits<T>::S2;
    using B = Bfly<T>;
    using V = typename B::V;
    constexpr bool RAW = Traits<T>::kRaw;
    constexpr int NB = (E + R - 1) / R;
    const int nr = P.L / R, pad = P.pad;
    S2 raw[NB][R];
#pragma unroll
    for (int i = 0; i < NB; ++i) {
        const int j = t + i * tpl;
        if (act && j < nr) {
            const char *p = base + (long long)j * is;
            const long long step = (long long)nr * is;
#pragma unroll
            for (int m = 0; m < R; ++m) raw[i][m] = ldg_s<S2>(p + m * step);
        }
    }
    int esc = 0;
    if constexpr (RAW) {
        unsigned mm = 0;  // largest magnitude word (dmag) of the thread's values
#pragma unroll
        for (int i = 0; i < NB; ++i) {
            const int j = t + i * tpl;
            if (act && j < nr) {
#pragma unroll
                for (int m = 0; m < R; ++m) mm = max(mm, max(dmag(raw[i][m].x), dmag(raw[i][m].y)));
            }
        }
        const int emax = dkey_mag(mm);
        // common case: every thread's largest value inside the safe window
        // 2^+-40 (all-zero threads are safe); otherwise the CTA takes the
        // exact per-line maximum
        constexpr int c = 1023 + kKeyOff;
        const bool out = emax != 0 && (emax > c + 40 || emax < c - 40);
        if (out) *s_flag = 1;
        __syncthreads();
        if (*s_flag) {
            if (act && emax != 0) atomicMax(&s_emax[g], emax);
            __syncthreads();
            const int ea = act ? s_emax[g] : 0;
            if (ea != 0 && (ea > c + 40 || ea < c - 40)) esc = c - ea;
        }
    }
#pragma unroll
    for (int i = 0; i < NB; ++i) {
        const int j = t + i * tpl;
        if (act && j < nr) {
            V v[R];
#pragma unroll
            for (int m = 0; m < R; ++m) {
                cx<T> z{Store<T>::in(raw[i][m].x, esc), Store<T>::in(raw[i][m].y, esc)};
                if (cc) z = conjx(z);
                if constexpr (std::is_same<T, df>::value) v[m] = to_p(z);
                else v[m] = z;
            }
            B::template dft<R>(v);
            const int base_i = j * R;
#pragma unroll
            for (int m = 0; m < R; ++m) B::st(line + sp(base_i + m, pad), v[m]);
        }
        asm volatile("" ::: "memory");
    }
    return esc;
}

// value of a butterfly output as a plain complex (double-float renormalised)
template <class T> __device__ __forceinline__ cx<T> line_val(const typename Bfly<T>::V &v)
{
    if constexpr (std::is_same<T, df>::value) return from_p(prenorm(v));
    else return v;
}

// Last stage of a complex line: butterfly j (q = 0, k = j) reads units
// j + m nr of `src`, twiddles, DFT, and writes units j + m nr of the output
// line with the output scale (conjugated for a backward transform).
template <class T, int E, int R>
__device__ __forceinline__ void line_last_c2c(const cx<T> *src, char *obase, long long os, const CoreDesc &P, int si,
                                              int tpl, int t, bool act, bool cc, const OutScale<T> &sc, int esc)
{
    using S2 = typename Traits<T>::S2;
    using B = Bfly<T>;
    using V = typename B::V;
    constexpr int NB = (E + R - 1) / R;
    const int nr = P.L / R, pad = P.pad;
    const typename B::W *tw = reinterpret_cast<const typename B::W *>(P.tw) + P.st[si].tw;
    if (!act) return;
#pragma unroll
    for (int i = 0; i < NB; ++i) {
        const int j = t + i * tpl;
        if (j < nr) {
            V v[R];
#pragma unroll
            for (int m = 0; m < R; ++m) v[m] = B::ld(src + sp(j + m * nr, pad));
            if (j) {
                const typename B::W *twk = tw + j * (R - 1) - 1;
#pragma unroll
                for (int m = 1; m < R; ++m) v[m] = B::tw(v[m], twk + m, P);
            }
            B::template dft<R>(v);
            char *p = obase + (long long)j * os;
            const long long step = (long long)nr * os;
#pragma unroll
            for (int m = 0; m < R; ++m) {
                cx<T> z = line_val<T>(v[m]);
                if (cc) z.i = -z.i;
                S2 o;
                o.x = sc.apply(z.r, esc);
                o.y = sc.apply(z.i, esc);
                stg_s<S2>(p + m * step, o);
            }
        }
        asm volatile("" ::: "memory");
    }
}

// real split of the partner bins a = Z[k], b = Z[M - k] and the halfcomplex
// stores of X[k] and X[M - k] (HS: as complex units k and M - k of a half
// spectrum, imaginary parts negated when cjo); sc carries fct / 2
template <class T, bool HS = false>
__device__ __forceinline__ void line_split_store(cx<T> a, cx<T> b, int k, int M, const cx<T> *rtw, char *obase,
                                                 long long os, const OutScale<T> &sc, int esc, const CoreDesc &P,
                                                 bool cjo = false)
{
    using S = typename Traits<T>::S;
    cx<T> X, Y;  // X[k], X[M - k]
    if constexpr (std::is_same<T, df>::value) {
        const f2p cj = pk(1.0f, -1.0f);
        const pcx pa = to_p(a), pc = plane(to_p(b), cj);  // a, conj b
        const pcx Ev = pa + pc, D = pa - pc;
        const pcx Tm = pmulw_cx<true>(prot<true>(D), rtw + k, P.neg1);  // w^k (-i) D
        X = from_p(prenorm(Ev + Tm));
        Y = from_p(prenorm(plane(Ev - Tm, cj)));
    } else {
        const cx<T> c{b.r, -b.i};
        const cx<T> Ev = a + c, D = a - c;
        const cx<T> Tm = cmul(cx<T>{D.i, -D.r}, rtw[k]);
        X = Ev + Tm;
        const cx<T> Z = Ev - Tm;
        Y = cx<T>{Z.r, -Z.i};
    }
    const int k2 = M - k;
    if constexpr (HS) {
        using S2 = typename Traits<T>::S2;
        const S zero = S(0);
        S2 o;
        o.x = sc.apply(X.r, esc);
        o.y = k == 0 ? zero : sc.apply(cjo ? -X.i : X.i, esc);
        stg_s<S2>(obase + (long long)k * os, o);
        if (k2 != k) {
            o.x = sc.apply(Y.r, esc);
            o.y = k2 == M ? zero : sc.apply(cjo ? -Y.i : Y.i, esc);
            stg_s<S2>(obase + (long long)k2 * os, o);
        }
        return;
    }
    if (k == 0) {
        stg_s<S>(obase, sc.apply(X.r, esc));
    } else {
        char *p = obase + (2 * (long long)k - 1) * os;
        stg_s<S>(p, sc.apply(X.r, esc));
        stg_s<S>(p + os, sc.apply(X.i, esc));
    }
    if (k2 != k) {
        if (k2 == M) {
            stg_s<S>(obase + (2 * (long long)M - 1) * os, sc.apply(Y.r, esc));
        } else {
            char *p = obase + (2 * (long long)k2 - 1) * os;
            stg_s<S>(p, sc.apply(Y.r, esc));
            stg_s<S>(p + os, sc.apply(Y.i, esc));
        }
    }
}

// Last stage of an even real line (M = L complex points of the packed line):
// pair slot p holds butterflies p and nr - p; output m of butterfly p is
// Z[p + m nr], whose partner Z[M - p - m nr] is output R - 1 - m of butterfly
// nr - p (for p = 0: output R - m of butterfly 0; for 2p = nr: output
// R - 1 - m of butterfly p itself).
template <class T, int E, int R, bool HS = false>
__device__ __forceinline__ void line_last_r2hc(const cx<T> *src, char *obase, long long os, const CoreDesc &P,
                                               int si, int tpl, int t, bool act, const OutScale<T> &sc, int esc,
                                               bool cjo = false)
{
    using B = Bfly<T>;
    using V = typename B::V;
    const int M = P.L, nr = M / R, pad = P.pad, nslot = nr / 2 + 1;
    const typename B::W *tw = reinterpret_cast<const typename B::W *>(P.tw) + P.st[si].tw;
    const cx<T> *rtw = reinterpret_cast<const cx<T> *>(P.rtw);
    if (!act) return;
    for (int p = t; p < nslot; p += tpl) {
        const int pb = nr - p;
        const bool two = p != 0 && 2 * p != nr;
        V va[R], vb[R];
#pragma unroll
        for (int m = 0; m < R; ++m) va[m] = B::ld(src + sp(p + m * nr, pad));
        if (two) {
#pragma unroll
            for (int m = 0; m < R; ++m) vb[m] = B::ld(src + sp(pb + m * nr, pad));
        }
        if (p) {
            const typename B::W *twk = tw + p * (R - 1) - 1;
#pragma unroll
            for (int m = 1; m < R; ++m) va[m] = B::tw(va[m], twk + m, P);
        }
        if (two) {
            const typename B::W *twk = tw + pb * (R - 1) - 1;
#pragma unroll
            for (int m = 1; m < R; ++m) vb[m] = B::tw(vb[m], twk + m, P);
        }
        B::template dft<R>(va);
        if (two) {
            B::template dft<R>(vb);
#pragma unroll
            for (int m = 0; m < R; ++m)
                line_split_store<T, HS>(line_val<T>(va[m]), line_val<T>(vb[R - 1 - m]), p + m * nr, M, rtw, obase, os, sc,
                                    esc, P, cjo);
        } else if (p == 0) {
            // k = m nr, partner (R - m) nr (m = 0: k = 0 with itself)
#pragma unroll
            for (int m = 0; m < R; ++m) {
                const int mp = m == 0 ? 0 : R - m;
                if (m <= mp)
                    line_split_store<T, HS>(line_val<T>(va[m]), line_val<T>(va[mp]), m * nr, M, rtw, obase, os, sc, esc, P, cjo);
            }
        } else {
            // 2 p = nr: k = p + m nr, partner p + (R - 1 - m) nr
#pragma unroll
            for (int m = 0; m < R; ++m) {
                const int mp = R - 1 - m;
                if (m <= mp)
                    line_split_store<T, HS>(line_val<T>(va[m]), line_val<T>(va[mp]), p + m * nr, M, rtw, obase, os, sc,
                                        esc, P, cjo);
            }
        }
        asm volatile("" ::: "memory");
    }
}

#define IG_LINE_RADIX_SWITCH(RV, CALL)                                                \
    switch (RV) {                                                                      \
    case 2: { constexpr int R_ = 2; CALL; } break;                                     \
    case 4: { constexpr int R_ = 4; CALL; } break;                                     \
    case 8: { constexpr int R_ = 8; CALL; } break;                                     \
    case 16: if constexpr (rs_has<E, RS>(16)) { constexpr int R_ = 16; CALL; } break;  \
    case 3: if constexpr (rs_has<E, RS>(3)) { constexpr int R_ = 3; CALL; } break;     \
    case 5: if constexpr (rs_has<E, RS>(5)) { constexpr int R_ = 5; CALL; } break;     \
    case 9: if constexpr (rs_has<E, RS>(9)) { constexpr int R_ = 9; CALL; } break;     \
    case 7: if constexpr (rs_has<E, RS>(7)) { constexpr int R_ = 7; CALL; } break;     \
    case 11: if constexpr (rs_has<E, RS>(11)) { constexpr int R_ = 11; CALL; } break;  \
    case 13: if constexpr (rs_has<E, RS>(13)) { constexpr int R_ = 13; CALL; } break;  \
    default: break;                                                                    \
    }

// first / last stages: radices 2, 4, 8, 16 and 3, 5 (plans with another first
// or last radix run k_fft_smem, see line_edge_ok)
#define IG_LINE_EDGE_SWITCH(RV, CALL)                                                \
    switch (RV) {                                                                      \
    case 2: { constexpr int R_ = 2; CALL; } break;                                     \
    case 4: { constexpr int R_ = 4; CALL; } break;                                     \
    case 8: { constexpr int R_ = 8; CALL; } break;                                     \
    case 16: if constexpr (rs_has<E, RS>(16)) { constexpr int R_ = 16; CALL; } break;  \
    case 3: if constexpr (rs_has<E, RS>(3)) { constexpr int R_ = 3; CALL; } break;     \
    case 5: if constexpr (rs_has<E, RS>(5)) { constexpr int R_ = 5; CALL; } break;     \
    default: break;                                                                    \
    }

// register caps: 512-thread CTAs (lines of 4096 / 8192 units) must fit the
// 64 K register file; FP32 8-element lines run two such CTAs per SM (four of
// 256 threads: the halfcomplex variant spills a few bytes at this cap, and
// measured faster with the extra CTA than without the spill)
template <class T, int E, int RS, int K, bool DB> constexpr int fft_line_regs()
{
    // double-float 8-element halfcomplex lines: 80 registers, three 256-thread
    // CTAs per SM like k_fft_smem's
    if constexpr (std::is_same<T, df>::value) return (K == LK_R2HC_S && E == 8) ? 80 : 128;
    return (E == 8 || DB) ? 64 : 128;
}

// One CTA: `lpc` lines of `tpl` threads; shared memory lpc * LSt complex slots
// (LSt = 2 LS with double-buffered middle stages).  Requires a Stockham core
// (no Bluestein / Rader steps) of at least two stages, lines addressed by the
// batch dimensions, complex units in (contiguous reals as pairs for LK_R2HC)
// and complex units (LK_C2C) or halfcomplex reals (LK_R2HC) out, and first and
// last radices with line_edge_ok (LK_R2HC: last radix with line_r2hc_last_ok).
template <class T, int E, int RS, int K, bool DB, int NT = 512>
__global__ void __launch_bounds__(NT) __maxnreg__((fft_line_regs<T, E, RS, K, DB>()))
    k_fft_line(const __grid_constant__ CoreDesc P, const __grid_constant__ IODesc io)
{
    constexpr bool RAW = Traits<T>::kRaw;
    extern __shared__ __align__(16) unsigned char smraw[];
    cx<T> *sm = reinterpret_cast<cx<T> *>(smraw);
    __shared__ int s_emax[kMaxLinesPerCta];
    __shared__ int s_flag;
    const int LS = P.LS, LSt = DB ? 2 * LS : LS;
    const int lpc = io.lpc, tpl = io.tpl;
    const long long line0 = (long long)blockIdx.x * lpc;
    const int nl = (int)min((long long)lpc, io.nlines - line0);
    const int g = threadIdx.x / tpl, t = threadIdx.x - g * tpl;
    const bool act = g < nl;
    // backward: forward stages on conjugated data
    const bool cc = (K == LK_C2C || K == LK_C2R) && !io.fwd;
    cx<T> *const line = sm + (size_t)(act ? g : 0) * LSt;
    const char *ibase = io.in + (act ? line_off(io, line0 + g, false) : 0);
    if constexpr (RAW) {
        for (int i = threadIdx.x; i < lpc; i += blockDim.x) s_emax[i] = 0;
        if (threadIdx.x == 0) s_flag = 0;
        __syncthreads();
    }
    int esc = 0;
    int s_first = 1;
    if constexpr (K == LK_C2R) {
        line_herm_pre<T>(line, ibase, io.is, P, tpl, t, act, io.conj_in != 0, cc);
        s_first = 0;
    } else {
        IG_LINE_EDGE_SWITCH(P.st[0].R,
                            (esc = line_first<T, E, R_>(line, ibase, io.is, P, tpl, t, act, cc, g, s_emax, &s_flag)))
    }
    __syncthreads();
    int cur = 0;
    const int nst = P.nst;
    for (int s = s_first; s < nst - 1; ++s) {
        if constexpr (DB) {
            const cx<T> *src = sm + cur;
            cx<T> *dst = sm + (LS - cur);
            IG_LINE_RADIX_SWITCH(P.st[s].R, (stage_db<T, E, R_>(src, dst, 2 * LS, P, s, nl, tpl, g, t)))
            cur = LS - cur;
            __syncthreads();
        } else {
            IG_LINE_RADIX_SWITCH(P.st[s].R, (stage<T, E, R_>(sm, P, s, nl, tpl, g, t, LS)))
        }
    }
    OutScale<T> sc;
    sc.init(io);
    char *obase = io.out + (act ? line_off(io, line0 + g, true) : 0);
    const cx<T> *src = line + cur;
    if constexpr (K == LK_C2C || K == LK_C2R) {
        IG_LINE_EDGE_SWITCH(P.st[nst - 1].R,
                            (line_last_c2c<T, E, R_>(src, obase, io.os, P, nst - 1, tpl, t, act, cc, sc, esc)))
    } else if constexpr (K == LK_R2HC_S) {
        // last stage into the other buffer (in place when the line has a
        // single buffer), then the real split from it
        if constexpr (std::is_same<T, df>::value) sc.e -= 1;
        else sc.f *= 0.5f;
        {
            const int s = nst - 1;
            if constexpr (DB) {
                const cx<T> *a = sm + cur;
                cx<T> *b = sm + (LS - cur);
                IG_LINE_RADIX_SWITCH(P.st[s].R, (stage_db<T, E, R_>(a, b, 2 * LS, P, s, nl, tpl, g, t)))
                cur = LS - cur;
                __syncthreads();
            } else {
                IG_LINE_RADIX_SWITCH(P.st[s].R, (stage<T, E, R_>(sm, P, s, nl, tpl, g, t, LS)))
            }
        }
        if (act) {
            const cx<T> *z = line + cur;
            const int M = P.L, pad = P.pad;
            const cx<T> *rtw = reinterpret_cast<const cx<T> *>(P.rtw);
            for (int k = t; 2 * k <= M; k += tpl) {
                const cx<T> a = sget(z + sp(k, pad)), b = sget(z + sp(k == 0 ? 0 : M - k, pad));
                line_split_store<T>(a, b, k, M, rtw, obase, io.os, sc, esc, P);
            }
        }
    } else {
        // the split's 1/2 joins the output scale
        if constexpr (std::is_same<T, df>::value) sc.e -= 1;
        else sc.f *= 0.5f;
        constexpr bool HS = K == LK_R2C;
        const bool cjo = HS && io.conj_out;
        switch (P.st[nst - 1].R) {
        case 2: line_last_r2hc<T, E, 2, HS>(src, obase, io.os, P, nst - 1, tpl, t, act, sc, esc, cjo); break;
        case 4: line_last_r2hc<T, E, 4, HS>(src, obase, io.os, P, nst - 1, tpl, t, act, sc, esc, cjo); break;
        case 8: line_last_r2hc<T, E, 8, HS>(src, obase, io.os, P, nst - 1, tpl, t, act, sc, esc, cjo); break;
        case 3:
            if constexpr (rs_has<E, RS>(3))
                line_last_r2hc<T, E, 3, HS>(src, obase, io.os, P, nst - 1, tpl, t, act, sc, esc, cjo);
            break;
        case 5:
            if constexpr (rs_has<E, RS>(5))
                line_last_r2hc<T, E, 5, HS>(src, obase, io.os, P, nst - 1, tpl, t, act, sc, esc, cjo);
            break;
        default: break;  // other last radices are not sent here (line_r2hc_last_ok)
        }
    }
}

// launch of one (arithmetic, elements per thread, buffering) family: radix
// class x kind; the radix-13 class has no line variant (line_edge_ok)
template <class T, int E, bool DB, int RS>
static void launch_line_rs(const CoreDesc &d, const IODesc &io, unsigned grid, unsigned blk, size_t smem,
                           cudaStream_t st)
{
    // double-float halfcomplex lines split after the last stage (LK_R2HC_S):
    // the fused mirror butterflies' two live butterflies cost a CTA per SM
    if (io.lay == LAY_R2HC) {
        if constexpr (std::is_same<T, df>::value) k_fft_line<T, E, RS, LK_R2HC_S, DB><<<grid, blk, smem, st>>>(d, io);
        else k_fft_line<T, E, RS, LK_R2HC, DB><<<grid, blk, smem, st>>>(d, io);
        return;
    }
    if constexpr (!std::is_same<T, df>::value) {
        if (io.lay == LAY_R2C) {
            k_fft_line<T, E, RS, LK_R2C, DB><<<grid, blk, smem, st>>>(d, io);
            return;
        }
        if (io.lay == LAY_C2R) {
            k_fft_line<T, E, RS, LK_C2R, DB><<<grid, blk, smem, st>>>(d, io);
            return;
        }
    }
    k_fft_line<T, E, RS, LK_C2C, DB><<<grid, blk, smem, st>>>(d, io);
}

template <class T, int E, bool DB>
cudaError_t launch_line_E(const CoreDesc &d, const IODesc &io, size_t smem, cudaStream_t st)
{
    const unsigned grid = (unsigned)((io.nlines + io.lpc - 1) / io.lpc), blk = (unsigned)(io.lpc * io.tpl);
    if (blk > 512) {
        if constexpr (std::is_same<T, df>::value && E == 8 && DB) return launch_line_wide<T>(d, io, smem, st);
        return cudaErrorInvalidConfiguration;
    }
    if (d.rs == RS_P2) launch_line_rs<T, E, DB, RS_P2>(d, io, grid, blk, smem, st);
    else if (E == 8 && d.rs == RS_P235) launch_line_rs<T, E, DB, (E == 8 ? RS_P235 : RS_ALL)>(d, io, grid, blk, smem, st);
    else if (d.rs == RS_ALL || d.rs == RS_P235) launch_line_rs<T, E, DB, RS_ALL>(d, io, grid, blk, smem, st);
    else return cudaErrorNotSupported;
    return cudaGetLastError();
}

// --------------------------------------------------------------------------
// k_fft_line_pipe: the same transform as k_fft_line on contiguous FP32 lines,
// with the input lines brought into shared memory by bulk copies (TMA) one or
// two tiles ahead.  A CTA is persistent: it walks tiles of `lpc` lines
// (blockIdx.x, + gridDim.x, ...).  Thread 0 issues one cp.async.bulk per
// line of a tile into a staging slot, completing on the slot's mbarrier;
// after the first stage has read slot s, the slot is refilled with the tile
// `nslot` steps ahead, so the copy of later lines overlaps the middle and
// last stages of this one.  k_fft_line keeps each thread's eight global
// loads in registers and waits on their latency with ~20 warps per SM; here
// the copy engine holds the bytes in flight.
// --------------------------------------------------------------------------

// number of bounded-wait give-ups seen by this translation unit's pipelined
// kernels (read and cleared by the host, ig_device_faults)
static __device__ unsigned g_pipe_wait_fault;

// polls of one mbarrier wait before a CTA gives up (each poll may suspend the
// thread for a while; a tile lands in microseconds)
constexpr unsigned kPipeWaitPolls = 1u << 22;

// first stage from a staged line: unit u of the line is src[u]
template <class T, int E, int R>
__device__ __forceinline__ void line_first_sm(cx<T> *line, const typename Traits<T>::S2 *src, const CoreDesc &P,
                                              int tpl, int t, bool act, bool cc)
{
    using S2 = typename Traits<T>::S2;
    using B = Bfly<T>;
    using V = typename B::V;
    constexpr int NB = (E + R - 1) / R;
    const int nr = P.L / R, pad = P.pad;
#pragma unroll
    for (int i = 0; i < NB; ++i) {
        const int j = t + i * tpl;
        if (act && j < nr) {
            V v[R];
#pragma unroll
            for (int m = 0; m < R; ++m) {
                const S2 r = src[j + m * nr];
                const cx<T> z{r.x, r.y};
                v[m] = cc ? conjx(z) : z;
            }
            B::template dft<R>(v);
            const int base_i = j * R;
#pragma unroll
            for (int m = 0; m < R; ++m) B::st(line + sp(base_i + m, pad), v[m]);
        }
        asm volatile("" ::: "memory");
    }
}

// Shared memory: [lpc line buffers of LSt slots][nslot staging slots of lpc
// lines x L units], the staging area starting at byte `stage_off` (a
// multiple of 128).  Requires FP32 (no per-line range scaling), input units
// contiguous along the line (io.is = 8 bytes), every line start and the
// line size 16-byte aligned.
// register cap of the pipelined variant: its staging slots already hold an
// 8-element line's CTAs at three per SM, which leaves 85 registers a thread
template <class T, int E, int RS, int K, bool DB> constexpr int fft_line_pipe_regs()
{
    return E == 8 ? 80 : 128;
}

template <class T, int E, int RS, int K, bool DB>
__global__ void __launch_bounds__(512) __maxnreg__((fft_line_pipe_regs<T, E, RS, K, DB>()))
    k_fft_line_pipe(const __grid_constant__ CoreDesc P, const __grid_constant__ IODesc io, int nslot, int stage_off)
{
    static_assert(!Traits<T>::kRaw, "pipelined lines carry no range scaling");
    using S2 = typename Traits<T>::S2;
    extern __shared__ __align__(16) unsigned char smraw[];
    __shared__ __align__(8) unsigned long long s_bar[2];
    cx<T> *sm = reinterpret_cast<cx<T> *>(smraw);
    S2 *stg = reinterpret_cast<S2 *>(smraw + stage_off);
    const int LS = P.LS, LSt = DB ? 2 * LS : LS;
    const int lpc = io.lpc, tpl = io.tpl;
    const int units = P.L;
    const unsigned line_bytes = (unsigned)units * (unsigned)sizeof(S2);
    const int ntiles = (int)((io.nlines + lpc - 1) / lpc);
    // tile `tile` into slot `s`: one bulk copy per line, one arrival
    auto issue = [&](int tile, int s) {
        const unsigned long long policy = l2_evict_first_policy();
        const long long l0 = (long long)tile * lpc;
        const int n = (int)min((long long)lpc, io.nlines - l0);
        mbar_arrive_expect_tx(&s_bar[s], (unsigned)n * line_bytes);
        S2 *dst = stg + (size_t)s * lpc * units;
        for (int i = 0; i < n; ++i)
            bulk_g2s(dst + (size_t)i * units, io.in + line_off(io, l0 + i, false), line_bytes, &s_bar[s], policy);
    };
    if (threadIdx.x == 0) {
        for (int s = 0; s < nslot; ++s) mbar_init(&s_bar[s], 1);
        mbar_init_fence();
        for (int s = 0; s < nslot; ++s) {
            const long long tile = blockIdx.x + (long long)s * gridDim.x;
            if (tile < ntiles) issue((int)tile, s);
        }
    }
    __syncthreads();
    int it = 0;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++it) {
        // per-thread line and position, recomputed per tile rather than kept
        // live across the stages
        const int g = threadIdx.x / tpl, t = threadIdx.x - g * tpl;
        const bool cc = K == LK_C2C && !io.fwd;
        cx<T> *const line = sm + (size_t)g * LSt;
        // the stage count is laundered per tile so that nothing derived from
        // the last stage's descriptor is hoisted out of the loop and kept live
        // across the stages
        int nst = P.nst;
        asm volatile("" : "+r"(nst));
        const int s = it % nslot;
        const unsigned par = (unsigned)(it / nslot) & 1u;
        // every thread waits for the slot (bounded); the vote is also the
        // barrier that keeps this tile's first stage behind the previous
        // tile's last-stage reads of the line buffers
        const bool ok = mbar_wait_bounded(&s_bar[s], par, kPipeWaitPolls);
        if (__syncthreads_or(!ok)) {
            if (threadIdx.x == 0) atomicAdd(&g_pipe_wait_fault, 1u);
            break;
        }
        const long long line0 = (long long)tile * lpc;
        const int nl = (int)min((long long)lpc, io.nlines - line0);
        const bool act = g < nl;
        const S2 *src0 = stg + ((size_t)s * lpc + (act ? g : 0)) * units;
        IG_LINE_EDGE_SWITCH(P.st[0].R, (line_first_sm<T, E, R_>(line, src0, P, tpl, t, act, cc)))
        __syncthreads();
        // slot s is consumed: refill it with the tile nslot steps ahead
        if (threadIdx.x == 0) {
            const long long nxt = tile + (long long)nslot * gridDim.x;
            if (nxt < ntiles) {
                fence_proxy_async_smem();
                issue((int)nxt, s);
            }
        }
        int cur = 0;
        for (int si = 1; si < nst - 1; ++si) {
            if constexpr (DB) {
                const cx<T> *a = sm + cur;
                cx<T> *b = sm + (LS - cur);
                IG_LINE_RADIX_SWITCH(P.st[si].R, (stage_db<T, E, R_>(a, b, 2 * LS, P, si, nl, tpl, g, t)))
                cur = LS - cur;
                __syncthreads();
            } else {
                IG_LINE_RADIX_SWITCH(P.st[si].R, (stage<T, E, R_>(sm, P, si, nl, tpl, g, t, LS)))
            }
        }
        OutScale<T> sc;
        sc.init(io);
        if constexpr (K == LK_R2HC) sc.f *= 0.5f;  // the split's 1/2 joins the output scale
        char *obase = io.out + (act ? line_off(io, line0 + g, true) : 0);
        const cx<T> *src = line + cur;
        if constexpr (K == LK_C2C) {
            IG_LINE_EDGE_SWITCH(P.st[nst - 1].R,
                                (line_last_c2c<T, E, R_>(src, obase, io.os, P, nst - 1, tpl, t, act, cc, sc, 0)))
        } else {
            switch (P.st[nst - 1].R) {
            case 2: line_last_r2hc<T, E, 2>(src, obase, io.os, P, nst - 1, tpl, t, act, sc, 0); break;
            case 4: line_last_r2hc<T, E, 4>(src, obase, io.os, P, nst - 1, tpl, t, act, sc, 0); break;
            case 8: line_last_r2hc<T, E, 8>(src, obase, io.os, P, nst - 1, tpl, t, act, sc, 0); break;
            case 3:
                if constexpr (rs_has<E, RS>(3)) line_last_r2hc<T, E, 3>(src, obase, io.os, P, nst - 1, tpl, t, act, sc, 0);
                break;
            case 5:
                if constexpr (rs_has<E, RS>(5)) line_last_r2hc<T, E, 5>(src, obase, io.os, P, nst - 1, tpl, t, act, sc, 0);
                break;
            default: break;
            }
        }
    }
    // a CTA that gave up still has copies in flight into its staging slots:
    // wait for them (bounded) before the shared memory is released
    if (threadIdx.x == 0) {
        for (int k = 0; k < nslot; ++k) {
            const int s = (it + k) % nslot;
            const long long tile = blockIdx.x + (long long)(it + k) * gridDim.x;
            if (tile < ntiles) mbar_wait_bounded(&s_bar[s], (unsigned)((it + k) / nslot) & 1u, kPipeWaitPolls);
        }
    }
}

template <class T, int E, bool DB, int RS, int K> static auto line_pipe_kernel()
{
    return k_fft_line_pipe<T, E, RS, K, DB>;
}

// Pipelined launch of one (arithmetic, elements per thread, buffering)
// family.  `work_bytes` = lpc line buffers; nslot staging slots of lpc lines
// follow at a 128-byte boundary; grid = SMs x resident CTAs (no more than
// the tiles).  Returns cudaErrorNotSupported for a core outside the family.
template <class T, int E, bool DB>
cudaError_t launch_line_pipe_E(const CoreDesc &d, const IODesc &io, size_t work_bytes, int nslot, int sms,
                               cudaStream_t st)
{
    if constexpr (Traits<T>::kRaw) {
        return cudaErrorNotSupported;
    } else {
        using S2 = typename Traits<T>::S2;
        const unsigned blk = (unsigned)(io.lpc * io.tpl);
        const int stage_off = (int)((work_bytes + 127) / 128 * 128);
        const size_t smem = (size_t)stage_off + (size_t)nslot * io.lpc * d.L * sizeof(S2);
        const long long ntiles = (io.nlines + io.lpc - 1) / io.lpc;
        const bool hc = io.lay == LAY_R2HC;
        void (*kern)(CoreDesc, IODesc, int, int) = nullptr;
        if (d.rs == RS_P2) kern = hc ? line_pipe_kernel<T, E, DB, RS_P2, LK_R2HC>() : line_pipe_kernel<T, E, DB, RS_P2, LK_C2C>();
        else if (E == 8 && d.rs == RS_P235)
            kern = hc ? line_pipe_kernel<T, E, DB, (E == 8 ? RS_P235 : RS_ALL), LK_R2HC>()
                      : line_pipe_kernel<T, E, DB, (E == 8 ? RS_P235 : RS_ALL), LK_C2C>();
        else if (d.rs == RS_ALL || d.rs == RS_P235)
            kern = hc ? line_pipe_kernel<T, E, DB, RS_ALL, LK_R2HC>() : line_pipe_kernel<T, E, DB, RS_ALL, LK_C2C>();
        else return cudaErrorNotSupported;
        int per_sm = 0;
        cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, (int)blk, smem);
        if (e != cudaSuccess) return e;
        if (per_sm < 1) return cudaErrorNotSupported;
        const long long grid = std::min<long long>(ntiles, (long long)per_sm * sms);
        kern<<<(unsigned)grid, blk, smem, st>>>(d, io, nslot, stage_off);
        return cudaGetLastError();
    }
}

// give-ups of this unit's pipelined waits since the last call (cleared)
template <class T, int E, bool DB> cudaError_t line_pipe_faults_E(unsigned *count)
{
    unsigned v = 0, z = 0;
    cudaError_t e = cudaMemcpyFromSymbol(&v, g_pipe_wait_fault, sizeof v);
    if (e == cudaSuccess && v) e = cudaMemcpyToSymbol(g_pipe_wait_fault, &z, sizeof z);
    *count += v;
    return e;
}

template <class K> static cudaError_t line_smem_attr(K kernel, int bytes)
{
    cudaFuncAttributes fa;
    cudaError_t e = cudaFuncGetAttributes(&fa, kernel);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes - (int)fa.sharedSizeBytes);
}
template <class T, int E, bool DB> cudaError_t set_smem_line_E(int bytes)
{
    cudaError_t e = cudaSuccess;
#define IG_SL(RS_)                                                                                        \
    if (e == cudaSuccess) e = line_smem_attr(k_fft_line<T, E, RS_, LK_C2C, DB>, bytes);                     \
    if constexpr (std::is_same<T, df>::value)                                                             \
        if (e == cudaSuccess) e = line_smem_attr(k_fft_line<T, E, RS_, LK_R2HC_S, DB>, bytes);              \
    if constexpr (!std::is_same<T, df>::value) {                                                          \
        if (e == cudaSuccess) e = line_smem_attr(k_fft_line<T, E, RS_, LK_R2HC, DB>, bytes);                \
        if (e == cudaSuccess) e = line_smem_attr(k_fft_line<T, E, RS_, LK_R2C, DB>, bytes);                 \
        if (e == cudaSuccess) e = line_smem_attr(k_fft_line<T, E, RS_, LK_C2R, DB>, bytes);                 \
        if (e == cudaSuccess) e = line_smem_attr(k_fft_line_pipe<T, E, RS_, LK_C2C, DB>, bytes);            \
        if (e == cudaSuccess) e = line_smem_attr(k_fft_line_pipe<T, E, RS_, LK_R2HC, DB>, bytes);           \
    }
    IG_SL(RS_P2)
    IG_SL(RS_ALL)
    if constexpr (E == 8) { IG_SL(RS_P235) }
#undef IG_SL
    return e;
}

}  // namespace ig
