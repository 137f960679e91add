// ig_pair.cuh -- k_fft_pair: FP32 Stockham lines with two butterflies per
// thread in the two lanes of Blackwell's paired FP32 instructions.
//
// The FP32 line kernel k_fft_line spends most of its ~136 instructions per
// complex point on scalar FP32 adds and products and on per-butterfly index
// arithmetic.  Here a thread runs butterflies j and j + 1 of a stage together:
// a value is cx<f2p>, the real parts of both butterflies' inputs in one
// 64-bit register pair and the imaginary parts in another, so every complex
// add, twiddle product and constant scaling of both butterflies is one
// add / mul / fma .f32x2 per component, and the index arithmetic is shared.
//
// Shared memory holds a line as 16-byte groups: group g has the real parts of
// elements 2g and 2g + 1, then their imaginary parts, so the two lanes of a
// stage's input m (elements j + m nr and j + 1 + m nr, j even, nr even) are
// one 128-bit load, and its outputs q ns R + k + m ns (k even, ns even) one
// 128-bit store.  One group of padding follows every eight, which keeps
// the 128-bit accesses of the radix-8/4/2 stages free of bank conflicts.
//
// Stages (the core's Stockham plan, radices 2/3/4/5/8 and the odd ones of
// the kernel's class):
//   * first stage (ns = 1) one butterfly per lane slot: units j + m nr read
//     from HBM (coalesced), scalar FP32 DFT, outputs j R + m written as
//     groups (two consecutive outputs per 128-bit store);
//   * middle stages in pairs through the two line buffers;
//   * last stage of a complex line (pocketfft::c2c, pocketfft_hdronly.h:3272):
//     pairs, outputs j + m nr and j + 1 + m nr interleaved into one 16-byte
//     HBM store; of an even real line written as halfcomplex (rfft_forward,
//     impulse/fft/c_pocketfft/pocketfft.c:2184): the last stage writes the
//     complex spectrum Z of the N/2-point transform to the other buffer, and
//     the real split X[k] = (Z[k] + conj Z[M-k]) / 2 - i w^k (Z[k] - conj
//     Z[M-k]) / 2, X[M-k] = conj(...) runs in pairs k, k + 1 with their
//     partners M - k, M - k - 1, written as halfcomplex.
// Requirements (checked by the host): FP32, first radix even (so ns is even
// in every later stage), L / R even in every later stage, radices <= 8 or
// odd, contiguous units in and out, output line starts 16-byte aligned
// (complex) or 8-byte aligned (halfcomplex).
#pragma once
#include "ig_line.cuh"

namespace ig {

template <> struct RealOps<f2p> {
    static __device__ __forceinline__ f2p k(double c) { return bcast((float)c); }
};
__device__ __forceinline__ f2p operator-(f2p a) { return a * bcast(-1.0f); }

using PV = cx<f2p>;  // lanes: butterfly j, butterfly j + 1

// padded group index
__device__ __forceinline__ int pgi(int g) { return g + (g >> 3); }

__device__ __forceinline__ PV pv_ld(const float4 *buf, int g)
{
    const ulonglong2 q = *reinterpret_cast<const ulonglong2 *>(buf + pgi(g));
    return PV{f2p{q.x}, f2p{q.y}};
}
__device__ __forceinline__ void pv_st(float4 *buf, int g, PV v)
{
    *reinterpret_cast<ulonglong2 *>(buf + pgi(g)) = make_ulonglong2(v.r.v, v.i.v);
}

// pair twiddle table: per stage from float4 offset P.st[s].twp (stages after
// the first), entry kp (R - 1) + m - 1 = {wr(2kp m), wr((2kp + 1) m), wi(2kp m),
// wi((2kp + 1) m)} of w(x) = exp(-2 pi i x / (ns R))
__device__ __forceinline__ PV pv_tw(const float4 *t, int e)
{
    const ulonglong2 q = __ldg(reinterpret_cast<const ulonglong2 *>(t + e));
    return PV{f2p{q.x}, f2p{q.y}};
}
// a * w: re = a.r wr - a.i wi, im = a.r wi + a.i wr
__device__ __forceinline__ PV pv_mul(PV a, PV w)
{
    const f2p nwi = -w.i;
    return PV{pfma(a.r, w.r, a.i * nwi), pfma(a.i, w.r, a.r * w.i)};
}

// lanes (x, y) of a pair -> (x0, y0, x1, y1) as float4 (interleaved complex)
__device__ __forceinline__ float4 pv_interleave(PV v)
{
    float r0, r1, i0, i1;
    upk(v.r, r0, r1);
    upk(v.i, i0, i1);
    return make_float4(r0, i0, r1, i1);
}

// First stage, butterflies j = t + i tpl (one per slot): units j + m nr from
// HBM, DFT, outputs j R + m (R even) as groups (j R + m) / 2.
template <int E, int R>
__device__ __forceinline__ void pair_first(float4 *dst, const char *base, int nr, int tpl, int t, bool cc,
                                           const char *pf)
{
    constexpr int NB = (E + R - 1) / R;
    float2 raw[NB][R];
#pragma unroll
    for (int i = 0; i < NB; ++i) {
        const int j = t + i * tpl;
        if (j < nr) {
            const float2 *p = reinterpret_cast<const float2 *>(base) + j;
#pragma unroll
            for (int m = 0; m < R; ++m) raw[i][m] = __ldcs(p + m * nr);
        }
    }
    // the same points of a line a wave of CTAs ahead, into L2
    if (pf) {
#pragma unroll
        for (int i = 0; i < NB; ++i) {
            const int j = t + i * tpl;
            if (j < nr) {
                const float2 *p = reinterpret_cast<const float2 *>(pf) + j;
#pragma unroll
                for (int m = 0; m < R; ++m) asm volatile("prefetch.global.L2 [%0];" ::"l"(p + m * nr));
            }
        }
    }
#pragma unroll
    for (int i = 0; i < NB; ++i) {
        const int j = t + i * tpl;
        if (j < nr) {
            cx<float> v[R];
#pragma unroll
            for (int m = 0; m < R; ++m) v[m] = cx<float>{raw[i][m].x, cc ? -raw[i][m].y : raw[i][m].y};
            dft<R, true>(v);
            const int g0 = j * (R / 2);
#pragma unroll
            for (int m = 0; m < R; m += 2)
                pv_st(dst, g0 + m / 2, PV{pk(v[m].r, v[m + 1].r), pk(v[m].i, v[m + 1].i)});
        }
    }
}

// Middle stage (ns even, nr even): pair p = butterflies 2p, 2p + 1.
template <int E, int R>
__device__ __forceinline__ void pair_mid(const float4 *src, float4 *dst, const float4 *tw, int L, int ns, FastDiv fns,
                                         int tpl, int t)
{
    constexpr int NP = (E + 2 * R - 1) / (2 * R);
    const int nr = L / R, hp = nr / 2, hns = ns / 2;
#pragma unroll
    for (int i = 0; i < NP; ++i) {
        const int p = t + i * tpl;
        if (p < hp) {
            PV v[R];
#pragma unroll
            for (int m = 0; m < R; ++m) v[m] = pv_ld(src, p + m * hp);
            const int j = 2 * p;
            const int q = (int)fdiv((unsigned)j, fns), k = j - q * ns;
            // lanes k, k + 1 (k even); the table's k = 0 lane is exactly 1 + 0i
            const int e0 = (k >> 1) * (R - 1) - 1;
#pragma unroll
            for (int m = 1; m < R; ++m) v[m] = pv_mul(v[m], pv_tw(tw, e0 + m));
            dft<R, true>(v);
            const int g0 = (q * ns * R + k) >> 1;
#pragma unroll
            for (int m = 0; m < R; ++m) pv_st(dst, g0 + m * hns, v[m]);
        }
        asm volatile("" ::: "memory");
    }
}

// Last stage of a complex line: pair p reads like pair_mid; outputs
// j + m nr (k = j, q = 0) go to HBM as interleaved pairs.
template <int E, int R>
__device__ __forceinline__ void pair_last_c2c(const float4 *src, char *obase, const float4 *tw, int L, int tpl, int t,
                                              bool cc, float fs)
{
    constexpr int NP = (E + 2 * R - 1) / (2 * R);
    const int nr = L / R, hp = nr / 2;
    const f2p sr = bcast(fs), si = bcast(cc ? -fs : fs);
#pragma unroll
    for (int i = 0; i < NP; ++i) {
        const int p = t + i * tpl;
        if (p < hp) {
            PV v[R];
#pragma unroll
            for (int m = 0; m < R; ++m) v[m] = pv_ld(src, p + m * hp);
            const int e0 = p * (R - 1) - 1;
#pragma unroll
            for (int m = 1; m < R; ++m) v[m] = pv_mul(v[m], pv_tw(tw, e0 + m));
            dft<R, true>(v);
            float4 *o = reinterpret_cast<float4 *>(obase) + p;
#pragma unroll
            for (int m = 0; m < R; ++m) __stcs(o + m * hp, pv_interleave(PV{v[m].r * sr, v[m].i * si}));
        }
        asm volatile("" ::: "memory");
    }
}

// four consecutive floats at float index `pos` (odd) of a halfcomplex line
__device__ __forceinline__ void st_hc4(float *o, int pos, float a, float b, float c, float d)
{
    __stcs(o + pos, a);
    __stcs(reinterpret_cast<float2 *>(o + pos + 1), make_float2(b, c));
    __stcs(o + pos + 3, d);
}

// Real split of an even real line of N = 2M reals from Z (complex spectrum
// of the M-point transform, group layout), pairs k = 2c, 2c + 1 with
// partners M - k, M - k - 1 (indices mod M), for k <= M / 2; halfcomplex out.
// sc = fct / 2.
__device__ __forceinline__ void pair_split(const float4 *z, char *obase, const float2 *rtw, int M, int tpl, int t,
                                           float sc)
{
    const int npair = M / 4 + 1;  // k = 0, 2, ..., covering k <= M / 2
    const f2p half = bcast(sc);
    float *o = reinterpret_cast<float *>(obase);
    for (int c = t; c < npair; c += tpl) {
        const int k = 2 * c;
        if (k > M / 2) break;
        const PV a = pv_ld(z, c);  // Z[k], Z[k + 1]
        // partners Z[(M - k) mod M] (lane 0 of group (M - k) / 2, or of group
        // 0 for k = 0) and Z[M - k - 1] (lane 1 of group (M - k) / 2 - 1):
        // two 128-bit loads, consecutive threads on consecutive groups
        const int gh = (M - k) >> 1;
        const float4 G1 = z[pgi(k == 0 ? 0 : gh)], G0 = z[pgi(gh - 1)];
        const PV cb = PV{pk(G1.x, G0.y), pk(-G1.z, -G0.w)};  // conj b
        const float4 w4 = __ldg(reinterpret_cast<const float4 *>(rtw + k));  // w^k, w^(k+1)
        const PV w = PV{pk(w4.x, w4.z), pk(w4.y, w4.w)};
        const PV Ev = a + cb, D = a - cb;
        // T = w (-i D) = w (D.i, -D.r)
        const PV Tm = pv_mul(PV{D.i, -D.r}, w);
        const PV X = Ev + Tm, Y = Ev - Tm;  // X[k], conj X[M - k]
        float xr0, xr1, xi0, xi1, yr0, yr1, yi0, yi1;
        upk(X.r * half, xr0, xr1);
        upk(X.i * half, xi0, xi1);
        upk(Y.r * half, yr0, yr1);
        upk(Y.i * half, yi0, yi1);
        // X[M - k] = conj(Y lane 0), X[M - k - 1] = conj(Y lane 1)
        if (k == 0) {
            // X[0] (real), X[1]; X[M] (real), X[M - 1]
            __stcs(o, xr0);
            __stcs(o + 1, xr1);
            __stcs(o + 2, xi1);
            __stcs(o + 2 * M - 1, yr0);
            __stcs(o + 2 * M - 3, yr1);
            __stcs(o + 2 * M - 2, -yi1);
        } else if (2 * k == M) {
            // X[M/2] alone (lane 1 and the partners belong to pair k - 2)
            __stcs(o + 2 * k - 1, xr0);
            __stcs(o + 2 * k, xi0);
        } else {
            st_hc4(o, 2 * k - 1, xr0, xi0, xr1, xi1);
            // X[M - k - 1] at 2 (M - k - 1) - 1, then X[M - k]
            st_hc4(o, 2 * (M - k) - 3, yr1, -yi1, yr0, -yi0);
        }
    }
}

// The same split to the half spectrum of r2c: X[k], k = 0..M, as complex
// units (DC and Nyquist imaginary parts 0), conjugated when cj (a backward
// r2c); 8-byte stores, since a line of M + 1 units starts 16-byte aligned
// only every other line.  sc = fct / 2.
__device__ __forceinline__ void pair_split_c(const float4 *z, char *obase, const float2 *rtw, int M, int tpl, int t,
                                             float sc, bool cj)
{
    const int npair = M / 4 + 1;
    const f2p half = bcast(sc);
    const float sg = cj ? -1.0f : 1.0f;
    float2 *o = reinterpret_cast<float2 *>(obase);
    for (int c = t; c < npair; c += tpl) {
        const int k = 2 * c;
        if (k > M / 2) break;
        const PV a = pv_ld(z, c);
        const int gh = (M - k) >> 1;
        const float4 G1 = z[pgi(k == 0 ? 0 : gh)], G0 = z[pgi(gh - 1)];
        const PV cb = PV{pk(G1.x, G0.y), pk(-G1.z, -G0.w)};
        const float4 w4 = __ldg(reinterpret_cast<const float4 *>(rtw + k));
        const PV w = PV{pk(w4.x, w4.z), pk(w4.y, w4.w)};
        const PV Ev = a + cb, D = a - cb;
        const PV Tm = pv_mul(PV{D.i, -D.r}, w);
        const PV X = Ev + Tm, Y = Ev - Tm;  // X[k], X[k + 1]; conj X[M - k], conj X[M - k - 1]
        float xr0, xr1, xi0, xi1, yr0, yr1, yi0, yi1;
        upk(X.r * half, xr0, xr1);
        upk(X.i * half, xi0, xi1);
        upk(Y.r * half, yr0, yr1);
        upk(Y.i * half, yi0, yi1);
        if (k == 0) {
            __stcs(o, make_float2(xr0, 0.0f));
            __stcs(o + 1, make_float2(xr1, sg * xi1));
            __stcs(o + M, make_float2(yr0, 0.0f));
            __stcs(o + M - 1, make_float2(yr1, -sg * yi1));
        } else if (2 * k == M) {
            __stcs(o + k, make_float2(xr0, sg * xi0));
        } else {
            __stcs(o + k, make_float2(xr0, sg * xi0));
            __stcs(o + k + 1, make_float2(xr1, sg * xi1));
            __stcs(o + M - k - 1, make_float2(yr1, -sg * yi1));
            __stcs(o + M - k, make_float2(yr0, -sg * yi0));
        }
    }
}

// register cap: the 16-element pairs fit in 64 registers (a few spilled
// bytes in the 7/11 class), which allows 32 resident warps per SM
constexpr int kPairRegs = 64;

constexpr int PK_C2C = 0, PK_R2HC = 1, PK_R2C = 2;

#define IG_PAIR_RADIX_SWITCH(RV, CALL)                                                 \
    switch (RV) {                                                                       \
    case 2: { constexpr int R_ = 2; CALL; } break;                                      \
    case 4: { constexpr int R_ = 4; CALL; } break;                                      \
    case 8: { constexpr int R_ = 8; CALL; } break;                                      \
    case 3: if constexpr (RS >= RS_P235) { constexpr int R_ = 3; CALL; } break;         \
    case 5: if constexpr (RS >= RS_P235) { constexpr int R_ = 5; CALL; } break;         \
    case 9: if constexpr (RS >= RS_P235) { constexpr int R_ = 9; CALL; } break;         \
    case 7: if constexpr (RS >= RS_ALL) { constexpr int R_ = 7; CALL; } break;          \
    case 11: if constexpr (RS >= RS_ALL) { constexpr int R_ = 11; CALL; } break;        \
    default: break;                                                                     \
    }

// One CTA: lpc lines of tpl = L / 16 threads; shared memory lpc x 2 buffers of
// GS = pgi(L / 2 - 1) + 1 groups.
template <int RS, int K>
__device__ __forceinline__ void pair_rest(const CoreDesc &P, const IODesc &io, float4 *bufA, float4 *bufB,
                                          long long line0, int g, int t, bool act, bool cc);

template <int RS, int K>
__global__ void __maxnreg__(kPairRegs)
    k_fft_pair(const __grid_constant__ CoreDesc P, const __grid_constant__ IODesc io, int GS)
{
    constexpr int E = 16;
    extern __shared__ __align__(16) unsigned char smraw[];
    float4 *sm = reinterpret_cast<float4 *>(smraw);
    const int lpc = io.lpc, tpl = io.tpl, L = P.L;
    const long long line0 = (long long)blockIdx.x * lpc;
    const int nl = (int)min((long long)lpc, io.nlines - line0);
    const int g = threadIdx.x / tpl, t = threadIdx.x - g * tpl;
    const bool act = g < nl;
    const bool cc = K == PK_C2C && !io.fwd;
    float4 *bufA = sm + (size_t)(act ? g : 0) * 2 * GS, *bufB = bufA + GS;
    const char *ibase = io.in + (act ? line_off(io, line0 + g, false) : 0);
    const char *pf = io.pf_lines && act && line0 + g + io.pf_lines < io.nlines
                         ? io.in + line_off(io, line0 + g + io.pf_lines, false)
                         : nullptr;
    if (act) {
        const int nr0 = L / P.st[0].R;
        switch (P.st[0].R) {
        case 2: pair_first<E, 2>(bufA, ibase, nr0, tpl, t, cc, pf); break;
        case 4: pair_first<E, 4>(bufA, ibase, nr0, tpl, t, cc, pf); break;
        case 8: pair_first<E, 8>(bufA, ibase, nr0, tpl, t, cc, pf); break;
        default: break;
        }
    }
    __syncthreads();
    pair_rest<RS, K>(P, io, bufA, bufB, line0, g, t, act, cc);
}

// stages after the first (middle stages, last stage to HBM or split); the
// first stage's output is in bufA
template <int RS, int K>
__device__ __forceinline__ void pair_rest(const CoreDesc &P, const IODesc &io, float4 *bufA, float4 *bufB,
                                          long long line0, int g, int t, bool act, bool cc)
{
    constexpr int E = 16;
    const int tpl = io.tpl, L = P.L;
    const float4 *twp = reinterpret_cast<const float4 *>(P.twp);
    const float2 *rtw = reinterpret_cast<const float2 *>(P.rtw);
    float4 *src = bufA, *dst = bufB;
    const int nst = P.nst;
    for (int s = 1; s < nst - 1; ++s) {
        if (act) {
            const float4 *tw = twp + P.st[s].twp;
            IG_PAIR_RADIX_SWITCH(P.st[s].R, (pair_mid<E, R_>(src, dst, tw, L, P.st[s].ns, P.st[s].fns, tpl, t)))
        }
        float4 *x = src;
        src = dst;
        dst = x;
        __syncthreads();
    }
    char *obase = io.out + (act ? line_off(io, line0 + g, true) : 0);
    const float4 *tw = twp + P.st[nst - 1].twp;
    if constexpr (K == PK_C2C) {
        if (act) IG_PAIR_RADIX_SWITCH(P.st[nst - 1].R, (pair_last_c2c<E, R_>(src, obase, tw, L, tpl, t, cc, io.fct_f)))
    } else {
        // last stage into the other buffer (the spectrum Z), then the split
        if (act) {
            const int s = nst - 1;
            IG_PAIR_RADIX_SWITCH(P.st[s].R, (pair_mid<E, R_>(src, dst, tw, L, P.st[s].ns, P.st[s].fns, tpl, t)))
        }
        __syncthreads();
        if (act) {
            if constexpr (K == PK_R2HC) pair_split(dst, obase, rtw, L, tpl, t, 0.5f * io.fct_f);
            else pair_split_c(dst, obase, rtw, L, tpl, t, 0.5f * io.fct_f, io.conj_out != 0);
        }
    }
}

// stage twiddles in pair form (see pv_tw); ns even
__global__ void k_gen_stage_twp(float4 *tw, int R, int ns)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (ns / 2) * (R - 1)) return;
    const int kp = e / (R - 1), m = e % (R - 1) + 1;
    const unsigned long long D = (unsigned long long)ns * R;
    double2 a = exp2pi_frac((unsigned long long)m * (2 * kp), D);
    double2 b = exp2pi_frac((unsigned long long)m * (2 * kp + 1), D);
    tw[e] = make_float4((float)a.x, (float)b.x, (float)-a.y, (float)-b.y);
}

}  // namespace ig
