// ig_pdf.cuh -- packed double-float complex arithmetic on Blackwell's paired
// FP32 instructions (add/sub/mul/fma .f32x2).
//
// A complex double-float value z = (re.h + re.l) + i (im.h + im.l) is held as
// two register pairs, H = (re.h, im.h) and L = (re.l, im.l).  The real and
// imaginary parts of a complex add, of a scale by a real constant and of the
// renormalisation run the same operation sequence, so one paired instruction
// does the work of two scalar ones.  The operation sequences are the scalar
// double-float ones of ig_arith.cuh (Knuth TwoSum, Dekker Fast2Sum, FMA exact
// products), lane by lane; only the lane crossings of a multiplication by
// +-i or by a complex twiddle need register moves.
//
// In shared memory a double-float complex is stored as (re.h, im.h, re.l,
// im.l), so that one 128-bit access moves both pairs without any move.
#pragma once
#include "ig_arith.cuh"

namespace ig {

#if defined(__CUDACC__)
#define IGP __device__ __forceinline__
struct f2p {
    unsigned long long v;
};
IGP f2p pk(float x, float y)
{
    f2p r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r.v) : "f"(x), "f"(y));
    return r;
}
IGP void upk(f2p a, float &x, float &y) { asm("mov.b64 {%0, %1}, %2;" : "=f"(x), "=f"(y) : "l"(a.v)); }
IGP f2p operator+(f2p a, f2p b)
{
    f2p r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
    return r;
}
IGP f2p operator-(f2p a, f2p b)
{
    f2p r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
    return r;
}
IGP f2p operator*(f2p a, f2p b)
{
    f2p r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
    return r;
}
// a * b + c, one rounding per lane
IGP f2p pfma(f2p a, f2p b, f2p c)
{
    f2p r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r.v) : "l"(a.v), "l"(b.v), "l"(c.v));
    return r;
}
#else
// host restatement (for host-side checks of the packed sequences): the same
// lane operations in scalar FP32
#define IGP inline
struct f2p {
    float x, y;
};
IGP f2p pk(float x, float y) { return f2p{x, y}; }
IGP void upk(f2p a, float &x, float &y) { x = a.x; y = a.y; }
IGP f2p operator+(f2p a, f2p b) { return f2p{IG_FADD(a.x, b.x), IG_FADD(a.y, b.y)}; }
IGP f2p operator-(f2p a, f2p b) { return f2p{IG_FSUB(a.x, b.x), IG_FSUB(a.y, b.y)}; }
IGP f2p operator*(f2p a, f2p b) { return f2p{IG_FMUL(a.x, b.x), IG_FMUL(a.y, b.y)}; }
IGP f2p pfma(f2p a, f2p b, f2p c) { return f2p{IG_FMA(a.x, b.x, c.x), IG_FMA(a.y, b.y, c.y)}; }
#endif
IGP f2p swp(f2p a)
{
    float x, y;
    upk(a, x, y);
    return pk(y, x);
}
IGP f2p bcast(float c) { return pk(c, c); }

struct pcx {
    f2p h, l;
};

// cx<df> <-> packed
IGP pcx to_p(cx<df> z) { return pcx{pk(z.r.h, z.i.h), pk(z.r.l, z.i.l)}; }
IGP cx<df> from_p(pcx z)
{
    cx<df> r;
    upk(z.h, r.r.h, r.i.h);
    upk(z.l, r.r.l, r.i.l);
    return r;
}
#if defined(__CUDACC__)
// shared-memory slot (re.h, im.h, re.l, im.l)
IGP pcx pld(const cx<df> *p)
{
    const ulonglong2 q = *reinterpret_cast<const ulonglong2 *>(p);
    return pcx{f2p{q.x}, f2p{q.y}};
}
IGP void pst(cx<df> *p, pcx z) { *reinterpret_cast<ulonglong2 *>(p) = make_ulonglong2(z.h.v, z.l.v); }
#endif

// lazy double-float add / subtract (TwoSum of the high pairs, low pairs added)
IGP pcx operator+(pcx a, pcx b)
{
    const f2p s = a.h + b.h, bb = s - a.h;
    const f2p e = (a.h - (s - bb)) + (b.h - bb);
    return pcx{s, e + (a.l + b.l)};
}
IGP pcx operator-(pcx a, pcx b)
{
    const f2p s = a.h - b.h, bb = s - a.h;
    const f2p e = (a.h - (s - bb)) - (b.h + bb);
    return pcx{s, e + (a.l - b.l)};
}
// Fast2Sum renormalisation
IGP pcx prenorm(pcx a)
{
    const f2p h = a.h + a.l;
    return pcx{h, a.l - (h - a.h)};
}
// lanes times exact constants (+-1, 1/2)
IGP pcx plane(pcx a, f2p s) { return pcx{a.h * s, a.l * s}; }
// multiply by -i (FWD) or +i: (im, -re) / (-im, re)
template <bool FWD> IGP pcx prot(pcx a)
{
    float rh, ih, rl, il;
    upk(a.h, rh, ih);
    upk(a.l, rl, il);
    return FWD ? pcx{pk(ih, -rh), pk(il, -rl)} : pcx{pk(-ih, rh), pk(-il, rl)};
}
IGP pcx pconj(pcx a)
{
    float rh, ih, rl, il;
    upk(a.h, rh, ih);
    upk(a.l, rl, il);
    return pcx{pk(rh, -ih), pk(rl, -il)};
}
// scale by the real double-float constant ch + cl (both lanes), renormalised
IGP pcx pscale(pcx a, float ch, float cl)
{
    const f2p Kh = bcast(ch), Kl = bcast(cl), nKh = bcast(-ch);
    const f2p np = a.h * nKh;         // -p, p = round(a.h ch)
    f2p e = pfma(a.h, Kh, np);        // a.h ch - p, exact
    e = pfma(a.h, Kl, e);
    e = pfma(a.l, Kh, e);
    const f2p h = e - np;             // p + e
    return pcx{h, e - (h + np)};      // e - (h - p)
}
// unrenormalised product a (ch + cl): (-np, e) with np = -round(a.h ch) and e
// its exact error plus the low terms (the renormalisation of pscale is left
// to the lazy add that consumes it)
IGP pcx pprod(pcx a, float ch, float cl)
{
    const f2p Kh = bcast(ch), Kl = bcast(cl), nKh = bcast(-ch);
    const f2p np = a.h * nKh;
    f2p e = pfma(a.h, Kh, np);
    e = pfma(a.h, Kl, e);
    e = pfma(a.l, Kh, e);
    return pcx{bcast(0.0f) - np, e};
}
// T + a (ch + cl): the product's high part enters the TwoSum directly and its
// error terms join the low parts (lazy add, no renormalisation of the product)
IGP pcx pacc(pcx T, pcx a, float ch, float cl)
{
    const f2p Kh = bcast(ch), Kl = bcast(cl), nKh = bcast(-ch);
    const f2p np = a.h * nKh;         // -p
    f2p e = pfma(a.h, Kh, np);        // a.h ch - p, exact
    e = pfma(a.h, Kl, e);
    e = pfma(a.l, Kh, e);
    const f2p s = T.h - np, bb = s - T.h;              // TwoSum(T.h, p)
    const f2p err = (T.h - (s - bb)) - (np + bb);
    return pcx{s, err + (T.l + e)};
}
// a * w with w = (wr, wi) given as the pairs W1 = (wr, wr) and W2 = (-wi, wi)
// (high and low parts) and the negated high pairs nW1 = -W1h, nW2 = -W2h:
// lanes (re, im) = a (wr, wr) + (a.im, a.re) (-wi, wi).  The lane sequence is
// the scalar df_mul_sub / df_mul_add one with the two high products formed
// negated (-p = a (-w), exactly) and the FMA error terms taken against them,
// so that no product is negated after the fact.  NORM = false returns the
// unrenormalised pair (s, T) for a lazy add to consume.
template <bool NORM = true>
IGP pcx pmulw(pcx a, f2p W1h, f2p W2h, f2p W1l, f2p W2l, f2p nW1h, f2p nW2h)
{
    const f2p ash = swp(a.h), asl = swp(a.l);
    const f2p np1 = a.h * nW1h, np2 = ash * nW2h;          // -p1, -p2
    const f2p e1 = pfma(a.h, W1h, np1), e2 = pfma(ash, W2h, np2);
    // TwoSum(-p1, -p2) = -(s, t)
    const f2p ns = np1 + np2, bb = ns - np1;
    const f2p nt = (np1 - (ns - bb)) + (np2 - bb);
    f2p T = (e1 + e2) - nt;
    T = pfma(a.h, W1l, T);
    T = pfma(a.l, W1h, T);
    T = pfma(ash, W2l, T);
    T = pfma(asl, W2h, T);
    if constexpr (!NORM) return pcx{bcast(0.0f) - ns, T};
    const f2p h = T - ns;                                    // s + T
    return pcx{h, T - (h + ns)};                             // T - (h - s)
}
// a * w, w as a cx<df>
IGP pcx pcmul(pcx a, cx<df> w)
{
    return pmulw(a, bcast(w.r.h), pk(-w.i.h, w.i.h), bcast(w.r.l), pk(-w.i.l, w.i.l), bcast(-w.r.h),
                 pk(w.i.h, -w.i.h));
}
// stage twiddle w = (wr, wi) as (wr.h, wi.h, wr.l, wi.l), 16 bytes (half the
// cache footprint of the pairs pmulw takes).  The pairs are formed in
// registers; the negations are products by `neg1` = -1, a value the kernels
// read from their parameters: a negation the compiler can see would let it
// cancel the FMA error term against the product it was taken from.
struct ptw {
    float rh, ih, rl, il;
};
#if defined(__CUDACC__)
template <bool NORM = true>
IGP pcx pmulw(pcx a, const ptw *w, float neg1)
{
    const float4 q = *reinterpret_cast<const float4 *>(w);
    const f2p m = pk(neg1, 1.0f), nn = pk(neg1, neg1);
    const f2p W1h = pk(q.x, q.x), W1l = pk(q.z, q.z);
    const f2p W2h = pk(q.y, q.y) * m, W2l = pk(q.w, q.w) * m;  // (-wi, wi)
    return pmulw<NORM>(a, W1h, W2h, W1l, W2l, W1h * nn, W2h * nn);
}
// a * w, w a cx<df> in memory (r.h, r.l, i.h, i.l), pairs formed as for ptw
template <bool NORM = true>
IGP pcx pmulw_cx(pcx a, const cx<df> *w, float neg1)
{
    const float4 q = *reinterpret_cast<const float4 *>(w);
    const f2p m = pk(neg1, 1.0f), nn = pk(neg1, neg1);
    const f2p W1h = pk(q.x, q.x), W1l = pk(q.y, q.y);
    const f2p W2h = pk(q.z, q.z) * m, W2l = pk(q.w, q.w) * m;  // (-wi, wi)
    return pmulw<NORM>(a, W1h, W2h, W1l, W2l, W1h * nn, W2h * nn);
}
#endif

// multiply by the constant c + i s (double constants split into double-float)
IGP pcx pcmulk(pcx a, double c, double s)
{
    const df C = df_const(c), S = df_const(s);
    // unrenormalised: the packed DFTs add the result lazily
    return pmulw<false>(a, bcast(C.h), pk(-S.h, S.h), bcast(C.l), pk(-S.l, S.l), bcast(-C.h), pk(S.h, -S.h));
}

// ---- packed small DFTs (forward sign only: the stages run forward) --------
IGP void pdft2(pcx &a, pcx &b)
{
    const pcx t = a;
    a = t + b;
    b = t - b;
}
IGP void pdft4(pcx &x0, pcx &x1, pcx &x2, pcx &x3)
{
    const pcx t0 = x0 + x2, t1 = x0 - x2, t2 = x1 + x3, t3 = prot<true>(x1 - x3);
    x0 = t0 + t2;
    x2 = t0 - t2;
    x1 = t1 + t3;
    x3 = t1 - t3;
}
// exp(-2 pi i/8) a = (a + rot(a)) / sqrt 2, exp(-6 pi i/8) a = (rot(a) - a) / sqrt 2
IGP pcx pw8_1(pcx a)
{
    const df h = df_const(kSqrtHalf);
    return pprod(a + prot<true>(a), h.h, h.l);  // consumed by lazy adds
}
IGP pcx pw8_3(pcx a)
{
    const df h = df_const(kSqrtHalf);
    return pprod(prot<true>(a) - a, h.h, h.l);
}
IGP void pdft8(pcx *v)
{
    pdft4(v[0], v[2], v[4], v[6]);
    pdft4(v[1], v[3], v[5], v[7]);
    const pcx o1 = pw8_1(v[3]), o2 = prot<true>(v[5]), o3 = pw8_3(v[7]);
    const pcx e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6];
    v[0] = e0 + v[1];
    v[4] = e0 - v[1];
    v[1] = e1 + o1;
    v[5] = e1 - o1;
    v[2] = e2 + o2;
    v[6] = e2 - o2;
    v[3] = e3 + o3;
    v[7] = e3 - o3;
}
IGP void pdft16(pcx *v)
{
#pragma unroll
    for (int m1 = 0; m1 < 4; ++m1) pdft4(v[m1], v[m1 + 4], v[m1 + 8], v[m1 + 12]);
    v[1 + 4 * 1] = pcmulk(v[1 + 4 * 1], kCos8, -kSin8);
    v[1 + 4 * 2] = pw8_1(v[1 + 4 * 2]);
    v[1 + 4 * 3] = pcmulk(v[1 + 4 * 3], kSin8, -kCos8);
    v[2 + 4 * 1] = pw8_1(v[2 + 4 * 1]);
    v[2 + 4 * 2] = prot<true>(v[2 + 4 * 2]);
    v[2 + 4 * 3] = pw8_3(v[2 + 4 * 3]);
    v[3 + 4 * 1] = pcmulk(v[3 + 4 * 1], kSin8, -kCos8);
    v[3 + 4 * 2] = pw8_3(v[3 + 4 * 2]);
    v[3 + 4 * 3] = pcmulk(v[3 + 4 * 3], -kCos8, kSin8);
#pragma unroll
    for (int q1 = 0; q1 < 4; ++q1) pdft4(v[4 * q1], v[4 * q1 + 1], v[4 * q1 + 2], v[4 * q1 + 3]);
    pcx t;
    t = v[1]; v[1] = v[4]; v[4] = t;
    t = v[2]; v[2] = v[8]; v[8] = t;
    t = v[3]; v[3] = v[12]; v[12] = t;
    t = v[6]; v[6] = v[9]; v[9] = t;
    t = v[7]; v[7] = v[13]; v[13] = t;
    t = v[11]; v[11] = v[14]; v[14] = t;
}
template <int P> IGP void pdft_odd(pcx *v)
{
    constexpr int H = (P - 1) / 2;
    pcx a[H], b[H];
#pragma unroll
    for (int k = 1; k <= H; ++k) {
        a[k - 1] = v[k] + v[P - k];
        b[k - 1] = v[k] - v[P - k];
    }
    const pcx x0 = v[0];
    pcx sum = x0;
#pragma unroll
    for (int k = 0; k < H; ++k) sum = sum + a[k];
#pragma unroll
    for (int q = 1; q <= H; ++q) {
        pcx T = x0, U;
#pragma unroll
        for (int k = 1; k <= H; ++k) {
            const int j = (k * q) % P;
            const int jj = j <= H ? j : P - j;
            const df ck = df_const(odd_cos(P, jj));
            const df sk = df_const(j <= H ? odd_sin(P, jj) : -odd_sin(P, jj));
            T = pacc(T, a[k - 1], ck.h, ck.l);
            U = k == 1 ? pprod(b[k - 1], sk.h, sk.l) : pacc(U, b[k - 1], sk.h, sk.l);
        }
        // forward: V_q = T - i U, V_{P-q} = T + i U
        const pcx iU = prot<true>(U);
        v[q] = T + iU;
        v[P - q] = T - iU;
    }
    v[0] = sum;
}
IGP void pdft3r(pcx &a, pcx &b, pcx &c)
{
    pcx t[3] = {a, b, c};
    pdft_odd<3>(t);
    a = t[0];
    b = t[1];
    c = t[2];
}
// radix 9 as 3 x 3 (scheme of dft9 in ig_dft.cuh), forward
IGP void pdft9(pcx *v)
{
#pragma unroll
    for (int m1 = 0; m1 < 3; ++m1) pdft3r(v[m1], v[m1 + 3], v[m1 + 6]);
    v[1 + 3 * 1] = pcmulk(v[1 + 3 * 1], kC9_1, -kS9_1);
    v[1 + 3 * 2] = pcmulk(v[1 + 3 * 2], kC9_2, -kS9_2);
    v[2 + 3 * 1] = pcmulk(v[2 + 3 * 1], kC9_2, -kS9_2);
    v[2 + 3 * 2] = pcmulk(v[2 + 3 * 2], kC9_4, -kS9_4);
#pragma unroll
    for (int q1 = 0; q1 < 3; ++q1) pdft3r(v[3 * q1], v[3 * q1 + 1], v[3 * q1 + 2]);
    pcx t;
    t = v[1]; v[1] = v[3]; v[3] = t;
    t = v[2]; v[2] = v[6]; v[6] = t;
    t = v[5]; v[5] = v[7]; v[7] = t;
}
template <int R> IGP void pdft(pcx *v)
{
    if constexpr (R == 2) pdft2(v[0], v[1]);
    else if constexpr (R == 4) pdft4(v[0], v[1], v[2], v[3]);
    else if constexpr (R == 8) pdft8(v);
    else if constexpr (R == 16) pdft16(v);
    else if constexpr (R == 9) pdft9(v);
    else pdft_odd<R>(v);
}


}  // namespace ig
