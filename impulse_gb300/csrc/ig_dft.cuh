// ig_dft.cuh -- register-resident small DFTs (radix 2, 3, 4, 5, 7, 8, 9, 11, 13, 16).
//
// dft<R, FWD>(v) replaces v[0..R) by V[q] = sum_m v[m] exp(-+2 pi i m q / R)
// (minus sign for the forward transform), the codelet set that PocketFFT's
// passes cover (impulse/fft/c_pocketfft/pocketfft.c:300-865 for radix
// 2/3/4/5/7/11; impulse/fft/cpp_pocketfft/pocketfft_hdronly.h:727-1305 adds
// radix 8).  Radices 9 (as 3 x 3), 13 and 16 are new here.  The odd prime radices use the symmetric
// pair form: with a_k = v_k + v_{R-k} and b_k = v_k - v_{R-k},
//   V_q = v_0 + sum_k a_k cos(2 pi k q/R) -+ i sum_k b_k sin(2 pi k q/R),
// and V_{R-q} the same with the sign of the second sum flipped.
#pragma once
#include "ig_arith.cuh"

namespace ig {

// cos / sin (2 pi k / P), k = 1 .. (P-1)/2, from a 25-digit evaluation
IGD constexpr double odd_cos(int P, int k)
{
    return P == 3 ? -0.5
         : P == 5 ? (k == 1 ? 0.3090169943749474241022934 : -0.8090169943749474241022934)
         : P == 7 ? (k == 1 ? 0.6234898018587335305250049 : k == 2 ? -0.2225209339563144042889026
                                                                     : -0.9009688679024191262361023)
         : P == 11 ? (k == 1 ? 0.8412535328311811688618117 : k == 2 ? 0.4154150130018864255292741
            : k == 3 ? -0.1423148382732851404437927 : k == 4 ? -0.6548607339452850640569251
                                                              : -0.9594929736144973898903681)
         : (k == 1 ? 0.8854560256532098959003755 : k == 2 ? 0.5680647467311558025118076
            : k == 3 ? 0.1205366802553230533490677 : k == 4 ? -0.3546048870425356259696379
            : k == 5 ? -0.7485107481711010986346306 : -0.9709418174260520271569823);
}
IGD constexpr double odd_sin(int P, int k)
{
    return P == 3 ? 0.8660254037844386467637232
         : P == 5 ? (k == 1 ? 0.9510565162951535721164393 : 0.5877852522924731291687060)
         : P == 7 ? (k == 1 ? 0.7818314824680298087084445 : k == 2 ? 0.9749279121818236070181317
                                                                     : 0.4338837391175581204757683)
         : P == 11 ? (k == 1 ? 0.5406408174555975821076360 : k == 2 ? 0.9096319953545183714117154
            : k == 3 ? 0.9898214418809327323760920 : k == 4 ? 0.7557495743542582837740358
                                                             : 0.2817325568414296977114179)
         : (k == 1 ? 0.4647231720437685456560153 : k == 2 ? 0.8229838658936563945796174
            : k == 3 ? 0.9927088740980539928007516 : k == 4 ? 0.9350162426854148234397846
            : k == 5 ? 0.6631226582407952023767855 : 0.2393156642875577671487537);
}

constexpr double kSqrtHalf = 0.7071067811865475244008444;
constexpr double kCos8 = 0.9238795325112867561281832;  // cos(pi/8)
constexpr double kSin8 = 0.3826834323650897717284600;  // sin(pi/8)

template <bool FWD, class R> IGD void dft2(cx<R> &a, cx<R> &b)
{
    cx<R> t = a;
    a = t + b;
    b = t - b;
}

template <bool FWD, class R> IGD void dft4(cx<R> &x0, cx<R> &x1, cx<R> &x2, cx<R> &x3)
{
    cx<R> t0 = x0 + x2, t1 = x0 - x2, t2 = x1 + x3, t3 = rot<FWD>(x1 - x3);
    x0 = t0 + t2;
    x2 = t0 - t2;
    x1 = t1 + t3;
    x3 = t1 - t3;
}

// multiply by exp(-+2 pi i e/8) for e = 1, 3 (e = 2 is rot)
template <bool FWD, class R> IGD cx<R> w8_1(cx<R> a)
{
    const R h = RealOps<R>::k(kSqrtHalf);
    if (FWD) return cx<R>{(a.r + a.i) * h, (a.i - a.r) * h};
    return cx<R>{(a.r - a.i) * h, (a.i + a.r) * h};
}
template <bool FWD, class R> IGD cx<R> w8_3(cx<R> a)
{
    const R h = RealOps<R>::k(kSqrtHalf);
    if (FWD) return cx<R>{(a.i - a.r) * h, (-(a.r + a.i)) * h};
    return cx<R>{(-(a.r + a.i)) * h, (a.r - a.i) * h};
}

// general constant complex multiply by (cr + i ci)
template <class R> IGD cx<R> cmulk(cx<R> a, R cr, R ci) { return cx<R>{a.r * cr - a.i * ci, a.r * ci + a.i * cr}; }

template <bool FWD, class R> IGD void dft8(cx<R> *v)
{
    // even / odd split: E = DFT4(v0, v2, v4, v6), O = DFT4(v1, v3, v5, v7)
    dft4<FWD>(v[0], v[2], v[4], v[6]);
    dft4<FWD>(v[1], v[3], v[5], v[7]);
    cx<R> o1 = w8_1<FWD>(v[3]), o2 = rot<FWD>(v[5]), o3 = w8_3<FWD>(v[7]);
    cx<R> e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6];
    v[0] = e0 + v[1];
    v[4] = e0 - v[1];
    v[1] = e1 + o1;
    v[5] = e1 - o1;
    v[2] = e2 + o2;
    v[6] = e2 - o2;
    v[3] = e3 + o3;
    v[7] = e3 - o3;
}

// radix 16 as 4 x 4: inner DFT4 over m2 of v[m1 + 4 m2], twiddle by
// w16^(m1 q1), outer DFT4 over m1; V[q1 + 4 q2].
template <bool FWD, class R> IGD void dft16(cx<R> *v)
{
#pragma unroll
    for (int m1 = 0; m1 < 4; ++m1) dft4<FWD>(v[m1], v[m1 + 4], v[m1 + 8], v[m1 + 12]);
    // now v[m1 + 4 q1] = Y[m1][q1]
    // w16^1 = (c, -+s), w16^2 = w8^1, w16^3 = (s, -+c), w16^4 = -+i, w16^6 = w8^3,
    // w16^9 = (-c, +-s), with c = cos(pi/8), s = sin(pi/8)
    const R c = RealOps<R>::k(kCos8), s = RealOps<R>::k(kSin8);
    const R w1i = RealOps<R>::k(FWD ? -kSin8 : kSin8);
    const R w3i = RealOps<R>::k(FWD ? -kCos8 : kCos8);
    const R w9r = RealOps<R>::k(-kCos8);
    const R w9i = RealOps<R>::k(FWD ? kSin8 : -kSin8);
    v[1 + 4 * 1] = cmulk(v[1 + 4 * 1], c, w1i);
    v[1 + 4 * 2] = w8_1<FWD>(v[1 + 4 * 2]);
    v[1 + 4 * 3] = cmulk(v[1 + 4 * 3], s, w3i);
    v[2 + 4 * 1] = w8_1<FWD>(v[2 + 4 * 1]);
    v[2 + 4 * 2] = rot<FWD>(v[2 + 4 * 2]);
    v[2 + 4 * 3] = w8_3<FWD>(v[2 + 4 * 3]);
    v[3 + 4 * 1] = cmulk(v[3 + 4 * 1], s, w3i);
    v[3 + 4 * 2] = w8_3<FWD>(v[3 + 4 * 2]);
    v[3 + 4 * 3] = cmulk(v[3 + 4 * 3], w9r, w9i);
#pragma unroll
    for (int q1 = 0; q1 < 4; ++q1) dft4<FWD>(v[4 * q1], v[4 * q1 + 1], v[4 * q1 + 2], v[4 * q1 + 3]);
    // v[4 q1 + q2] = V[q1 + 4 q2] -> transpose the 4x4 index
    cx<R> t;
    t = v[1]; v[1] = v[4]; v[4] = t;
    t = v[2]; v[2] = v[8]; v[8] = t;
    t = v[3]; v[3] = v[12]; v[12] = t;
    t = v[6]; v[6] = v[9]; v[9] = t;
    t = v[7]; v[7] = v[13]; v[13] = t;
    t = v[11]; v[11] = v[14]; v[14] = t;
}

// radix 9 as 3 x 3 (the dft16 scheme): inner DFT3 over m2 of v[m1 + 3 m2],
// twiddle by w9^(m1 q1), outer DFT3 over m1; V[q1 + 3 q2]
constexpr double kC9_1 = 0.7660444431189780352023927, kS9_1 = 0.6427876096865393263226434;
constexpr double kC9_2 = 0.1736481776669303488517166, kS9_2 = 0.9848077530122080593667430;
constexpr double kC9_4 = -0.9396926207859083840541093, kS9_4 = 0.3420201433256687330440996;
template <int P, bool FWD, class R> IGD void dft_odd(cx<R> *v);
template <bool FWD, class R> IGD void dft3r(cx<R> &a, cx<R> &b, cx<R> &c)
{
    cx<R> t[3] = {a, b, c};
    dft_odd<3, FWD>(t);
    a = t[0];
    b = t[1];
    c = t[2];
}
template <bool FWD, class R> IGD void dft9(cx<R> *v)
{
#pragma unroll
    for (int m1 = 0; m1 < 3; ++m1) dft3r<FWD>(v[m1], v[m1 + 3], v[m1 + 6]);
    // now v[m1 + 3 q1] = Y[m1][q1]
    constexpr double sg = FWD ? -1.0 : 1.0;
    v[1 + 3 * 1] = cmulk(v[1 + 3 * 1], RealOps<R>::k(kC9_1), RealOps<R>::k(sg * kS9_1));
    v[1 + 3 * 2] = cmulk(v[1 + 3 * 2], RealOps<R>::k(kC9_2), RealOps<R>::k(sg * kS9_2));
    v[2 + 3 * 1] = cmulk(v[2 + 3 * 1], RealOps<R>::k(kC9_2), RealOps<R>::k(sg * kS9_2));
    v[2 + 3 * 2] = cmulk(v[2 + 3 * 2], RealOps<R>::k(kC9_4), RealOps<R>::k(sg * kS9_4));
#pragma unroll
    for (int q1 = 0; q1 < 3; ++q1) dft3r<FWD>(v[3 * q1], v[3 * q1 + 1], v[3 * q1 + 2]);
    // v[3 q1 + q2] = V[q1 + 3 q2] -> transpose the 3x3 index
    cx<R> t;
    t = v[1]; v[1] = v[3]; v[3] = t;
    t = v[2]; v[2] = v[6]; v[6] = t;
    t = v[5]; v[5] = v[7]; v[7] = t;
}

template <int P, bool FWD, class R> IGD void dft_odd(cx<R> *v)
{
    constexpr int H = (P - 1) / 2;
    cx<R> a[H], b[H];
#pragma unroll
    for (int k = 1; k <= H; ++k) {
        a[k - 1] = v[k] + v[P - k];
        b[k - 1] = v[k] - v[P - k];
    }
    cx<R> x0 = v[0];
    cx<R> sum = x0;
#pragma unroll
    for (int k = 0; k < H; ++k) sum = sum + a[k];
#pragma unroll
    for (int q = 1; q <= H; ++q) {
        cx<R> T = x0, U;
#pragma unroll
        for (int k = 1; k <= H; ++k) {
            int j = (k * q) % P;  // cos(2 pi j/P) = cos(2 pi (P-j)/P), sin flips sign
            int jj = j <= H ? j : P - j;
            double cs = odd_cos(P, jj);
            double sn = j <= H ? odd_sin(P, jj) : -odd_sin(P, jj);
            R ck = RealOps<R>::k(cs), sk = RealOps<R>::k(sn);
            T = T + cx<R>{a[k - 1].r * ck, a[k - 1].i * ck};
            if (k == 1) U = cx<R>{b[0].r * sk, b[0].i * sk};
            else U = U + cx<R>{b[k - 1].r * sk, b[k - 1].i * sk};
        }
        // forward: V_q = T - i U, V_{P-q} = T + i U
        cx<R> iU = cx<R>{-U.i, U.r};
        if (FWD) {
            v[q] = T - iU;
            v[P - q] = T + iU;
        } else {
            v[q] = T + iU;
            v[P - q] = T - iU;
        }
    }
    v[0] = sum;
}

template <int R, bool FWD, class T> IGD void dft(cx<T> *v)
{
    if constexpr (R == 2) dft2<FWD>(v[0], v[1]);
    else if constexpr (R == 4) dft4<FWD>(v[0], v[1], v[2], v[3]);
    else if constexpr (R == 8) dft8<FWD>(v);
    else if constexpr (R == 16) dft16<FWD>(v);
    else if constexpr (R == 9) dft9<FWD>(v);
    else dft_odd<R, FWD>(v);
}

}  // namespace ig
