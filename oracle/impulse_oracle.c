/*
 * impulse_oracle.c -- CPU oracle for the impulse FFT path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker that the GPU engine is
 * compared against; it is linked only by the test-suite, by the smoke check
 * and by the CPU-baseline leg of the benchmark.  The product (libimpulse_gpu)
 * never links or calls it.
 *
 * It is an independent FP64 restatement of the algorithms behind impulse's
 * FFT path (PocketFFT as vendored by impulse, plus impulse's Nim glue):
 *
 *   - plan heuristics: largest prime factor, cost guess, good size and the
 *     FFTPACK-vs-Bluestein rule
 *       (impulse/fft/c_pocketfft/pocketfft.c:205-260, 2066-2153);
 *   - mixed-radix complex FFT (the reference runs FFTPACK passes,
 *     pocketfft.c:300-929; this oracle runs a Stockham autosort formulation
 *     of the same factorisation, with radix-2/3/4/5 butterflies and a direct
 *     generic-radix DFT for every other prime factor);
 *   - accurate twiddles exp(-2 pi i t/n) with exact integer octant reduction
 *       (pocketfft.c:62-203 computes the same table by a different method);
 *   - Bluestein for lengths with a large prime factor: chirp exp(i pi m^2/n)
 *     with m^2 mod 2n kept as an exact integer, zero padded to
 *     n2 = good_size(2n-1)  (pocketfft.c:1880-2008);
 *   - real transforms in FFTPACK "halfcomplex" order
 *     [r0, r1, i1, r2, i2, ..., (r_{n/2})]  (pocketfft.c:1701-1766,
 *     impulse/fft/c_pocketfft/pocketfft.nim:216-288);
 *   - the N-d strided drivers of the C++ backend: c2c over several axes with
 *     the scale factor applied on the first axis only, r2c on the last axis
 *     followed by c2c on the others, c2r as c2c into a contiguous temporary
 *     followed by c2r on the last axis, byte strides
 *       (impulse/fft/cpp_pocketfft/pocketfft_hdronly.h:3012-3050,
 *        3125-3250, 3272-3390);
 *   - impulse's Nim glue: unpackFFT, symmetrize, symmTargetSize,
 *     initNormalize  (impulse/fft/c_pocketfft/pocketfft.nim:126-204).
 *
 * Everything is double precision.  Batched entry points run over POSIX
 * threads so that the oracle can also serve as the timed CPU baseline.
 */
#include <math.h>
#include <pthread.h>
#include <stddef.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

typedef struct { double r, i; } oc_t;

/* ------------------------------------------------------------------ */
/* plan heuristics (pocketfft.c:205-260)                               */
/* ------------------------------------------------------------------ */

size_t io_largest_prime_factor(size_t n)
{
    size_t res = 1;
    while (n > 1 && (n & 1) == 0) { res = 2; n >>= 1; }
    for (size_t x = 3; x * x <= n; x += 2)
        while (n % x == 0) { res = x; n /= x; }
    if (n > 1) res = n;
    return res;
}

double io_cost_guess(size_t n)
{
    const double lfp = 1.1; /* penalty for factors without a dedicated pass */
    size_t ni = n;
    double result = 0.0;
    while (n > 1 && (n & 1) == 0) { result += 2; n >>= 1; }
    for (size_t x = 3; x * x <= n; x += 2)
        while (n % x == 0) { result += (x <= 5) ? (double)x : lfp * (double)x; n /= x; }
    if (n > 1) result += (n <= 5) ? (double)n : lfp * (double)n;
    return result * (double)ni;
}

/* smallest 2^a 3^b 5^c 7^d 11^e >= n (pocketfft.c:245-260) */
size_t io_good_size(size_t n)
{
    if (n <= 6) return n;
    size_t best = 2 * n;
    for (size_t f2 = 1; f2 < best; f2 *= 2)
        for (size_t f3 = f2; f3 < best; f3 *= 3)
            for (size_t f5 = f3; f5 < best; f5 *= 5)
                for (size_t f7 = f5; f7 < best; f7 *= 7)
                    for (size_t f11 = f7; f11 < best; f11 *= 11)
                        if (f11 >= n) best = f11;
    return best;
}

/* Bluestein decision of make_cfft_plan / make_rfft_plan (pocketfft.c:2066-2153):
   FFTPACK when n < 50 or lpf^2 <= n; otherwise Bluestein iff
   1.5 * 2 * cost(good_size(2n-1)) < cost(n)   (complex)
   1.5 * 2 * cost(good_size(2n-1)) < 0.5 * cost(n)   (real). */
int io_use_bluestein(size_t n, int real)
{
    if (n < 50) return 0;
    size_t lpf = io_largest_prime_factor(n);
    if ((double)lpf <= sqrt((double)n)) return 0;
    double comp1 = io_cost_guess(n) * (real ? 0.5 : 1.0);
    double comp2 = 2.0 * io_cost_guess(io_good_size(2 * n - 1)) * 1.5;
    return comp2 < comp1;
}

/* ------------------------------------------------------------------ */
/* twiddles                                                            */
/* ------------------------------------------------------------------ */

/* exp(+2 pi i t / n) with exact integer reduction to the first octant. */
static void io_sincos_2pi(size_t t, size_t n, double *c, double *s)
{
    t %= n;
    int neg_s = 0;
    if (2 * t > n) { t = n - t; neg_s = 1; }              /* angle -> 2pi - angle */
    double cc, ss;
    /* now t/n in [0, 1/2] */
    if (4 * t > n) {
        /* angle = pi/2 + 2pi*(4t-n)/(4n) */
        size_t num = 4 * t - n, den = 4 * n;
        /* num/den in (0, 1/4] */
        double cq, sq;
        if (8 * num > den) { /* reflect around 1/8: 2pi*num/den = pi/2 - 2pi*(den-4num)/(4den) */
            double a = 2.0 * M_PI * (double)(den - 4 * num) / (double)(4 * den);
            cq = sin(a); sq = cos(a);
        } else {
            double a = 2.0 * M_PI * (double)num / (double)den;
            cq = cos(a); sq = sin(a);
        }
        cc = -sq; ss = cq;
    } else {
        if (8 * t > n) {
            double a = 2.0 * M_PI * (double)(n - 4 * t) / (double)(4 * n);
            cc = sin(a); ss = cos(a);
        } else {
            double a = 2.0 * M_PI * (double)t / (double)n;
            cc = cos(a); ss = sin(a);
        }
    }
    *c = cc;
    *s = neg_s ? -ss : ss;
}

/* ------------------------------------------------------------------ */
/* complex plan: Stockham mixed radix or Bluestein                     */
/* ------------------------------------------------------------------ */

#define IO_MAXFCT 64

typedef struct io_cplan {
    size_t n;
    int blue;
    size_t nfct;
    size_t fct[IO_MAXFCT];
    oc_t *tw;             /* tw[t] = exp(-2 pi i t/n), t < n (Stockham plans) */
    size_t maxr;          /* largest radix, for generic-radix scratch */
    oc_t *stw;            /* stage twiddles: stage s at stw + twoff[s], entry
                             k (r-1) + m - 1 = exp(-2 pi i m k / (ns r)), k < ns */
    size_t twoff[IO_MAXFCT];
    /* Bluestein */
    size_t n2;
    oc_t *bk;             /* exp(+i pi m^2/n), m < n */
    oc_t *bkf;            /* FFT_n2 of the symmetric zero-padded bk, scaled 1/n2 */
    struct io_cplan *sub; /* Stockham plan of length n2 */
} io_cplan;

static void io_factorize(io_cplan *p)
{
    /* 8s, then 4s, then a single 2 moved to the front, then odd divisors
       (the C++ backend's cfftp::factorize, pocketfft_hdronly.h:1360-1381;
       the C backend's pocketfft.c:954-983 takes 4s only) */
    size_t n = p->n, nf = 0;
    while (n % 8 == 0) { p->fct[nf++] = 8; n /= 8; }
    while (n % 4 == 0) { p->fct[nf++] = 4; n /= 4; }
    if (n % 2 == 0) {
        n /= 2;
        p->fct[nf++] = 2;
        size_t t = p->fct[0]; p->fct[0] = p->fct[nf - 1]; p->fct[nf - 1] = t;
    }
    for (size_t d = 3; n > 1 && d * d <= n; d += 2)
        while (n % d == 0) { p->fct[nf++] = d; n /= d; }
    if (n > 1) p->fct[nf++] = n;
    p->nfct = nf;
    p->maxr = 1;
    for (size_t k = 0; k < nf; ++k) if (p->fct[k] > p->maxr) p->maxr = p->fct[k];
}

void io_destroy_cplan(io_cplan *p);

static io_cplan *io_make_stockham(size_t n)
{
    io_cplan *p = (io_cplan *)calloc(1, sizeof(io_cplan));
    if (!p) return NULL;
    p->n = n;
    io_factorize(p);
    p->tw = (oc_t *)malloc(sizeof(oc_t) * (n ? n : 1));
    if (!p->tw) { free(p); return NULL; }
    for (size_t t = 0; t < n; ++t) {
        double c, s;
        io_sincos_2pi(t, n, &c, &s);
        p->tw[t].r = c;
        p->tw[t].i = -s;
    }
    /* per-stage tables, read in order by the k-major stage loops: the same
       values as tw[m k n/(ns r)] */
    size_t tot = 0, ns = 1;
    for (size_t f = 0; f < p->nfct; ++f) { p->twoff[f] = tot; tot += ns * (p->fct[f] - 1); ns *= p->fct[f]; }
    p->stw = (oc_t *)malloc(sizeof(oc_t) * (tot ? tot : 1));
    if (!p->stw) { free(p->tw); free(p); return NULL; }
    ns = 1;
    for (size_t f = 0; f < p->nfct; ++f) {
        const size_t r = p->fct[f], step = n / (ns * r);
        oc_t *t = p->stw + p->twoff[f];
        for (size_t k = 0; k < ns; ++k)
            for (size_t m = 1; m < r; ++m) t[k * (r - 1) + m - 1] = p->tw[(m * k * step) % n];
        ns *= r;
    }
    return p;
}

static int io_stockham_exec(const io_cplan *p, oc_t *x, oc_t *scratch, int forward, double fct);

io_cplan *io_make_cplan(size_t n)
{
    if (n == 0) return NULL;
    if (!io_use_bluestein(n, 0)) return io_make_stockham(n);
    io_cplan *p = (io_cplan *)calloc(1, sizeof(io_cplan));
    if (!p) return NULL;
    p->n = n;
    p->blue = 1;
    p->n2 = io_good_size(2 * n - 1);
    p->sub = io_make_stockham(p->n2);
    p->bk = (oc_t *)malloc(sizeof(oc_t) * n);
    p->bkf = (oc_t *)calloc(p->n2, sizeof(oc_t));
    oc_t *scr = (oc_t *)malloc(sizeof(oc_t) * p->n2);
    if (!p->sub || !p->bk || !p->bkf || !scr) { free(scr); io_destroy_cplan(p); return NULL; }
    /* chirp: m^2 mod 2n as an exact integer recurrence (pocketfft.c:1907-1914) */
    size_t coeff = 0;
    for (size_t m = 0; m < n; ++m) {
        if (m > 0) { coeff += 2 * m - 1; if (coeff >= 2 * n) coeff -= 2 * n; }
        double c, s;
        io_sincos_2pi(coeff, 2 * n, &c, &s);
        p->bk[m].r = c;
        p->bk[m].i = s;
    }
    double xn2 = 1.0 / (double)p->n2;
    p->bkf[0].r = p->bk[0].r * xn2;
    p->bkf[0].i = p->bk[0].i * xn2;
    for (size_t m = 1; m < n; ++m) {
        oc_t v = { p->bk[m].r * xn2, p->bk[m].i * xn2 };
        p->bkf[m] = v;
        p->bkf[p->n2 - m] = v;
    }
    io_stockham_exec(p->sub, p->bkf, scr, 1, 1.0);
    free(scr);
    return p;
}

void io_destroy_cplan(io_cplan *p)
{
    if (!p) return;
    free(p->tw);
    free(p->stw);
    free(p->bk);
    free(p->bkf);
    if (p->sub) io_destroy_cplan(p->sub);
    free(p);
}

size_t io_cplan_n2(const io_cplan *p) { return p->blue ? p->n2 : 0; }
size_t io_cplan_nfct(const io_cplan *p) { return p->blue ? p->sub->nfct : p->nfct; }
size_t io_cplan_fct(const io_cplan *p, size_t k) { return p->blue ? p->sub->fct[k] : p->fct[k]; }

static inline oc_t cmul(oc_t a, oc_t b) { oc_t r = { a.r * b.r - a.i * b.i, a.r * b.i + a.i * b.r }; return r; }
static inline oc_t cmulc(oc_t a, oc_t b) { oc_t r = { a.r * b.r + a.i * b.i, a.i * b.r - a.r * b.i }; return r; } /* a*conj(b) */

/* One Stockham stage of radix r (stage s of the plan): x -> y.  ns = product
   of the radices already applied.  Butterfly j = q ns + k (j < n/r) reads
   x[j + m n/r], twiddles input m by w^(m k) (w = exp(-+2 pi i/(ns r)), from
   the stage table), runs a radix-r DFT and writes y[q ns r + k + m ns].  The
   loops run k outermost so that one butterfly's twiddles serve all q.  The
   DFTs: radix 2 and 4 directly, odd radices in the symmetric-pair form
   V[q] = v0 + sum_k a_k cos(2 pi k q/r) -+ i sum_k b_k sin(2 pi k q/r),
   V[r-q] with the second sum's sign flipped (a_k = v_k + v_{r-k},
   b_k = v_k - v_{r-k}), written out for 3 and 5 (pocketfft.c:300-865 covers
   radices 2, 3, 4, 5, 7, 11 with passes of the same arithmetic). */
static void io_stage(const io_cplan *p, size_t s, size_t ns, const oc_t *x, oc_t *y, int forward, oc_t *v, oc_t *tk)
{
    const size_t r = p->fct[s], n = p->n, nr = n / r, nq = nr / ns;
    const oc_t *tws = p->stw + p->twoff[s];
    const double sg = forward ? 1.0 : -1.0; /* sign of the imaginary part of the table */
    /* odd radices: cos / sin (2 pi t / r), t < r, from the plan's table */
    double cs[IO_MAXFCT + 2], sn[IO_MAXFCT + 2];
    double *cr = cs, *sr = sn, *heap = NULL;
    if (r % 2 == 1 && r > IO_MAXFCT + 2) {
        heap = (double *)malloc(2 * r * sizeof(double));
        cr = heap;
        sr = heap + r;
    }
    if (r % 2 == 1)
        for (size_t t = 0; t < r; ++t) { cr[t] = p->tw[t * nr].r; sr[t] = -p->tw[t * nr].i; }
    for (size_t k = 0; k < ns; ++k) {
        for (size_t m = 1; m < r; ++m) {
            oc_t t = k ? tws[k * (r - 1) + m - 1] : (oc_t){ 1.0, 0.0 };
            t.i *= sg;
            tk[m] = t;
        }
        if (r == 8) {
            /* radix 8 = radix-2 butterflies (m, m + 4), w8^m on the
               differences, two radix-4 DFTs on the sums and differences */
            const double h = 0.70710678118654752440; /* sqrt(1/2) */
            for (size_t q = 0; q < nq; ++q) {
                const size_t j = q * ns + k;
                const oc_t *xi = x + j;
                oc_t *yo = y + q * ns * r + k;
                oc_t w[8];
                w[0] = xi[0];
                if (k) for (size_t m = 1; m < 8; ++m) w[m] = cmul(xi[m * nr], tk[m]);
                else for (size_t m = 1; m < 8; ++m) w[m] = xi[m * nr];
                oc_t a[4], b[4];
                for (size_t m = 0; m < 4; ++m) {
                    a[m].r = w[m].r + w[m + 4].r; a[m].i = w[m].i + w[m + 4].i;
                    b[m].r = w[m].r - w[m + 4].r; b[m].i = w[m].i - w[m + 4].i;
                }
                /* b1 w8, b2 w8^2 = -+i, b3 w8^3 (forward: w8 = (1 - i)/sqrt 2) */
                oc_t t1, t2, t3;
                if (forward) {
                    t1.r = h * (b[1].r + b[1].i); t1.i = h * (b[1].i - b[1].r);
                    t2.r = b[2].i; t2.i = -b[2].r;
                    t3.r = h * (b[3].i - b[3].r); t3.i = -h * (b[3].r + b[3].i);
                } else {
                    t1.r = h * (b[1].r - b[1].i); t1.i = h * (b[1].i + b[1].r);
                    t2.r = -b[2].i; t2.i = b[2].r;
                    t3.r = -h * (b[3].r + b[3].i); t3.i = h * (b[3].r - b[3].i);
                }
                b[1] = t1; b[2] = t2; b[3] = t3;
                for (int half = 0; half < 2; ++half) {
                    const oc_t *u = half ? b : a;
                    oc_t s0 = { u[0].r + u[2].r, u[0].i + u[2].i }, s1 = { u[0].r - u[2].r, u[0].i - u[2].i };
                    oc_t s2 = { u[1].r + u[3].r, u[1].i + u[3].i }, s3 = { u[1].r - u[3].r, u[1].i - u[3].i };
                    oc_t s3r = forward ? (oc_t){ s3.i, -s3.r } : (oc_t){ -s3.i, s3.r };
                    oc_t *o = yo + (size_t)half * ns;
                    o[0].r = s0.r + s2.r; o[0].i = s0.i + s2.i;
                    o[4 * ns].r = s0.r - s2.r; o[4 * ns].i = s0.i - s2.i;
                    o[2 * ns].r = s1.r + s3r.r; o[2 * ns].i = s1.i + s3r.i;
                    o[6 * ns].r = s1.r - s3r.r; o[6 * ns].i = s1.i - s3r.i;
                }
            }
            continue;
        }
        for (size_t q = 0; q < nq; ++q) {
            const size_t j = q * ns + k;
            const oc_t *xi = x + j;
            oc_t *yo = y + q * ns * r + k;
            v[0] = xi[0];
            if (k) for (size_t m = 1; m < r; ++m) v[m] = cmul(xi[m * nr], tk[m]);
            else for (size_t m = 1; m < r; ++m) v[m] = xi[m * nr];
            if (r == 2) {
                yo[0].r = v[0].r + v[1].r; yo[0].i = v[0].i + v[1].i;
                yo[ns].r = v[0].r - v[1].r; yo[ns].i = v[0].i - v[1].i;
            } else if (r == 4) {
                oc_t t0 = { v[0].r + v[2].r, v[0].i + v[2].i }, t1 = { v[0].r - v[2].r, v[0].i - v[2].i };
                oc_t t2 = { v[1].r + v[3].r, v[1].i + v[3].i }, t3 = { v[1].r - v[3].r, v[1].i - v[3].i };
                /* t3 times -i (forward) or +i (backward) */
                oc_t t3r = forward ? (oc_t){ t3.i, -t3.r } : (oc_t){ -t3.i, t3.r };
                yo[0].r = t0.r + t2.r; yo[0].i = t0.i + t2.i;
                yo[2 * ns].r = t0.r - t2.r; yo[2 * ns].i = t0.i - t2.i;
                yo[ns].r = t1.r + t3r.r; yo[ns].i = t1.i + t3r.i;
                yo[3 * ns].r = t1.r - t3r.r; yo[3 * ns].i = t1.i - t3r.i;
            } else if (r == 3) {
                const double c1 = cr[1], s1 = sg * sr[1];
                oc_t a = { v[1].r + v[2].r, v[1].i + v[2].i }, b = { v[1].r - v[2].r, v[1].i - v[2].i };
                oc_t u = { v[0].r + c1 * a.r, v[0].i + c1 * a.i };
                yo[0].r = v[0].r + a.r; yo[0].i = v[0].i + a.i;
                /* -+ i s1 b */
                yo[ns].r = u.r + s1 * b.i; yo[ns].i = u.i - s1 * b.r;
                yo[2 * ns].r = u.r - s1 * b.i; yo[2 * ns].i = u.i + s1 * b.r;
            } else if (r == 5) {
                const double c1 = cr[1], c2 = cr[2], s1 = sg * sr[1], s2 = sg * sr[2];
                oc_t a1 = { v[1].r + v[4].r, v[1].i + v[4].i }, b1 = { v[1].r - v[4].r, v[1].i - v[4].i };
                oc_t a2 = { v[2].r + v[3].r, v[2].i + v[3].i }, b2 = { v[2].r - v[3].r, v[2].i - v[3].i };
                yo[0].r = v[0].r + a1.r + a2.r; yo[0].i = v[0].i + a1.i + a2.i;
                oc_t u1 = { v[0].r + c1 * a1.r + c2 * a2.r, v[0].i + c1 * a1.i + c2 * a2.i };
                oc_t w1 = { s1 * b1.r + s2 * b2.r, s1 * b1.i + s2 * b2.i };
                oc_t u2 = { v[0].r + c2 * a1.r + c1 * a2.r, v[0].i + c2 * a1.i + c1 * a2.i };
                oc_t w2 = { s2 * b1.r - s1 * b2.r, s2 * b1.i - s1 * b2.i };
                yo[ns].r = u1.r + w1.i; yo[ns].i = u1.i - w1.r;
                yo[4 * ns].r = u1.r - w1.i; yo[4 * ns].i = u1.i + w1.r;
                yo[2 * ns].r = u2.r + w2.i; yo[2 * ns].i = u2.i - w2.r;
                yo[3 * ns].r = u2.r - w2.i; yo[3 * ns].i = u2.i + w2.r;
            } else if (r % 2 == 1) {
                const size_t h = (r - 1) / 2;
                oc_t *a = v + r, *b = v + r + h; /* a_k, b_k at index k - 1 */
                oc_t y0 = v[0];
                for (size_t kk = 1; kk <= h; ++kk) {
                    a[kk - 1].r = v[kk].r + v[r - kk].r; a[kk - 1].i = v[kk].i + v[r - kk].i;
                    b[kk - 1].r = v[kk].r - v[r - kk].r; b[kk - 1].i = v[kk].i - v[r - kk].i;
                    y0.r += a[kk - 1].r; y0.i += a[kk - 1].i;
                }
                yo[0] = y0;
                for (size_t qq = 1; qq <= h; ++qq) {
                    oc_t u = v[0], w = { 0.0, 0.0 };
                    size_t t = 0;
                    for (size_t kk = 1; kk <= h; ++kk) {
                        t += qq;
                        if (t >= r) t -= r;
                        u.r += cr[t] * a[kk - 1].r; u.i += cr[t] * a[kk - 1].i;
                        w.r += sr[t] * b[kk - 1].r; w.i += sr[t] * b[kk - 1].i;
                    }
                    w.r *= sg; w.i *= sg;
                    yo[qq * ns].r = u.r + w.i; yo[qq * ns].i = u.i - w.r;
                    yo[(r - qq) * ns].r = u.r - w.i; yo[(r - qq) * ns].i = u.i + w.r;
                }
            } else {
                /* other even radices (the planner makes none but 2, 4 and 8): direct DFT */
                for (size_t qq = 0; qq < r; ++qq) {
                    oc_t acc = v[0];
                    for (size_t m = 1; m < r; ++m) {
                        oc_t t = p->tw[((m * qq) % r) * nr];
                        t.i *= sg;
                        oc_t pr = cmul(v[m], t);
                        acc.r += pr.r; acc.i += pr.i;
                    }
                    yo[qq * ns] = acc;
                }
            }
        }
    }
    free(heap);
}

static int io_stockham_exec(const io_cplan *p, oc_t *x, oc_t *scratch, int forward, double fct)
{
    size_t n = p->n;
    if (n == 1) { x[0].r *= fct; x[0].i *= fct; return 0; }
    /* butterfly values (r), symmetric-pair sums (r - 1) and twiddles (r) */
    oc_t vbuf[64];
    oc_t *v = 3 * p->maxr <= 64 ? vbuf : (oc_t *)malloc(sizeof(oc_t) * 3 * p->maxr);
    if (!v) return -1;
    oc_t *a = x, *b = scratch;
    size_t ns = 1;
    for (size_t s = 0; s < p->nfct; ++s) {
        io_stage(p, s, ns, a, b, forward, v, v + 2 * p->maxr);
        ns *= p->fct[s];
        oc_t *t = a; a = b; b = t;
    }
    if (a != x) {
        for (size_t i = 0; i < n; ++i) { x[i].r = a[i].r * fct; x[i].i = a[i].i * fct; }
    } else if (fct != 1.0) {
        for (size_t i = 0; i < n; ++i) { x[i].r *= fct; x[i].i *= fct; }
    }
    if (v != vbuf) free(v);
    return 0;
}

/* per-thread scratch of at least `count` complex values, kept between calls
   (the batch workers are persistent pool threads) */
static __thread oc_t *io_tls_buf = NULL;
static __thread size_t io_tls_len = 0;
static oc_t *io_scratch(size_t count)
{
    if (count > io_tls_len) {
        free(io_tls_buf);
        io_tls_buf = (oc_t *)malloc(sizeof(oc_t) * count);
        io_tls_len = io_tls_buf ? count : 0;
    }
    return io_tls_buf;
}
/* a second one for the real transforms' packed line (the complex plan
   uses the first) */
static __thread oc_t *io_tls_buf2 = NULL;
static __thread size_t io_tls_len2 = 0;
static oc_t *io_scratch2(size_t count)
{
    if (count > io_tls_len2) {
        free(io_tls_buf2);
        io_tls_buf2 = (oc_t *)malloc(sizeof(oc_t) * count);
        io_tls_len2 = io_tls_buf2 ? count : 0;
    }
    return io_tls_buf2;
}
static __thread oc_t *io_tls_blue = NULL;
static __thread size_t io_tls_blue_len = 0;

/* Bluestein (pocketfft.c:1945-2008): premultiply by the chirp, convolve with
   the chirp through two length-n2 FFTs, postmultiply by the chirp. */
static int io_blue_exec(const io_cplan *p, oc_t *c, int forward, double fct)
{
    size_t n = p->n, n2 = p->n2;
    if (2 * n2 > io_tls_blue_len) {  /* per-thread, kept between calls */
        free(io_tls_blue);
        io_tls_blue = (oc_t *)malloc(sizeof(oc_t) * 2 * n2);
        io_tls_blue_len = io_tls_blue ? 2 * n2 : 0;
    }
    oc_t *akf = io_tls_blue;
    if (!akf) return -1;
    oc_t *scr = akf + n2;
    for (size_t m = 0; m < n; ++m)
        akf[m] = forward ? cmulc(c[m], p->bk[m]) : cmul(c[m], p->bk[m]);
    memset(akf + n, 0, (n2 - n) * sizeof(oc_t));
    io_stockham_exec(p->sub, akf, scr, 1, fct);
    for (size_t m = 0; m < n2; ++m)
        akf[m] = forward ? cmul(akf[m], p->bkf[m]) : cmulc(akf[m], p->bkf[m]);
    io_stockham_exec(p->sub, akf, scr, 0, 1.0);
    for (size_t m = 0; m < n; ++m)
        c[m] = forward ? cmulc(akf[m], p->bk[m]) : cmul(akf[m], p->bk[m]);
    return 0;
}

/* In-place complex transform of one line with an existing plan. */
int io_cplan_exec(const io_cplan *p, double *c, int forward, double fct)
{
    if (p->blue) return io_blue_exec(p, (oc_t *)c, forward, fct);
    oc_t *scr = io_scratch(p->n);
    if (!scr) return -1;
    return io_stockham_exec(p, (oc_t *)c, scr, forward, fct);
}

/* ------------------------------------------------------------------ */
/* real plan: halfcomplex layout                                       */
/* ------------------------------------------------------------------ */

typedef struct io_rplan {
    size_t n;
    io_cplan *cp;   /* complex plan of length n/2 (even n) or n (odd n) */
    oc_t *wn;       /* exp(-2 pi i k/n), k <= n/2 (even n) */
} io_rplan;

io_rplan *io_make_rplan(size_t n)
{
    if (n == 0) return NULL;
    io_rplan *p = (io_rplan *)calloc(1, sizeof(io_rplan));
    if (!p) return NULL;
    p->n = n;
    if (n == 1) return p;
    size_t h = (n % 2 == 0) ? n / 2 : n;
    p->cp = io_make_cplan(h);
    if (n % 2 == 0) {
        p->wn = (oc_t *)malloc(sizeof(oc_t) * (n / 2 + 1));
        for (size_t k = 0; k <= n / 2; ++k) {
            double c, s;
            io_sincos_2pi(k, n, &c, &s);
            p->wn[k].r = c;
            p->wn[k].i = -s;
        }
    }
    return p;
}

void io_destroy_rplan(io_rplan *p)
{
    if (!p) return;
    io_destroy_cplan(p->cp);
    free(p->wn);
    free(p);
}

/* r2hc / hc2r in place on n doubles (pocketfft.c:2176-2190 semantics):
   forward: halfcomplex of sum_m x[m] exp(-2 pi i m k/n), times fct;
   backward: x[m] = fct * sum_k X[k] exp(+2 pi i m k/n) over the full
   Hermitian spectrum described by the halfcomplex input. */
int io_rplan_exec(const io_rplan *p, double *c, int forward, double fct)
{
    size_t n = p->n;
    if (n == 1) { c[0] *= fct; return 0; }
    if (n % 2 == 1) {
        oc_t *z = io_scratch2(n);
        if (!z) return -1;
        if (forward) {
            for (size_t m = 0; m < n; ++m) { z[m].r = c[m]; z[m].i = 0.0; }
            io_cplan_exec(p->cp, (double *)z, 1, fct);
            c[0] = z[0].r;
            for (size_t k = 1; 2 * k < n + 1; ++k) { c[2 * k - 1] = z[k].r; c[2 * k] = z[k].i; }
        } else {
            z[0].r = c[0]; z[0].i = 0.0;
            for (size_t k = 1; 2 * k < n + 1; ++k) {
                z[k].r = c[2 * k - 1]; z[k].i = c[2 * k];
                z[n - k].r = c[2 * k - 1]; z[n - k].i = -c[2 * k];
            }
            io_cplan_exec(p->cp, (double *)z, 0, fct);
            for (size_t m = 0; m < n; ++m) c[m] = z[m].r;
        }
        return 0;
    }
    size_t h = n / 2;
    oc_t *z = io_scratch2(h);
    if (!z) return -1;
    if (forward) {
        /* z[m] = x[2m] + i x[2m+1] is the line itself read as complex values:
           Z = FFT_h(z) in place, split into X[0..h] through the packed buffer */
        oc_t *zc = (oc_t *)c;
        if (io_cplan_exec(p->cp, c, 1, 1.0)) return -1;
        double *xo = (double *)z;
        for (size_t k = 0; k <= h; ++k) {
            oc_t zk = zc[k == h ? 0 : k], zm = zc[k == 0 ? 0 : h - k];
            /* E = (zk + conj(zm))/2, O = (zk - conj(zm))/(2i) */
            oc_t e = { 0.5 * (zk.r + zm.r), 0.5 * (zk.i - zm.i) };
            oc_t o = { 0.5 * (zk.i + zm.i), -0.5 * (zk.r - zm.r) };
            oc_t t = cmul(o, p->wn[k]);
            double xr = (e.r + t.r) * fct, xi = (e.i + t.i) * fct;
            if (k == 0) xo[0] = xr;
            else if (k == h) xo[n - 1] = xr;
            else { xo[2 * k - 1] = xr; xo[2 * k] = xi; }
        }
        memcpy(c, xo, n * sizeof(double));
    } else {
        /* X from halfcomplex; Z[k] = A + i exp(+2 pi i k/n) B,
           A = X[k] + conj(X[h-k]), B = X[k] - conj(X[h-k]); z = IFFT_h(Z) */
        for (size_t k = 0; k < h; ++k) {
            oc_t xk, xm;
            if (k == 0) { xk.r = c[0]; xk.i = 0.0; } else { xk.r = c[2 * k - 1]; xk.i = c[2 * k]; }
            size_t q = h - k;
            if (q == h) { xm.r = c[n - 1]; xm.i = 0.0; } else if (q == 0) { xm.r = c[0]; xm.i = 0.0; }
            else { xm.r = c[2 * q - 1]; xm.i = c[2 * q]; }
            oc_t a = { xk.r + xm.r, xk.i - xm.i };
            oc_t b = { xk.r - xm.r, xk.i + xm.i };
            oc_t wc = { p->wn[k].r, -p->wn[k].i }; /* exp(+2 pi i k/n) */
            oc_t t = cmul(b, wc);
            z[k].r = a.r - t.i;
            z[k].i = a.i + t.r;
        }
        io_cplan_exec(p->cp, (double *)z, 0, fct);
        for (size_t m = 0; m < h; ++m) { c[2 * m] = z[m].r; c[2 * m + 1] = z[m].i; }
    }
    return 0;
}

/* ------------------------------------------------------------------ */
/* pocketfft.h-shaped one-shot entry points (plan built per call, as  */
/* impulse's C backend does: pocketfft.nim:206-214)                    */
/* ------------------------------------------------------------------ */

int io_cfft(size_t n, double *c, int forward, double fct)
{
    io_cplan *p = io_make_cplan(n);
    if (!p) return -1;
    int rc = io_cplan_exec(p, c, forward, fct);
    io_destroy_cplan(p);
    return rc;
}

int io_rfft(size_t n, double *c, int forward, double fct)
{
    io_rplan *p = io_make_rplan(n);
    if (!p) return -1;
    int rc = io_rplan_exec(p, c, forward, fct);
    io_destroy_rplan(p);
    return rc;
}

/* ------------------------------------------------------------------ */
/* threaded batch drivers                                              */
/* ------------------------------------------------------------------ */

typedef struct {
    const void *plan;
    int real;
    double *base;
    size_t batch, dist; /* dist in doubles */
    int forward;
    double fct;
    size_t t, nt;
    int rc;
} io_batch_job;

/* Two real lines a, b of odd length n in one complex transform: forward,
   Z = FFT(a + i b), A[k] = (Z[k] + conj Z[n-k]) / 2, B[k] = (Z[k] - conj Z[n-k]) / 2i;
   backward, Z[k] = A[k] + i B[k] over the full Hermitian spectra, a = Re IFFT(Z),
   b = Im IFFT(Z).  Exact in the same way as one line per transform. */
static int io_rplan_exec_pair(const io_rplan *p, double *ca, double *cb, int forward, double fct)
{
    const size_t n = p->n;
    oc_t *z = io_scratch2(n);
    if (!z) return -1;
    if (forward) {
        for (size_t m = 0; m < n; ++m) { z[m].r = ca[m]; z[m].i = cb[m]; }
        int rc = io_cplan_exec(p->cp, (double *)z, 1, fct);
        if (rc) return rc;
        ca[0] = z[0].r;
        cb[0] = z[0].i;
        for (size_t k = 1; 2 * k < n + 1; ++k) {
            const oc_t zk = z[k], zm = z[n - k];
            ca[2 * k - 1] = 0.5 * (zk.r + zm.r);
            ca[2 * k] = 0.5 * (zk.i - zm.i);
            cb[2 * k - 1] = 0.5 * (zk.i + zm.i);
            cb[2 * k] = 0.5 * (zm.r - zk.r);
        }
    } else {
        z[0].r = ca[0];
        z[0].i = cb[0];
        for (size_t k = 1; 2 * k < n + 1; ++k) {
            const double ar = ca[2 * k - 1], ai = ca[2 * k], br = cb[2 * k - 1], bi = cb[2 * k];
            z[k].r = ar - bi;       /* A[k] + i B[k] */
            z[k].i = ai + br;
            z[n - k].r = ar + bi;   /* conj A[k] + i conj B[k] */
            z[n - k].i = br - ai;
        }
        int rc = io_cplan_exec(p->cp, (double *)z, 0, fct);
        if (rc) return rc;
        for (size_t m = 0; m < n; ++m) { ca[m] = z[m].r; cb[m] = z[m].i; }
    }
    return 0;
}

static void *io_batch_worker(void *arg)
{
    io_batch_job *j = (io_batch_job *)arg;
    size_t lo = j->batch * j->t / j->nt, hi = j->batch * (j->t + 1) / j->nt;
    const int pair = j->real && ((const io_rplan *)j->plan)->n % 2 == 1 && ((const io_rplan *)j->plan)->n > 1;
    for (size_t b = lo; b < hi; ++b) {
        double *line = j->base + b * j->dist;
        int rc;
        if (pair && b + 1 < hi) {
            rc = io_rplan_exec_pair((const io_rplan *)j->plan, line, line + j->dist, j->forward, j->fct);
            ++b;
        } else {
            rc = j->real ? io_rplan_exec((const io_rplan *)j->plan, line, j->forward, j->fct)
                         : io_cplan_exec((const io_cplan *)j->plan, line, j->forward, j->fct);
        }
        if (rc) j->rc = rc;
    }
    return NULL;
}

/* A persistent worker pool for the batch drivers (the C++ backend keeps one
   too, pocketfft_hdronly.h:651-667): workers sleep on a condition variable;
   a batch call hands out its job slices and waits for them.  One batch call
   at a time uses the pool (others run their slices on their own thread). */
#define IO_POOL_MAX 256
static pthread_mutex_t io_pool_mu = PTHREAD_MUTEX_INITIALIZER;
static pthread_cond_t io_pool_cv = PTHREAD_COND_INITIALIZER, io_pool_done = PTHREAD_COND_INITIALIZER;
static pthread_mutex_t io_pool_busy = PTHREAD_MUTEX_INITIALIZER;
static int io_pool_size = 0;              /* workers started */
static unsigned long long io_pool_gen = 0; /* bumped per batch call */
static io_batch_job *io_pool_jobs = NULL;
static int io_pool_njobs = 0, io_pool_pending = 0;

static void *io_pool_main(void *arg)
{
    const int me = (int)(size_t)arg; /* serves job slot me (slot 0 is the caller's) */
    unsigned long long seen = 0;
    pthread_mutex_lock(&io_pool_mu);
    for (;;) {
        while (io_pool_gen == seen) pthread_cond_wait(&io_pool_cv, &io_pool_mu);
        seen = io_pool_gen;
        if (me < io_pool_njobs) {
            io_batch_job *j = &io_pool_jobs[me];
            pthread_mutex_unlock(&io_pool_mu);
            io_batch_worker(j);
            pthread_mutex_lock(&io_pool_mu);
            if (--io_pool_pending == 0) pthread_cond_signal(&io_pool_done);
        }
    }
    return NULL;
}

static int io_run_batch(const void *plan, int real, double *c, size_t batch, size_t dist, int forward, double fct, int nthreads)
{
    if (nthreads < 1) nthreads = 1;
    if ((size_t)nthreads > batch) nthreads = (int)(batch ? batch : 1);
    if (nthreads > IO_POOL_MAX) nthreads = IO_POOL_MAX;
    io_batch_job *jobs = (io_batch_job *)calloc((size_t)nthreads, sizeof(io_batch_job));
    if (!jobs) return -1;
    for (int t = 0; t < nthreads; ++t) {
        io_batch_job v = { plan, real, c, batch, dist, forward, fct, (size_t)t, (size_t)nthreads, 0 };
        jobs[t] = v;
    }
    int rc = 0;
    if (nthreads > 1 && pthread_mutex_trylock(&io_pool_busy) == 0) {
        pthread_mutex_lock(&io_pool_mu);
        while (io_pool_size < nthreads - 1) {
            pthread_t th;
            if (pthread_create(&th, NULL, io_pool_main, (void *)(size_t)(io_pool_size + 1)) != 0) break;
            pthread_detach(th);
            ++io_pool_size;
        }
        const int njobs = io_pool_size + 1 < nthreads ? io_pool_size + 1 : nthreads;
        /* slices are re-cut for the workers available */
        for (int t = 0; t < njobs; ++t) { jobs[t].t = (size_t)t; jobs[t].nt = (size_t)njobs; }
        io_pool_jobs = jobs;
        io_pool_njobs = njobs;
        io_pool_pending = njobs - 1;
        ++io_pool_gen;
        pthread_cond_broadcast(&io_pool_cv);
        pthread_mutex_unlock(&io_pool_mu);
        io_batch_worker(&jobs[0]);
        pthread_mutex_lock(&io_pool_mu);
        while (io_pool_pending > 0) pthread_cond_wait(&io_pool_done, &io_pool_mu);
        io_pool_jobs = NULL;
        io_pool_njobs = 0;
        pthread_mutex_unlock(&io_pool_mu);
        pthread_mutex_unlock(&io_pool_busy);
        for (int t = 0; t < njobs; ++t) if (jobs[t].rc) rc = jobs[t].rc;
    } else {
        /* single-threaded, or the pool is serving another call */
        jobs[0].t = 0;
        jobs[0].nt = 1;
        io_batch_worker(&jobs[0]);
        rc = jobs[0].rc;
    }
    free(jobs);
    return rc;
}

/* Plan cache of the batch drivers, like the C++ backend's get_plan LRU
   (pocketfft_hdronly.h:2655-2706): a few recent plans per kind, shared by
   callers (plans are read-only while they execute), reference-counted so
   that an evicted plan lives until its last user is done. */
#define IO_CACHE 8
typedef struct {
    int real;
    size_t n;
    void *plan;
    unsigned long long used;
    int refs;
    int dead;
} io_cache_ent;
static io_cache_ent io_cache[IO_CACHE];
static unsigned long long io_cache_clock = 0;
static pthread_mutex_t io_cache_mu = PTHREAD_MUTEX_INITIALIZER;

static void io_plan_free(int real, void *plan)
{
    if (real) io_destroy_rplan((io_rplan *)plan);
    else io_destroy_cplan((io_cplan *)plan);
}

static void *io_plan_get(int real, size_t n, int *slot)
{
    pthread_mutex_lock(&io_cache_mu);
    for (int i = 0; i < IO_CACHE; ++i)
        if (io_cache[i].plan && !io_cache[i].dead && io_cache[i].real == real && io_cache[i].n == n) {
            io_cache[i].used = ++io_cache_clock;
            io_cache[i].refs++;
            *slot = i;
            pthread_mutex_unlock(&io_cache_mu);
            return io_cache[i].plan;
        }
    pthread_mutex_unlock(&io_cache_mu);
    void *plan = real ? (void *)io_make_rplan(n) : (void *)io_make_cplan(n);
    if (!plan) return NULL;
    pthread_mutex_lock(&io_cache_mu);
    int victim = -1;
    for (int i = 0; i < IO_CACHE; ++i) {
        if (!io_cache[i].plan) { victim = i; break; }
        if (io_cache[i].refs == 0 && (victim < 0 || io_cache[i].used < io_cache[victim].used)) victim = i;
    }
    if (victim < 0) {  /* every entry in use: run uncached */
        pthread_mutex_unlock(&io_cache_mu);
        *slot = -1;
        return plan;
    }
    if (io_cache[victim].plan) io_plan_free(io_cache[victim].real, io_cache[victim].plan);
    io_cache_ent e = { real, n, plan, ++io_cache_clock, 1, 0 };
    io_cache[victim] = e;
    *slot = victim;
    pthread_mutex_unlock(&io_cache_mu);
    return plan;
}

static void io_plan_put(int real, void *plan, int slot)
{
    if (slot < 0) { io_plan_free(real, plan); return; }
    pthread_mutex_lock(&io_cache_mu);
    io_cache[slot].refs--;
    pthread_mutex_unlock(&io_cache_mu);
}

/* batch lines of n complex numbers, line b at c + 2*b*dist doubles */
int io_cfft_batch(size_t n, size_t batch, double *c, size_t dist, int forward, double fct, int nthreads)
{
    int slot;
    io_cplan *p = (io_cplan *)io_plan_get(0, n, &slot);
    if (!p) return -1;
    int rc = io_run_batch(p, 0, c, batch, 2 * dist, forward, fct, nthreads);
    io_plan_put(0, p, slot);
    return rc;
}

/* batch lines of n reals (halfcomplex in place), line b at c + b*dist doubles */
int io_rfft_batch(size_t n, size_t batch, double *c, size_t dist, int forward, double fct, int nthreads)
{
    int slot;
    io_rplan *p = (io_rplan *)io_plan_get(1, n, &slot);
    if (!p) return -1;
    int rc = io_run_batch(p, 1, c, batch, dist, forward, fct, nthreads);
    io_plan_put(1, p, slot);
    return rc;
}

/* ------------------------------------------------------------------ */
/* N-d strided drivers (pocketfft_hdronly.h:3012-3050, 3125-3390)       */
/* ------------------------------------------------------------------ */

typedef struct {
    size_t ndim;
    const size_t *shape;
    const ptrdiff_t *sin, *sout; /* byte strides */
    size_t axis;
    size_t nlines;
} io_lines;

/* byte offsets (in, out) of line number l along `axis` */
static void io_line_offsets(const io_lines *L, size_t l, ptrdiff_t *oi, ptrdiff_t *oo)
{
    ptrdiff_t a = 0, b = 0;
    for (size_t d = L->ndim; d-- > 0;) {
        if (d == L->axis) continue;
        size_t idx = l % L->shape[d];
        l /= L->shape[d];
        a += (ptrdiff_t)idx * L->sin[d];
        b += (ptrdiff_t)idx * L->sout[d];
    }
    *oi = a;
    *oo = b;
}

/* kind: 0 c2c, 1 r2c (real in -> n/2+1 complex out), 2 c2r (n/2+1 complex in -> real out)
   `len` is the logical transform length (real length for r2c/c2r). */
typedef struct {
    io_lines L;
    int kind;
    size_t len;
    const char *in;
    char *out;
    int forward;
    double fct;
    const void *plan;
    size_t t, nt;
    int rc;
    int type, cosine, ortho, r2c; /* kinds 3-5 */
} io_nd_job;

/* ------------------------------------------------------------------ */
/* DCT / DST I-IV by their defining sums (compensated, exact tables),  */
/* scaling steps of pocketfft_hdronly.h:2424-2650: fct on every output; */
/* ortho: DCT-I scales x[0], x[n-1] by sqrt2 and y[0], y[n-1] by       */
/* 1/sqrt2; types II (DCT and DST) scale y[0] by 1/sqrt2; types III    */
/* scale x[0] by sqrt2; DST-I and types IV ignore ortho.                */
/* ------------------------------------------------------------------ */
static void io_dcst_line(int type, int cosine, int ortho, size_t n, const double *x, double *y, double fct)
{
    const long double PI = 3.14159265358979323846264338327950288L;
    const double R2 = 1.41421356237309504880168872420969808;
    /* every angle is pi * q / P for an integer q: one table of cos / sin(pi q / P), q < 2P
       (long double, rounded once); the sums are compensated (Neumaier) in double */
    size_t P = type == 1 ? (cosine ? n - 1 : n + 1) : type == 4 ? 4 * n : 2 * n;
    double *cs = (double *)malloc(sizeof(double) * (4 * P + n));
    if (!cs) { for (size_t k = 0; k < n; ++k) y[k] = 0.0 / 0.0; return; }
    double *sn = cs + 2 * P, *xs = cs + 4 * P;
    for (size_t q = 0; q < 2 * P; ++q) {
        cs[q] = (double)cosl(PI * (long double)q / (long double)P);
        sn[q] = (double)sinl(PI * (long double)q / (long double)P);
    }
    for (size_t j = 0; j < n; ++j) {
        double xj = x[j];
        if (type == 1 && cosine) {
            if (ortho && (j == 0 || j == n - 1)) xj *= R2;
            xj *= (j == 0 || j == n - 1) ? 1.0 : 2.0;
        } else if (type == 3 && cosine) {
            if (ortho && j == 0) xj *= R2;
            xj *= j == 0 ? 1.0 : 2.0;
        } else if (type == 3) {
            if (ortho && j == 0) xj *= R2;
            xj *= j == n - 1 ? 1.0 : 2.0;
        } else {
            xj *= 2.0;
        }
        xs[j] = xj;
    }
    const size_t M2 = 2 * P;
    const double *tab = cosine ? cs : sn;
    for (size_t k = 0; k < n; ++k) {
        double acc = 0.0, comp = 0.0;
        for (size_t j = 0; j < n; ++j) {
            size_t q;
            if (type == 1) q = cosine ? k * j : (k + 1) * (j + 1);
            else if (type == 2) q = (cosine ? k : k + 1) * (2 * j + 1);
            else if (type == 3) q = cosine ? j * (2 * k + 1) : (j + 1) * (2 * k + 1);
            else q = (2 * j + 1) * (2 * k + 1);
            const double t = xs[j] * tab[q % M2];
            const double s2 = acc + t;
            comp += fabs(acc) >= fabs(t) ? (acc - s2) + t : (t - s2) + acc;
            acc = s2;
        }
        double r = (acc + comp) * fct;
        if (ortho && type == 1 && cosine && (k == 0 || k == n - 1)) r /= R2;
        if (ortho && type == 2 && k == 0) r /= R2;
        y[k] = r;
    }
    free(cs);
}

static void *io_nd_worker(void *arg)
{
    io_nd_job *j = (io_nd_job *)arg;
    const size_t len = j->len, ax = j->L.axis;
    const ptrdiff_t si = j->L.sin[ax], so = j->L.sout[ax];
    double *buf = (double *)malloc(sizeof(double) * 2 * (len + 1));
    if (!buf) { j->rc = -1; return NULL; }
    size_t lo = j->L.nlines * j->t / j->nt, hi = j->L.nlines * (j->t + 1) / j->nt;
    for (size_t l = lo; l < hi; ++l) {
        ptrdiff_t oi, oo;
        io_line_offsets(&j->L, l, &oi, &oo);
        const char *pi = j->in + oi;
        char *po = j->out + oo;
        if (j->kind == 0) {
            for (size_t m = 0; m < len; ++m) {
                const double *s = (const double *)(pi + (ptrdiff_t)m * si);
                buf[2 * m] = s[0]; buf[2 * m + 1] = s[1];
            }
            if (io_cplan_exec((const io_cplan *)j->plan, buf, j->forward, j->fct)) j->rc = -1;
            for (size_t m = 0; m < len; ++m) {
                double *d = (double *)(po + (ptrdiff_t)m * so);
                d[0] = buf[2 * m]; d[1] = buf[2 * m + 1];
            }
        } else if (j->kind == 1) {
            /* general_r2c: always the forward r2hc, conjugate when !forward */
            for (size_t m = 0; m < len; ++m) buf[m] = *(const double *)(pi + (ptrdiff_t)m * si);
            if (io_rplan_exec((const io_rplan *)j->plan, buf, 1, j->fct)) j->rc = -1;
            double sg = j->forward ? 1.0 : -1.0;
            double *d = (double *)po;
            d[0] = buf[0]; d[1] = 0.0;
            size_t i = 1, ii = 1;
            for (; i + 1 < len; i += 2, ++ii) {
                d = (double *)(po + (ptrdiff_t)ii * so);
                d[0] = buf[i]; d[1] = sg * buf[i + 1];
            }
            if (i < len) { d = (double *)(po + (ptrdiff_t)ii * so); d[0] = buf[i]; d[1] = 0.0; }
        } else if (j->kind == 3 || j->kind == 4) {
            /* r2r_fftpack (ExecR2R, pocketfft_hdronly.h:3252-3270): the halfcomplex transform in
               the direction `forward`; real2hermitian=false negates the odd imaginary slots
               before a forward pass, real2hermitian=true after a backward pass.
               separable Hartley (ExecHartley, copy_hartley, pocketfft_hdronly.h:3066-3106):
               forward halfcomplex, then h[0]; h[i] +- h[i+1] into i1 / n - i1; h[n-1] for even n */
            for (size_t m = 0; m < len; ++m) buf[m] = *(const double *)(pi + (ptrdiff_t)m * si);
            int fwd = j->kind == 4 ? 1 : j->forward;
            if (j->kind == 3 && !j->r2c && fwd) for (size_t i = 2; i < len; i += 2) buf[i] = -buf[i];
            if (io_rplan_exec((const io_rplan *)j->plan, buf, fwd, j->fct)) j->rc = -1;
            if (j->kind == 3) {
                if (j->r2c && !fwd) for (size_t i = 2; i < len; i += 2) buf[i] = -buf[i];
                for (size_t m = 0; m < len; ++m) *(double *)(po + (ptrdiff_t)m * so) = buf[m];
            } else {
                double *o = buf + len;  /* second half of the 2(len+1) buffer */
                o[0] = buf[0];
                size_t i = 1, i1 = 1, i2 = len - 1;
                for (; i + 1 < len; i += 2, ++i1, --i2) {
                    o[i1] = buf[i] + buf[i + 1];
                    o[i2] = buf[i] - buf[i + 1];
                }
                if (i < len) o[i1] = buf[i];
                for (size_t m = 0; m < len; ++m) *(double *)(po + (ptrdiff_t)m * so) = o[m];
            }
        } else if (j->kind == 5) {
            for (size_t m = 0; m < len; ++m) buf[m] = *(const double *)(pi + (ptrdiff_t)m * si);
            io_dcst_line(j->type, j->cosine, j->ortho, len, buf, buf + len, j->fct);
            for (size_t m = 0; m < len; ++m) *(double *)(po + (ptrdiff_t)m * so) = buf[len + m];
        } else {
            /* general_c2r: halfcomplex from the input (conjugated when forward), then hc2r */
            double sg = j->forward ? -1.0 : 1.0;
            buf[0] = ((const double *)pi)[0];
            size_t i = 1, ii = 1;
            for (; i + 1 < len; i += 2, ++ii) {
                const double *s = (const double *)(pi + (ptrdiff_t)ii * si);
                buf[i] = s[0]; buf[i + 1] = sg * s[1];
            }
            if (i < len) buf[i] = ((const double *)(pi + (ptrdiff_t)ii * si))[0];
            if (io_rplan_exec((const io_rplan *)j->plan, buf, 0, j->fct)) j->rc = -1;
            for (size_t m = 0; m < len; ++m) *(double *)(po + (ptrdiff_t)m * so) = buf[m];
        }
    }
    free(buf);
    return NULL;
}

static int io_run_axis_x(int kind, size_t ndim, const size_t *shape_lines, const ptrdiff_t *sin, const ptrdiff_t *sout,
                         size_t axis, size_t len, const void *in, void *out, int forward, double fct, int nthreads,
                         int type, int cosine, int ortho, int r2c);
static int io_run_axis(int kind, size_t ndim, const size_t *shape_lines, const ptrdiff_t *sin, const ptrdiff_t *sout,
                       size_t axis, size_t len, const void *in, void *out, int forward, double fct, int nthreads)
{
    return io_run_axis_x(kind, ndim, shape_lines, sin, sout, axis, len, in, out, forward, fct, nthreads, 0, 0, 0, 0);
}
static int io_run_axis_x(int kind, size_t ndim, const size_t *shape_lines, const ptrdiff_t *sin, const ptrdiff_t *sout,
                         size_t axis, size_t len, const void *in, void *out, int forward, double fct, int nthreads,
                         int type, int cosine, int ortho, int r2c)
{
    size_t nlines = 1;
    for (size_t d = 0; d < ndim; ++d) if (d != axis) nlines *= shape_lines[d];
    const void *plan = (kind == 0) ? (const void *)io_make_cplan(len)
                     : (kind == 5) ? (const void *)"direct" : (const void *)io_make_rplan(len);
    if (!plan) return -1;
    if (nthreads < 1) nthreads = 1;
    if ((size_t)nthreads > nlines) nthreads = (int)(nlines ? nlines : 1);
    io_nd_job *jobs = (io_nd_job *)calloc((size_t)nthreads, sizeof(io_nd_job));
    pthread_t *th = (pthread_t *)calloc((size_t)nthreads, sizeof(pthread_t));
    int rc = 0;
    if (!jobs || !th) rc = -1;
    else {
        for (int t = 0; t < nthreads; ++t) {
            io_nd_job v;
            memset(&v, 0, sizeof v);
            v.L.ndim = ndim; v.L.shape = shape_lines; v.L.sin = sin; v.L.sout = sout; v.L.axis = axis; v.L.nlines = nlines;
            v.kind = kind; v.len = len; v.in = (const char *)in; v.out = (char *)out;
            v.forward = forward; v.fct = fct; v.plan = plan; v.t = (size_t)t; v.nt = (size_t)nthreads;
            v.type = type; v.cosine = cosine; v.ortho = ortho; v.r2c = r2c;
            jobs[t] = v;
        }
        for (int t = 1; t < nthreads; ++t) pthread_create(&th[t], NULL, io_nd_worker, &jobs[t]);
        io_nd_worker(&jobs[0]);
        rc = jobs[0].rc;
        for (int t = 1; t < nthreads; ++t) { pthread_join(th[t], NULL); if (jobs[t].rc) rc = jobs[t].rc; }
    }
    free(jobs);
    free(th);
    if (kind == 0) io_destroy_cplan((io_cplan *)plan);
    else if (kind != 5) io_destroy_rplan((io_rplan *)plan);
    return rc;
}

/* error codes shared with the product's C ABI */
#define IO_EINVAL_AXIS   (-2)
#define IO_EREPEAT_AXIS  (-3)
#define IO_ESTRIDE       (-4)
#define IO_ENDIM         (-7)

static int io_check_axes(size_t ndim, size_t naxes, const size_t *axes)
{
    if (ndim < 1) return IO_ENDIM;
    unsigned char seen[64] = { 0 };
    for (size_t a = 0; a < naxes; ++a) {
        if (axes[a] >= ndim) return IO_EINVAL_AXIS;
        if (axes[a] < 64 && seen[axes[a]]++) return IO_EREPEAT_AXIS;
    }
    return 0;
}

/* pocketfft::c2c (pocketfft_hdronly.h:3272-3282): axes in order, the first
   axis reads `in`, later axes read and write `out`, fct on the first axis. */
int io_c2c(size_t ndim, const size_t *shape, const ptrdiff_t *sin, const ptrdiff_t *sout,
           size_t naxes, const size_t *axes, int forward, const double *in, double *out, double fct, int nthreads)
{
    size_t tot = 1;
    for (size_t d = 0; d < ndim; ++d) tot *= shape[d];
    if (ndim >= 1 && tot == 0) return 0;
    int rc = io_check_axes(ndim, naxes, axes);
    if (rc) return rc;
    if (in == out) for (size_t d = 0; d < ndim; ++d) if (sin[d] != sout[d]) return IO_ESTRIDE;
    for (size_t a = 0; a < naxes; ++a) {
        const void *src = a == 0 ? (const void *)in : (const void *)out;
        const ptrdiff_t *ss = a == 0 ? sin : sout;
        rc = io_run_axis(0, ndim, shape, ss, sout, axes[a], shape[axes[a]], src, out, forward, a == 0 ? fct : 1.0, nthreads);
        if (rc) return rc;
    }
    return 0;
}

/* pocketfft::r2c over axes (pocketfft_hdronly.h:3320-3350) */
int io_r2c(size_t ndim, const size_t *shape_in, const ptrdiff_t *sin, const ptrdiff_t *sout,
           size_t naxes, const size_t *axes, int forward, const double *in, double *out, double fct, int nthreads)
{
    size_t tot = 1;
    for (size_t d = 0; d < ndim; ++d) tot *= shape_in[d];
    if (ndim >= 1 && tot == 0) return 0;
    int rc = io_check_axes(ndim, naxes, axes);
    if (rc) return rc;
    if (naxes == 0) return 0;
    size_t last = axes[naxes - 1];
    size_t shape_out[64];
    for (size_t d = 0; d < ndim; ++d) shape_out[d] = shape_in[d];
    shape_out[last] = shape_in[last] / 2 + 1;
    /* the line iterator walks the non-transformed axes, which share the shape */
    rc = io_run_axis(1, ndim, shape_in, sin, sout, last, shape_in[last], in, out, forward, fct, nthreads);
    if (rc || naxes == 1) return rc;
    return io_c2c(ndim, shape_out, sout, sout, naxes - 1, axes, forward, out, out, 1.0, nthreads);
}

/* pocketfft::c2r over axes (pocketfft_hdronly.h:3352-3390) */
int io_c2r(size_t ndim, const size_t *shape_out, const ptrdiff_t *sin, const ptrdiff_t *sout,
           size_t naxes, const size_t *axes, int forward, const double *in, double *out, double fct, int nthreads)
{
    size_t tot = 1;
    for (size_t d = 0; d < ndim; ++d) tot *= shape_out[d];
    if (ndim >= 1 && tot == 0) return 0;
    int rc = io_check_axes(ndim, naxes, axes);
    if (rc) return rc;
    if (naxes == 0) return 0;
    size_t last = axes[naxes - 1];
    if (naxes == 1)
        return io_run_axis(2, ndim, shape_out, sin, sout, last, shape_out[last], in, out, forward, fct, nthreads);
    size_t shape_in[64];
    for (size_t d = 0; d < ndim; ++d) shape_in[d] = shape_out[d];
    shape_in[last] = shape_out[last] / 2 + 1;
    size_t nval = 1;
    for (size_t d = 0; d < ndim; ++d) nval *= shape_in[d];
    ptrdiff_t sinter[64];
    sinter[ndim - 1] = 16;
    for (size_t d = ndim - 1; d-- > 0;) sinter[d] = sinter[d + 1] * (ptrdiff_t)shape_in[d + 1];
    double *tmp = (double *)malloc(sizeof(double) * 2 * nval);
    if (!tmp) return -1;
    rc = io_c2c(ndim, shape_in, sin, sinter, naxes - 1, axes, forward, in, tmp, 1.0, nthreads);
    if (!rc) rc = io_run_axis(2, ndim, shape_out, sinter, sout, last, shape_out[last], tmp, out, forward, fct, nthreads);
    free(tmp);
    return rc;
}

/* real-to-real transforms over axes (pocketfft_hdronly.h:3284-3318, 3392-3445): every axis
   in order, the first reads `in`, later ones read and write `out`, fct on the first axis */
static int io_r2r_axes(int kind, size_t ndim, const size_t *shape, const ptrdiff_t *sin, const ptrdiff_t *sout,
                       size_t naxes, const size_t *axes, const double *in, double *out, double fct, int nthreads,
                       int forward, int type, int cosine, int ortho, int r2c)
{
    size_t tot = 1;
    for (size_t d = 0; d < ndim; ++d) tot *= shape[d];
    if (ndim >= 1 && tot == 0) return 0;
    int rc = io_check_axes(ndim, naxes, axes);
    if (rc) return rc;
    if (in == out) for (size_t d = 0; d < ndim; ++d) if (sin[d] != sout[d]) return IO_ESTRIDE;
    for (size_t a = 0; a < naxes; ++a) {
        const void *src = a == 0 ? (const void *)in : (const void *)out;
        const ptrdiff_t *ss = a == 0 ? sin : sout;
        rc = io_run_axis_x(kind, ndim, shape, ss, sout, axes[a], shape[axes[a]], src, out, forward, a == 0 ? fct : 1.0,
                           nthreads, type, cosine, ortho, r2c);
        if (rc) return rc;
    }
    return 0;
}
/* DCT / DST types 1-4 (pocketfft::dct / dst); DCT-I needs length >= 2 */
int io_dct(size_t ndim, const size_t *shape, const ptrdiff_t *sin, const ptrdiff_t *sout, size_t naxes,
           const size_t *axes, int type, const double *in, double *out, double fct, int ortho, int nthreads)
{
    if (type < 1 || type > 4) return -1;
    for (size_t a = 0; a < naxes; ++a) if (axes[a] < ndim && type == 1 && shape[axes[a]] < 2) return -10;
    return io_r2r_axes(5, ndim, shape, sin, sout, naxes, axes, in, out, fct, nthreads, 1, type, 1, ortho, 0);
}
int io_dst(size_t ndim, const size_t *shape, const ptrdiff_t *sin, const ptrdiff_t *sout, size_t naxes,
           const size_t *axes, int type, const double *in, double *out, double fct, int ortho, int nthreads)
{
    if (type < 1 || type > 4) return -1;
    return io_r2r_axes(5, ndim, shape, sin, sout, naxes, axes, in, out, fct, nthreads, 1, type, 0, ortho, 0);
}
int io_r2r_fftpack(size_t ndim, const size_t *shape, const ptrdiff_t *sin, const ptrdiff_t *sout, size_t naxes,
                   const size_t *axes, int real2hermitian, int forward, const double *in, double *out, double fct,
                   int nthreads)
{
    return io_r2r_axes(3, ndim, shape, sin, sout, naxes, axes, in, out, fct, nthreads, forward, 0, 0, 0,
                       real2hermitian);
}
int io_r2r_separable_hartley(size_t ndim, const size_t *shape, const ptrdiff_t *sin, const ptrdiff_t *sout,
                             size_t naxes, const size_t *axes, const double *in, double *out, double fct, int nthreads)
{
    return io_r2r_axes(4, ndim, shape, sin, sout, naxes, axes, in, out, fct, nthreads, 1, 0, 0, 0, 0);
}
/* genuine Hartley over axes (pocketfft_hdronly.h:3420-3445): Re + Im of the forward DFT over the
   axes, taken here from the full complex transform of the real input */
int io_r2r_genuine_hartley(size_t ndim, const size_t *shape, const ptrdiff_t *sin, const ptrdiff_t *sout,
                           size_t naxes, const size_t *axes, const double *in, double *out, double fct, int nthreads)
{
    size_t tot = 1;
    for (size_t d = 0; d < ndim; ++d) tot *= shape[d];
    if (ndim >= 1 && tot == 0) return 0;
    int rc = io_check_axes(ndim, naxes, axes);
    if (rc) return rc;
    if (naxes == 1) return io_r2r_separable_hartley(ndim, shape, sin, sout, naxes, axes, in, out, fct, nthreads);
    double *c = (double *)malloc(sizeof(double) * 2 * tot);
    if (!c) return -1;
    ptrdiff_t cs[64];
    cs[ndim - 1] = 16;
    for (size_t d = ndim - 1; d-- > 0;) cs[d] = cs[d + 1] * (ptrdiff_t)shape[d + 1];
    size_t idx[64] = { 0 };
    for (size_t e = 0; e < tot; ++e) {
        ptrdiff_t o = 0;
        size_t r = e;
        for (size_t d = ndim; d-- > 0;) { idx[d] = r % shape[d]; r /= shape[d]; o += (ptrdiff_t)idx[d] * sin[d]; }
        c[2 * e] = *(const double *)((const char *)in + o);
        c[2 * e + 1] = 0.0;
    }
    rc = io_c2c(ndim, shape, cs, cs, naxes, axes, 1, c, c, fct, nthreads);
    if (!rc)
        for (size_t e = 0; e < tot; ++e) {
            ptrdiff_t o = 0;
            size_t r = e;
            for (size_t d = ndim; d-- > 0;) { idx[d] = r % shape[d]; r /= shape[d]; o += (ptrdiff_t)idx[d] * sout[d]; }
            *(double *)((char *)out + o) = c[2 * e] + c[2 * e + 1];
        }
    free(c);
    return rc;
}

/* upfirdn (impulse signal.nim:545-594): upsample by `up` (up - 1 zeros between samples,
   length (n - 1) up + 1), full convolution with h, every `down`-th sample from index 0;
   direct sums with compensated accumulation.  Rows b at x + b dx, y + b dy. */
size_t io_upfirdn_length(size_t n, size_t nh, int up, int down)
{
    size_t lc = (n - 1) * (size_t)up + nh;
    return (lc + (size_t)down - 1) / (size_t)down;
}
int io_upfirdn(size_t batch, size_t n, const double *x, size_t dx, size_t nh, const double *h, int up, int down,
               double *y, size_t dy)
{
    if (up < 1 || down < 1 || n < 1 || nh < 1) return -1;
    size_t ny = io_upfirdn_length(n, nh, up, down);
    for (size_t b = 0; b < batch; ++b) {
        const double *xb = x + b * dx;
        for (size_t j = 0; j < ny; ++j) {
            size_t m = j * (size_t)down; /* full-convolution index: c[m] = sum_i u[i] h[m - i] */
            double acc = 0.0, comp = 0.0;
            for (size_t q = 0; q < n; ++q) {
                size_t i = q * (size_t)up;
                if (i > m) break;
                if (m - i >= nh) continue;
                double t = xb[q] * h[m - i], s2 = acc + t;
                comp += fabs(acc) >= fabs(t) ? (acc - s2) + t : (t - s2) + acc;
                acc = s2;
            }
            y[b * dy + j] = acc + comp;
        }
    }
    return 0;
}

/* ------------------------------------------------------------------ */
/* impulse's Nim glue (pocketfft.nim:126-204)                          */
/* ------------------------------------------------------------------ */

/* unpackFFT: halfcomplex of length in_len -> in_len/2+1 (even) or (in_len+1)/2 (odd) complex */
void io_unpack_fft(const double *data, double *out, size_t in_len)
{
    size_t k = 0;
    double re = data[0], im = 0.0;
    out[0] = re; out[1] = im;
    ++k;
    for (size_t i = 1; i < in_len; ++i) {
        if (i & 1) re = data[i];
        else { im = data[i]; out[2 * k] = re; out[2 * k + 1] = im; ++k; }
    }
    if ((in_len & 1) == 0) { out[2 * k] = re; out[2 * k + 1] = 0.0; }
}

/* symmTargetSize (pocketfft.nim:173-180) */
size_t io_symm_target_size_real(size_t len) { return len; }
size_t io_symm_target_size_complex(double last_im, size_t len) { return len * 2 - (last_im == 0.0 ? 2 : 1); }

/* symmetrize: mirror conj(res[i]) into res[out_len-i] for i in 1 ..< ceil(out_len/2)
   (pocketfft.nim:160-171); `is_real` selects the unpackFFT pre-step. */
void io_symmetrize(const double *data, int is_real, size_t in_len, double *res, size_t out_len)
{
    if (is_real) io_unpack_fft(data, res, in_len);
    else memcpy(res, data, in_len * 2 * sizeof(double));
    size_t k = out_len - 1;
    for (size_t i = 1; i < (out_len + 1) / 2; ++i) {
        res[2 * k] = res[2 * i];
        res[2 * k + 1] = -res[2 * i + 1];
        --k;
    }
}

/* initNormalize (pocketfft.nim:199-204): kind 0 backward, 1 ortho, 2 forward, 3 custom */
double io_init_normalize(int kind, int forward, double value, size_t length)
{
    switch (kind) {
    case 0: return forward ? 1.0 : 1.0 / (double)length;
    case 1: return 1.0 / sqrt((double)length);
    case 2: return forward ? 1.0 / (double)length : 1.0;
    default: return value;
    }
}
