// ig_types.h -- plain descriptors shared by the host engine and the kernels.
#pragma once

namespace ig {

// q = n / d for 0 <= n < 2^31 as (n * m) >> s, m = ceil(2^s / d), s = 31 + ceil(log2 d):
// the error term n (m - 2^s/d) / 2^s stays below 1/d, so the quotient is exact
struct FastDiv {
    unsigned m;
    int s;
};

constexpr int kMaxStages = 24;
constexpr int kMaxLinesPerCta = 128;
constexpr int kEMax = 16;  // largest complex-elements-per-thread variant of the core kernel

struct StageDesc {
    int R, ns, tw;  // radix, product of previous radices, twiddle offset (cx units)
    int twp;        // offset into the FP32 pair twiddle table (16-byte entries; ns even)
    FastDiv fns;    // division by ns
};

// layout classes of the kernel variants: the common layouts compile without
// per-element runtime checks
constexpr int LAY_GEN = 0;    // any layout (runtime kinds, pre / post steps, pairs, twiddles)
constexpr int LAY_C2C = 1;    // complex in, complex out, nothing else
constexpr int LAY_R2HC = 2;   // contiguous reals as complex pairs, real split, halfcomplex out
constexpr int LAY_PR2HC = 3;  // two real lines per complex line, pair split, halfcomplex out
constexpr int LAY_TW = 4;     // complex in / out with the four-step twiddle or a pointwise table
constexpr int LAY_C2R = 6;    // half spectrum in (Hermitian pre-step), real pairs out (c2r; as LAY_R2C)
constexpr int LAY_RC = 7;     // LAY_TW with the row-convolution mode (IODesc::rowconv) compiled in

// Threads a CTA may have: 512; the wide double-float 8-element variants (a
// separate instantiation at 80-96 registers) run lines of up to 8 x 672 =
// 5376 points as one 672-thread CTA instead of 16-element threads at half the
// warps
constexpr int kMaxThreadsE8 = 672;
constexpr int LAY_R2C = 5;    // contiguous reals as complex pairs, real split, half spectrum out (r2c; the
                              // shared-memory kernel runs it as LAY_GEN, the FP32 line kernel natively)

// radix classes of the kernel variants
constexpr int RS_P2 = 0;   // 2, 4, 8, 16
constexpr int RS_P235 = 1; // 2, 4, 8, 16, 3, 5, 9
constexpr int RS_ALL = 2;  // 2, 3, 4, 5, 7, 8, 9, 11, 16
constexpr int RS_FULL = 3; // all of RS_ALL, 13, and the Rader steps (also the generic-layout kernels)
constexpr int RS_ALLR = 4; // the radices of RS_ALL and the Rader steps (double-float 8-element cores only)

// last radices of k_fft_line's halfcomplex variant: the two mirror
// butterflies of a pair slot stay in registers, so larger radices would spill
constexpr bool line_r2hc_last_ok(int R) { return R == 2 || R == 3 || R == 4 || R == 5 || R == 8; }
// first and last radices k_fft_line compiles
constexpr bool line_edge_ok(int R) { return R == 2 || R == 3 || R == 4 || R == 5 || R == 8 || R == 16; }

enum InKind { IN_C = 0, IN_R = 1, IN_P = 2, IN_HC = 3 };
enum OutKind { OUT_C = 0, OUT_R = 1, OUT_P = 2, OUT_HC = 3 };
enum PreKind { PRE_NONE = 0, PRE_HERM_EVEN = 1, PRE_HERM_ODD = 2 };
enum PostKind { POST_NONE = 0, POST_SPLIT = 1, POST_PAIR = 2, POST_SPLIT4 = 3 };
// POST_SPLIT4: the real split fused into the second pass of a four-step core:
// the lines of a CTA come in pairs (row r, row N1 - r) of the transform's
// N1 x N2 layout (rows 0 and N1/2 paired with themselves), and the epilogue
// writes X[k], X[M - k] (k = r + N1 u) as halfcomplex.  Line l is row slot
// l mod bn0 (bn0 = N1 + (1 or 2)) of transform l / bn0; the input offset of a
// slot is its row times bsi0

struct CoreDesc {
    int M;    // logical complex length of the core transform
    int L;    // Stockham length run in shared memory (M, or n2 for Bluestein)
    int LS;   // shared-memory complex slots per line (>= max(L, M + 1))
    int blue; // 1: Bluestein core, 2: Rader core (prime M, Stockham length M - 1)
    int pad;  // shared-memory padding: slot i is stored at i + (i >> pad)
    int E;    // complex elements per thread (kernel variant 8 or 16): L / E threads per line
    int rs;   // radix class of the kernel variant (0: 2/4/8/16, 1: + 3/5, 2: all)
    int lpc_pref;  // lines per CTA chosen by the autotuner (0: planner default)
    int db;   // 1: double-buffered stages (two line buffers; always with E = 8)
    float neg1;  // -1 (a runtime value for the packed double-float twiddle products)
    int nst;
    StageDesc st[kMaxStages];
    const void *tw;     // cx<T> stage twiddles, forward sign
    const void *twp;    // FP32: the same twiddles for butterfly pairs (k_fft_pair), stages with ns even
    const void *chirp;  // cx<T> exp(+i pi m^2 / M), m < M  (Bluestein)
    const void *chirpf; // cx<T> FFT_L of the padded chirp / L  (Bluestein)
    const void *rtw;    // cx<T> exp(-2 pi i k / (2M)), k <= M  (real split)
    const int *rin;     // Rader (blue = 2): g^-q mod M, q < M - 1
    const int *rout;    // Rader: p with g^p = u, 0 < u < M
};

struct IODesc {
    const char *in;
    char *out;
    long long is, os;       // byte stride along the line (between storage units of the kind)
    long long ps_in, ps_out;  // IN_P / OUT_P: bytes from a unit's real value to its second real
    long long nlines;
    long long bn[3];        // batch dims: line l -> (l % bn0, (l / bn0) % bn1, l / (bn0 bn1))
    long long bsi[3], bso[3];
    FastDiv fb0, fb1;       // division by bn[0], bn[1] (line numbers are < 2^31)
    int in_kind, out_kind, pre, post;
    int cnt_in, cnt_out;    // storage units per line
    int conj_in, conj_out;
    int real_out;           // output is the spectrum of real data (zero DC / Nyquist imaginary parts)
    // two real lines per complex line (odd real lengths): line l of the
    // kernel covers real lines a (at the line's offset) and b (at +pair_in /
    // +pair_out); b is absent when 2 * (l mod bn0) + 1 >= pair_n0
    int pair;
    long long pair_in, pair_out, pair_n0;
    int cols_in, cols_out;  // 1: consecutive threads walk consecutive lines
    int lpc, tpl;           // lines per CTA, threads per line
    long long nreal;        // real length N for halfcomplex units
    int fwd;                // direction of the core transform
    double fct;             // output scale
    // fct pre-split on the host (the device never compares or converts
    // doubles: those instructions issue on GB300's narrow FP64 pipe):
    // FP32 value, and mantissa (hi, lo) in [1, 2) with exponent for double-float
    float fct_f, fct_h, fct_l;
    int fct_e;
    int lay;                // layout class of the kernel variant (set by the host)
    int pf_lines;           // paired-lane kernel: prefetch into L2 the points of line l + pf_lines (0: none)
    // four-step inter-pass twiddle on output unit u of line l:
    // t = ((l % bn0) * u) mod tw4N, value w_hi[t / tw4S] * w_lo[t % tw4S]
    int tw4;
    int tw4_dim1;           // the twiddle's row index is batch dim 1 ((l / bn0) % bn1), not dim 0
    long long tw4N, tw4S;
    FastDiv fdS;            // division by tw4S
    const void *tw4hi, *tw4lo;
    const void *tw4tab;     // when set: the full table, N1 entries a line (stage-twiddle format)
    // pointwise product on output unit u of line l with tab[(l % bn0) * mul_a + u * mul_b]
    // (conjugated when mul_conj); Bluestein's convolution step on a four-step core
    const void *mul;
    long long mul_a, mul_b;
    int mul_conj;
    // storage complex of output unit 0 of each transform's first line (before
    // the product), one per transform: Rader's A[0] on a multi-pass core
    void *keep0;
    int keep0_rows;  // lines per transform: 1 (one-pass core) or N1 (four-step second pass)
    // row convolution (twiddle / table layout only): the lines are rows k1 of
    // a four-step core (or whole lines, N1 = 1); forward FFT, the `mul` product
    // (and keep0) between two stage passes, inverse FFT, and the inverse
    // four-step twiddle (tw4) in the epilogue
    int rowconv;
    // per-line byte offsets (device arrays) replacing the batch dims when set
    const long long *loff_in, *loff_out;
    // POST_SPLIT4 (when split_N1 != 0): the real-split twiddles exp(-2 pi i k / 2M), k <= M, and N1
    const void *split_tw;
    int split_N1;
};

// one group of the persistent work list: a core, a line set, its block count;
// io.in / io.out are byte offsets from base in_base / out_base
// (0 input, 1 output, 2 scratch) of the launch
struct WorkGroup {
    CoreDesc P;
    IODesc io;
    int in_base, out_base;
};

// Elementwise line maps of the multi-pass paths (k_gather / k_scatter).
// `ext` is the user-facing side (IODesc fields in/out, is/os, bn/bsi/bso,
// kinds, conj, nreal); `scr` is a scratch array of contiguous complex lines.
enum MapKind {
    MAP_PLAIN = 0,      // unit u <-> scratch[u]
    MAP_BLUE = 1,       // times chirp (Bluestein pre / post); gather zero-pads to scr_len
    MAP_HERM_EVEN = 2,  // gather: halfcomplex X[0..M] -> Z[0..M) (inverse of the real split)
    MAP_SPLIT_EVEN = 3, // scatter: Z[0..M) -> X[0..M] (real split), written as halfcomplex or half spectrum
    MAP_RADER = 4,      // gather: scratch[q] = x[ridx[q]], x[0] to x0buf; scatter: X[0] = x0 + A0,
                        // X[u] = x0 + scratch[ridx[u]]; conjugated on both sides for the backward direction
};
struct MapDesc {
    int kind;
    long long M;        // complex units per line on the scratch side
    long long scr_len;  // scratch line length (elements)
    char *scr;          // scratch base (storage complex)
    const void *chirp;  // cx<T>, MAP_BLUE
    const void *rtw;    // cx<T> exp(-2 pi i k/2M), k <= M, real split
    int fwd;            // Bluestein / Rader direction
    const int *ridx;    // MAP_RADER: g^-q (gather) or the discrete log (scatter)
    void *x0buf;        // MAP_RADER: storage complex x[0] of each scratch line
    void *a0buf;        // MAP_RADER: storage complex A[0] of each scratch line
    FastDiv fsl, fcnt;  // division by scr_len and by the user side's unit count (set by the launchers)
};


// real-to-real transforms along one axis (pocketfft's dct / dst / r2r_fftpack /
// Hartley): a pre-map from the user's lines into contiguous scratch lines, one
// FFT of the scratch lines, a post-map back to the user's lines
enum R2RMode {
    R2R_DCT1 = 1, R2R_DCT2, R2R_DCT3, R2R_DCT4,   // complex scratch of length L2, FFT forward
    R2R_DST1 = 5, R2R_DST2, R2R_DST3, R2R_DST4,
    R2R_COPY = 9,     // real scratch; halfcomplex FFT; elements 2, 4, ... negated when neg_even
    R2R_HARTLEY = 10, // real scratch; forward halfcomplex FFT; post-map h[i] +- h[i+1]
};
struct R2RDesc {
    int mode;
    int ortho;
    int neg_even;       // R2R_COPY: negate elements 2, 4, ... in this map
    long long N;        // length along the axis
    long long L2;       // scratch elements per line
    char *scr;          // scratch lines (storage type), line l at l * L2
    const void *tw1;    // cx<T> exp(-2 pi i m / 4N), m <= N
    const void *tw2;    // cx<T> exp(-2 pi i (2k + 1) / 8N), k < N
    double fct;         // DCT / DST: scale applied by the post-map
    FastDiv fL2, fN;    // division by L2 and N (set by the launcher)
};
// genuine Hartley over several axes: the r2c half spectrum (contiguous, shape
// `tshp`) folded into the real output: out[i] = re + im, out[-i] = re - im
struct HartleyDesc {
    int ndim;
    long long tshp[8];
    long long shape[8];
    long long sout[8];  // bytes
    int rev[8];         // 1: transformed axis (index reversed for the mirror)
    long long total;
};

enum Arith { A_F32 = 0, A_DF = 1, A_F64 = 2 };

}  // namespace ig
