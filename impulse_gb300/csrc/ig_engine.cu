// ig_engine.cu -- host side of the GPU FFT engine: planner, plan cache,
// workspace, executor and the C ABI declared in include/impulse_gpu.h.
//
// Planning follows the reference's structure (factorise, build twiddles,
// choose FFTPACK-style passes or Bluestein: impulse/fft/c_pocketfft/
// pocketfft.c:954-983, 2066-2153; pocketfft_hdronly.h:2349-2417, 2655-2706)
// but targets the GPU: a length is run as one shared-memory Stockham kernel
// when it fits on one SM, as a four-step decomposition of two such kernels
// otherwise, and through Bluestein when it has a prime factor above 11.  All
// tables are built on the GPU in FP64.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <functional>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <list>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/impulse_gpu.h"
#include "ig_launch.h"

namespace ig {

static thread_local std::string g_err;
static std::atomic<unsigned long long> g_launches{0};
static int g_f64_arith = 0;  // 0 double-float, 1 native FP64

struct Error {
    int code;
    std::string msg;
};
[[noreturn]] static void raise(int code, const std::string &msg) { throw Error{code, msg}; }
static void ck(cudaError_t e, const char *what)
{
    if (e != cudaSuccess) {
        cudaGetLastError();
        if (e == cudaErrorMemoryAllocation) raise(IG_ENOMEM, std::string(what) + ": " + cudaGetErrorString(e));
        raise(IG_ECUDA, std::string(what) + ": " + cudaGetErrorString(e));
    }
}
static void count_launch()
{
    g_launches.fetch_add(1, std::memory_order_relaxed);
    ck(cudaGetLastError(), "kernel launch");
}

static size_t slot_bytes(Arith a) { return a == A_F32 ? 8 : 16; }
static size_t store_real_bytes(Arith a) { return a == A_F32 ? 4 : 8; }

// --------------------------------------------------------------------------
// device memory
// --------------------------------------------------------------------------
struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
    DevBuf() = default;
    explicit DevBuf(size_t n)
    {
        bytes = n;
        if (n) {
            if (getenv("IG_FAIL_MALLOC")) raise(IG_ENOMEM, "cudaMalloc: injected failure (IG_FAIL_MALLOC)");
            ck(cudaMalloc(&p, n), "cudaMalloc");
        }
    }
    ~DevBuf()
    {
        if (p) cudaFree(p);
    }
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
};

static int device_id()
{
    int d = 0;
    ck(cudaGetDevice(&d), "cudaGetDevice");
    return d;
}

// shared memory of one SM (all resident CTAs together)
static long long smem_per_sm()
{
    static long long v = 0;
    if (!v) {
        int x = 0;
        ck(cudaDeviceGetAttribute(&x, cudaDevAttrMaxSharedMemoryPerMultiprocessor, device_id()), "smem attr");
        v = x;
    }
    return v;
}

static int g_max_smem = 0;
static int max_smem()
{
    if (!g_max_smem) {
        int v = 0;
        ck(cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, device_id()), "smem attr");
        g_max_smem = v - 1024;  // room for the kernels' static shared memory
    }
    return g_max_smem;
}

// --------------------------------------------------------------------------
// cores: complex transforms of one length
// --------------------------------------------------------------------------
// ---- autotuner configuration --------------------------------------------------
// Per (arithmetic, Stockham or four-step length): radix order (0 large radices
// first, 1 reversed), elements per thread (0 default, 8, 16), lines per CTA
// (0 default) and the four-step split N1 (0 default).
struct TuneCfg {
    int order = 0, E = 0, lpc = 0, no9 = 0;
    long long N1 = 0;
    double ms = 0.0;
};
static std::mutex g_tune_mu;
static std::map<std::pair<int, long long>, TuneCfg> g_tune;
static thread_local const TuneCfg *g_cfg_override = nullptr;
static thread_local long long g_cfg_override_len = 0;
static thread_local int g_cfg_override_arith = -1;

static TuneCfg tune_lookup(int a, long long L)
{
    TuneCfg c;
    if (g_cfg_override && g_cfg_override_len == L && g_cfg_override_arith == a) {
        c = *g_cfg_override;
    } else {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_tune.find(std::make_pair(a, L));
        if (it != g_tune.end()) c = it->second;
    }
    // 8 elements a thread beyond 4096 points: the wide variants exist for
    // double-float only (elsewhere the default, 16 beyond 4096, applies)
    if (a != A_DF && c.E == 8) c.E = 0;
    return c;
}

static int elems_per_thread(long long L, int cfgE = 0)
{
    // (tuned plans may take 8 elements a thread up to kMaxThreadsE8 threads)
    if (cfgE == 8 && L <= 8LL * kMaxThreadsE8) return 8;
    if (cfgE == 16) return 16;
    return L <= 4096 ? 8 : 16;
}

// Radices for a Stockham length L.  Cores of 8 elements per thread (up to
// 4096 points by default) use radix 8 at most, since a radix-16 stage would
// leave half the threads idle.
static bool gpu_factor(long long L, std::vector<int> &rad, int E = 0, int order = 0, int no9 = 0)
{
    rad.clear();
    long long n = L;
    const bool small = elems_per_thread(L, E) == 8;
    while (!small && n % 16 == 0) { rad.push_back(16); n /= 16; }
    while (small && n % 8 == 0) { rad.push_back(8); n /= 8; }
    if (n % 8 == 0) { rad.push_back(8); n /= 8; }
    if (n % 4 == 0) { rad.push_back(4); n /= 4; }
    if (n % 2 == 0) { rad.push_back(2); n /= 2; }
    for (int p : {13, 11, 7, 5, 9, 3}) {
        if (p == 9 && no9) continue;  // tuned plans may prefer two radix-3 stages
        while (n % p == 0) { rad.push_back(p); n /= p; }
    }
    if (order == 1) std::reverse(rad.begin(), rad.end());
    return n == 1;
}

static long long good_size_gpu(long long n)
{
    // smallest 2^a 3^b 5^c 7^d 11^e >= n (pocketfft.c:245-260)
    if (n <= 6) return n;
    long long best = 2 * n;
    for (long long f2 = 1; f2 < best; f2 *= 2)
        for (long long f3 = f2; f3 < best; f3 *= 3)
            for (long long f5 = f3; f5 < best; f5 *= 5)
                for (long long f7 = f5; f7 < best; f7 *= 7)
                    for (long long f11 = f7; f11 < best; f11 *= 11)
                        if (f11 >= n) best = f11;
    return best;
}

struct Core {
    Arith a;
    long long M = 0;
    bool real_tw = false;  // rtw built (core of an even real transform of length 2M)
    int kind = 0;          // 0 smem, 1 four-step, 2 Bluestein / 3 Rader over a multi-pass core
    CoreDesc d{};
    std::vector<std::unique_ptr<DevBuf>> mem;
    // four-step
    long long N1 = 0, N2 = 0;
    std::shared_ptr<Core> c1, c2;
    const void *whi = nullptr, *wlo = nullptr, *tw4tab = nullptr;
    // Bluestein over a large core
    long long n2 = 0;
    std::shared_ptr<Core> sub;
    const void *chirp = nullptr, *chirpf = nullptr;
    const void *rtw = nullptr;

    void *alloc(size_t bytes)
    {
        mem.emplace_back(new DevBuf(bytes));
        return mem.back()->p;
    }
};

static std::mutex g_mu;
static std::map<std::tuple<int, int, long long, bool>, std::shared_ptr<Core>> g_cores;

static std::shared_ptr<Core> get_core(Arith a, long long M, bool real_tw);

static void launch_stage_tw(Arith a, void *tw, int R, int ns)
{
    cudaError_t e = a == A_F32 ? Launch<TagF32>::stage_tw(tw, R, ns)
                  : a == A_DF  ? Launch<TagDF>::stage_tw(tw, R, ns)
                               : Launch<TagF64>::stage_tw(tw, R, ns);
    ck(e, "twiddle table");
    count_launch();
}
static void launch_roots_a(Arith a, void *out, long long count, unsigned long long mult, unsigned long long D)
{
    cudaError_t e = a == A_F32 ? Launch<TagF32>::roots(out, count, mult, D)
                  : a == A_DF  ? Launch<TagDF>::roots(out, count, mult, D)
                               : Launch<TagF64>::roots(out, count, mult, D);
    ck(e, "roots table");
    count_launch();
}
static void launch_convert_a(Arith a, const void *in, void *out, long long n)
{
    cudaError_t e = a == A_F32 ? Launch<TagF32>::convert64(in, out, n)
                  : a == A_DF  ? Launch<TagDF>::convert64(in, out, n)
                               : Launch<TagF64>::convert64(in, out, n);
    ck(e, "table conversion");
    count_launch();
}

static constexpr int kMaxThreads = 512;

// smem slots a core of Stockham length L needs per line
static long long smem_slots(long long L, long long M) { return std::max(L, M + 1); }


static bool fits_smem(Arith a, long long L, long long M)
{
    long long tpl = (L + kEMax - 1) / kEMax;
    if (tpl > kMaxThreads) return false;
    long long slots = smem_slots(L, M);
    slots += (slots >> 3) + 1;  // worst-case padding, and the odd per-line stride
    return slots * (long long)slot_bytes(a) <= (long long)max_smem();
}

struct Exec;
static void run_core_on_device(const Core &c, const void *in, void *out, long long batch, int fwd, double fct,
                               cudaStream_t st);

static FastDiv make_fdiv(unsigned d)
{
    int lg = 0;
    while ((1ull << lg) < d) ++lg;
    FastDiv f;
    f.s = 31 + lg;
    f.m = (unsigned)(((1ull << f.s) + d - 1) / d);
    return f;
}

// fct as the kernels consume it: FP32 value, and m * 2^e with m in [1, 2)
// split into two floats for double-float
static void set_fct_parts(IODesc &io)
{
    io.fct_f = (float)io.fct;
    if (io.fct == 0.0 || !std::isfinite(io.fct)) {
        io.fct_h = (float)io.fct;
        io.fct_l = 0.0f;
        io.fct_e = 0;
        return;
    }
    int ex = 0;
    double m = std::frexp(io.fct, &ex);  // fct = m 2^ex, |m| in [0.5, 1)
    m *= 2.0;
    ex -= 1;
    io.fct_h = (float)m;
    io.fct_l = (float)(m - (double)io.fct_h);
    io.fct_e = ex;
}

// layout class of the kernel variant for a line descriptor (the specialised
// variants compile the common layouts without per-element runtime checks)
static int choose_layout(Arith a, const IODesc &io)
{
    if (a == A_F64) return LAY_GEN;
    const bool plain = !io.conj_in && !io.conj_out && !io.real_out && io.pre == PRE_NONE;
    // the twiddle / table variant also keeps Rader's unit 0 (keep0) before the product
    if (io.keep0 && !(io.tw4 || io.mul)) return LAY_GEN;
    if (io.rowconv)
        return (plain && !io.pair && io.post == POST_NONE && io.in_kind == IN_C && io.out_kind == OUT_C) ? LAY_RC
                                                                                                          : LAY_GEN;
    if (io.tw4 || io.mul)
        return (plain && !io.pair && io.post == POST_NONE && io.in_kind == IN_C && io.out_kind == OUT_C) ? LAY_TW
                                                                                                          : LAY_GEN;
    // r2c's last axis: contiguous reals, real split, half spectrum with real DC
    // and Nyquist bins (conjugated for a backward r2c)
    if (a != A_F64 && !io.pair && io.in_kind == IN_C && io.out_kind == OUT_C && io.post == POST_SPLIT && io.real_out &&
        !io.conj_in && io.pre == PRE_NONE && !io.keep0 && !io.mul && !io.tw4)
        return LAY_R2C;
    // c2r's last axis: half spectrum in (Hermitian pre-step), real pairs out
    if (a != A_F64 && !io.pair && io.in_kind == IN_C && io.out_kind == OUT_C && io.pre == PRE_HERM_EVEN &&
        io.post == POST_NONE && !io.conj_out && !io.real_out && !io.keep0 && !io.mul && !io.tw4)
        return LAY_C2R;
    if (!plain) return LAY_GEN;
    if (!io.pair && io.in_kind == IN_C && io.out_kind == OUT_C && io.post == POST_NONE) return LAY_C2C;
    // the fused four-step split reads complex rows and has its own epilogue
    if (!io.pair && io.in_kind == IN_C && io.out_kind == OUT_HC && io.post == POST_SPLIT4) return LAY_C2C;
    if (!io.pair && io.in_kind == IN_C && io.out_kind == OUT_HC && io.post == POST_SPLIT) return LAY_R2HC;
    if (io.pair && io.in_kind == IN_R && io.out_kind == OUT_HC && io.post == POST_PAIR) return LAY_PR2HC;
    return LAY_GEN;
}

// line-number decomposition of the kernels uses 32-bit fast division
static void set_line_divs(IODesc &io)
{
    set_fct_parts(io);
    if (io.nlines >= (1LL << 31) || io.bn[0] >= (1LL << 31) || io.bn[1] >= (1LL << 31))
        raise(IG_ETOOLARGE, "more than 2^31 lines in one launch");
    io.fb0 = make_fdiv((unsigned)std::max<long long>(1, io.bn[0]));
    io.fb1 = make_fdiv((unsigned)std::max<long long>(1, io.bn[1]));
}

// shared-memory wavefronts of one warp-wide access (quarter-warp phases for
// 16-byte slots, half-warp phases for 8-byte slots)
static int wavefronts(const int *addr, int n, int slot)
{
    const int group = slot == 16 ? 8 : 16, nslot = group;
    int tot = 0;
    for (int q = 0; q < n; q += group) {
        int cnt[16] = {0}, worst = 0;
        for (int a = q; a < std::min(n, q + group); ++a) {
            bool dup = false;
            for (int b = q; b < a; ++b) dup |= addr[b] == addr[a];
            if (dup) continue;
            int c = ++cnt[addr[a] % nslot];
            worst = std::max(worst, c);
        }
        tot += worst;
    }
    return tot;
}

// pick the padding shift (i -> i + (i >> pad)) with the fewest simulated
// shared-memory wavefronts over the stages of the first warp
static int choose_pad(const CoreDesc &d, int slot)
{
    const int L = d.L;
    const int tpl = (L + d.E - 1) / d.E;
    int best_pad = 31;
    long long best = -1;
    for (int pad : {31, 5, 4, 3}) {
        long long cost = 0;
        for (int s = 0; s < d.nst; ++s) {
            const int R = d.st[s].R, ns = d.st[s].ns, nr = L / R;
            int la[32], sa[32];
            for (int w = 0; w < std::min(tpl, 64); w += 32) {
                int n = 0;
                for (int l = 0; l < 32; ++l) {
                    int j = w + l;
                    if (j >= nr || j >= tpl) break;
                    ++n;
                }
                if (!n) continue;
                for (int m = 0; m < R; ++m) {
                    for (int l = 0; l < n; ++l) {
                        int j = w + l;
                        int a = j + m * nr, b = (j / ns) * ns * R + (j % ns) + m * ns;
                        la[l] = a + (a >> pad);
                        sa[l] = b + (b >> pad);
                    }
                    cost += wavefronts(la, n, slot) + wavefronts(sa, n, slot);
                }
            }
        }
        if (best < 0 || cost < best) {
            best = cost;
            best_pad = pad;
        }
    }
    return best_pad;
}

static void finish_layout(Core &c, long long L, long long M, const TuneCfg &cfg = TuneCfg())
{
    c.d.E = elems_per_thread(L, cfg.E);
    c.d.lpc_pref = cfg.lpc;
    bool odd35 = false, odd711 = false, full = c.d.blue == 2;
    for (int s = 0; s < c.d.nst; ++s) {
        odd35 |= c.d.st[s].R == 3 || c.d.st[s].R == 5 || c.d.st[s].R == 9;
        odd711 |= c.d.st[s].R == 7 || c.d.st[s].R == 11;
        full |= c.d.st[s].R == 13;
    }
    c.d.rs = full ? RS_FULL : odd711 ? RS_ALL : odd35 ? (c.d.E == 8 ? RS_P235 : RS_ALL) : RS_P2;
    // Rader in one CTA without radix 13, double-float 8-element cores: the
    // 7/11 class with the Rader steps, at 80 registers instead of the full
    // class's 96 (three CTAs per SM instead of two; IG_NO_RADER_ALL=1: full)
    static const bool rader_all = getenv("IG_NO_RADER_ALL") == nullptr;
    if (c.d.blue == 2 && rader_all && c.a == A_DF && c.d.E == 8) {
        bool r13 = false;
        for (int s = 0; s < c.d.nst; ++s) r13 |= c.d.st[s].R == 13;
        if (!r13) c.d.rs = RS_ALLR;
    }
    // double-float 8-element kernels: the 2/3/5 variant fits the register cap
    // without spills where the power-of-two one does not
    if (c.a == A_DF && c.d.E == 8 && c.d.rs == RS_P2) c.d.rs = RS_P235;
    c.d.pad = choose_pad(c.d, (int)slot_bytes(c.a));
    long long last = std::max(L, M + 1) - 1;
    c.d.LS = (int)(last + (last >> c.d.pad) + 1);
    // double-buffered stages whenever two line buffers fit (always for E = 8)
    // (margin: the kernels' static shared memory comes out of the same budget)
    const long long db_cap = (long long)max_smem() - 4096;
    c.d.db = c.d.E == 8 || 2LL * c.d.LS * (long long)slot_bytes(c.a) <= db_cap;
    if (!c.d.db) {
        // less padding (more bank conflicts) when that lets the stages double-buffer
        for (int pad : {5, 31}) {
            if (pad <= c.d.pad) continue;
            const long long ls = last + (last >> pad) + 1;
            if (2LL * ls * (long long)slot_bytes(c.a) <= db_cap) {
                c.d.pad = pad;
                c.d.LS = (int)ls;
                c.d.db = 1;
                break;
            }
        }
    }
}

static void build_stockham(Core &c, long long L, const std::vector<int> &rad)
{
    c.d.L = (int)L;
    c.d.nst = (int)rad.size();
    if (c.d.nst > kMaxStages) raise(IG_ETOOLARGE, "too many FFT stages");
    long long ns = 1, off = 0;
    for (size_t s = 0; s < rad.size(); ++s) {
        c.d.st[s].R = rad[s];
        c.d.st[s].ns = (int)ns;
        c.d.st[s].tw = (int)off;
        c.d.st[s].fns = make_fdiv((unsigned)ns);
        off += ns * (rad[s] - 1);
        ns *= rad[s];
    }
    // one complex per twiddle (double-float: (wr.h, wi.h, wr.l, wi.l), 16 bytes)
    const size_t twb = slot_bytes(c.a);
    c.d.neg1 = -1.0f;
    void *tw = c.alloc(std::max<long long>(off, 1) * twb);
    c.d.tw = tw;
    for (size_t s = 0; s < rad.size(); ++s) {
        void *p = (char *)tw + (size_t)c.d.st[s].tw * twb;
        launch_stage_tw(c.a, p, rad[s], c.d.st[s].ns);
    }
    // FP32 cores with an even first radix: the same twiddles laid out for
    // butterfly pairs (k_fft_pair), stages after the first
    c.d.twp = nullptr;
    if (c.a == A_F32 && !rad.empty() && rad[0] % 2 == 0) {
        long long offp = 0;
        for (size_t s = 1; s < rad.size(); ++s) {
            c.d.st[s].twp = (int)offp;
            offp += (c.d.st[s].ns / 2) * (long long)(rad[s] - 1);
        }
        void *twp = c.alloc(std::max<long long>(offp, 1) * 16);
        c.d.twp = twp;
        for (size_t s = 1; s < rad.size(); ++s) {
            ck(launch_stage_twp((char *)twp + (size_t)c.d.st[s].twp * 16, rad[s], c.d.st[s].ns), "pair twiddle table");
            count_launch();
        }
    }
}

// Bluestein tables for a logical length M over a Stockham/four-step length L:
// chirp[m] = exp(+i pi m^2/M), chirpf = FFT_L(padded chirp)/L, computed from
// FP64 tables with the double-float engine, then rounded to the core type.
static void build_chirp(Core &c, long long M, long long L, void *&chirp, void *&chirpf)
{
    DevBuf bk64(M * 16), pad(L * 16);
    ck(launch_chirp64(bk64.p, M), "chirp");
    count_launch();
    ck(launch_pad_chirp64(bk64.p, pad.p, M, L), "chirp padding");
    count_launch();
    // the padded chirp's spectrum in FP64-class arithmetic: native FP64 for
    // native-FP64 plans, double-float otherwise
    auto dfcore = get_core(c.a == A_F64 ? A_F64 : A_DF, L, false);
    run_core_on_device(*dfcore, pad.p, pad.p, 1, 1, 1.0, 0);
    chirp = c.alloc(M * slot_bytes(c.a));
    chirpf = c.alloc(L * slot_bytes(c.a));
    launch_convert_a(c.a, bk64.p, chirp, M);
    launch_convert_a(c.a, pad.p, chirpf, L);
    ck(cudaDeviceSynchronize(), "chirp tables");
}

// Rader tables for a prime M over the Stockham length L = M - 1: the index
// maps of the generator g and B = FFT_L(exp(-2 pi i g^m / M)) / L, computed
// from long-double roots with the double-float engine, then rounded to the
// core type.
static bool is_prime(long long n)
{
    if (n < 2) return false;
    for (long long d = 2; d * d <= n; ++d)
        if (n % d == 0) return false;
    return true;
}
static long long powmod(long long b, long long e, long long m)
{
    long long r = 1;
    b %= m;
    while (e) {
        if (e & 1) r = r * b % m;
        b = b * b % m;
        e >>= 1;
    }
    return r;
}
static long long primitive_root(long long p)
{
    std::vector<long long> fac;
    long long n = p - 1;
    for (long long d = 2; d * d <= n; ++d)
        if (n % d == 0) {
            fac.push_back(d);
            while (n % d == 0) n /= d;
        }
    if (n > 1) fac.push_back(n);
    for (long long g = 2; g < p; ++g) {
        bool ok = true;
        for (long long f : fac)
            if (powmod(g, (p - 1) / f, p) == 1) { ok = false; break; }
        if (ok) return g;
    }
    return 1;
}
// Rader in one CTA when M - 1 factors into the kernel radices and its core
// runs double-buffered (a single-buffered 16-element core spills registers);
// over a multi-pass core when M - 1 splits into two such factors.
static bool rader_single(Arith a, long long M, const TuneCfg &cfg)
{
    std::vector<int> rad;
    if (!gpu_factor(M - 1, rad, cfg.E, cfg.order, cfg.no9) || !fits_smem(a, M - 1, M)) return false;
    if (elems_per_thread(M - 1, cfg.E) == 8) return true;
    if (getenv("IG_RADER_SB")) return true;  // single-buffered 16-element Rader core (measurement)
    const long long slots = (M + 1) + ((M + 1) >> 3);
    return 2 * slots * (long long)slot_bytes(a) <= (long long)max_smem() - 4096;
}
static bool rader_multi(Arith a, long long M)
{
    const long long L = M - 1;
    for (long long d = 2; d * d <= L; ++d) {
        if (L % d) continue;
        std::vector<int> r1, r2;
        if (gpu_factor(d, r1) && gpu_factor(L / d, r2) && fits_smem(a, d, d) && fits_smem(a, L / d, L / d))
            return true;
    }
    return false;
}

static void build_rader(Core &c, long long M)
{
    const long long L = M - 1;
    const long long g = primitive_root(M), gi = powmod(g, M - 2, M);
    std::vector<int> rin(L), rout(M, 0);
    std::vector<double> b(2 * L);
    long long x = 1, y = 1;
    for (long long q = 0; q < L; ++q) {
        rin[q] = (int)x;        // g^-q
        rout[y] = (int)q;       // g^q = y
        const long double ang = -2.0L * 3.14159265358979323846264338327950288L * (long double)y / (long double)M;
        b[2 * q] = (double)cosl(ang);
        b[2 * q + 1] = (double)sinl(ang);
        x = x * gi % M;
        y = y * g % M;
    }
    int *din = (int *)c.alloc(L * sizeof(int)), *dout = (int *)c.alloc(M * sizeof(int));
    ck(cudaMemcpy(din, rin.data(), L * sizeof(int), cudaMemcpyHostToDevice), "rader tables");
    ck(cudaMemcpy(dout, rout.data(), M * sizeof(int), cudaMemcpyHostToDevice), "rader tables");
    DevBuf b64(L * 16);
    ck(cudaMemcpy(b64.p, b.data(), L * 16, cudaMemcpyHostToDevice), "rader tables");
    auto dfcore = get_core(c.a == A_F64 ? A_F64 : A_DF, L, false);
    run_core_on_device(*dfcore, b64.p, b64.p, 1, 1, 1.0 / (double)L, 0);
    void *bf = c.alloc(L * slot_bytes(c.a));
    launch_convert_a(c.a, b64.p, bf, L);
    ck(cudaDeviceSynchronize(), "rader tables");
    c.d.rin = din;
    c.d.rout = dout;
    c.d.chirpf = bf;
}

static std::shared_ptr<Core> make_core(Arith a, long long M, bool real_tw)
{
    auto c = std::make_shared<Core>();
    c->a = a;
    c->M = M;
    c->real_tw = real_tw;
    c->d.M = (int)std::min<long long>(M, 1 << 30);
    const TuneCfg cfg = tune_lookup(a, M);
    std::vector<int> rad;
    bool smooth = gpu_factor(M, rad, cfg.E, cfg.order, cfg.no9);
    if (real_tw) {
        void *rtw = c->alloc((M + 1) * slot_bytes(a));
        launch_roots_a(a, rtw, M + 1, 1, 2 * (unsigned long long)M);
        c->rtw = rtw;
        c->d.rtw = rtw;
    }
    // a tuned four-step split may replace a single-CTA core
    bool force4 = false;
    if (smooth && cfg.N1 > 1 && M % cfg.N1 == 0 && fits_smem(a, cfg.N1, cfg.N1) && fits_smem(a, M / cfg.N1, M / cfg.N1)) {
        std::vector<int> r1, r2;
        force4 = gpu_factor(cfg.N1, r1) && gpu_factor(M / cfg.N1, r2);
    }
    if (smooth && fits_smem(a, M, M) && !force4) {
        c->kind = 0;
        build_stockham(*c, M, rad);
        c->d.blue = 0;
        finish_layout(*c, M, M, cfg);
    } else if (!smooth && M > 2 && is_prime(M) && rader_single(a, M, cfg)) {
        // prime length: Rader over the Stockham length M - 1 in one CTA
        c->kind = 0;
        c->d.blue = 2;
        gpu_factor(M - 1, rad, cfg.E, cfg.order, cfg.no9);
        build_stockham(*c, M - 1, rad);
        finish_layout(*c, M - 1, M, cfg);
        build_rader(*c, M);
        c->n2 = M - 1;
    } else if (!smooth && M > 2 && is_prime(M) && rader_multi(a, M)) {
        // prime length: Rader over a multi-pass core of length M - 1
        c->kind = 3;
        c->n2 = M - 1;
        c->sub = get_core(a, M - 1, false);
        build_rader(*c, M);
    } else if (!smooth) {
        long long L = good_size_gpu(2 * M - 1);
        std::vector<int> radL;
        gpu_factor(L, radL, cfg.E, cfg.order, cfg.no9);
        if (fits_smem(a, L, M)) {
            c->kind = 0;
            c->d.blue = 1;
            build_stockham(*c, L, radL);
            finish_layout(*c, L, M, cfg);
            void *ch, *chf;
            build_chirp(*c, M, L, ch, chf);
            c->d.chirp = ch;
            c->d.chirpf = chf;
            c->n2 = L;
        } else {
            // Bluestein over a length-L core that itself runs as a four-step
            c->kind = 2;
            c->n2 = L;
            c->sub = get_core(a, L, false);
            void *ch, *chf;
            build_chirp(*c, M, L, ch, chf);
            c->chirp = ch;
            c->chirpf = chf;
        }
    } else {
        // four-step: M = N1 * N2, both run as shared-memory cores
        long long best = 0;
        for (long long d = 2; d * d <= M; ++d) {
            if (M % d) continue;
            std::vector<int> r1, r2;
            if (gpu_factor(d, r1) && gpu_factor(M / d, r2) && fits_smem(a, d, d) && fits_smem(a, M / d, M / d))
                best = d;
        }
        if (!best) raise(IG_ETOOLARGE, "no four-step split of this length fits the GPU kernels");
        if (cfg.N1 > 1 && M % cfg.N1 == 0 && fits_smem(a, cfg.N1, cfg.N1) && fits_smem(a, M / cfg.N1, M / cfg.N1)) {
            std::vector<int> r1, r2;
            if (gpu_factor(cfg.N1, r1) && gpu_factor(M / cfg.N1, r2)) best = cfg.N1;
        }
        c->kind = 1;
        c->N1 = best;
        c->N2 = M / best;
        c->c1 = get_core(a, c->N1, false);
        c->c2 = get_core(a, c->N2, false);
        void *whi = c->alloc(c->N1 * slot_bytes(a));
        void *wlo = c->alloc(c->N2 * slot_bytes(a));
        launch_roots_a(a, whi, c->N1, 1, (unsigned long long)c->N1);
        launch_roots_a(a, wlo, c->N2, 1, (unsigned long long)M);
        c->whi = whi;
        c->wlo = wlo;
        // the full twiddle table when it stays modest (one table read per element)
        if (M <= (1LL << 22)) {
            const size_t twb = slot_bytes(a);
            void *tab = c->alloc((size_t)M * twb);
            cudaError_t e = a == A_F32 ? Launch<TagF32>::tw4_table(tab, c->N1, c->N2)
                          : a == A_DF  ? Launch<TagDF>::tw4_table(tab, c->N1, c->N2)
                                       : Launch<TagF64>::tw4_table(tab, c->N1, c->N2);
            ck(e, "four-step twiddles");
            count_launch();
            c->tw4tab = tab;
        }
    }
    ck(cudaDeviceSynchronize(), "plan tables");
    return c;
}

static std::shared_ptr<Core> get_core(Arith a, long long M, bool real_tw)
{
    auto key = std::make_tuple(device_id(), (int)a, M, real_tw);
    {
        std::lock_guard<std::mutex> lk(g_mu);
        auto it = g_cores.find(key);
        if (it != g_cores.end()) return it->second;
    }
    auto c = make_core(a, M, real_tw);
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_cores.find(key);
    if (it != g_cores.end()) return it->second;
    g_cores[key] = c;
    return c;
}

// --------------------------------------------------------------------------
// launching the shared-memory kernel
// --------------------------------------------------------------------------
// k_fft_line serves Stockham cores of two or more stages on lines addressed
// by the batch dimensions (rows: consecutive threads walk a line's units)
// with the plain complex layout or the even real -> halfcomplex one
static const bool g_line_kernel = getenv("IG_NO_LINE_KERNEL") == nullptr;
static int line_pf_env()
{
    const char *v = getenv("IG_LINE_PF");
    return v ? std::max(0, std::min(8, atoi(v))) : 1;
}
static const int g_line_pf = line_pf_env();
static const bool g_df_line_hc = getenv("IG_NO_DF_LINE_HC") == nullptr;
static bool line_kernel_ok(Arith a, const CoreDesc &d, const IODesc &io)
{
    if (!g_line_kernel || (a != A_F32 && a != A_DF) || d.blue != 0 || d.nst < 2 || d.L != d.M) return false;
    if (d.rs == RS_FULL || !line_edge_ok(d.st[0].R) || !line_edge_ok(d.st[d.nst - 1].R)) return false;
    if (io.cols_in || io.cols_out || io.loff_in || io.loff_out || io.pair || io.split_N1) return false;
    // the double-float line variants other than the 8-element halfcomplex one
    // run at 128 registers: 512 threads a CTA at most
    if (a == A_DF && !(io.lay == LAY_R2HC && d.E == 8) && (d.L + d.E - 1) / d.E > 512) return false;
    if (io.lay == LAY_C2C) return io.post == POST_NONE && io.in_kind == IN_C && io.out_kind == OUT_C;
    // r2c half spectra (FP32): the halfcomplex butterflies storing complex units
    if (io.lay == LAY_R2C)
        return a == A_F32 && io.nreal == 2LL * d.M && line_r2hc_last_ok(d.st[d.nst - 1].R);
    // c2r half spectra (FP32): the pre-step from HBM, every stage from shared memory
    if (io.lay == LAY_C2R) return a == A_F32 && d.rtw && io.cnt_in == d.M + 1 && io.cnt_out == d.M;
    // halfcomplex lines: FP32 with the split fused into the last stage's
    // mirror butterflies (last radix with line_r2hc_last_ok), double-float
    // with a split pass after the last stage (IG_NO_DF_LINE_HC=1: k_fft_smem)
    if (io.lay == LAY_R2HC) {
        if (io.post != POST_SPLIT || io.in_kind != IN_C || io.out_kind != OUT_HC || io.nreal != 2LL * d.M) return false;
        // (double-float: double-buffered cores only; the single-buffered
        // 16-element line variants spill kilobytes a thread)
        return a == A_F32 ? line_r2hc_last_ok(d.st[d.nst - 1].R) : g_df_line_hc && d.db;
    }
    return false;
}

// k_fft_line_pipe: FP32 lines whose input units are contiguous and whose
// starts and sizes allow 16-byte bulk copies.  Off by default (IG_PIPE=1
// turns it on, IG_PIPE_SLOTS=1|2 fixes the staging depth): its staging slots
// cost CTAs per SM, and k_fft_line measured faster on every length tried
// (rfft 4096: 2601 vs 1850 GB/s, c2c 4096: 3217 vs 2603, rfft 256: 3162 vs
// 1960).
static bool pipe_env()
{
    const char *v = getenv("IG_PIPE");
    return v && atoi(v) != 0;
}
static const bool g_pipe_kernel = pipe_env();
static int pipe_slots_env()
{
    const char *v = getenv("IG_PIPE_SLOTS");
    return v ? std::max(1, std::min(2, atoi(v))) : 0;
}
static const int g_pipe_slots = pipe_slots_env();
static bool pipe_ok(Arith a, const CoreDesc &d, const IODesc &io)
{
    if (!g_pipe_kernel || a != A_F32 || io.is != 8 || (io.lay != LAY_C2C && io.lay != LAY_R2HC)) return false;
    const long long line_bytes = (long long)d.L * 8;
    if (line_bytes % 16 || ((uintptr_t)io.in & 15)) return false;
    for (int k = 0; k < 3; ++k)
        if (io.bn[k] > 1 && (io.bsi[k] & 15)) return false;
    return true;
}
static int sm_count()
{
    static int n = 0;
    if (!n) ck(cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, device_id()), "SM count");
    return n;
}

// k_fft_pair: FP32 complex lines and even real lines to halfcomplex whose
// core has an even first radix, radices up to 8 or odd (the 7/11 class at
// most), L / R even in every later stage, contiguous units in and out and
// output line starts aligned for the 16-byte (complex) or 8-byte
// (halfcomplex) stores (IG_NO_PAIR=1 turns it off)
static const bool g_pair_kernel = getenv("IG_NO_PAIR") == nullptr;
static bool pair_ok(Arith a, const CoreDesc &d, const IODesc &io)
{
    if (io.lay != LAY_C2C && io.lay != LAY_R2HC && io.lay != LAY_R2C) return false;
    // below 512 points k_fft_line measured faster (a line's 16-element
    // threads are too few: N = 96 real 1966 vs 1679 GB/s, 256 3070 vs 2675);
    // from 512 on the pairs win (1200 real 1927 -> 2178, 1280 2145 -> 2421,
    // 1680 1867 -> 2070, complex 4096 3263 -> 3529) or tie (4096 real)
    if (!g_pair_kernel || a != A_F32 || !d.twp || d.L < 512 || d.rs > RS_ALL || io.is != 8) return false;
    const int R0 = d.st[0].R;
    if (R0 != 2 && R0 != 4 && R0 != 8) return false;
    for (int s = 1; s < d.nst; ++s) {
        const int R = d.st[s].R;
        if (R == 16 || R == 13 || (d.L / R) % 2) return false;
    }
    // (r2c: half-spectrum units, 8-byte stores)
    const long long oal = io.lay == LAY_C2C ? 16 : 8;
    if (io.lay == LAY_R2HC && (io.os != 4 || !d.rtw)) return false;
    if (io.lay == LAY_R2C && (io.os != 8 || !d.rtw || io.cnt_out != d.M + 1)) return false;
    if (io.lay == LAY_C2C && io.os != 8) return false;
    if ((uintptr_t)io.out % oal) return false;
    for (int k = 0; k < 3; ++k)
        if (io.bn[k] > 1 && io.bso[k] % oal) return false;
    return true;
}

// lines per CTA of a shared-memory launch of core d
static long long smem_lpc(Arith a, const CoreDesc &d, const IODesc &io, long long &line_bytes)
{
    const long long tpl = (d.L + d.E - 1) / d.E;
    // double-buffered stages: two line buffers
    // (k_fft_smem's per-line stride is odd in slots: 2 LS + 1, or LS rounded up to odd)
    line_bytes = (long long)(d.db ? 2LL * d.LS + 1 : (long long)(d.LS | 1)) * (long long)slot_bytes(a);
    const int smax = max_smem();
    long long lpc = std::max<long long>(1, 256 / tpl);
    if (d.lpc_pref > 0) lpc = d.lpc_pref;
    // column-mapped launches need several lines per CTA for coalescing, whatever
    // the tuner chose for the core's contiguous lines
    if (io.cols_in || io.cols_out) lpc = std::max<long long>(lpc, 8);
    lpc = std::min<long long>(lpc, kMaxLinesPerCta);
    lpc = std::min<long long>(lpc, std::max<long long>(1, kMaxThreads / tpl));
    // keep three (or two) CTAs per SM when a line is small enough: a third
    // (half) of the SM's shared memory less what each CTA holds besides its
    // line buffers (the reserved 1 KB and the kernels' static arrays, at most
    // 4 KB); a third of the per-block limit let only two CTAs in
    const long long per_cta = 1024 + 4096, sm_total = smem_per_sm();
    const long long b3 = sm_total / 3 - per_cta, b2 = sm_total / 2 - per_cta;
    long long budget = line_bytes <= b3 ? b3 : line_bytes <= b2 ? b2 : smax;
    lpc = std::min<long long>(lpc, std::max<long long>(1, budget / line_bytes));
    return std::min<long long>(lpc, std::max<long long>(1, io.nlines));
}

// Prefetch distance of the paired-lane kernel, in lines: SMs x resident CTAs
// (shared memory, threads and registers at `regs` a thread) x lines a CTA,
// times the IG_LINE_PF waves to prefetch ahead (default 1; 0 turns it off)
static int line_pf_lines(size_t smem, long long threads, int regs, long long lpc)
{
    if (g_line_pf <= 0) return 0;
    const long long by_smem = (smem_per_sm() - 1024) / (long long)(smem + 1024);
    const long long by_thr = 2048 / std::max<long long>(1, threads);
    const long long by_reg = 65536 / std::max<long long>(1, (long long)regs * threads);
    const long long res = std::max<long long>(1, std::min(by_smem, std::min(by_thr, by_reg)));
    return (int)std::min<long long>(0x3fffffff, g_line_pf * sm_count() * res * lpc);
}

static void launch_smem(Arith a, const CoreDesc &d_in, IODesc io, cudaStream_t st)
{
    if (io.nlines <= 0) return;
    CoreDesc dv = d_in;
    long long line_bytes = 0;
    long long lpc = smem_lpc(a, dv, io, line_bytes);
    // lines walked across (strided axes): each row of a CTA's lines should fill
    // a 32-byte sector; when double buffering or 8 elements per thread leave
    // room for fewer lines, single-buffered 16-element stages take more
    if ((io.cols_in || io.cols_out) && d_in.lpc_pref <= 0 && (dv.E == 8 || dv.db)) {
        const long long ue = io.in_kind == IN_C || io.in_kind == IN_P ? 2 * (long long)store_real_bytes(a)
                                                                      : (long long)store_real_bytes(a);
        const long long want = std::max<long long>(1, 32 / ue);
        if (lpc < want && lpc < io.nlines) {
            CoreDesc d2 = dv;
            d2.E = 16;
            d2.db = 0;
            long long lb2 = 0;
            const long long lpc2 = smem_lpc(a, d2, io, lb2);
            if (lpc2 > lpc) {
                dv = d2;
                lpc = lpc2;
                line_bytes = lb2;
            }
        }
    }
    const CoreDesc &d = dv;
    const long long tpl = (d.L + d.E - 1) / d.E;
    const int smax = max_smem();
    if (io.post == POST_SPLIT4) lpc = std::max<long long>(2, lpc & ~1LL);  // whole row pairs per CTA
    io.lpc = (int)lpc;
    io.tpl = (int)tpl;
    set_line_divs(io);
    io.lay = choose_layout(a, io);
    if (io.rowconv && io.lay != LAY_RC) raise(IG_EINVAL, "internal: row convolution outside its layout class");
    size_t smem = (size_t)(lpc * line_bytes);
    static std::once_flag once[3];
    std::call_once(once[a], [&] {
        int optin = smax + 1024;
        cudaError_t e = a == A_F32 ? Launch<TagF32>::set_max_smem(optin)
                      : a == A_DF  ? Launch<TagDF>::set_max_smem(optin)
                                   : Launch<TagF64>::set_max_smem(optin);
        ck(e, "cudaFuncSetAttribute");
    });
    long long grid = (io.nlines + lpc - 1) / lpc;
    if (grid > 0x7fffffffLL) raise(IG_ETOOLARGE, "too many lines for one launch");
    cudaError_t e;
    // staging slots of the pipelined line kernel: two while the CTAs per SM
    // that the line buffers allow stay the same with them (at most three are
    // counted), else one; none when even one slot does not fit
    int nslot = 0;
    if (line_kernel_ok(a, d, io) && pipe_ok(a, d, io) && grid < (1LL << 30)) {
        const size_t stage = (size_t)lpc * d.L * 8;
        const size_t w = (smem + 127) / 128 * 128;
        const size_t cap = (size_t)smax, per_sm = cap + 1024;
        if (w + stage <= cap) {
            nslot = g_pipe_slots ? g_pipe_slots : 1;
            if (!g_pipe_slots && w + 2 * stage <= cap &&
                per_sm / (w + 2 * stage + 1024) >= std::min<size_t>(3, per_sm / (w + stage + 1024)))
                nslot = 2;
            if (w + nslot * stage > cap) nslot = 1;
        }
    }
    if (nslot) {
        e = Launch<TagF32>::fft_line_pipe(d, io, smem, nslot, sm_count(), st);
    } else if (line_kernel_ok(a, d, io) && pair_ok(a, d, io)) {
        // 16 elements a thread; line buffers of GS padded 16-byte groups, two a line
        const int GS = (d.L / 2 - 1) + ((d.L / 2 - 1) >> 3) + 1;
        const long long tplp = (d.L + 15) / 16, lb = 2LL * GS * 16;
        const long long per_cta = 1024 + 1024, b3 = smem_per_sm() / 3 - per_cta;
        long long lp = d.lpc_pref > 0 ? d.lpc_pref : std::max<long long>(1, 256 / tplp);
        lp = std::min<long long>(lp, std::max<long long>(1, kMaxThreads / tplp));
        lp = std::min<long long>(lp, std::max<long long>(1, (lb <= b3 ? b3 : (long long)smax) / lb));
        lp = std::min<long long>(std::min<long long>(lp, kMaxLinesPerCta), std::max<long long>(1, io.nlines));
        IODesc iop = io;
        iop.lpc = (int)lp;
        iop.tpl = (int)tplp;
        iop.pf_lines = line_pf_lines((size_t)(lp * lb), lp * tplp, 64, lp);
        static std::once_flag once_pair;
        std::call_once(once_pair, [&] { ck(set_smem_pair(smax + 1024), "cudaFuncSetAttribute"); });
        e = launch_pair(d, iop, GS, (size_t)(lp * lb), st);
    } else if (line_kernel_ok(a, d, io)) {
        e = a == A_F32 ? Launch<TagF32>::fft_line(d, io, smem, st) : Launch<TagDF>::fft_line(d, io, smem, st);
    }
    else
        e = a == A_F32 ? Launch<TagF32>::fft_smem(d, io, smem, st)
          : a == A_DF  ? Launch<TagDF>::fft_smem(d, io, smem, st)
                       : Launch<TagF64>::fft_smem(d, io, smem, st);
    ck(e, "fft kernel launch");
    count_launch();
}

static IODesc blank_io()
{
    IODesc io;
    memset(&io, 0, sizeof io);
    io.bn[0] = io.bn[1] = io.bn[2] = 1;
    io.fct = 1.0;
    return io;
}

// --------------------------------------------------------------------------
// scratch for the multi-pass paths: per (device, stream), grow-only
// --------------------------------------------------------------------------
struct Scratch {
    std::unique_ptr<DevBuf> buf[8];
    void *get(int i, size_t bytes)
    {
        if (!buf[i] || buf[i]->bytes < bytes) {
            buf[i].reset();
            buf[i].reset(new DevBuf(bytes));
        }
        return buf[i]->p;
    }
};
static std::mutex g_scr_mu;
static std::map<std::pair<int, cudaStream_t>, std::unique_ptr<Scratch>> g_scratch;
static Scratch &scratch_for(cudaStream_t st)
{
    std::lock_guard<std::mutex> lk(g_scr_mu);
    auto &p = g_scratch[std::make_pair(device_id(), st)];
    if (!p) p.reset(new Scratch);
    return *p;
}

static void launch_map(Arith a, bool gather, const IODesc &io_in, const MapDesc &mp_in, cudaStream_t st)
{
    IODesc io = io_in;
    set_line_divs(io);
    MapDesc mp = mp_in;
    mp.fsl = make_fdiv((unsigned)std::max<long long>(1, std::min<long long>(mp.scr_len, 0x7fffffffLL)));
    mp.fcnt = make_fdiv((unsigned)std::max<long long>(1, std::min<long long>(io.cnt_out, 0x7fffffffLL)));
    cudaError_t e;
    if (gather)
        e = a == A_F32 ? Launch<TagF32>::gather(io, mp, st)
          : a == A_DF  ? Launch<TagDF>::gather(io, mp, st)
                       : Launch<TagF64>::gather(io, mp, st);
    else
        e = a == A_F32 ? Launch<TagF32>::scatter(io, mp, st)
          : a == A_DF  ? Launch<TagDF>::scatter(io, mp, st)
                       : Launch<TagF64>::scatter(io, mp, st);
    ck(e, gather ? "gather launch" : "scatter launch");
    count_launch();
}

static void run_complex(const Core &c, const IODesc &io, cudaStream_t st);

static void launch_pair_map(Arith a, int which, const IODesc &io_in, const MapDesc &mp_in, int *esc, cudaStream_t st)
{
    IODesc io = io_in;
    set_line_divs(io);
    MapDesc mp = mp_in;
    mp.fsl = make_fdiv((unsigned)std::max<long long>(1, std::min<long long>(mp.scr_len, 0x7fffffffLL)));
    mp.fcnt = make_fdiv((unsigned)std::max<long long>(1, std::min<long long>(io.cnt_out, 0x7fffffffLL)));
    cudaError_t e;
    if (which == 0)
        e = a == A_F32 ? Launch<TagF32>::line_exp(io, esc, st)
          : a == A_DF  ? Launch<TagDF>::line_exp(io, esc, st)
                       : Launch<TagF64>::line_exp(io, esc, st);
    else if (which == 1)
        e = a == A_F32 ? Launch<TagF32>::gather_pair(io, mp, esc, st)
          : a == A_DF  ? Launch<TagDF>::gather_pair(io, mp, esc, st)
                       : Launch<TagF64>::gather_pair(io, mp, esc, st);
    else
        e = a == A_F32 ? Launch<TagF32>::scatter_pair(io, mp, esc, st)
          : a == A_DF  ? Launch<TagDF>::scatter_pair(io, mp, esc, st)
                       : Launch<TagF64>::scatter_pair(io, mp, esc, st);
    ck(e, "paired line map");
    count_launch();
}

// contiguous scratch lines as an IODesc side
static void contig_side(IODesc &io, bool out, char *base, long long es, long long len, long long nl)
{
    if (out) {
        io.out = base;
        io.os = es;
        io.bso[0] = len * es;
    } else {
        io.in = (const char *)base;
        io.is = es;
        io.bsi[0] = len * es;
    }
    io.bn[0] = nl;
    io.bn[1] = io.bn[2] = 1;
    if (out) io.bso[1] = io.bso[2] = 0; else io.bsi[1] = io.bsi[2] = 0;
}

// Four-step over M = N1 * N2 (column FFTs of length N1 with the inter-pass
// twiddle, then row FFTs of length N2 written transposed).  io describes
// the user-facing sides with kinds IN_C/IN_R/IN_P and OUT_C/OUT_R/OUT_P and
// at most two batch dims; `B` is a scratch of nlines * M complex elements.
static void fourstep_passes(const Core &c, const IODesc &io, char *B, IODesc &p1, IODesc &p2);

static void run_fourstep(const Core &c, const IODesc &io, char *B, cudaStream_t st)
{
    IODesc p1, p2;
    fourstep_passes(c, io, B, p1, p2);
    launch_smem(c.a, c.c1->d, p1, st);
    launch_smem(c.a, c.c2->d, p2, st);
}

static void fourstep_passes(const Core &c, const IODesc &io, char *B, IODesc &p1, IODesc &p2)
{
    const long long N1 = c.N1, N2 = c.N2, M = c.M;
    const long long ES = 2 * (long long)store_real_bytes(c.a);
    const long long nl = io.nlines;
    // pass 1: columns
    p1 = io;
    const long long ub_in = io.is;  // bytes between units
    p1.nlines = nl * N2;
    p1.bn[0] = N2;
    p1.bsi[0] = ub_in;
    p1.bn[1] = io.bn[0];
    p1.bsi[1] = io.bsi[0];
    p1.bn[2] = io.bn[1];
    p1.bsi[2] = io.bsi[1];
    p1.is = N2 * io.is;
    p1.cnt_in = p1.cnt_out = (int)N1;
    p1.out = B;
    p1.out_kind = OUT_C;
    p1.os = N2 * ES;
    p1.bso[0] = ES;
    p1.bso[1] = M * ES;
    p1.bso[2] = M * ES * io.bn[0];
    p1.pre = PRE_NONE;
    p1.post = POST_NONE;
    p1.conj_out = 0;
    p1.real_out = 0;
    p1.mul = nullptr;
    p1.keep0 = nullptr;
    p1.fct = 1.0;
    p1.tw4 = 1;
    p1.tw4N = M;
    p1.tw4S = N2;
    p1.fdS = make_fdiv((unsigned)N2);
    p1.tw4hi = c.whi;
    p1.tw4lo = c.wlo;
    p1.tw4tab = c.tw4tab;
    p1.cols_in = 1;
    p1.cols_out = 1;
    // pass 2: rows, transposed write
    p2 = io;
    const long long ub_out = io.os;
    p2.in = B;
    p2.in_kind = IN_C;
    p2.conj_in = 0;
    p2.is = ES;
    p2.nlines = nl * N1;
    p2.bn[0] = N1;
    p2.bsi[0] = N2 * ES;
    p2.bn[1] = io.bn[0];
    p2.bsi[1] = M * ES;
    p2.bn[2] = io.bn[1];
    p2.bsi[2] = M * ES * io.bn[0];
    p2.bso[0] = ub_out;
    p2.bso[1] = io.bso[0];
    p2.bso[2] = io.bso[1];
    p2.os = N1 * io.os;
    p2.cnt_in = p2.cnt_out = (int)N2;
    p2.pre = PRE_NONE;
    p2.post = POST_NONE;
    p2.tw4 = 0;
    p2.cols_in = 0;
    p2.cols_out = 1;
    if (io.mul) {
        p2.mul_a = 1;
        p2.mul_b = N1;
    }
    p2.keep0_rows = (int)N1;
}

// Strided-axis FP32 transforms (lines = adjacent columns, elements a row
// apart) of 2048 points and more as a four-step split M = N1 N2 with the
// columns as the fastest line index of both passes.  A single-CTA launch of
// such columns holds only a few whole columns per CTA (four 4096-point FP32
// columns fill 128 KB: one CTA per SM) and is latency-bound; here each CTA
// transforms 32 adjacent columns of N1 (then N2) elements, every row segment
// read or written is a run of adjacent columns, and the scratch B holds
// element e of column c at e C + c (C = columns of a batch row).  Pass 1:
// columns of length N1 with the inter-pass twiddle (row index n2 = batch dim
// 1), into B; pass 2: length N2, written transposed to the output.
static const bool g_col4 = getenv("IG_NO_COL_FOURSTEP") == nullptr;
static std::mutex g_colcore_mu;
static std::map<std::tuple<int, int, long long>, std::shared_ptr<Core>> g_colcores;

static bool col_fourstep_ok(Arith a, const Core &c, const IODesc &io)
{
    return g_col4 && a == A_F32 && c.kind == 0 && c.d.blue == 0 && c.M >= 2048 && io.cols_in && io.cols_out &&
           io.in_kind == IN_C && io.out_kind == OUT_C && io.pre == PRE_NONE && io.post == POST_NONE && !io.pair &&
           !io.loff_in && !io.loff_out && !io.tw4 && !io.mul && !io.keep0 && !io.split_N1 && !io.real_out &&
           io.bn[0] >= 32;
}

// the four-step core of a column transform: N1 the divisor of M nearest its
// square root with both factors on single-CTA cores (nullptr if none)
static std::shared_ptr<Core> col_core(Arith a, long long M)
{
    const auto key = std::make_tuple(device_id(), (int)a, M);
    {
        std::lock_guard<std::mutex> lk(g_colcore_mu);
        auto it = g_colcores.find(key);
        if (it != g_colcores.end()) return it->second;
    }
    long long best = 0;
    for (long long d = 2; d * d <= M; ++d) {
        if (M % d) continue;
        std::vector<int> r1, r2;
        if (gpu_factor(d, r1) && gpu_factor(M / d, r2) && fits_smem(a, d, d) && fits_smem(a, M / d, M / d)) best = d;
    }
    std::shared_ptr<Core> c;
    if (best) {
        TuneCfg cfg;
        cfg.N1 = best;
        g_cfg_override = &cfg;
        g_cfg_override_len = M;
        g_cfg_override_arith = a;
        try {
            c = make_core(a, M, false);
        } catch (...) {
            g_cfg_override = nullptr;
            throw;
        }
        g_cfg_override = nullptr;
        if (c->kind != 1) c.reset();
    }
    std::lock_guard<std::mutex> lk(g_colcore_mu);
    auto it = g_colcores.find(key);
    if (it != g_colcores.end()) return it->second;
    g_colcores[key] = c;
    return c;
}

static void run_fourstep_cols(const Core &c, const IODesc &io, char *B, cudaStream_t st)
{
    const long long N1 = c.N1, N2 = c.N2, M = c.M;
    const long long ES = 2 * (long long)store_real_bytes(c.a);
    const long long C = io.bn[0], NB1 = io.bn[1];
    IODesc p1 = io;
    p1.nlines = C * N2 * NB1;
    p1.bn[0] = C;
    p1.bsi[0] = io.bsi[0];
    p1.bn[1] = N2;
    p1.bsi[1] = io.is;
    p1.bn[2] = NB1;
    p1.bsi[2] = io.bsi[1];
    p1.is = N2 * io.is;
    p1.cnt_in = p1.cnt_out = (int)N1;
    p1.out = B;
    p1.out_kind = OUT_C;
    p1.os = N2 * C * ES;
    p1.bso[0] = ES;
    p1.bso[1] = C * ES;
    p1.bso[2] = M * C * ES;
    p1.pre = PRE_NONE;
    p1.post = POST_NONE;
    p1.conj_out = 0;
    p1.real_out = 0;
    p1.mul = nullptr;
    p1.keep0 = nullptr;
    p1.fct = 1.0;
    p1.tw4 = 1;
    p1.tw4_dim1 = 1;
    p1.tw4N = M;
    p1.tw4S = N2;
    p1.fdS = make_fdiv((unsigned)N2);
    p1.tw4hi = c.whi;
    p1.tw4lo = c.wlo;
    p1.tw4tab = c.tw4tab;
    p1.cols_in = p1.cols_out = 1;
    IODesc p2 = io;
    p2.in = B;
    p2.in_kind = IN_C;
    p2.conj_in = 0;
    p2.pre = PRE_NONE;
    p2.is = C * ES;
    p2.nlines = C * N1 * NB1;
    p2.bn[0] = C;
    p2.bsi[0] = ES;
    p2.bn[1] = N1;
    p2.bsi[1] = N2 * C * ES;
    p2.bn[2] = NB1;
    p2.bsi[2] = M * C * ES;
    p2.os = N1 * io.os;
    p2.bso[0] = io.bso[0];
    p2.bso[1] = io.os;
    p2.bso[2] = io.bso[1];
    p2.cnt_in = p2.cnt_out = (int)N2;
    p2.tw4 = 0;
    p2.tw4_dim1 = 0;
    p2.cols_in = p2.cols_out = 1;
    launch_smem(c.a, c.c1->d, p1, st);
    launch_smem(c.a, c.c2->d, p2, st);
}

// Forward real halfcomplex transform over a four-step core of length M = N1 N2
// (N = 2M reals): column pass into scratch B, then a row pass whose CTAs hold
// each row r next to its mirror N1 - r and write X[k], X[M - k] directly.
static bool g_fused_split = getenv("IG_NO_FUSED_SPLIT") == nullptr;
static void run_fourstep_split(const Core &c, const IODesc &io, char *B, cudaStream_t st)
{
    IODesc p1, p2;
    fourstep_passes(c, io, B, p1, p2);
    launch_smem(c.a, c.c1->d, p1, st);
    const long long N1 = c.N1, N2 = c.N2, M = c.M, nl = io.nlines;
    const long long ES = 2 * (long long)store_real_bytes(c.a);
    // row slots of one transform: pairs (r, N1 - r) for 0 < r < N1 / 2, (0, 0), and (N1 / 2, N1 / 2)
    const long long LT = 2 * ((N1 - 1) / 2) + 2 + (N1 % 2 == 0 ? 2 : 0);
    IODesc q = p2;
    q.nlines = nl * LT;
    q.bn[0] = LT;
    q.bn[1] = io.bn[0];
    q.bn[2] = io.bn[1];
    q.bsi[0] = N2 * ES;
    q.bsi[1] = M * ES;
    q.bsi[2] = io.bn[0] * M * ES;
    q.bso[0] = 0;
    q.bso[1] = io.bso[0];
    q.bso[2] = io.bso[1];
    q.loff_in = q.loff_out = nullptr;
    q.in = B;
    q.out = io.out;
    q.in_kind = IN_C;
    q.is = ES;
    q.out_kind = OUT_HC;
    q.os = io.os;
    q.nreal = io.nreal;
    q.cnt_in = q.cnt_out = (int)N2;
    q.post = POST_SPLIT4;
    q.split_tw = c.rtw;
    q.split_N1 = (int)N1;
    q.fct = io.fct;
    q.cols_in = q.cols_out = 0;
    q.mul = nullptr;
    q.keep0 = nullptr;
    q.tw4 = 0;
    launch_smem(c.a, c.c2->d, q, st);
}

// The convolution of Bluestein (kind 2) and Rader (kind 3) on nl contiguous
// scratch lines of length L, in place: forward FFT_L with the product by the
// transformed kernel (chirpf / B) fused into its last pass, then the
// backward FFT_L.  Bluestein conjugates the kernel for the backward
// direction; Rader always runs forward (its maps conjugate) and keeps each
// line's A[0] from before the product in a0buf.
// The convolution of Rader / Bluestein over a multi-pass core of length L:
// forward FFT_L, product with the table (A[0] kept first for Rader), inverse
// FFT_L, in place on the contiguous scratch lines A.  With the row-convolution
// mode of the shared-memory kernel (IG_NO_ROWCONV=1 turns it off) a four-step
// core L = N1 N2 takes three passes instead of four: columns forward with the
// twiddle (A -> B), then per row k1 of B the forward FFT_N2, the product in
// the natural spectrum order k1 + N1 k2, the inverse FFT_N2 and the inverse
// twiddle w^-(k1 n2) (B in place), then columns inverse (B -> A), which leaves
// x[n2 + N2 n1] in natural order; a one-CTA core takes one launch instead of two.
static const bool g_rowconv = getenv("IG_NO_ROWCONV") == nullptr;

static void convolve_passes(const Core &c, char *A, long long L, long long nl, int fwd, void *a0buf,
                            cudaStream_t st)
{
    const long long ES = 2 * (long long)store_real_bytes(c.a);
    const bool rader = c.kind == 3;
    const Core &s = *c.sub;
    if (g_rowconv && c.a != A_F64 && (s.kind == 0 || s.kind == 1) && (s.kind == 1 || s.d.blue == 0)) {
        IODesc q = blank_io();
        contig_side(q, false, A, ES, L, nl);
        contig_side(q, true, A, ES, L, nl);
        q.nlines = nl;
        q.in_kind = IN_C;
        q.out_kind = OUT_C;
        q.cnt_in = q.cnt_out = (int)L;
        q.nreal = L;
        q.fwd = 1;
        const void *tab = rader ? c.d.chirpf : c.chirpf;
        const int tconj = (!rader && !fwd) ? 1 : 0;
        if (s.kind == 0) {
            q.mul = tab;
            q.mul_a = 0;
            q.mul_b = 1;
            q.mul_conj = tconj;
            q.keep0 = a0buf;
            q.keep0_rows = 1;
            q.rowconv = 1;
            launch_smem(c.a, s.d, q, st);
            return;
        }
        const long long N1 = s.N1, N2 = s.N2;
        char *B = (char *)scratch_for(st).get(1, (size_t)(nl * L * ES));
        IODesc p1, p2;
        fourstep_passes(s, q, B, p1, p2);
        launch_smem(c.a, s.c1->d, p1, st);
        // rows of B in place
        IODesc r = p2;
        r.out = B;
        r.out_kind = OUT_C;
        r.os = ES;
        r.bso[0] = N2 * ES;
        r.bso[1] = L * ES;
        r.bso[2] = L * ES * q.bn[0];
        r.cols_out = 0;
        r.mul = tab;
        r.mul_a = 1;
        r.mul_b = N1;
        r.mul_conj = tconj;
        r.keep0 = a0buf;
        r.keep0_rows = (int)N1;
        r.rowconv = 1;
        r.tw4 = 1;
        r.tw4N = L;
        r.tw4S = N2;
        r.fdS = make_fdiv((unsigned)N2);
        r.tw4hi = s.whi;
        r.tw4lo = s.wlo;
        r.tw4tab = nullptr;
        r.tw4_dim1 = 0;
        launch_smem(c.a, s.c2->d, r, st);
        // columns inverse, B -> A, natural order
        IODesc p3 = p1;
        p3.in = B;
        p3.out = A;
        p3.tw4 = 0;
        p3.tw4hi = p3.tw4lo = p3.tw4tab = nullptr;
        p3.fwd = 0;
        launch_smem(c.a, s.c1->d, p3, st);
        return;
    }
    for (int pass = 0; pass < 2; ++pass) {
        IODesc q = blank_io();
        contig_side(q, false, A, ES, L, nl);
        contig_side(q, true, A, ES, L, nl);
        q.nlines = nl;
        q.in_kind = IN_C;
        q.out_kind = OUT_C;
        q.cnt_in = q.cnt_out = (int)L;
        q.nreal = L;
        q.fwd = pass == 0 ? 1 : 0;
        if (pass == 0) {
            q.mul = rader ? c.d.chirpf : c.chirpf;
            q.mul_a = 0;
            q.mul_b = 1;
            q.mul_conj = (!rader && !fwd) ? 1 : 0;
            q.keep0 = a0buf;
            q.keep0_rows = 1;  // four-step cores set N1 for their second pass
        }
        run_complex(*c.sub, q, st);
    }
}

// Run a complex core of any kind.  io: user-facing sides, kinds, pre/post,
// conj flags and fct, as for the shared-memory kernel.
static void run_complex(const Core &c, const IODesc &io_all, cudaStream_t st)
{
    if (io_all.nlines <= 0) return;
    if (c.kind == 0) {
        launch_smem(c.a, c.d, io_all, st);
        return;
    }
    // at most two batch dims on the user side per multi-pass run
    for (long long i2 = 0; i2 < io_all.bn[2]; ++i2) {
        IODesc io = io_all;
        io.in += i2 * io_all.bsi[2];
        io.out += i2 * io_all.bso[2];
        io.bn[2] = 1;
        io.bsi[2] = io.bso[2] = 0;
        io.nlines = io.bn[0] * io.bn[1];
        const long long nl = io.nlines;
        const long long ES = 2 * (long long)store_real_bytes(c.a);
        Scratch &scr = scratch_for(st);
        if (io.pair) {
            // two real lines per complex line: per-line scales, paired gather,
            // complex core on contiguous scratch, paired scatter
            const bool rader = c.kind == 3;
            const long long L = (c.kind == 2 || rader) ? c.n2 : c.M;
            int *esc = (int *)scr.get(3, (size_t)(2 * nl * sizeof(int)));
            char *A = (char *)scr.get(0, (size_t)(nl * L * ES));
            MapDesc mp{};
            mp.kind = c.kind == 2 ? MAP_BLUE : rader ? MAP_RADER : MAP_PLAIN;
            mp.M = c.M;
            mp.scr_len = L;
            mp.scr = A;
            mp.chirp = c.chirp;
            mp.fwd = io.fwd;
            if (rader) {
                mp.ridx = c.d.rin;
                mp.x0buf = scr.get(4, (size_t)(nl * ES));
                mp.a0buf = scr.get(5, (size_t)(nl * ES));
            }
            launch_pair_map(c.a, 0, io, mp, esc, st);
            launch_pair_map(c.a, 1, io, mp, esc, st);
            if (rader) mp.ridx = c.d.rout;
            if (c.kind == 1) {
                char *B = (char *)scr.get(1, (size_t)(nl * L * ES));
                IODesc q = blank_io();
                contig_side(q, false, A, ES, L, nl);
                contig_side(q, true, A, ES, L, nl);
                q.nlines = nl;
                q.in_kind = IN_C;
                q.out_kind = OUT_C;
                q.cnt_in = q.cnt_out = (int)L;
                q.nreal = L;
                q.fwd = io.fwd;
                run_fourstep(c, q, B, st);
            } else {
                convolve_passes(c, A, L, nl, io.fwd, rader ? mp.a0buf : nullptr, st);
            }
            launch_pair_map(c.a, 2, io, mp, esc, st);
            continue;
        }
        if (c.kind == 1) {
            const long long M = c.M;
            bool gath = io.pre != PRE_NONE || io.in_kind == IN_HC;
            bool scat = io.post != POST_NONE || io.out_kind == OUT_HC || io.cnt_out != (int)M || io.real_out;
            char *B = (char *)scr.get(1, (size_t)(nl * M * ES));
            // scratch lines keep the user's (bn0, bn1) line numbering: line l at l * M * ES
            IODesc f = io;
            if (gath) {
                char *A = (char *)scr.get(0, (size_t)(nl * M * ES));
                MapDesc mp{};
                mp.kind = io.pre == PRE_HERM_EVEN ? MAP_HERM_EVEN : MAP_PLAIN;
                mp.M = M;
                mp.scr_len = M;
                mp.scr = A;
                mp.rtw = c.rtw;
                launch_map(c.a, true, io, mp, st);
                f.in = A;
                f.is = ES;
                f.bsi[0] = M * ES;
                f.bsi[1] = M * ES * io.bn[0];
                f.in_kind = IN_C;
                f.conj_in = 0;
                f.pre = PRE_NONE;
                f.cnt_in = (int)M;
            }
            if (scat && io.post == POST_SPLIT && io.out_kind == OUT_HC && !gath && !io.conj_out && !io.real_out &&
                !io.loff_out && io.bn[2] == 1 && c.rtw && g_fused_split) {
                // the real split fused into the row pass: rows paired with their mirrors
                run_fourstep_split(c, io, B, st);
            } else if (scat) {
                char *C = (char *)scr.get(2, (size_t)(nl * M * ES));
                f.out = C;
                f.os = ES;
                f.bso[0] = M * ES;
                f.bso[1] = M * ES * io.bn[0];
                f.out_kind = OUT_C;
                f.conj_out = 0;
                f.real_out = 0;
                f.post = POST_NONE;
                f.fct = 1.0;
                f.cnt_out = (int)M;
                run_fourstep(c, f, B, st);
                MapDesc mp{};
                mp.kind = io.post == POST_SPLIT ? MAP_SPLIT_EVEN : MAP_PLAIN;
                mp.M = M;
                mp.scr_len = M;
                mp.scr = C;
                mp.rtw = c.rtw;
                IODesc h = io;
                h.pre = PRE_NONE;
                launch_map(c.a, false, h, mp, st);
            } else {
                run_fourstep(c, f, B, st);
            }
        } else {
            // Bluestein (kind 2) or Rader (kind 3) over a multi-pass core of length n2
            const bool rader = c.kind == 3;
            const long long M = c.M, L = c.n2;
            char *A = (char *)scr.get(0, (size_t)(nl * L * ES));
            IODesc src = io;
            if (io.pre == PRE_HERM_EVEN) {
                char *C = (char *)scr.get(2, (size_t)(nl * M * ES));
                MapDesc mp{};
                mp.kind = MAP_HERM_EVEN;
                mp.M = M;
                mp.scr_len = M;
                mp.scr = C;
                mp.rtw = c.rtw;
                launch_map(c.a, true, io, mp, st);
                contig_side(src, false, C, ES, M, nl);
                src.in_kind = IN_C;
                src.conj_in = 0;
                src.pre = PRE_NONE;
                src.cnt_in = (int)M;
            }
            MapDesc mp{};
            mp.kind = rader ? MAP_RADER : MAP_BLUE;
            mp.M = M;
            mp.scr_len = L;
            mp.scr = A;
            mp.chirp = c.chirp;
            mp.fwd = io.fwd;
            if (rader) {
                mp.ridx = c.d.rin;
                mp.x0buf = scr.get(4, (size_t)(nl * ES));
                mp.a0buf = scr.get(5, (size_t)(nl * ES));
            }
            launch_map(c.a, true, src, mp, st);
            if (rader) mp.ridx = c.d.rout;
            convolve_passes(c, A, L, nl, io.fwd, rader ? mp.a0buf : nullptr, st);
            IODesc h = io;
            h.pre = PRE_NONE;
            if (io.post == POST_SPLIT) {
                char *C = (char *)scr.get(2, (size_t)(nl * M * ES));
                IODesc g = blank_io();
                contig_side(g, true, C, ES, M, nl);
                g.nlines = nl;
                g.out_kind = OUT_C;
                g.cnt_out = (int)M;
                MapDesc mb = mp;
                launch_map(c.a, false, g, mb, st);
                MapDesc ms{};
                ms.kind = MAP_SPLIT_EVEN;
                ms.M = M;
                ms.scr_len = M;
                ms.scr = C;
                ms.rtw = c.rtw;
                launch_map(c.a, false, h, ms, st);
            } else {
                launch_map(c.a, false, h, mp, st);
            }
        }
    }
}

// contiguous batch of complex lines of length M (used for table building)
static void run_core_on_device(const Core &c, const void *in, void *out, long long batch, int fwd, double fct,
                               cudaStream_t st)
{
    IODesc io = blank_io();
    size_t sb = 2 * store_real_bytes(c.a);
    io.in = (const char *)in;
    io.out = (char *)out;
    io.is = io.os = (long long)sb;
    io.nlines = batch;
    io.bn[0] = batch;
    io.bsi[0] = io.bso[0] = c.M * (long long)sb;
    io.in_kind = IN_C;
    io.out_kind = OUT_C;
    io.cnt_in = io.cnt_out = (int)c.M;
    io.fwd = fwd;
    io.fct = fct;
    run_complex(c, io, st);
}

// --------------------------------------------------------------------------
// transforms over lines
// --------------------------------------------------------------------------
enum Op { OP_C2C = 0, OP_R2HC = 1, OP_HC2R = 2, OP_R2C = 3, OP_C2R = 4 };

struct Lines {
    // a set of lines of logical length N: line l starts at in/out + offset(l),
    // consecutive elements `es_in` / `es_out` bytes apart (storage elements:
    // complex for complex sides, real for real sides)
    const char *in;
    char *out;
    long long es_in, es_out;
    long long nlines;
    long long bn[3], bsi[3], bso[3];
};

static Arith arith_for(int dtype)
{
    if (dtype == IG_F32) return A_F32;
    return g_f64_arith == 1 ? A_F64 : A_DF;
}

// every line start and element of one side at a multiple of `align` bytes
static bool side_aligned(const void *p, long long es, const long long *bn, const long long *bs, long long align)
{
    if ((uintptr_t)p % (uintptr_t)align || std::llabs(es) % align) return false;
    for (int i = 0; i < 3; ++i)
        if (bn[i] > 1 && std::llabs(bs[i]) % align) return false;
    return true;
}

static void require_aligned(const void *p, size_t align, const char *what)
{
    if ((uintptr_t)p % align) raise(IG_EINVAL, std::string(what) + " not aligned to its element size");
}

static void exec_op(Arith a, Op op, long long N, const Lines &ln, int forward, double fct, cudaStream_t st,
                    std::shared_ptr<Core> forced = nullptr)
{
    if (ln.nlines <= 0 || N <= 0) return;
    // scalar accesses need natural alignment; complex (pair) accesses need
    // twice that, else the kernels read and write the two halves separately
    {
        const long long sr0 = (long long)store_real_bytes(a);
        if (!side_aligned(ln.in, ln.es_in, ln.bn, ln.bsi, sr0) || !side_aligned(ln.out, ln.es_out, ln.bn, ln.bso, sr0))
            raise(IG_EINVAL, "data pointer or stride not aligned to the element size");
    }
    const bool pair_in = side_aligned(ln.in, ln.es_in, ln.bn, ln.bsi, 2 * (long long)store_real_bytes(a));
    const bool pair_out = side_aligned(ln.out, ln.es_out, ln.bn, ln.bso, 2 * (long long)store_real_bytes(a));
    IODesc io = blank_io();
    io.in = ln.in;
    io.out = ln.out;
    io.nlines = ln.nlines;
    for (int i = 0; i < 3; ++i) {
        io.bn[i] = ln.bn[i];
        io.bsi[i] = ln.bsi[i];
        io.bso[i] = ln.bso[i];
    }
    io.fct = fct;
    io.nreal = N;
    io.is = ln.es_in;
    io.os = ln.es_out;
    const long long sr = (long long)store_real_bytes(a);
    bool even = (N % 2 == 0) && N > 1;
    long long M = N;
    std::shared_ptr<Core> core;
    switch (op) {
    case OP_C2C:
        core = forced ? forced : get_core(a, N, false);
        io.in_kind = IN_C;
        io.out_kind = OUT_C;
        if (!pair_in) {
            io.in_kind = IN_P;
            io.ps_in = sr;
        }
        if (!pair_out) {
            io.out_kind = OUT_P;
            io.ps_out = sr;
        }
        io.cnt_in = io.cnt_out = (int)N;
        io.fwd = forward;
        break;
    case OP_R2HC:
    case OP_R2C:
        M = even ? N / 2 : N;
        core = forced ? forced : get_core(a, M, even);
        if (even && ln.es_in == sr &&
            side_aligned(ln.in, 2 * sr, ln.bn, ln.bsi, 2 * sr)) {
            io.in_kind = IN_C;  // contiguous reals read as complex pairs
            io.is = 2 * sr;
        } else if (even) {
            io.in_kind = IN_P;
            io.is = 2 * ln.es_in;
            io.ps_in = ln.es_in;
        } else {
            io.in_kind = IN_R;
        }
        io.cnt_in = (int)M;
        io.post = even ? POST_SPLIT : POST_NONE;
        io.fwd = 1;
        if (op == OP_R2HC) {
            io.out_kind = OUT_HC;
            io.cnt_out = (int)(even ? N / 2 + 1 : (N + 1) / 2);
        } else {
            io.out_kind = pair_out ? OUT_C : OUT_P;
            if (!pair_out) io.ps_out = sr;
            io.cnt_out = (int)(N / 2 + 1);
            io.conj_out = forward ? 0 : 1;
            io.real_out = 1;
        }
        break;
    case OP_HC2R:
    case OP_C2R:
        M = even ? N / 2 : N;
        core = forced ? forced : get_core(a, M, even);
        io.in_kind = op == OP_HC2R ? IN_HC : (pair_in ? IN_C : IN_P);
        if (io.in_kind == IN_P) io.ps_in = sr;
        io.cnt_in = (int)(even ? N / 2 + 1 : (N + 1) / 2);
        if (op == OP_C2R) io.conj_in = forward ? 1 : 0;
        io.pre = even ? PRE_HERM_EVEN : PRE_HERM_ODD;
        io.fwd = 0;
        if (even) {
            if (ln.es_out == sr && side_aligned(ln.out, 2 * sr, ln.bn, ln.bso, 2 * sr)) {
                io.out_kind = OUT_C;
                io.os = 2 * sr;
            } else {
                io.out_kind = OUT_P;
                io.os = 2 * ln.es_out;
                io.ps_out = ln.es_out;
            }
            io.cnt_out = (int)M;
        } else {
            io.out_kind = OUT_R;
            io.cnt_out = (int)N;
        }
        break;
    }
    if (N == 1 && (op == OP_R2HC || op == OP_HC2R)) {
        io.in_kind = IN_R;
        io.out_kind = OUT_R;
        io.pre = PRE_NONE;
        io.post = POST_NONE;
        io.cnt_in = io.cnt_out = 1;
    }
    if (N == 1 && op == OP_C2R) {
        io.in_kind = IN_C;
        io.out_kind = OUT_R;
        io.pre = PRE_NONE;
        io.conj_in = 0;
        io.cnt_in = io.cnt_out = 1;
    }
    if (N == 1 && op == OP_R2C) {
        io.in_kind = IN_R;
        io.post = POST_NONE;
        io.cnt_in = 1;
    }
    // odd real lengths on a single-CTA core: two real lines per complex line
    if (N > 1 && N % 2 == 1 && op != OP_C2C && ln.bn[0] >= 2) {
        io.pair = 1;
        io.pair_n0 = ln.bn[0];
        io.pair_in = ln.bsi[0];
        io.pair_out = ln.bso[0];
        io.bn[0] = (ln.bn[0] + 1) / 2;
        io.bsi[0] = 2 * ln.bsi[0];
        io.bso[0] = 2 * ln.bso[0];
        io.nlines = io.bn[0] * io.bn[1] * io.bn[2];
        if (op == OP_R2HC || op == OP_R2C) {
            io.post = POST_PAIR;
        } else {
            io.pre = PRE_HERM_ODD;  // both half spectra completed to Z in the prologue
        }
    }
    // coalescing mode: lines adjacent in memory and elements strided
    long long ue_in = (io.in_kind == IN_C || io.in_kind == IN_P) ? 2 * sr : sr;
    long long ue_out = (io.out_kind == OUT_C || io.out_kind == OUT_P) ? 2 * sr : sr;
    io.cols_in = (ln.bn[0] > 1 && std::llabs(ln.bsi[0]) <= ue_in && std::llabs(io.is) > ue_in) ? 1 : 0;
    io.cols_out = (ln.bn[0] > 1 && std::llabs(ln.bso[0]) <= ue_out && std::llabs(io.os) > ue_out) ? 1 : 0;
    if (!forced && col_fourstep_ok(a, *core, io)) {
        auto c4 = col_core(a, core->M);
        if (c4) {
            const long long ES = 2 * (long long)store_real_bytes(a);
            for (long long i2 = 0; i2 < io.bn[2]; ++i2) {
                IODesc q = io;
                q.in += i2 * io.bsi[2];
                q.out += i2 * io.bso[2];
                q.bn[2] = 1;
                q.bsi[2] = q.bso[2] = 0;
                q.nlines = q.bn[0] * q.bn[1];
                char *B = (char *)scratch_for(st).get(1, (size_t)(q.nlines * c4->M * ES));
                run_fourstep_cols(*c4, q, B, st);
            }
            return;
        }
    }
    run_complex(*core, io, st);
}

// --------------------------------------------------------------------------
// N-d driver (pocketfft_hdronly.h:3012-3050 semantics)
// --------------------------------------------------------------------------
static void check_axes(size_t ndim, size_t naxes, const size_t *axes)
{
    if (ndim < 1) raise(IG_ENDIM, "ndim must be >= 1");
    std::vector<int> seen(ndim, 0);
    for (size_t i = 0; i < naxes; ++i) {
        if (axes[i] >= ndim) raise(IG_EINVAL_AXIS, "bad axis number");
        if (++seen[axes[i]] > 1) raise(IG_EREPEAT_AXIS, "axis specified repeatedly");
    }
}

// lines along `axis` of an array with `shape`, element strides in bytes
static void for_lines(size_t ndim, const size_t *shape, const ptrdiff_t *sin, const ptrdiff_t *sout, size_t axis,
                      const char *in, char *out, const std::function<void(const Lines &)> &fn)
{
    // collect the other dims, innermost (smallest |out stride|) first
    std::vector<size_t> dims;
    for (size_t d = 0; d < ndim; ++d)
        if (d != axis && shape[d] > 1) dims.push_back(d);
    std::sort(dims.begin(), dims.end(), [&](size_t x, size_t y) {
        long long ax = std::llabs((long long)sout[x]), ay = std::llabs((long long)sout[y]);
        if (ax != ay) return ax < ay;
        return std::llabs((long long)sin[x]) < std::llabs((long long)sin[y]);
    });
    // merge dims that are contiguous in both arrays
    struct D { long long n, si, so; };
    std::vector<D> m;
    for (size_t d : dims) {
        if (!m.empty() && m.back().si * m.back().n == (long long)sin[d] && m.back().so * m.back().n == (long long)sout[d]) {
            m.back().n *= (long long)shape[d];
        } else {
            m.push_back(D{(long long)shape[d], (long long)sin[d], (long long)sout[d]});
        }
    }
    Lines ln;
    ln.es_in = sin[axis];
    ln.es_out = sout[axis];
    for (int i = 0; i < 3; ++i) { ln.bn[i] = 1; ln.bsi[i] = 0; ln.bso[i] = 0; }
    size_t inner = std::min<size_t>(m.size(), 3);
    ln.nlines = 1;
    for (size_t i = 0; i < inner; ++i) {
        ln.bn[i] = m[i].n;
        ln.bsi[i] = m[i].si;
        ln.bso[i] = m[i].so;
        ln.nlines *= m[i].n;
    }
    // remaining outer dims: host loop
    std::vector<long long> idx(m.size() > 3 ? m.size() - 3 : 0, 0);
    while (true) {
        long long oi = 0, oo = 0;
        for (size_t k = 0; k < idx.size(); ++k) {
            oi += idx[k] * m[3 + k].si;
            oo += idx[k] * m[3 + k].so;
        }
        ln.in = in + oi;
        ln.out = out + oo;
        fn(ln);
        size_t k = 0;
        for (; k < idx.size(); ++k) {
            if (++idx[k] < m[3 + k].n) break;
            idx[k] = 0;
        }
        if (k == idx.size()) break;
    }
}

static cudaStream_t as_stream(void *s) { return (cudaStream_t)s; }

static void nd_c2c_device(Arith a, size_t ndim, const size_t *shape, const ptrdiff_t *sin, const ptrdiff_t *sout,
                          size_t naxes, const size_t *axes, int forward, const void *in, void *out, double fct,
                          cudaStream_t st)
{
    for (size_t k = 0; k < naxes; ++k) {
        size_t ax = axes[k];
        const char *src = k == 0 ? (const char *)in : (const char *)out;
        const ptrdiff_t *ss = k == 0 ? sin : sout;
        for_lines(ndim, shape, ss, sout, ax, src, (char *)out, [&](const Lines &ln) {
            exec_op(a, OP_C2C, (long long)shape[ax], ln, forward, k == 0 ? fct : 1.0, st);
        });
    }
}

// --------------------------------------------------------------------------
// workspace for host-memory entry points
// --------------------------------------------------------------------------
struct Workspace {
    DevBuf *buf = nullptr;
    size_t cap = 0;
    void *get(size_t n)
    {
        if (n > cap) {
            delete buf;
            buf = nullptr;
            cap = 0;
            buf = new DevBuf(n);
            cap = n;
        }
        return buf->p;
    }
    void release()
    {
        delete buf;
        buf = nullptr;
        cap = 0;
    }
};
static std::mutex g_ws_mu;
static Workspace g_ws;

// streams and chunk buffers of the pipelined host-memory batches
static const int kPipe = 3;
// chunk size of the pipeline: IG_PIPE_CHUNK_MB (default 16 MiB)
static size_t pipe_chunk_bytes()
{
    static size_t v = [] {
        const char *e = getenv("IG_PIPE_CHUNK_MB");
        long mb = e ? atol(e) : 16;
        return (size_t)std::max<long>(1, mb) << 20;
    }();
    return v;
}
struct Pipe {
    cudaStream_t st[kPipe] = {};
    Workspace ws[kPipe];
};
static std::map<int, std::unique_ptr<Pipe>> g_pipes;

static Pipe &pipe_for_device()
{
    auto &p = g_pipes[device_id()];
    if (!p) {
        p.reset(new Pipe);
        for (int i = 0; i < kPipe; ++i)
            ck(cudaStreamCreateWithFlags(&p->st[i], cudaStreamNonBlocking), "pipeline stream");
    }
    return *p;
}


// byte span [lo, hi) covered by a strided array
static void span_of(size_t ndim, const size_t *shape, const ptrdiff_t *st, size_t elem, long long &lo, long long &hi)
{
    lo = 0;
    hi = 0;
    for (size_t d = 0; d < ndim; ++d) {
        if (shape[d] == 0) { lo = hi = 0; return; }
        long long ext = (long long)(shape[d] - 1) * (long long)st[d];
        if (ext < 0) lo += ext; else hi += ext;
    }
    hi += (long long)elem;
}
static bool dense(size_t ndim, const size_t *shape, const ptrdiff_t *st, size_t elem)
{
    long long lo, hi;
    span_of(ndim, shape, st, elem, lo, hi);
    long long tot = (long long)elem;
    for (size_t d = 0; d < ndim; ++d) tot *= (long long)shape[d];
    return hi - lo == tot;
}

}  // namespace ig

using namespace ig;

// ----------------------------------------------------------------------------
// C ABI
// ----------------------------------------------------------------------------
struct ig_cfft_plan_i {
    size_t n;
    Arith a;
    int dtype;
    std::shared_ptr<Core> core;
};
struct ig_rfft_plan_i {
    size_t n;
    Arith a;
    int dtype;
    std::shared_ptr<Core> core;
};

template <class F> static int guarded(F &&f)
{
    try {
        f();
        g_err.clear();
        return IG_OK;
    } catch (const Error &e) {
        g_err = e.msg;
        return e.code;
    } catch (const std::bad_alloc &) {
        g_err = "host allocation failed";
        return IG_ENOMEM;
    } catch (const std::exception &e) {
        g_err = e.what();
        return IG_EINVAL;
    }
}

extern "C" {

const char *ig_last_error_string(void) { return g_err.c_str(); }
int ig_version(void) { return 100; }

int ig_set_f64_arith(int mode)
{
    if (mode != 0 && mode != 1) {
        g_err = "f64 arithmetic mode must be 0 or 1";
        return IG_EINVAL;
    }
    g_f64_arith = mode;
    return IG_OK;
}

void ig_release_caches(void)
{
    std::lock_guard<std::mutex> lk(g_mu);
    g_cores.clear();
    std::lock_guard<std::mutex> lk2(g_ws_mu);
    g_ws.release();
    for (auto &kv : g_pipes)
        for (int i = 0; i < kPipe; ++i) kv.second->ws[i].release();
}

unsigned long long ig_launch_count(int reset)
{
    return reset ? g_launches.exchange(0) : g_launches.load();
}

int ig_device_faults(unsigned *count)
{
    return guarded([&] {
        if (!count) raise(IG_EINVAL, "null count");
        *count = 0;
        ck(cudaDeviceSynchronize(), "device synchronize");
        ck(Launch<TagF32>::pipe_faults(count), "fault counters");
    });
}

// ---- 1-D plans ----
ig_cfft_plan ig_make_cfft_plan(size_t length, int dtype)
{
    ig_cfft_plan p = nullptr;
    int rc = guarded([&] {
        if (length == 0) raise(IG_EZERO_LEN, "zero-length FFT requested");
        if (dtype != IG_F64 && dtype != IG_F32) raise(IG_EINVAL, "bad dtype");
        auto pl = std::make_unique<ig_cfft_plan_i>();
        pl->n = length;
        pl->dtype = dtype;
        pl->a = arith_for(dtype);
        pl->core = get_core(pl->a, (long long)length, false);
        p = pl.release();
    });
    (void)rc;
    return p;
}
void ig_destroy_cfft_plan(ig_cfft_plan plan) { delete plan; }
size_t ig_cfft_length(ig_cfft_plan plan) { return plan ? plan->n : 0; }

ig_rfft_plan ig_make_rfft_plan(size_t length, int dtype)
{
    ig_rfft_plan p = nullptr;
    guarded([&] {
        if (length == 0) raise(IG_EZERO_LEN, "zero-length FFT requested");
        if (dtype != IG_F64 && dtype != IG_F32) raise(IG_EINVAL, "bad dtype");
        auto pl = std::make_unique<ig_rfft_plan_i>();
        pl->n = length;
        pl->dtype = dtype;
        pl->a = arith_for(dtype);
        bool even = length % 2 == 0 && length > 1;
        pl->core = get_core(pl->a, even ? (long long)length / 2 : (long long)length, even);
        p = pl.release();
    });
    return p;
}
void ig_destroy_rfft_plan(ig_rfft_plan plan) { delete plan; }
size_t ig_rfft_length(ig_rfft_plan plan) { return plan ? plan->n : 0; }

int ig_cfft_uses_bluestein(ig_cfft_plan plan, size_t *n2)
{
    if (!plan) return IG_EINVAL;
    bool b = plan->core->d.blue == 1 || plan->core->kind == 2;
    if (n2) *n2 = b ? (size_t)plan->core->n2 : 0;
    return b ? 1 : 0;
}
int ig_rfft_uses_bluestein(ig_rfft_plan plan, size_t *n2)
{
    if (!plan) return IG_EINVAL;
    bool b = plan->core->d.blue == 1 || plan->core->kind == 2;
    if (n2) *n2 = b ? (size_t)plan->core->n2 : 0;
    return b ? 1 : 0;
}

static Lines contiguous_lines(const void *in, void *out, long long batch, long long dist_in, long long dist_out,
                              long long es_in, long long es_out)
{
    Lines ln;
    ln.in = (const char *)in;
    ln.out = (char *)out;
    ln.es_in = es_in;
    ln.es_out = es_out;
    ln.nlines = batch;
    ln.bn[0] = batch;
    ln.bn[1] = ln.bn[2] = 1;
    ln.bsi[0] = dist_in * es_in;
    ln.bso[0] = dist_out * es_out;
    ln.bsi[1] = ln.bsi[2] = ln.bso[1] = ln.bso[2] = 0;
    return ln;
}

int ig_cfft_exec_device(ig_cfft_plan plan, const void *in, void *out, size_t batch, size_t dist_in, size_t dist_out,
                        int forward, double fct, void *stream)
{
    return guarded([&] {
        if (!plan || !in || !out) raise(IG_EINVAL, "null argument");
        long long es = 2 * (long long)store_real_bytes(plan->a);
        exec_op(plan->a, OP_C2C, (long long)plan->n,
                contiguous_lines(in, out, (long long)batch, (long long)dist_in, (long long)dist_out, es, es), forward,
                fct, as_stream(stream));
    });
}

// ---- allocation-free complex execution ------------------------------------
// Some callers cannot allocate device memory at call time: a process that
// reserves its whole device-memory budget up front in a pool that must not
// grow, or a latency-bound loop where cudaMalloc / cudaFree (which can
// synchronise the device and take unbounded time) are not allowed.
// ig_cfft_exec_device_noalloc serves them: its four-step scratch is this
// file-scope device array instead of the cached per-stream workspace.  Every
// GPU that loads the library holds the array until the process exits.
#define IG_NOALLOC_SCRATCH_BYTES (64ull << 20)
#define IG_NOALLOC_MAX_DEVICES 64
static __device__ __align__(256) unsigned char g_noalloc_scratch[IG_NOALLOC_SCRATCH_BYTES];
static std::mutex g_noalloc_mu;
static void *g_noalloc_ptr[IG_NOALLOC_MAX_DEVICES];

// Device address of g_noalloc_scratch on the current device.  In host code
// the array's name is only a host-side stand-in, so the address is looked up
// once per device (with that device current) and cached.
static void *noalloc_scratch()
{
    int dev = device_id();
    if (dev < 0 || dev >= IG_NOALLOC_MAX_DEVICES) raise(IG_EINVAL, "device index beyond the no-allocation table");
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void *p = nullptr;
        ck(cudaGetSymbolAddress(&p, g_noalloc_scratch), "cudaGetSymbolAddress(no-allocation scratch)");
        g_noalloc_ptr[dev] = p;
    }
    return g_noalloc_ptr[dev];
}

// Same transform as ig_cfft_exec_device, with no device-memory allocation:
// single-CTA plans need no scratch, four-step plans use the static array
// (at most IG_NOALLOC_SCRATCH_BYTES = batch * length * complex size).  Plans
// that run Bluestein or Rader over a multi-pass core are rejected.  The first call on
// a device (whatever its plan) looks up the array's address there; make that
// first call before any stream capture.  All calls share the array and it keeps
// the previous call's contents (this path writes every scratch element before
// reading it, so nothing needs clearing); calls that overlap on the GPU race.
int ig_cfft_exec_device_noalloc(ig_cfft_plan plan, const void *in, void *out, size_t batch, size_t dist_in,
                                size_t dist_out, int forward, double fct, void *stream)
{
    return guarded([&] {
        if (!plan || !in || !out) raise(IG_EINVAL, "null argument");
        const Core &c = *plan->core;
        const long long es = 2 * (long long)store_real_bytes(plan->a);
        if (c.kind == 2 || c.kind == 3)
            raise(IG_EINVAL, "no-allocation execution does not cover Bluestein or Rader over a multi-pass core");
        // the per-device set-up runs on the first call, for every kind of plan
        char *const arr = (char *)noalloc_scratch();
        if (batch == 0) return;
        char *scr = nullptr;
        if (c.kind == 1) {
            unsigned long long need = (unsigned long long)batch * (unsigned long long)c.M * (unsigned long long)es;
            if (need > IG_NOALLOC_SCRATCH_BYTES)
                raise(IG_ETOOLARGE, "batch * length * element size exceeds the 64 MiB no-allocation scratch");
            scr = arr;
        }
        require_aligned(in, (size_t)es, "input");
        require_aligned(out, (size_t)es, "output");
        IODesc io = blank_io();
        io.in = (const char *)in;
        io.out = (char *)out;
        io.is = io.os = es;
        io.nlines = (long long)batch;
        io.bn[0] = (long long)batch;
        io.bsi[0] = (long long)dist_in * es;
        io.bso[0] = (long long)dist_out * es;
        io.in_kind = IN_C;
        io.out_kind = OUT_C;
        io.cnt_in = io.cnt_out = (int)c.M;
        io.nreal = c.M;
        io.fwd = forward;
        io.fct = fct;
        if (c.kind == 0) launch_smem(c.a, c.d, io, as_stream(stream));
        else run_fourstep(c, io, scr, as_stream(stream));
    });
}

int ig_rfft_exec_device(ig_rfft_plan plan, const void *in, void *out, size_t batch, size_t dist_in, size_t dist_out,
                        int forward, double fct, void *stream)
{
    return guarded([&] {
        if (!plan || !in || !out) raise(IG_EINVAL, "null argument");
        long long es = (long long)store_real_bytes(plan->a);
        exec_op(plan->a, forward ? OP_R2HC : OP_HC2R, (long long)plan->n,
                contiguous_lines(in, out, (long long)batch, (long long)dist_in, (long long)dist_out, es, es), forward,
                fct, as_stream(stream));
    });
}

// Pageable host memory that the device reaches through the host's page tables
// (address translation services): the pipeline's copies then run as SM copy
// kernels, since a copy engine moving pageable memory waits for the host and
// the two directions would not overlap.  IG_PAGEABLE_CE=1 keeps the copy
// engines.
static bool pageable_by_sms(const void *c)
{
    static const bool off = getenv("IG_PAGEABLE_CE") != nullptr;
    if (off) return false;
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, c) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    if (at.type != cudaMemoryTypeUnregistered) return false;
    int dev = device_id(), pageable = 0, host_pt = 0;
    ck(cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, dev), "device attribute");
    ck(cudaDeviceGetAttribute(&host_pt, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev), "device attribute");
    return pageable && host_pt;
}

// Host-memory batches.  Batches longer than one chunk run as a pipeline of
// line chunks over three streams, so that the host-to-device copy of one
// chunk, the transform of the next and the device-to-host copy of a third
// overlap (fully so for page-locked memory; copies from pageable memory may
// serialise with the host); shorter batches take one copy each way.
static int host_batch(bool real, size_t n, Arith a, void *c, size_t batch, size_t dist, int forward, double fct)
{
    return guarded([&] {
        if (!c) raise(IG_EINVAL, "null data pointer");
        if (batch == 0) return;
        long long es = (real ? 1 : 2) * (long long)store_real_bytes(a);
        if (dist < n) raise(IG_EINVAL, "line distance smaller than the length");
        size_t bytes = ((batch - 1) * dist + n) * (size_t)es;
        const Op op = real ? (forward ? OP_R2HC : OP_HC2R) : OP_C2C;
        std::lock_guard<std::mutex> lk(g_ws_mu);
        const size_t line_bytes = dist * (size_t)es;
        const size_t chunk_lines = std::max<size_t>(1, pipe_chunk_bytes() / line_bytes);
        if (batch <= chunk_lines) {
            void *d = g_ws.get(bytes);
            ck(cudaMemcpy(d, c, bytes, cudaMemcpyHostToDevice), "H2D copy");
            Lines ln = contiguous_lines(d, d, (long long)batch, (long long)dist, (long long)dist, es, es);
            exec_op(a, op, (long long)n, ln, forward, fct, 0);
            ck(cudaMemcpy(c, d, bytes, cudaMemcpyDeviceToHost), "D2H copy");
            return;
        }
        Pipe &pp = pipe_for_device();
        const bool by_sms = pageable_by_sms(c);
        const int sms = sm_count() / 2;  // copy grids of 4 CTAs per SM
        const size_t cbytes = ((chunk_lines - 1) * dist + n) * (size_t)es;
        void *dbuf[kPipe];
        for (int i = 0; i < kPipe; ++i) dbuf[i] = pp.ws[i].get(cbytes);
        try {
            size_t i = 0;
            for (size_t l0 = 0; l0 < batch; l0 += chunk_lines, ++i) {
                const size_t nl = std::min(chunk_lines, batch - l0);
                const size_t nb = ((nl - 1) * dist + n) * (size_t)es;
                char *h = (char *)c + l0 * line_bytes;
                cudaStream_t st = pp.st[i % kPipe];
                void *d = dbuf[i % kPipe];
                if (by_sms) {
                    ck(launch_copy(h, d, nb, sms, st), "H2D copy kernel");
                    count_launch();
                } else {
                    ck(cudaMemcpyAsync(d, h, nb, cudaMemcpyHostToDevice, st), "H2D copy");
                }
                Lines ln = contiguous_lines(d, d, (long long)nl, (long long)dist, (long long)dist, es, es);
                exec_op(a, op, (long long)n, ln, forward, fct, st);
                if (by_sms) {
                    ck(launch_copy(d, h, nb, sms, st), "D2H copy kernel");
                    count_launch();
                } else {
                    ck(cudaMemcpyAsync(h, d, nb, cudaMemcpyDeviceToHost, st), "D2H copy");
                }
            }
            for (int k = 0; k < kPipe; ++k) ck(cudaStreamSynchronize(pp.st[k]), "pipeline");
        } catch (...) {
            for (int k = 0; k < kPipe; ++k) cudaStreamSynchronize(pp.st[k]);
            throw;
        }
    });
}

int ig_cfft_forward(ig_cfft_plan plan, void *c, double fct)
{
    if (!plan) { g_err = "null plan"; return IG_EINVAL; }
    return host_batch(false, plan->n, plan->a, c, 1, plan->n, 1, fct);
}
int ig_cfft_backward(ig_cfft_plan plan, void *c, double fct)
{
    if (!plan) { g_err = "null plan"; return IG_EINVAL; }
    return host_batch(false, plan->n, plan->a, c, 1, plan->n, 0, fct);
}
int ig_rfft_forward(ig_rfft_plan plan, void *c, double fct)
{
    if (!plan) { g_err = "null plan"; return IG_EINVAL; }
    return host_batch(true, plan->n, plan->a, c, 1, plan->n, 1, fct);
}
int ig_rfft_backward(ig_rfft_plan plan, void *c, double fct)
{
    if (!plan) { g_err = "null plan"; return IG_EINVAL; }
    return host_batch(true, plan->n, plan->a, c, 1, plan->n, 0, fct);
}
int ig_cfft_exec_batch(ig_cfft_plan plan, void *c, size_t batch, size_t dist, int forward, double fct)
{
    if (!plan) { g_err = "null plan"; return IG_EINVAL; }
    return host_batch(false, plan->n, plan->a, c, batch, dist, forward, fct);
}
int ig_rfft_exec_batch(ig_rfft_plan plan, void *c, size_t batch, size_t dist, int forward, double fct)
{
    if (!plan) { g_err = "null plan"; return IG_EINVAL; }
    return host_batch(true, plan->n, plan->a, c, batch, dist, forward, fct);
}

// ---- N-d ----
static void nd_checks(int dtype, size_t ndim, const size_t *shape, const ptrdiff_t *sin, const ptrdiff_t *sout,
                      size_t naxes, const size_t *axes, const void *in, void *out, bool allow_inplace)
{
    if (dtype != IG_F64 && dtype != IG_F32) raise(IG_EINVAL, "bad dtype");
    if (ndim < 1) raise(IG_ENDIM, "ndim must be >= 1");
    if (!shape || !sin || !sout || (naxes && !axes)) raise(IG_EINVAL, "null argument");
    check_axes(ndim, naxes, axes);
    if (in == out) {
        if (!allow_inplace) raise(IG_ESTRIDE_INPLACE, "stride mismatch");
        for (size_t d = 0; d < ndim; ++d)
            if (sin[d] != sout[d]) raise(IG_ESTRIDE_INPLACE, "stride mismatch");
    }
    if (!in || !out) raise(IG_EINVAL, "null data pointer");
}

static size_t prod(size_t ndim, const size_t *shape)
{
    size_t p = 1;
    for (size_t d = 0; d < ndim; ++d) p *= shape[d];
    return p;
}

int ig_c2c_device(int dtype, size_t ndim, const size_t *shape, const ptrdiff_t *sin, const ptrdiff_t *sout,
                  size_t naxes, const size_t *axes, int forward, const void *in, void *out, double fct, void *stream)
{
    return guarded([&] {
        if (ndim >= 1 && shape && prod(ndim, shape) == 0) return;
        nd_checks(dtype, ndim, shape, sin, sout, naxes, axes, in, out, true);
        nd_c2c_device(arith_for(dtype), ndim, shape, sin, sout, naxes, axes, forward, in, out, fct,
                      as_stream(stream));
    });
}

static void nd_r2c_device(Arith a, size_t ndim, const size_t *shape_in, const ptrdiff_t *sin, const ptrdiff_t *sout,
                          size_t naxes, const size_t *axes, int forward, const void *in, void *out, double fct,
                          cudaStream_t st)
{
    if (naxes == 0) return;
    size_t last = axes[naxes - 1];
    for_lines(ndim, shape_in, sin, sout, last, (const char *)in, (char *)out, [&](const Lines &ln) {
        exec_op(a, OP_R2C, (long long)shape_in[last], ln, forward, fct, st);
    });
    if (naxes == 1) return;
    std::vector<size_t> shape_out(shape_in, shape_in + ndim);
    shape_out[last] = shape_in[last] / 2 + 1;
    nd_c2c_device(a, ndim, shape_out.data(), sout, sout, naxes - 1, axes, forward, out, out, 1.0, st);
}

int ig_r2c_device(int dtype, size_t ndim, const size_t *shape_in, const ptrdiff_t *sin, const ptrdiff_t *sout,
                  size_t naxes, const size_t *axes, int forward, const void *in, void *out, double fct, void *stream)
{
    return guarded([&] {
        if (ndim >= 1 && shape_in && prod(ndim, shape_in) == 0) return;
        nd_checks(dtype, ndim, shape_in, sin, sout, naxes, axes, in, out, false);
        nd_r2c_device(arith_for(dtype), ndim, shape_in, sin, sout, naxes, axes, forward, in, out, fct,
                      as_stream(stream));
    });
}

static void nd_c2r_device(Arith a, size_t ndim, const size_t *shape_out, const ptrdiff_t *sin, const ptrdiff_t *sout,
                          size_t naxes, const size_t *axes, int forward, const void *in, void *out, double fct,
                          cudaStream_t st)
{
    if (naxes == 0) return;
    size_t last = axes[naxes - 1];
    if (naxes == 1) {
        for_lines(ndim, shape_out, sin, sout, last, (const char *)in, (char *)out, [&](const Lines &ln) {
            exec_op(a, OP_C2R, (long long)shape_out[last], ln, forward, fct, st);
        });
        return;
    }
    // c2c over the other axes into a contiguous temporary, then c2r on the last axis
    std::vector<size_t> shape_in(shape_out, shape_out + ndim);
    shape_in[last] = shape_out[last] / 2 + 1;
    size_t ce = 2 * store_real_bytes(a);
    std::vector<ptrdiff_t> sinter(ndim);
    sinter[ndim - 1] = (ptrdiff_t)ce;
    for (size_t d = ndim - 1; d-- > 0;) sinter[d] = sinter[d + 1] * (ptrdiff_t)shape_in[d + 1];
    // the temporary (pocketfft_hdronly.h:3384 allocates it per call) is a grow-only
    // workspace of the stream, kept between calls (slot 7: the multi-pass paths
    // of the line transforms use slots 0-6)
    void *tmp = scratch_for(st).get(7, prod(ndim, shape_in.data()) * ce);
    nd_c2c_device(a, ndim, shape_in.data(), sin, sinter.data(), naxes - 1, axes, forward, in, tmp, 1.0, st);
    for_lines(ndim, shape_out, sinter.data(), sout, last, (const char *)tmp, (char *)out, [&](const Lines &ln) {
        exec_op(a, OP_C2R, (long long)shape_out[last], ln, forward, fct, st);
    });
}

int ig_c2r_device(int dtype, size_t ndim, const size_t *shape_out, const ptrdiff_t *sin, const ptrdiff_t *sout,
                  size_t naxes, const size_t *axes, int forward, const void *in, void *out, double fct, void *stream)
{
    return guarded([&] {
        if (ndim >= 1 && shape_out && prod(ndim, shape_out) == 0) return;
        nd_checks(dtype, ndim, shape_out, sin, sout, naxes, axes, in, out, false);
        nd_c2r_device(arith_for(dtype), ndim, shape_out, sin, sout, naxes, axes, forward, in, out, fct,
                      as_stream(stream));
    });
}

// host-memory N-d: copy the byte spans to the GPU, run, copy back
// host arrays: copy the spans the strides cover to the device, run `fn` on
// device pointers with the same strides, copy the output span back
static void host_nd_run(size_t ndim, const std::vector<size_t> &shp_in, const std::vector<size_t> &shp_out,
                        const ptrdiff_t *sin, const ptrdiff_t *sout, size_t e_in, size_t e_out, const void *in,
                        void *out, const std::function<void(const void *, void *)> &fn)
{
    long long ilo, ihi, olo, ohi;
    span_of(ndim, shp_in.data(), sin, e_in, ilo, ihi);
    span_of(ndim, shp_out.data(), sout, e_out, olo, ohi);
    bool inplace = in == out;
    std::lock_guard<std::mutex> lk(g_ws_mu);
    size_t ibytes = (size_t)(ihi - ilo), obytes = (size_t)(ohi - olo);
    size_t oalign = inplace ? 0 : ((ibytes + 255) / 256) * 256;
    char *d = (char *)g_ws.get(oalign + (inplace ? std::max(ibytes, obytes) : obytes));
    char *din = d - ilo;
    char *dout = inplace ? din : d + oalign - olo;
    ck(cudaMemcpy(d, (const char *)in + ilo, ibytes, cudaMemcpyHostToDevice), "H2D copy");
    if (!inplace && !dense(ndim, shp_out.data(), sout, e_out))
        ck(cudaMemcpy(dout + olo, (char *)out + olo, obytes, cudaMemcpyHostToDevice), "H2D copy (output gaps)");
    fn(din, dout);
    ck(cudaMemcpy((char *)out + olo, dout + olo, obytes, cudaMemcpyDeviceToHost), "D2H copy");
}

static void host_nd(int kind, int dtype, size_t ndim, const size_t *shape, const ptrdiff_t *sin, const ptrdiff_t *sout,
                    size_t naxes, const size_t *axes, int forward, const void *in, void *out, double fct)
{
    Arith a = arith_for(dtype);
    size_t sr = store_real_bytes(a);
    std::vector<size_t> shp_in(shape, shape + ndim), shp_out(shape, shape + ndim);
    size_t e_in = 2 * sr, e_out = 2 * sr;
    if (kind == 1) {  // r2c
        e_in = sr;
        if (naxes) shp_out[axes[naxes - 1]] = shape[axes[naxes - 1]] / 2 + 1;
    } else if (kind == 2) {  // c2r
        e_out = sr;
        if (naxes) shp_in[axes[naxes - 1]] = shape[axes[naxes - 1]] / 2 + 1;
    }
    host_nd_run(ndim, shp_in, shp_out, sin, sout, e_in, e_out, in, out, [&](const void *din, void *dout) {
        if (kind == 0) nd_c2c_device(a, ndim, shape, sin, sout, naxes, axes, forward, din, dout, fct, 0);
        else if (kind == 1) nd_r2c_device(a, ndim, shape, sin, sout, naxes, axes, forward, din, dout, fct, 0);
        else nd_c2r_device(a, ndim, shape, sin, sout, naxes, axes, forward, din, dout, fct, 0);
    });
}


// ---- real-to-real transforms (pocketfft::dct / dst / r2r_fftpack / Hartley) ------
// One axis at a time, like the reference's general_nd (pocketfft_hdronly.h:3012-3050):
// the first axis reads the input, later axes read and write the output, fct on
// the first axis only.  Per axis: pre-map into contiguous scratch lines, one
// FFT of the scratch lines, post-map into the output lines (kernels k_r2r_pre /
// k_r2r_post; the DCT / DST forms run a complex FFT of length 2N, 2(N-1) or 2(N+1)).
struct R2RTables {
    std::unique_ptr<DevBuf> tw1, tw2;
};
static std::map<std::tuple<int, int, long long>, std::shared_ptr<R2RTables>> g_r2r_tw;

static std::shared_ptr<R2RTables> r2r_tables(Arith a, long long N)
{
    std::lock_guard<std::mutex> lk(g_mu);
    auto key = std::make_tuple(device_id(), (int)a, N);
    auto it = g_r2r_tw.find(key);
    if (it != g_r2r_tw.end()) return it->second;
    auto t = std::make_shared<R2RTables>();
    t->tw1.reset(new DevBuf((size_t)(N + 1) * slot_bytes(a)));
    t->tw2.reset(new DevBuf((size_t)std::max<long long>(N, 1) * slot_bytes(a)));
    cudaError_t e = a == A_F32 ? Launch<TagF32>::r2r_tw(t->tw1->p, t->tw2->p, N)
                  : a == A_DF  ? Launch<TagDF>::r2r_tw(t->tw1->p, t->tw2->p, N)
                               : Launch<TagF64>::r2r_tw(t->tw1->p, t->tw2->p, N);
    ck(e, "r2r tables");
    count_launch();
    ck(cudaDeviceSynchronize(), "r2r tables");
    g_r2r_tw[key] = t;
    return t;
}

static void launch_r2r(Arith a, bool pre, const IODesc &io_in, const R2RDesc &d_in, cudaStream_t st)
{
    IODesc io = io_in;
    set_line_divs(io);
    R2RDesc d = d_in;
    d.fL2 = make_fdiv((unsigned)std::max<long long>(1, std::min<long long>(d.L2, 0x7fffffffLL)));
    d.fN = make_fdiv((unsigned)std::max<long long>(1, std::min<long long>(d.N, 0x7fffffffLL)));
    cudaError_t e;
    if (pre)
        e = a == A_F32 ? Launch<TagF32>::r2r_pre(io, d, st)
          : a == A_DF  ? Launch<TagDF>::r2r_pre(io, d, st)
                       : Launch<TagF64>::r2r_pre(io, d, st);
    else
        e = a == A_F32 ? Launch<TagF32>::r2r_post(io, d, st)
          : a == A_DF  ? Launch<TagDF>::r2r_post(io, d, st)
                       : Launch<TagF64>::r2r_post(io, d, st);
    ck(e, "r2r map");
    count_launch();
}

// one axis over the lines `ln` (length N along the axis).  mode: R2RMode;
// COPY runs the halfcomplex FFT in direction fwd with the negations the
// reference's ExecR2R applies (neg_pre before, neg_post after).
static void r2r_axis(Arith a, const Lines &ln, long long N, int mode, int ortho, int neg_pre, int neg_post, int fwd,
                     double fct, cudaStream_t st)
{
    if (ln.nlines <= 0 || N <= 0) return;
    const long long sr = (long long)store_real_bytes(a), ES = 2 * sr, nl = ln.nlines;
    if (!side_aligned(ln.in, ln.es_in, ln.bn, ln.bsi, sr) || !side_aligned(ln.out, ln.es_out, ln.bn, ln.bso, sr))
        raise(IG_EINVAL, "data pointer or stride not aligned to the element size");
    const bool cplx = mode <= R2R_DST4;
    R2RDesc d{};
    d.mode = mode;
    d.ortho = ortho;
    d.N = N;
    d.L2 = mode == R2R_DCT1 ? 2 * (N - 1) : mode == R2R_DST1 ? 2 * (N + 1) : cplx ? 2 * N : N;
    d.fct = fct;
    std::shared_ptr<R2RTables> tb;
    if (cplx && mode != R2R_DCT1 && mode != R2R_DST1) {
        tb = r2r_tables(a, N);
        d.tw1 = tb->tw1->p;
        d.tw2 = tb->tw2->p;
    }
    char *A = (char *)scratch_for(st).get(6, (size_t)(nl * d.L2 * (cplx ? ES : sr)));
    d.scr = A;
    IODesc io = blank_io();
    io.in = ln.in;
    io.out = ln.out;
    io.is = ln.es_in;
    io.os = ln.es_out;
    io.nlines = nl;
    for (int i = 0; i < 3; ++i) {
        io.bn[i] = ln.bn[i];
        io.bsi[i] = ln.bsi[i];
        io.bso[i] = ln.bso[i];
    }
    d.neg_even = neg_pre;
    launch_r2r(a, true, io, d, st);
    if (cplx) {
        Lines s = contiguous_lines(A, A, nl, d.L2, d.L2, ES, ES);
        exec_op(a, OP_C2C, d.L2, s, 1, 1.0, st);
    } else {
        Lines s = contiguous_lines(A, A, nl, N, N, sr, sr);
        exec_op(a, fwd ? OP_R2HC : OP_HC2R, N, s, fwd, fct, st);
    }
    d.neg_even = neg_post;
    launch_r2r(a, false, io, d, st);
}

static void r2r_nd_device(Arith a, size_t ndim, const size_t *shape, const ptrdiff_t *sin, const ptrdiff_t *sout,
                          size_t naxes, const size_t *axes, const void *in, void *out, double fct, cudaStream_t st,
                          int mode, int ortho, int neg_pre, int neg_post, int fwd)
{
    for (size_t i = 0; i < naxes; ++i) {
        const size_t ax = axes[i];
        const long long N = (long long)shape[ax];
        if (mode == R2R_DCT1 && N < 2) raise(IG_EZERO_LEN, "zero-length FFT requested");
        for_lines(ndim, shape, i == 0 ? sin : sout, sout, ax, i == 0 ? (const char *)in : (const char *)out,
                  (char *)out, [&](const Lines &ln) {
                      r2r_axis(a, ln, N, mode, ortho, neg_pre, neg_post, fwd, i == 0 ? fct : 1.0, st);
                  });
    }
}

static void hartley_gen_device(Arith a, size_t ndim, const size_t *shape, const ptrdiff_t *sin, const ptrdiff_t *sout,
                               size_t naxes, const size_t *axes, const void *in, void *out, double fct, cudaStream_t st)
{
    if (naxes == 1) {
        r2r_nd_device(a, ndim, shape, sin, sout, naxes, axes, in, out, fct, st, R2R_HARTLEY, 0, 0, 0, 1);
        return;
    }
    if (ndim > 8) raise(IG_ENDIM, "genuine Hartley over more than 8 dimensions");
    const size_t last = axes[naxes - 1];
    std::vector<size_t> tshp(shape, shape + ndim);
    tshp[last] = shape[last] / 2 + 1;
    const long long ES = 2 * (long long)store_real_bytes(a);
    std::vector<ptrdiff_t> tst(ndim);
    tst[ndim - 1] = (ptrdiff_t)ES;
    for (size_t d = ndim - 1; d-- > 0;) tst[d] = tst[d + 1] * (ptrdiff_t)tshp[d + 1];
    DevBuf tmp(prod(ndim, tshp.data()) * (size_t)ES);
    nd_r2c_device(a, ndim, shape, sin, tst.data(), naxes, axes, 1, in, tmp.p, fct, st);
    HartleyDesc h{};
    h.ndim = (int)ndim;
    h.total = (long long)prod(ndim, tshp.data());
    for (size_t d = 0; d < ndim; ++d) {
        h.tshp[d] = (long long)tshp[d];
        h.shape[d] = (long long)shape[d];
        h.sout[d] = (long long)sout[d];
        h.rev[d] = 0;
    }
    for (size_t i = 0; i < naxes; ++i) h.rev[axes[i]] = 1;
    cudaError_t e = a == A_F32 ? Launch<TagF32>::hartley_fold(tmp.p, out, h, st)
                  : a == A_DF  ? Launch<TagDF>::hartley_fold(tmp.p, out, h, st)
                               : Launch<TagF64>::hartley_fold(tmp.p, out, h, st);
    ck(e, "Hartley fold");
    count_launch();
    ck(cudaStreamSynchronize(st), "Hartley fold");  // tmp is released on return
}

enum { R2R_OP_DCT = 0, R2R_OP_DST, R2R_OP_FFTPACK, R2R_OP_HSEP, R2R_OP_HGEN };
static void r2r_dispatch(int op, Arith a, size_t ndim, const size_t *shape, const ptrdiff_t *sin, const ptrdiff_t *sout,
                         size_t naxes, const size_t *axes, int type, int ortho, int r2h, int fwd, const void *in,
                         void *out, double fct, cudaStream_t st)
{
    switch (op) {
    case R2R_OP_DCT:
    case R2R_OP_DST:
        r2r_nd_device(a, ndim, shape, sin, sout, naxes, axes, in, out, fct, st,
                      (op == R2R_OP_DST ? R2R_DST1 : R2R_DCT1) + type - 1, ortho, 0, 0, 1);
        break;
    case R2R_OP_FFTPACK:
        // ExecR2R (pocketfft_hdronly.h:3252-3270)
        r2r_nd_device(a, ndim, shape, sin, sout, naxes, axes, in, out, fct, st, R2R_COPY, 0, !r2h && fwd,
                      r2h && !fwd, fwd);
        break;
    case R2R_OP_HSEP:
        r2r_nd_device(a, ndim, shape, sin, sout, naxes, axes, in, out, fct, st, R2R_HARTLEY, 0, 0, 0, 1);
        break;
    default: hartley_gen_device(a, ndim, shape, sin, sout, naxes, axes, in, out, fct, st); break;
    }
}

static int r2r_entry(int op, int dtype, size_t ndim, const size_t *shape, const ptrdiff_t *sin, const ptrdiff_t *sout,
                     size_t naxes, const size_t *axes, int type, int ortho, int r2h, int fwd, const void *in,
                     void *out, double fct, bool host, void *stream)
{
    return guarded([&] {
        if ((op == R2R_OP_DCT || op == R2R_OP_DST) && (type < 1 || type > 4))
            raise(IG_EINVAL, op == R2R_OP_DCT ? "invalid DCT type" : "invalid DST type");
        if (ndim >= 1 && shape && prod(ndim, shape) == 0) return;
        nd_checks(dtype, ndim, shape, sin, sout, naxes, axes, in, out, true);
        Arith a = arith_for(dtype);
        if (!host) {
            r2r_dispatch(op, a, ndim, shape, sin, sout, naxes, axes, type, ortho, r2h, fwd, in, out, fct,
                         as_stream(stream));
            return;
        }
        const size_t sr = store_real_bytes(a);
        std::vector<size_t> shp(shape, shape + ndim);
        host_nd_run(ndim, shp, shp, sin, sout, sr, sr, in, out, [&](const void *din, void *dout) {
            r2r_dispatch(op, a, ndim, shape, sin, sout, naxes, axes, type, ortho, r2h, fwd, din, dout, fct, 0);
        });
    });
}

// ---- upfirdn (impulse signal.nim:545-594) -----------------------------------------
// upsample (up - 1 zeros between samples), full convolution with the FIR
// filter h, every down-th sample: by FFT, the rows and the filter zero-padded
// to an even smooth length P >= (n - 1) up + nh, r2c, product, c2r (1/P),
// decimation.  One filter for all rows.
static long long upfirdn_len(long long n, long long nh, int up, int down)
{
    const long long lc = (n - 1) * up + nh;
    return (lc + down - 1) / down;
}

static void upfirdn_device(Arith a, long long B, long long n, const void *x, long long dx, long long nh, const void *h,
                           int up, int down, void *y, long long dy, cudaStream_t st)
{
    if (up < 1 || down < 1) raise(IG_EINVAL, "up and down must be >= 1");
    if (n < 1 || nh < 1) raise(IG_EINVAL, "empty signal or filter");
    if (B == 0) return;
    const long long sr = (long long)store_real_bytes(a), lc = (n - 1) * up + nh;
    const long long P = 2 * good_size_gpu((lc + 1) / 2), PH = P / 2 + 1, ny = upfirdn_len(n, nh, up, down);
    require_aligned(x, (size_t)sr, "signal");
    require_aligned(h, (size_t)sr, "filter");
    require_aligned(y, (size_t)sr, "output");
    DevBuf U((size_t)(B * P * sr)), H((size_t)(P * sr)), FU((size_t)(B * PH * 2 * sr)), FH((size_t)(PH * 2 * sr));
    auto pad = [&](const void *src, long long d, long long len, int u, void *dst, long long nb) {
        cudaError_t e = a == A_F32 ? Launch<TagF32>::upsample_pad(src, d, len, u, dst, P, nb, st)
                      : a == A_DF  ? Launch<TagDF>::upsample_pad(src, d, len, u, dst, P, nb, st)
                                   : Launch<TagF64>::upsample_pad(src, d, len, u, dst, P, nb, st);
        ck(e, "upsample");
        count_launch();
    };
    pad(x, dx, n, up, U.p, B);
    pad(h, nh, nh, 1, H.p, 1);
    exec_op(a, OP_R2C, P, contiguous_lines(U.p, FU.p, B, P, PH, sr, 2 * sr), 1, 1.0, st);
    exec_op(a, OP_R2C, P, contiguous_lines(H.p, FH.p, 1, P, PH, sr, 2 * sr), 1, 1.0, st);
    cudaError_t e = a == A_F32 ? Launch<TagF32>::spec_mul(FU.p, FH.p, FU.p, B, 1, PH, 0, st)
                  : a == A_DF  ? Launch<TagDF>::spec_mul(FU.p, FH.p, FU.p, B, 1, PH, 0, st)
                               : Launch<TagF64>::spec_mul(FU.p, FH.p, FU.p, B, 1, PH, 0, st);
    ck(e, "spectrum product");
    count_launch();
    exec_op(a, OP_C2R, P, contiguous_lines(FU.p, U.p, B, PH, P, 2 * sr, sr), 0, 1.0 / (double)P, st);
    e = a == A_F32 ? Launch<TagF32>::decimate(U.p, P, down, y, dy, ny, B, st)
      : a == A_DF  ? Launch<TagDF>::decimate(U.p, P, down, y, dy, ny, B, st)
                   : Launch<TagF64>::decimate(U.p, P, down, y, dy, ny, B, st);
    ck(e, "decimate");
    count_launch();
    ck(cudaStreamSynchronize(st), "upfirdn");  // temporaries are released on return
}

// ---- adjoints of the real transforms ------------------------------------------
static void launch_half_weight(Arith a, void *x, long long lines, long long n_half, long long nreal, double w,
                               int drop_im, cudaStream_t st)
{
    cudaError_t e = a == A_F32 ? Launch<TagF32>::half_weight(x, lines, n_half, nreal, w, drop_im, st)
                  : a == A_DF  ? Launch<TagDF>::half_weight(x, lines, n_half, nreal, w, drop_im, st)
                               : Launch<TagF64>::half_weight(x, lines, n_half, nreal, w, drop_im, st);
    ck(e, "Hermitian weighting");
    count_launch();
}

// adjoint of c2c(axes, forward, fct): c2c(axes, !forward, fct).  The
// transform is complex-linear with a symmetric matrix F, so its adjoint under
// the real inner product Re <a, b> is conj(F) = the opposite direction.
int ig_c2c_adjoint_device(int dtype, size_t ndim, const size_t *shape, const ptrdiff_t *stride_g,
                          const ptrdiff_t *stride_x, size_t naxes, const size_t *axes, int forward, const void *g,
                          void *x, double fct, void *stream)
{
    return guarded([&] {
        if (ndim >= 1 && shape && prod(ndim, shape) == 0) return;
        nd_checks(dtype, ndim, shape, stride_g, stride_x, naxes, axes, g, x, true);
        nd_c2c_device(arith_for(dtype), ndim, shape, stride_g, stride_x, naxes, axes, forward ? 0 : 1, g, x, fct,
                      as_stream(stream));
    });
}

// adjoint of r2c(axes, forward): halve the inner bins of the last axis (the
// Hermitian weighting), then c2r(axes, !forward), which reads only the real
// parts of the DC / Nyquist bins after its c2c over the other axes.  g has the half-spectrum
// shape; x is real with shape_in.
int ig_r2c_adjoint_device(int dtype, size_t ndim, const size_t *shape_in, const ptrdiff_t *stride_g,
                          const ptrdiff_t *stride_x, size_t naxes, const size_t *axes, int forward, const void *g,
                          void *x, double fct, void *stream)
{
    return guarded([&] {
        if (ndim >= 1 && shape_in && prod(ndim, shape_in) == 0) return;
        nd_checks(dtype, ndim, shape_in, stride_g, stride_x, naxes, axes, g, x, false);
        require_aligned(g, 2 * store_real_bytes(arith_for(dtype)), "gradient");
        require_aligned(x, store_real_bytes(arith_for(dtype)), "output");
        if (naxes == 0) return;
        Arith a = arith_for(dtype);
        cudaStream_t st = as_stream(stream);
        size_t last = axes[naxes - 1];
        std::vector<size_t> sh(shape_in, shape_in + ndim);
        sh[last] = shape_in[last] / 2 + 1;
        const size_t ce = 2 * store_real_bytes(a);
        // contiguous copy with the last axis innermost-of-the-copy: c2c the strided input into it
        std::vector<ptrdiff_t> sc(ndim);
        sc[ndim - 1] = (ptrdiff_t)ce;
        for (size_t d = ndim - 1; d-- > 0;) sc[d] = sc[d + 1] * (ptrdiff_t)sh[d + 1];
        DevBuf tmp(prod(ndim, sh.data()) * ce);
        // identity copy through a zero-axis c2c is not available: copy line by line with the gather map
        for_lines(ndim, sh.data(), stride_g, sc.data(), last, (const char *)g, (char *)tmp.p, [&](const Lines &ln) {
            IODesc io = blank_io();
            io.in = ln.in;
            io.out = ln.out;
            io.is = ln.es_in;
            io.os = ln.es_out;
            io.nlines = ln.nlines;
            for (int i = 0; i < 3; ++i) { io.bn[i] = ln.bn[i]; io.bsi[i] = ln.bsi[i]; io.bso[i] = ln.bso[i]; }
            const long long sr = (long long)store_real_bytes(a);
            io.in_kind = side_aligned(ln.in, ln.es_in, ln.bn, ln.bsi, 2 * sr) ? IN_C : IN_P;
            io.ps_in = sr;
            io.out_kind = OUT_C;
            io.cnt_in = io.cnt_out = (int)sh[last];
            io.nreal = (long long)shape_in[last];
            MapDesc mp{};
            mp.kind = MAP_PLAIN;
            mp.M = (long long)sh[last];
            mp.scr_len = (long long)sh[last];
            // gather writes scratch line l at l * scr_len: the copy is contiguous in line order
            mp.scr = ln.out;
            launch_map(a, true, io, mp, st);
        });
        // the gather above wrote lines in the engine's line order, which for a
        // contiguous destination whose last axis is innermost is the array order
        long long nh = (long long)sh[last];
        // DC / Nyquist imaginary parts are kept: the c2c over the other axes
        // mixes them into real values; c2r drops them after that step
        launch_half_weight(a, tmp.p, (long long)(prod(ndim, sh.data()) / sh[last]), nh, (long long)shape_in[last], 0.5,
                           0, st);
        nd_c2r_device(a, ndim, shape_in, sc.data(), stride_x, naxes, axes, forward ? 0 : 1, tmp.p, x, fct, st);
        ck(cudaStreamSynchronize(st), "r2c adjoint");
    });
}

// adjoint of c2r(axes, forward): r2c(axes, !forward), then double the inner
// bins of the last axis.  y is real with shape_out; g has the half-spectrum shape.
int ig_c2r_adjoint_device(int dtype, size_t ndim, const size_t *shape_out, const ptrdiff_t *stride_y,
                          const ptrdiff_t *stride_g, size_t naxes, const size_t *axes, int forward, const void *y,
                          void *g, double fct, void *stream)
{
    return guarded([&] {
        if (ndim >= 1 && shape_out && prod(ndim, shape_out) == 0) return;
        nd_checks(dtype, ndim, shape_out, stride_y, stride_g, naxes, axes, y, g, false);
        require_aligned(y, store_real_bytes(arith_for(dtype)), "gradient");
        require_aligned(g, 2 * store_real_bytes(arith_for(dtype)), "output");
        if (naxes == 0) return;
        Arith a = arith_for(dtype);
        cudaStream_t st = as_stream(stream);
        size_t last = axes[naxes - 1];
        nd_r2c_device(a, ndim, shape_out, stride_y, stride_g, naxes, axes, forward ? 0 : 1, y, g, fct, st);
        std::vector<size_t> sh(shape_out, shape_out + ndim);
        sh[last] = shape_out[last] / 2 + 1;
        // weighting along the last axis of a possibly strided array: one launch per line set
        const long long es = 2 * (long long)store_real_bytes(a);
        bool contiguous_last = stride_g[last] == es;
        if (!contiguous_last) raise(IG_EINVAL, "c2r adjoint needs a unit-stride last axis in the spectrum");
        for_lines(ndim, sh.data(), stride_g, stride_g, last, (const char *)g, (char *)g, [&](const Lines &ln) {
            // lines here are rows of sh[last] contiguous bins; weight each row set
            for (long long i1 = 0; i1 < ln.bn[1] * ln.bn[2]; ++i1) {
                long long i1a = i1 % ln.bn[1], i2 = i1 / ln.bn[1];
                char *base = ln.out + i1a * ln.bso[1] + i2 * ln.bso[2];
                if (ln.bso[0] == (long long)sh[last] * es || ln.bn[0] == 1)
                    launch_half_weight(a, base, ln.bn[0], (long long)sh[last], (long long)shape_out[last], 2.0, 0, st);
                else
                    for (long long i0 = 0; i0 < ln.bn[0]; ++i0)
                        launch_half_weight(a, base + i0 * ln.bso[0], 1, (long long)sh[last], (long long)shape_out[last],
                                           2.0, 0, st);
            }
        });
    });
}

// ---- differentiable FFT convolution --------------------------------------------
struct ig_fftconv_i {
    Arith a;
    int dtype;
    long long B, H, W, NF, K, P0, P1;
    int recompute;
    std::unique_ptr<DevBuf> xpad, kpad, FX, FK, FG, Z, zpad;
    bool have_spectra = false;
};

static void conv_r2c2d(Arith a, long long nb, long long P0, long long P1, const void *in, void *out, cudaStream_t st)
{
    const size_t sr = store_real_bytes(a), ce = 2 * sr;
    size_t shape[3] = {(size_t)nb, (size_t)P0, (size_t)P1};
    ptrdiff_t si[3] = {(ptrdiff_t)(P0 * P1 * sr), (ptrdiff_t)(P1 * sr), (ptrdiff_t)sr};
    ptrdiff_t so[3] = {(ptrdiff_t)(P0 * (P1 / 2 + 1) * ce), (ptrdiff_t)((P1 / 2 + 1) * ce), (ptrdiff_t)ce};
    size_t axes[2] = {1, 2};
    nd_r2c_device(a, 3, shape, si, so, 2, axes, 1, in, out, 1.0, st);
}
static void conv_c2r2d(Arith a, long long nb, long long P0, long long P1, const void *in, void *out, cudaStream_t st)
{
    const size_t sr = store_real_bytes(a), ce = 2 * sr;
    size_t shape[3] = {(size_t)nb, (size_t)P0, (size_t)P1};
    ptrdiff_t si[3] = {(ptrdiff_t)(P0 * (P1 / 2 + 1) * ce), (ptrdiff_t)((P1 / 2 + 1) * ce), (ptrdiff_t)ce};
    ptrdiff_t so[3] = {(ptrdiff_t)(P0 * P1 * sr), (ptrdiff_t)(P1 * sr), (ptrdiff_t)sr};
    size_t axes[2] = {1, 2};
    nd_c2r_device(a, 3, shape, si, so, 2, axes, 0, in, out, 1.0 / ((double)P0 * (double)P1), st);
}
static void conv_pad(Arith a, const void *in, void *out, long long B, long long H, long long W, long long P0,
                     long long P1, long long r0, long long c0, cudaStream_t st)
{
    cudaError_t e = a == A_F32 ? Launch<TagF32>::pad2d(in, out, B, H, W, P0, P1, r0, c0, st)
                  : a == A_DF  ? Launch<TagDF>::pad2d(in, out, B, H, W, P0, P1, r0, c0, st)
                               : Launch<TagF64>::pad2d(in, out, B, H, W, P0, P1, r0, c0, st);
    ck(e, "pad");
    count_launch();
}
static void conv_crop(Arith a, const void *in, void *out, long long B, long long H, long long W, long long P0,
                      long long P1, long long r0, long long c0, cudaStream_t st)
{
    cudaError_t e = a == A_F32 ? Launch<TagF32>::crop2d(in, out, B, H, W, P0, P1, r0, c0, st)
                  : a == A_DF  ? Launch<TagDF>::crop2d(in, out, B, H, W, P0, P1, r0, c0, st)
                               : Launch<TagF64>::crop2d(in, out, B, H, W, P0, P1, r0, c0, st);
    ck(e, "crop");
    count_launch();
}
static void conv_mul(Arith a, const void *x, const void *f, void *out, long long B, long long nf, long long n, int mode,
                     cudaStream_t st)
{
    cudaError_t e = a == A_F32 ? Launch<TagF32>::spec_mul(x, f, out, B, nf, n, mode, st)
                  : a == A_DF  ? Launch<TagDF>::spec_mul(x, f, out, B, nf, n, mode, st)
                               : Launch<TagF64>::spec_mul(x, f, out, B, nf, n, mode, st);
    ck(e, "spectrum product");
    count_launch();
}

static void conv_spectra(ig_fftconv_i &c, const void *x, const void *k, cudaStream_t st)
{
    conv_pad(c.a, x, c.xpad->p, c.B, c.H, c.W, c.P0, c.P1, 0, 0, st);
    conv_r2c2d(c.a, c.B, c.P0, c.P1, c.xpad->p, c.FX->p, st);
    conv_pad(c.a, k, c.kpad->p, c.NF, c.K, c.K, c.P0, c.P1, 0, 0, st);
    conv_r2c2d(c.a, c.NF, c.P0, c.P1, c.kpad->p, c.FK->p, st);
}

ig_fftconv ig_fftconv_create(int dtype, size_t batch, size_t height, size_t width, size_t nfilters, size_t ksize,
                             size_t pad_rows, size_t pad_cols, int recompute)
{
    ig_fftconv c = nullptr;
    guarded([&] {
        if (dtype != IG_F64 && dtype != IG_F32) raise(IG_EINVAL, "bad dtype");
        if (!batch || !height || !width || !ksize) raise(IG_EZERO_LEN, "zero-length FFT requested");
        if (ksize % 2 == 0) raise(IG_EINVAL, "filter size must be odd ('same' convolution)");
        if (nfilters != 1 && nfilters != batch) raise(IG_EINVAL, "nfilters must be 1 or the batch size");
        auto o = std::make_unique<ig_fftconv_i>();
        o->a = arith_for(dtype);
        o->dtype = dtype;
        o->B = (long long)batch;
        o->H = (long long)height;
        o->W = (long long)width;
        o->NF = (long long)nfilters;
        o->K = (long long)ksize;
        long long need0 = o->H + o->K - 1, need1 = o->W + o->K - 1;
        o->P0 = pad_rows ? (long long)pad_rows : good_size_gpu(need0);
        o->P1 = pad_cols ? (long long)pad_cols : good_size_gpu(need1);
        if (o->P0 < need0 || o->P1 < need1) raise(IG_EINVAL, "padded size smaller than height/width + ksize - 1");
        o->recompute = recompute;
        const size_t sr = store_real_bytes(o->a), ce = 2 * sr;
        const size_t half = (size_t)(o->P0 * (o->P1 / 2 + 1));
        o->xpad.reset(new DevBuf(o->B * o->P0 * o->P1 * sr));
        o->kpad.reset(new DevBuf(o->NF * o->P0 * o->P1 * sr));
        o->FX.reset(new DevBuf(o->B * half * ce));
        o->FK.reset(new DevBuf(o->NF * half * ce));
        o->FG.reset(new DevBuf(o->B * half * ce));
        o->Z.reset(new DevBuf(o->B * half * ce));
        o->zpad.reset(new DevBuf(o->B * o->P0 * o->P1 * sr));
        c = o.release();
    });
    return c;
}

void ig_fftconv_destroy(ig_fftconv c) { delete c; }

int ig_fftconv_padded_size(ig_fftconv c, size_t *rows, size_t *cols)
{
    if (!c) return IG_EINVAL;
    if (rows) *rows = (size_t)c->P0;
    if (cols) *cols = (size_t)c->P1;
    return IG_OK;
}

// y = crop_c(c2r(r2c(pad x) * r2c(pad k))) / (P0 P1), c = (K - 1) / 2  ('same' convolution)
int ig_fftconv_forward(ig_fftconv c, const void *x, const void *k, void *y, void *stream)
{
    return guarded([&] {
        if (!c || !x || !k || !y) raise(IG_EINVAL, "null argument");
        for (const void *p : {x, k, (const void *)y}) require_aligned(p, store_real_bytes(c->a), "array");
        cudaStream_t st = as_stream(stream);
        conv_spectra(*c, x, k, st);
        const long long n = c->P0 * (c->P1 / 2 + 1);
        conv_mul(c->a, c->FX->p, c->FK->p, c->Z->p, c->B, c->NF, n, 0, st);
        conv_c2r2d(c->a, c->B, c->P0, c->P1, c->Z->p, c->zpad->p, st);
        const long long off = (c->K - 1) / 2;
        conv_crop(c->a, c->zpad->p, y, c->B, c->H, c->W, c->P0, c->P1, off, off, st);
        c->have_spectra = !c->recompute;
    });
}

// gx = crop_0(c2r(r2c(pad_c gy) * conj(r2c(pad k)))) / (P0 P1)
// gk = crop_0(sum_b c2r(r2c(pad_c gy_b) * conj(r2c(pad x_b)))) / (P0 P1)  (per image when nfilters == batch)
// The spectra of x and k are recomputed unless the object keeps them.
int ig_fftconv_backward(ig_fftconv c, const void *x, const void *k, const void *gy, void *gx, void *gk, void *stream)
{
    return guarded([&] {
        if (!c || !x || !k || !gy) raise(IG_EINVAL, "null argument");
        for (const void *p : {x, k, gy, (const void *)gx, (const void *)gk}) require_aligned(p, store_real_bytes(c->a), "array");
        cudaStream_t st = as_stream(stream);
        if (!c->have_spectra) conv_spectra(*c, x, k, st);
        const long long off = (c->K - 1) / 2;
        const long long n = c->P0 * (c->P1 / 2 + 1);
        conv_pad(c->a, gy, c->zpad->p, c->B, c->H, c->W, c->P0, c->P1, off, off, st);
        conv_r2c2d(c->a, c->B, c->P0, c->P1, c->zpad->p, c->FG->p, st);
        if (gx) {
            conv_mul(c->a, c->FG->p, c->FK->p, c->Z->p, c->B, c->NF, n, 1, st);
            conv_c2r2d(c->a, c->B, c->P0, c->P1, c->Z->p, c->zpad->p, st);
            conv_crop(c->a, c->zpad->p, gx, c->B, c->H, c->W, c->P0, c->P1, 0, 0, st);
        }
        if (gk) {
            if (c->NF == 1) {
                conv_mul(c->a, c->FG->p, c->FX->p, c->Z->p, c->B, c->B, n, 2, st);
                conv_c2r2d(c->a, 1, c->P0, c->P1, c->Z->p, c->zpad->p, st);
                conv_crop(c->a, c->zpad->p, gk, 1, c->K, c->K, c->P0, c->P1, 0, 0, st);
            } else {
                conv_mul(c->a, c->FG->p, c->FX->p, c->Z->p, c->B, c->B, n, 1, st);
                conv_c2r2d(c->a, c->B, c->P0, c->P1, c->Z->p, c->zpad->p, st);
                conv_crop(c->a, c->zpad->p, gk, c->B, c->K, c->K, c->P0, c->P1, 0, 0, st);
            }
        }
        if (c->recompute) c->have_spectra = false;
    });
}

// ---- batched transforms of uneven lengths ---------------------------------------
// Transforms whose length fits one CTA are grouped by length (lines at
// arbitrary offsets through per-line offset tables); four-step transforms
// contribute a column-pass group and a row-pass group; all run through the
// persistent work-list kernel in two launches (phase 0: single-CTA groups and
// column passes; phase 1: row passes).  Lengths needing Bluestein over a
// multi-pass core run on the general path.  The whole sequence can be
// captured once into a CUDA graph.
// one persistent work-list launch: the groups of a phase that run the same
// shared-memory kernel variant (elements per thread, buffering, radix class,
// layout class)
struct MultiPart {
    int E = 16, db = 0, rs = RS_FULL, lay = LAY_GEN;
    std::vector<WorkGroup> groups;
    std::vector<long long> prefix;
    std::unique_ptr<DevBuf> d_groups, d_prefix;
    unsigned long long total = 0;
    size_t smem = 0;
    int block = 0, grid = 0, slot = 0;  // slot: its counter
};
struct MultiPhase {
    std::vector<WorkGroup> groups;  // before partitioning
    std::vector<MultiPart> parts;
};

struct ig_multi_plan_i {
    Arith a;
    int dtype, fwd;
    double fct;
    std::vector<long long> len, off;
    std::vector<std::shared_ptr<Core>> cores;
    MultiPhase ph[2];
    std::vector<std::unique_ptr<DevBuf>> tables;
    std::vector<long long> general;
    // general transforms run on up to 16 side streams (fork / join around the work
    // list): their launches are small, so several run at once
    std::vector<int> gstream;  // side stream of general[k]
    std::vector<cudaStream_t> side;
    std::vector<cudaEvent_t> ev;  // ev[0] fork, ev[1 + i] join of side[i]
    std::unique_ptr<DevBuf> scratch, counter;
    int nslots = 0;  // work-list counters, one per partition
    size_t n_wl = 0, n_4s = 0;
    cudaGraphExec_t gexec = nullptr;
    const void *g_in = nullptr;
    void *g_out = nullptr;
    cudaStream_t g_st = nullptr;
    ~ig_multi_plan_i()
    {
        if (gexec) cudaGraphExecDestroy(gexec);
        for (cudaStream_t s : side) cudaStreamDestroy(s);
        for (cudaEvent_t e : ev) cudaEventDestroy(e);
    }
};

static const int kMultiSide = 16;

// Partition a phase's groups by kernel variant.  Each group keeps its core's
// tuned configuration (elements per thread, buffering) and gets the lines per
// CTA a stand-alone launch would; a partition's launch takes the largest
// block and shared-memory size of its groups and as many CTAs as fit the GPU.
static void finish_phase(Arith a, MultiPhase &ph, int &nslots)
{
    std::map<std::tuple<int, int, int, int>, size_t> index;
    int sms = 0;
    ck(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device_id()), "SM count");
    for (WorkGroup g : ph.groups) {
        long long line_bytes = 0;
        const long long lpc = smem_lpc(a, g.P, g.io, line_bytes);
        const long long tpl = (g.P.L + g.P.E - 1) / g.P.E;
        g.io.lpc = (int)lpc;
        g.io.tpl = (int)tpl;
        set_line_divs(g.io);
        g.io.lay = choose_layout(a, g.io);
        int lay = g.io.lay == LAY_C2C || g.io.lay == LAY_TW ? g.io.lay : LAY_GEN;
        if (a == A_F64) lay = LAY_GEN;
        // the full radix class for every partition: work-list instantiations of
        // the narrower classes gave wrong results on twiddled radix-8 (FP32) and
        // radix-7 (double-float) stages, although the same device code is exact
        // in the stand-alone kernel; the cause is not found
        const int rs = RS_FULL;
        // groups of 512-thread blocks (lines of 4096 points at 8 elements a
        // thread) get their own partition: a partition launches with its
        // largest block, and one 512-thread block per SM left the 256-thread
        // groups at a third of the warps they could have
        const int big = lpc * tpl > 256 ? 1 : 0;
        const auto key = std::make_tuple(g.P.E, g.P.db, rs, lay * 2 + big);
        auto it = index.find(key);
        if (it == index.end()) {
            it = index.emplace(key, ph.parts.size()).first;
            ph.parts.emplace_back();
            MultiPart &np = ph.parts.back();
            np.E = g.P.E;
            np.db = g.P.db;
            np.rs = rs;
            np.lay = lay;
            np.slot = nslots++;
        }
        MultiPart &pt = ph.parts[it->second];
        pt.smem = std::max(pt.smem, (size_t)(lpc * line_bytes));
        pt.block = std::max(pt.block, (int)(lpc * tpl));
        pt.groups.push_back(g);
    }
    for (MultiPart &pt : ph.parts) {
        pt.prefix.clear();
        unsigned long long tot = 0;
        for (auto &g : pt.groups) {
            pt.prefix.push_back((long long)tot);
            tot += (unsigned long long)((g.io.nlines + g.io.lpc - 1) / g.io.lpc);
        }
        pt.total = tot;
        pt.d_groups.reset(new DevBuf(pt.groups.size() * sizeof(WorkGroup)));
        pt.d_prefix.reset(new DevBuf(pt.prefix.size() * sizeof(long long)));
        ck(cudaMemcpy(pt.d_groups->p, pt.groups.data(), pt.groups.size() * sizeof(WorkGroup), cudaMemcpyHostToDevice),
           "work list upload");
        ck(cudaMemcpy(pt.d_prefix->p, pt.prefix.data(), pt.prefix.size() * sizeof(long long), cudaMemcpyHostToDevice),
           "work list upload");
        int per_sm = 0;
        cudaError_t e = a == A_F32 ? Launch<TagF32>::worklist_occupancy(pt.E, pt.db, pt.rs, pt.lay, pt.block, pt.smem, &per_sm)
                      : a == A_DF  ? Launch<TagDF>::worklist_occupancy(pt.E, pt.db, pt.rs, pt.lay, pt.block, pt.smem, &per_sm)
                                   : Launch<TagF64>::worklist_occupancy(pt.E, pt.db, pt.rs, pt.lay, pt.block, pt.smem, &per_sm);
        ck(e, "work list occupancy");
        pt.grid = (int)std::min<unsigned long long>((unsigned long long)sms * (unsigned long long)std::max(1, per_sm),
                                                    std::max<unsigned long long>(1, pt.total));
    }
    ph.groups.clear();
}

// parts: 1 work-list phase 0 (single-CTA groups, four-step column passes),
// 2 phase 1 (four-step row passes), 4 general transforms
static void multi_launch(ig_multi_plan_i &m, const void *in, void *out, cudaStream_t st, int parts = 7)
{
    const long long es = 2 * (long long)store_real_bytes(m.a);
    const bool gen = (parts & 4) && !m.general.empty();
    if (gen) {
        ck(cudaEventRecord(m.ev[0], st), "fork");
        for (cudaStream_t s : m.side) ck(cudaStreamWaitEvent(s, m.ev[0], 0), "fork");
        for (size_t k = 0; k < m.general.size(); ++k) {
            const long long i = m.general[k];
            Lines ln = contiguous_lines((const char *)in + m.off[i] * es, (char *)out + m.off[i] * es, 1, m.len[i],
                                        m.len[i], es, es);
            exec_op(m.a, OP_C2C, m.len[i], ln, m.fwd, m.fct, m.side[m.gstream[k]]);
        }
    }
    if (m.nslots) ck(cudaMemsetAsync(m.counter->p, 0, m.nslots * sizeof(unsigned long long), st), "work list counter");
    for (int k = 0; k < 2; ++k) {
        if (!(parts & (1 << k))) continue;
        for (MultiPart &pt : m.ph[k].parts) {
            if (!pt.total) continue;
            unsigned long long *ctr = (unsigned long long *)m.counter->p + pt.slot;
            void *scr = m.scratch ? m.scratch->p : nullptr;
            const WorkGroup *gd = (const WorkGroup *)pt.d_groups->p;
            const long long *pd = (const long long *)pt.d_prefix->p;
            const int ng = (int)pt.groups.size();
            cudaError_t e =
                m.a == A_F32 ? Launch<TagF32>::fft_worklist(pt.E, pt.db, pt.rs, pt.lay, gd, pd, ng, pt.total, ctr, in, out,
                                                            scr, pt.grid, pt.block, pt.smem, st)
              : m.a == A_DF  ? Launch<TagDF>::fft_worklist(pt.E, pt.db, pt.rs, pt.lay, gd, pd, ng, pt.total, ctr, in, out,
                                                           scr, pt.grid, pt.block, pt.smem, st)
                             : Launch<TagF64>::fft_worklist(pt.E, pt.db, pt.rs, pt.lay, gd, pd, ng, pt.total, ctr, in,
                                                            out, scr, pt.grid, pt.block, pt.smem, st);
            ck(e, "work list launch");
            count_launch();
        }
    }
    if (gen) {
        for (size_t i = 0; i < m.side.size(); ++i) {
            ck(cudaEventRecord(m.ev[1 + i], m.side[i]), "join");
            ck(cudaStreamWaitEvent(st, m.ev[1 + i], 0), "join");
        }
    }
}

ig_multi_plan ig_make_multi_plan(int dtype, size_t count, const size_t *lengths, const size_t *offsets, int forward,
                                 double fct)
{
    ig_multi_plan plan = nullptr;
    guarded([&] {
        if (dtype != IG_F64 && dtype != IG_F32) raise(IG_EINVAL, "bad dtype");
        if (!count || !lengths) raise(IG_EINVAL, "empty transform list");
        auto m = std::make_unique<ig_multi_plan_i>();
        m->a = arith_for(dtype);
        m->dtype = dtype;
        m->fwd = forward;
        m->fct = fct;
        const long long es = 2 * (long long)store_real_bytes(m->a);
        long long pos = 0;
        for (size_t i = 0; i < count; ++i) {
            if (!lengths[i]) raise(IG_EZERO_LEN, "zero-length FFT requested");
            m->len.push_back((long long)lengths[i]);
            m->off.push_back(offsets ? (long long)offsets[i] : pos);
            pos += (long long)lengths[i];
        }
        // group single-CTA lengths; collect four-step and general transforms
        std::map<long long, std::vector<long long>> by_len;
        std::vector<long long> four;
        for (size_t i = 0; i < count; ++i) {
            auto c = get_core(m->a, m->len[i], false);
            m->cores.push_back(c);
            // (wide cores, more than 512 threads a line, take the general path:
            // the work-list kernel is bounded at 512 threads)
            if (c->kind == 0 && (c->d.L + c->d.E - 1) / c->d.E <= 512) by_len[m->len[i]].push_back((long long)i);
            else if (c->kind == 1) four.push_back((long long)i);
            else m->general.push_back((long long)i);
        }
        for (auto &kv : by_len) {
            const long long L = kv.first;
            const auto &ids = kv.second;
            std::vector<long long> lo(ids.size());
            for (size_t j = 0; j < ids.size(); ++j) lo[j] = m->off[ids[j]] * es;
            m->tables.emplace_back(new DevBuf(lo.size() * sizeof(long long)));
            ck(cudaMemcpy(m->tables.back()->p, lo.data(), lo.size() * sizeof(long long), cudaMemcpyHostToDevice),
               "offset table");
            WorkGroup g;
            memset(&g, 0, sizeof g);
            g.P = m->cores[ids[0]]->d;
            g.io = blank_io();
            g.io.loff_in = g.io.loff_out = (const long long *)m->tables.back()->p;
            g.io.nlines = (long long)ids.size();
            g.io.bn[0] = g.io.nlines;
            g.io.is = g.io.os = es;
            g.io.in_kind = IN_C;
            g.io.out_kind = OUT_C;
            g.io.cnt_in = g.io.cnt_out = (int)L;
            g.io.nreal = L;
            g.io.fwd = forward;
            g.io.fct = fct;
            g.in_base = 0;
            g.out_base = 1;
            m->ph[0].groups.push_back(g);
            m->n_wl += ids.size();
        }
        long long soff = 0;
        for (long long i : four) soff += m->len[i];
        if (soff) m->scratch.reset(new DevBuf((size_t)(soff * es)));
        soff = 0;
        for (long long i : four) {
            const Core &c = *m->cores[i];
            IODesc io = blank_io();
            io.in = (const char *)(m->off[i] * es);  // offsets from the bases
            io.out = (char *)(m->off[i] * es);
            io.is = io.os = es;
            io.nlines = 1;
            io.bn[0] = 1;
            io.bsi[0] = io.bso[0] = c.M * es;
            io.in_kind = IN_C;
            io.out_kind = OUT_C;
            io.cnt_in = io.cnt_out = (int)c.M;
            io.nreal = c.M;
            io.fwd = forward;
            io.fct = fct;
            IODesc p1, p2;
            fourstep_passes(c, io, (char *)(soff * es), p1, p2);
            WorkGroup g1, g2;
            memset(&g1, 0, sizeof g1);
            memset(&g2, 0, sizeof g2);
            g1.P = c.c1->d;
            g1.io = p1;
            g1.in_base = 0;
            g1.out_base = 2;
            g2.P = c.c2->d;
            g2.io = p2;
            g2.in_base = 2;
            g2.out_base = 1;
            m->ph[0].groups.push_back(g1);
            m->ph[1].groups.push_back(g2);
            soff += c.M;
            ++m->n_4s;
        }
        int optin0 = max_smem() + 1024;
        static std::once_flag once0[3];
        std::call_once(once0[m->a], [&] {
            cudaError_t e = m->a == A_F32 ? Launch<TagF32>::set_max_smem(optin0)
                          : m->a == A_DF  ? Launch<TagDF>::set_max_smem(optin0)
                                          : Launch<TagF64>::set_max_smem(optin0);
            ck(e, "cudaFuncSetAttribute");
        });
        finish_phase(m->a, m->ph[0], m->nslots);
        finish_phase(m->a, m->ph[1], m->nslots);
        if (!m->general.empty()) {
            // longest first onto the least loaded side stream (cost ~ N log N)
            const int ns = (int)std::min<size_t>(kMultiSide, m->general.size());
            for (int i = 0; i < ns; ++i) {
                cudaStream_t sst;
                ck(cudaStreamCreateWithFlags(&sst, cudaStreamNonBlocking), "side stream");
                m->side.push_back(sst);
            }
            for (int i = 0; i <= ns; ++i) {
                cudaEvent_t e;
                ck(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "side event");
                m->ev.push_back(e);
            }
            std::vector<size_t> order(m->general.size());
            for (size_t k = 0; k < order.size(); ++k) order[k] = k;
            std::sort(order.begin(), order.end(), [&](size_t x, size_t y) {
                return m->len[m->general[x]] > m->len[m->general[y]];
            });
            std::vector<double> load(ns, 0.0);
            m->gstream.assign(m->general.size(), 0);
            for (size_t k : order) {
                const int best = (int)(std::min_element(load.begin(), load.end()) - load.begin());
                const double n = (double)m->len[m->general[k]];
                load[best] += n * std::log2(n + 1.0);
                m->gstream[k] = best;
            }
        }
        m->counter.reset(new DevBuf(std::max(1, m->nslots) * sizeof(unsigned long long)));
        plan = m.release();
    });
    return plan;
}

void ig_destroy_multi_plan(ig_multi_plan plan) { delete plan; }

int ig_multi_info(ig_multi_plan plan, size_t *n_worklist, size_t *n_fourstep, size_t *n_general)
{
    if (!plan) return IG_EINVAL;
    if (n_worklist) *n_worklist = plan->n_wl;
    if (n_fourstep) *n_fourstep = plan->n_4s;
    if (n_general) *n_general = plan->general.size();
    return IG_OK;
}

int ig_multi_exec_device(ig_multi_plan plan, const void *in, void *out, void *stream)
{
    return guarded([&] {
        if (!plan || !in || !out) raise(IG_EINVAL, "null argument");
        require_aligned(in, 2 * store_real_bytes(plan->a), "input");
        require_aligned(out, 2 * store_real_bytes(plan->a), "output");
        multi_launch(*plan, in, out, as_stream(stream));
    });
}

// Capture the work-list sequence for (in, out) into a CUDA graph once, then
// replay it.  The first call runs the sequence eagerly (sizing every
// workspace) before capturing; `stream` must not be the legacy default stream.
int ig_multi_exec_graph(ig_multi_plan plan, const void *in, void *out, void *stream)
{
    return guarded([&] {
        if (!plan || !in || !out) raise(IG_EINVAL, "null argument");
        require_aligned(in, 2 * store_real_bytes(plan->a), "input");
        require_aligned(out, 2 * store_real_bytes(plan->a), "output");
        cudaStream_t st = as_stream(stream);
        if (!st) raise(IG_EINVAL, "graph capture needs a created stream, not the default stream");
        if (!plan->gexec || plan->g_in != in || plan->g_out != out || plan->g_st != st) {
            if (plan->gexec) {
                cudaGraphExecDestroy(plan->gexec);
                plan->gexec = nullptr;
            }
            multi_launch(*plan, in, out, st);
            ck(cudaStreamSynchronize(st), "eager run before capture");
            cudaGraph_t graph = nullptr;
            ck(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal), "begin capture");
            try {
                multi_launch(*plan, in, out, st);
            } catch (...) {
                cudaStreamEndCapture(st, &graph);
                if (graph) cudaGraphDestroy(graph);
                throw;
            }
            ck(cudaStreamEndCapture(st, &graph), "end capture");
            cudaError_t e = cudaGraphInstantiate(&plan->gexec, graph, 0);
            cudaGraphDestroy(graph);
            ck(e, "graph instantiate");
            plan->g_in = in;
            plan->g_out = out;
            plan->g_st = st;
        }
        ck(cudaGraphLaunch(plan->gexec, st), "graph launch");
        count_launch();
    });
}

// One part of the sequence (bit mask: 1 work-list phase 0, 2 phase 1, 4 the
// general transforms), for timing the parts apart.
int ig_multi_exec_part(ig_multi_plan plan, const void *in, void *out, int parts, void *stream)
{
    return guarded([&] {
        if (!plan || !in || !out) raise(IG_EINVAL, "null argument");
        if (parts < 0 || parts > 7) raise(IG_EINVAL, "parts must be a mask of 1, 2 and 4");
        require_aligned(in, 2 * store_real_bytes(plan->a), "input");
        require_aligned(out, 2 * store_real_bytes(plan->a), "output");
        multi_launch(*plan, in, out, as_stream(stream), parts);
    });
}

// Reference launch pattern: one call of the single-transform path per transform.
int ig_multi_exec_loop_device(ig_multi_plan plan, const void *in, void *out, void *stream)
{
    return guarded([&] {
        if (!plan || !in || !out) raise(IG_EINVAL, "null argument");
        require_aligned(in, 2 * store_real_bytes(plan->a), "input");
        require_aligned(out, 2 * store_real_bytes(plan->a), "output");
        const long long es = 2 * (long long)store_real_bytes(plan->a);
        for (size_t i = 0; i < plan->len.size(); ++i) {
            Lines ln = contiguous_lines((const char *)in + plan->off[i] * es, (char *)out + plan->off[i] * es, 1,
                                        plan->len[i], plan->len[i], es, es);
            exec_op(plan->a, OP_C2C, plan->len[i], ln, plan->fwd, plan->fct, as_stream(stream));
        }
    });
}

// ---- autotuner -------------------------------------------------------------------
static std::string gpu_name()
{
    cudaDeviceProp p;
    if (cudaGetDeviceProperties(&p, device_id()) != cudaSuccess) return "unknown";
    return p.name;
}

static std::string tune_cache_path(const char *path)
{
    if (path && *path) return path;
    const char *e = getenv("IG_AUTOTUNE_CACHE");
    return e ? std::string(e) : std::string();
}

// one entry per line: gpu<TAB>arith<TAB>length<TAB>order<TAB>E<TAB>lpc<TAB>no9<TAB>N1<TAB>ms
int ig_autotune_save(const char *path)
{
    return guarded([&] {
        std::string f = tune_cache_path(path);
        if (f.empty()) raise(IG_EINVAL, "no autotune cache path (argument or IG_AUTOTUNE_CACHE)");
        FILE *fp = fopen(f.c_str(), "w");
        if (!fp) raise(IG_EINVAL, "cannot write " + f);
        std::string g = gpu_name();
        std::lock_guard<std::mutex> lk(g_tune_mu);
        for (auto &kv : g_tune)
            fprintf(fp, "%s\t%d\t%lld\t%d\t%d\t%d\t%d\t%lld\t%.6f\n", g.c_str(), kv.first.first, kv.first.second,
                    kv.second.order, kv.second.E, kv.second.lpc, kv.second.no9, kv.second.N1, kv.second.ms);
        fclose(fp);
    });
}

int ig_autotune_load(const char *path)
{
    return guarded([&] {
        std::string f = tune_cache_path(path);
        if (f.empty()) raise(IG_EINVAL, "no autotune cache path (argument or IG_AUTOTUNE_CACHE)");
        FILE *fp = fopen(f.c_str(), "r");
        if (!fp) raise(IG_EINVAL, "cannot read " + f);
        std::string g = gpu_name();
        char name[256];
        int a, order, E, lpc, no9;
        long long len, N1;
        double ms;
        std::lock_guard<std::mutex> lk(g_tune_mu);
        while (fscanf(fp, " %255[^\t]\t%d\t%lld\t%d\t%d\t%d\t%d\t%lld\t%lf", name, &a, &len, &order, &E, &lpc, &no9,
                      &N1, &ms) == 9) {
            if (g != name) continue;
            TuneCfg c;
            c.order = order;
            c.E = E;
            c.lpc = lpc;
            c.no9 = no9;
            c.N1 = N1;
            c.ms = ms;
            g_tune[std::make_pair(a, len)] = c;
        }
        fclose(fp);
        std::lock_guard<std::mutex> lk2(g_mu);
        g_cores.clear();
    });
}

// Tune the transform of `length` (kind 0: complex, 1: real halfcomplex
// forward) for dtype: every candidate (radix order x elements per thread x
// lines per CTA, or the four-step split) is built, timed with CUDA events on
// a synthetic batch of ~64 MiB, and the fastest is kept for later plans.
int ig_autotune(int dtype, size_t length, int kind, double *best_ms)
{
    return guarded([&] {
        if (dtype != IG_F64 && dtype != IG_F32) raise(IG_EINVAL, "bad dtype");
        if (!length) raise(IG_EZERO_LEN, "zero-length FFT requested");
        const Arith a = arith_for(dtype);
        const long long N = (long long)length;
        const bool even = kind == 1 && N % 2 == 0 && N > 1;
        const long long M = even ? N / 2 : N;
        const Op op = kind == 1 ? OP_R2HC : OP_C2C;
        const long long es = (kind == 1 ? 1 : 2) * (long long)store_real_bytes(a);
        const long long batch = std::max<long long>(2, (64ll << 20) / (N * es));
        DevBuf in((size_t)(batch * N * es)), out((size_t)(batch * N * es));
        ck(cudaMemset(in.p, 0x3f, in.bytes), "tuning data");
        Lines ln = contiguous_lines(in.p, out.p, batch, N, N, es, es);
        // candidates
        auto base = make_core(a, M, even);
        std::vector<TuneCfg> cands;
        if (base->kind == 2 || base->kind == 3) {
            // Bluestein or Rader over a multi-pass core: tune the core's complex length
            double sub_ms = 0.0;
            int rc = ig_autotune(dtype, (size_t)base->n2, 0, &sub_ms);
            if (rc != IG_OK) raise(rc, ig_last_error_string());
        } else if (base->kind == 1) {
            for (long long d = 2; d * d <= M; ++d)
                if (M % d == 0 && fits_smem(a, d, d) && fits_smem(a, M / d, M / d)) {
                    std::vector<int> r1, r2;
                    if (gpu_factor(d, r1) && gpu_factor(M / d, r2)) {
                        for (long long n1 : {d, M / d}) {
                            TuneCfg c;
                            c.N1 = n1;
                            cands.push_back(c);
                            if (d * d == M) break;
                        }
                    }
                }
        } else {
            const long long L = base->d.L;
            // long single-CTA cores also try four-step splits (fewer lines per SM
            // in shared memory against a second pass)
            if (!base->d.blue && L > 2048) {
                for (long long d = 2; d * d <= M; ++d)
                    if (M % d == 0 && fits_smem(a, d, d) && fits_smem(a, M / d, M / d)) {
                        std::vector<int> r1, r2;
                        if (gpu_factor(d, r1) && gpu_factor(M / d, r2))
                            for (long long n1 : {d, M / d}) {
                                TuneCfg c;
                                c.N1 = n1;
                                cands.push_back(c);
                                if (d * d == M) break;
                            }
                    }
            }
            for (int order : {0, 1})
                for (int E : {8, 16}) {
                    const long long e8max = a == A_DF ? 8LL * kMaxThreadsE8 : 4096;
                    if (E == 8 && L > e8max) continue;
                    for (int lpc : {0, 1, 2, 4, 8, 16, 32}) {
                        long long tpl = (L + E - 1) / E;
                        if (lpc * tpl > (E == 8 && L > 4096 ? kMaxThreadsE8 : 512)) continue;
                        for (int no9 : {0, 1}) {
                            if (no9 && L % 9) continue;
                            TuneCfg c;
                            c.order = order;
                            c.E = E;
                            c.lpc = lpc;
                            c.no9 = no9;
                            cands.push_back(c);
                        }
                    }
                }
        }
        if (cands.empty()) cands.push_back(TuneCfg());
        cudaEvent_t e0, e1;
        ck(cudaEventCreate(&e0), "event");
        ck(cudaEventCreate(&e1), "event");
        TuneCfg best;
        best.ms = -1.0;
        for (const TuneCfg &c : cands) {
            g_cfg_override = &c;
            g_cfg_override_len = M;
            g_cfg_override_arith = a;
            std::shared_ptr<Core> core;
            try {
                core = make_core(a, M, even);
            } catch (...) {
                g_cfg_override = nullptr;
                continue;
            }
            g_cfg_override = nullptr;
            float round_ms = 0.f;
            try {
                exec_op(a, op, N, ln, 1, 1.0, 0, core);
                // best of two rounds of two calls
                float best_round = -1.f;
                for (int round = 0; round < 2; ++round) {
                    ck(cudaEventRecord(e0, 0), "event");
                    for (int r = 0; r < 2; ++r) exec_op(a, op, N, ln, 1, 1.0, 0, core);
                    ck(cudaEventRecord(e1, 0), "event");
                    ck(cudaEventSynchronize(e1), "event");
                    float rms = 0.f;
                    cudaEventElapsedTime(&rms, e0, e1);
                    if (best_round < 0 || rms < best_round) best_round = rms;
                }
                round_ms = best_round / 2.0f;
            } catch (const Error &err) {
                // a configuration the kernels cannot launch is skipped
                if (getenv("IG_TUNE_VERBOSE"))
                    fprintf(stderr, "ig_autotune: N=%lld order=%d E=%d lpc=%d N1=%lld skipped: %s\n", N, c.order, c.E,
                            c.lpc, c.N1, err.msg.c_str());
                cudaGetLastError();
                continue;
            }
            TuneCfg r = c;
            r.ms = round_ms;
            if (best.ms < 0 || r.ms < best.ms) best = r;
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        {
            std::lock_guard<std::mutex> lk(g_tune_mu);
            g_tune[std::make_pair((int)a, M)] = best;
        }
        {
            std::lock_guard<std::mutex> lk(g_mu);
            g_cores.clear();  // cores that embed the tuned length are rebuilt on next use
        }
        if (best_ms) *best_ms = best.ms;
    });
}

int ig_c2c(int dtype, size_t ndim, const size_t *shape, const ptrdiff_t *sin, const ptrdiff_t *sout, size_t naxes,
           const size_t *axes, int forward, const void *in, void *out, double fct, size_t nthreads)
{
    (void)nthreads;
    return guarded([&] {
        if (ndim >= 1 && shape && prod(ndim, shape) == 0) return;
        nd_checks(dtype, ndim, shape, sin, sout, naxes, axes, in, out, true);
        host_nd(0, dtype, ndim, shape, sin, sout, naxes, axes, forward, in, out, fct);
    });
}
int ig_r2c(int dtype, size_t ndim, const size_t *shape_in, const ptrdiff_t *sin, const ptrdiff_t *sout, size_t naxes,
           const size_t *axes, int forward, const void *in, void *out, double fct, size_t nthreads)
{
    (void)nthreads;
    return guarded([&] {
        if (ndim >= 1 && shape_in && prod(ndim, shape_in) == 0) return;
        nd_checks(dtype, ndim, shape_in, sin, sout, naxes, axes, in, out, false);
        host_nd(1, dtype, ndim, shape_in, sin, sout, naxes, axes, forward, in, out, fct);
    });
}
int ig_c2r(int dtype, size_t ndim, const size_t *shape_out, const ptrdiff_t *sin, const ptrdiff_t *sout, size_t naxes,
           const size_t *axes, int forward, const void *in, void *out, double fct, size_t nthreads)
{
    (void)nthreads;
    return guarded([&] {
        if (ndim >= 1 && shape_out && prod(ndim, shape_out) == 0) return;
        nd_checks(dtype, ndim, shape_out, sin, sout, naxes, axes, in, out, false);
        host_nd(2, dtype, ndim, shape_out, sin, sout, naxes, axes, forward, in, out, fct);
    });
}

// ---- upfirdn ----
int ig_upfirdn_length(size_t n, size_t nh, int up, int down, size_t *out_len)
{
    return guarded([&] {
        if (!out_len) raise(IG_EINVAL, "null argument");
        if (up < 1 || down < 1) raise(IG_EINVAL, "up and down must be >= 1");
        if (n < 1 || nh < 1) raise(IG_EINVAL, "empty signal or filter");
        *out_len = (size_t)upfirdn_len((long long)n, (long long)nh, up, down);
    });
}
int ig_upfirdn_device(int dtype, size_t batch, size_t n, const void *x, size_t dist_x, size_t nh, const void *h,
                      int up, int down, void *y, size_t dist_y, void *stream)
{
    return guarded([&] {
        if (dtype != IG_F64 && dtype != IG_F32) raise(IG_EINVAL, "bad dtype");
        if (!x || !h || !y) raise(IG_EINVAL, "null argument");
        upfirdn_device(arith_for(dtype), (long long)batch, (long long)n, x, (long long)dist_x, (long long)nh, h, up,
                       down, y, (long long)dist_y, as_stream(stream));
    });
}
int ig_upfirdn(int dtype, size_t batch, size_t n, const void *x, size_t dist_x, size_t nh, const void *h, int up,
               int down, void *y, size_t dist_y)
{
    return guarded([&] {
        if (dtype != IG_F64 && dtype != IG_F32) raise(IG_EINVAL, "bad dtype");
        if (!x || !h || !y) raise(IG_EINVAL, "null argument");
        if (up < 1 || down < 1) raise(IG_EINVAL, "up and down must be >= 1");
        if (n < 1 || nh < 1) raise(IG_EINVAL, "empty signal or filter");
        if (batch == 0) return;
        const Arith a = arith_for(dtype);
        const size_t sr = store_real_bytes(a);
        const long long ny = upfirdn_len((long long)n, (long long)nh, up, down);
        DevBuf dx(((batch - 1) * dist_x + n) * sr), dh(nh * sr), dyb(((batch - 1) * dist_y + (size_t)ny) * sr);
        ck(cudaMemcpy(dx.p, x, dx.bytes, cudaMemcpyHostToDevice), "H2D copy");
        ck(cudaMemcpy(dh.p, h, dh.bytes, cudaMemcpyHostToDevice), "H2D copy");
        if (dist_y > (size_t)ny) ck(cudaMemcpy(dyb.p, y, dyb.bytes, cudaMemcpyHostToDevice), "H2D copy (output gaps)");
        upfirdn_device(a, (long long)batch, (long long)n, dx.p, (long long)dist_x, (long long)nh, dh.p, up, down, dyb.p,
                       (long long)dist_y, 0);
        ck(cudaMemcpy(y, dyb.p, dyb.bytes, cudaMemcpyDeviceToHost), "D2H copy");
    });
}

// ---- real-to-real transforms ----
int ig_dct(int dtype, size_t ndim, const size_t *shape, const ptrdiff_t *sin, const ptrdiff_t *sout, size_t naxes,
           const size_t *axes, int type, const void *in, void *out, double fct, int ortho, size_t nthreads)
{
    (void)nthreads;
    return r2r_entry(R2R_OP_DCT, dtype, ndim, shape, sin, sout, naxes, axes, type, ortho, 0, 1, in, out, fct, true,
                     nullptr);
}
int ig_dst(int dtype, size_t ndim, const size_t *shape, const ptrdiff_t *sin, const ptrdiff_t *sout, size_t naxes,
           const size_t *axes, int type, const void *in, void *out, double fct, int ortho, size_t nthreads)
{
    (void)nthreads;
    return r2r_entry(R2R_OP_DST, dtype, ndim, shape, sin, sout, naxes, axes, type, ortho, 0, 1, in, out, fct, true,
                     nullptr);
}
int ig_r2r_fftpack(int dtype, size_t ndim, const size_t *shape, const ptrdiff_t *sin, const ptrdiff_t *sout,
                   size_t naxes, const size_t *axes, int real2hermitian, int forward, const void *in, void *out,
                   double fct, size_t nthreads)
{
    (void)nthreads;
    return r2r_entry(R2R_OP_FFTPACK, dtype, ndim, shape, sin, sout, naxes, axes, 0, 0, real2hermitian, forward, in,
                     out, fct, true, nullptr);
}
int ig_r2r_separable_hartley(int dtype, size_t ndim, const size_t *shape, const ptrdiff_t *sin,
                             const ptrdiff_t *sout, size_t naxes, const size_t *axes, const void *in, void *out,
                             double fct, size_t nthreads)
{
    (void)nthreads;
    return r2r_entry(R2R_OP_HSEP, dtype, ndim, shape, sin, sout, naxes, axes, 0, 0, 0, 1, in, out, fct, true, nullptr);
}
int ig_r2r_genuine_hartley(int dtype, size_t ndim, const size_t *shape, const ptrdiff_t *sin, const ptrdiff_t *sout,
                           size_t naxes, const size_t *axes, const void *in, void *out, double fct, size_t nthreads)
{
    (void)nthreads;
    return r2r_entry(R2R_OP_HGEN, dtype, ndim, shape, sin, sout, naxes, axes, 0, 0, 0, 1, in, out, fct, true, nullptr);
}
int ig_dct_device(int dtype, size_t ndim, const size_t *shape, const ptrdiff_t *sin, const ptrdiff_t *sout,
                  size_t naxes, const size_t *axes, int type, const void *in, void *out, double fct, int ortho,
                  void *stream)
{
    return r2r_entry(R2R_OP_DCT, dtype, ndim, shape, sin, sout, naxes, axes, type, ortho, 0, 1, in, out, fct, false,
                     stream);
}
int ig_dst_device(int dtype, size_t ndim, const size_t *shape, const ptrdiff_t *sin, const ptrdiff_t *sout,
                  size_t naxes, const size_t *axes, int type, const void *in, void *out, double fct, int ortho,
                  void *stream)
{
    return r2r_entry(R2R_OP_DST, dtype, ndim, shape, sin, sout, naxes, axes, type, ortho, 0, 1, in, out, fct, false,
                     stream);
}
int ig_r2r_fftpack_device(int dtype, size_t ndim, const size_t *shape, const ptrdiff_t *sin, const ptrdiff_t *sout,
                          size_t naxes, const size_t *axes, int real2hermitian, int forward, const void *in, void *out,
                          double fct, void *stream)
{
    return r2r_entry(R2R_OP_FFTPACK, dtype, ndim, shape, sin, sout, naxes, axes, 0, 0, real2hermitian, forward, in,
                     out, fct, false, stream);
}
int ig_r2r_hartley_device(int dtype, size_t ndim, const size_t *shape, const ptrdiff_t *sin, const ptrdiff_t *sout,
                          size_t naxes, const size_t *axes, int genuine, const void *in, void *out, double fct,
                          void *stream)
{
    return r2r_entry(genuine ? R2R_OP_HGEN : R2R_OP_HSEP, dtype, ndim, shape, sin, sout, naxes, axes, 0, 0, 0, 1, in,
                     out, fct, false, stream);
}

}  // extern "C"
