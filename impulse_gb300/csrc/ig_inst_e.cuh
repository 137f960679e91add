// ig_inst_e.cuh -- k_fft_smem variants of one arithmetic and elements-per-thread
// count: radix classes x layout classes (double uses the generic variant only).
#pragma once
#include <type_traits>

#include "ig_inst.cuh"

namespace ig {

template <class T, int E> struct Variants {
    static constexpr bool kSpecialised = !std::is_same<T, double>::value;
};

#define IG_K(RS_, LAY_) k_fft_smem<T, E, RS_, LAY_, DB><<<grid, blk, smem, st>>>(d, io)
template <class T, int E, bool DB, int RS>
static void launch_rs(const CoreDesc &d, const IODesc &io, unsigned grid, unsigned blk, size_t smem, cudaStream_t st)
{
    switch (io.lay) {
    case LAY_C2C: IG_K(RS, LAY_C2C); break;
    case LAY_R2HC: IG_K(RS, LAY_R2HC); break;
    case LAY_PR2HC: IG_K(RS, LAY_PR2HC); break;
    case LAY_TW: IG_K(RS, LAY_TW); break;
    case LAY_RC: IG_K(RS, LAY_RC); break;
    default: IG_K(RS_FULL, LAY_GEN); break;
    }
}
#undef IG_K

template <class T, int E, bool DB>
cudaError_t launch_fft_E(const CoreDesc &d, const IODesc &io, size_t smem, cudaStream_t st)
{
    const unsigned grid = (unsigned)((io.nlines + io.lpc - 1) / io.lpc), blk = (unsigned)(io.lpc * io.tpl);
    if (blk > 512) {
        if constexpr (std::is_same<T, df>::value && E == 8 && DB) return launch_fft_wide<T>(d, io, smem, st);
        return cudaErrorInvalidConfiguration;
    }
    if constexpr (!Variants<T, E>::kSpecialised) {
        k_fft_smem<T, E, RS_FULL, LAY_GEN, DB><<<grid, blk, smem, st>>>(d, io);
    } else {
        if (io.lay == LAY_GEN) k_fft_smem<T, E, RS_FULL, LAY_GEN, DB><<<grid, blk, smem, st>>>(d, io);
        else if (d.rs == RS_P2) launch_rs<T, E, DB, RS_P2>(d, io, grid, blk, smem, st);
        else if (E == 8 && d.rs == RS_P235) launch_rs<T, E, DB, (E == 8 ? RS_P235 : RS_ALL)>(d, io, grid, blk, smem, st);
        else if (d.rs == RS_ALL) launch_rs<T, E, DB, RS_ALL>(d, io, grid, blk, smem, st);
        else if constexpr (std::is_same<T, df>::value && E == 8 && DB) {
            if (d.rs == RS_ALLR) launch_rs<T, E, DB, RS_ALLR>(d, io, grid, blk, smem, st);
            else launch_rs<T, E, DB, RS_FULL>(d, io, grid, blk, smem, st);
        } else
            launch_rs<T, E, DB, RS_FULL>(d, io, grid, blk, smem, st);
    }
    return cudaGetLastError();
}

// work-list variants: the same (radix class, layout class) choice as
// launch_fft_E; with per_sm set, report CTAs per SM instead of launching
template <class T, int E, bool DB, int RS, int LAY>
static cudaError_t worklist_one(const WorkGroup *groups, const long long *prefix, int ngroups, unsigned long long total,
                                unsigned long long *counter, const char *in, char *out, char *scr, int grid, int block,
                                size_t smem, cudaStream_t st, int *per_sm)
{
    auto k = k_fft_worklist<T, E, RS, LAY, DB>;
    if (per_sm) return cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, k, block, smem);
    k<<<grid, block, smem, st>>>(groups, prefix, ngroups, total, counter, in, out, scr);
    return cudaGetLastError();
}

template <class T, int E, bool DB, int RS>
static cudaError_t worklist_rs(int lay, const WorkGroup *groups, const long long *prefix, int ngroups,
                               unsigned long long total, unsigned long long *counter, const char *in, char *out,
                               char *scr, int grid, int block, size_t smem, cudaStream_t st, int *per_sm)
{
#define IG_W(LAY_) worklist_one<T, E, DB, RS, LAY_>(groups, prefix, ngroups, total, counter, in, out, scr, grid, block, smem, st, per_sm)
    switch (lay) {
    case LAY_C2C: return IG_W(LAY_C2C);
    case LAY_TW: return IG_W(LAY_TW);
    default: return worklist_one<T, E, DB, RS_FULL, LAY_GEN>(groups, prefix, ngroups, total, counter, in, out, scr,
                                                            grid, block, smem, st, per_sm);
    }
#undef IG_W
}

template <class T, int E, bool DB>
cudaError_t launch_worklist_E(int rs, int lay, const WorkGroup *groups, const long long *prefix, int ngroups,
                              unsigned long long total, unsigned long long *counter, const char *in, char *out,
                              char *scr, int grid, int block, size_t smem, cudaStream_t st, int *per_sm)
{
    if constexpr (!Variants<T, E>::kSpecialised) {
        return worklist_one<T, E, DB, RS_FULL, LAY_GEN>(groups, prefix, ngroups, total, counter, in, out, scr, grid,
                                                       block, smem, st, per_sm);
    } else {
        (void)rs;  // the host sends every partition with the full radix class
        if (lay != LAY_C2C && lay != LAY_TW)
            return worklist_one<T, E, DB, RS_FULL, LAY_GEN>(groups, prefix, ngroups, total, counter, in, out, scr,
                                                           grid, block, smem, st, per_sm);
        return worklist_rs<T, E, DB, RS_FULL>(lay, groups, prefix, ngroups, total, counter, in, out, scr, grid, block,
                                              smem, st, per_sm);
    }
}

template <class T, int E, bool DB> cudaError_t set_smem_E(int bytes)
{
    cudaError_t e = set_smem_attr(k_fft_smem<T, E, RS_FULL, LAY_GEN, DB>, bytes);
    if constexpr (Variants<T, E>::kSpecialised) {
#define IG_S(RS_)                                                                                         \
    if (e == cudaSuccess) e = set_smem_attr(k_fft_smem<T, E, RS_, LAY_C2C, DB>, bytes);                     \
    if (e == cudaSuccess) e = set_smem_attr(k_fft_smem<T, E, RS_, LAY_R2HC, DB>, bytes);                    \
    if (e == cudaSuccess) e = set_smem_attr(k_fft_smem<T, E, RS_, LAY_PR2HC, DB>, bytes);                   \
    if (e == cudaSuccess) e = set_smem_attr(k_fft_smem<T, E, RS_, LAY_TW, DB>, bytes);                     \
    if (e == cudaSuccess) e = set_smem_attr(k_fft_smem<T, E, RS_, LAY_RC, DB>, bytes);
        IG_S(RS_P2)
        IG_S(RS_ALL)
        IG_S(RS_FULL)
        if constexpr (E == 8) { IG_S(RS_P235) }
        if constexpr (std::is_same<T, df>::value && E == 8 && DB) { IG_S(RS_ALLR) }
#undef IG_S
        if (e == cudaSuccess) e = set_smem_attr(k_fft_worklist<T, E, RS_FULL, LAY_C2C, DB>, bytes);
        if (e == cudaSuccess) e = set_smem_attr(k_fft_worklist<T, E, RS_FULL, LAY_TW, DB>, bytes);
    }
    if (e == cudaSuccess) e = set_smem_attr(k_fft_worklist<T, E, RS_FULL, LAY_GEN, DB>, bytes);
    return e;
}

}  // namespace ig
