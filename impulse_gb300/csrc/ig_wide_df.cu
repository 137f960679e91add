// ig_wide_df.cu -- the wide double-float variants: 8 elements a thread,
// double-buffered, launch bound kMaxThreadsE8 (672) instead of 512, for
// tuned cores of 4097-5376 points (one line per CTA, twice the warps of the
// 16-element variants).  A separate instantiation with its own launch bound:
// raising the bound of the regular variants changed their register
// allocation (more spills) and cost 3-10 % on other lengths.
#include "ig_inst.cuh"
#include "ig_line.cuh"

namespace ig {

#define IG_KW(RS_, LAY_) k_fft_smem<T, 8, RS_, LAY_, true, kMaxThreadsE8><<<grid, blk, smem, st>>>(d, io)
template <class T, int RS>
static void wide_rs(const CoreDesc &d, const IODesc &io, unsigned grid, unsigned blk, size_t smem, cudaStream_t st)
{
    switch (io.lay) {
    case LAY_C2C: IG_KW(RS, LAY_C2C); break;
    case LAY_R2HC: IG_KW(RS, LAY_R2HC); break;
    case LAY_PR2HC: IG_KW(RS, LAY_PR2HC); break;
    case LAY_TW: IG_KW(RS, LAY_TW); break;
    case LAY_RC: IG_KW(RS, LAY_RC); break;
    default: IG_KW(RS_FULL, LAY_GEN); break;
    }
}

template <class T> cudaError_t launch_fft_wide(const CoreDesc &d, const IODesc &io, size_t smem, cudaStream_t st)
{
    const unsigned grid = (unsigned)((io.nlines + io.lpc - 1) / io.lpc), blk = (unsigned)(io.lpc * io.tpl);
    if (blk > (unsigned)kMaxThreadsE8) return cudaErrorInvalidConfiguration;
    // (double-float 8-element cores are never of the power-of-two class)
    if (io.lay == LAY_GEN) IG_KW(RS_FULL, LAY_GEN);
    else if (d.rs == RS_P2 || d.rs == RS_P235) wide_rs<T, RS_P235>(d, io, grid, blk, smem, st);
    else if (d.rs == RS_ALL) wide_rs<T, RS_ALL>(d, io, grid, blk, smem, st);
    else wide_rs<T, RS_FULL>(d, io, grid, blk, smem, st);
    return cudaGetLastError();
}
#undef IG_KW

template <class T> cudaError_t set_smem_wide(int bytes)
{
    cudaError_t e = set_smem_attr(k_fft_smem<T, 8, RS_FULL, LAY_GEN, true, kMaxThreadsE8>, bytes);
#define IG_SW(RS_)                                                                                          \
    if (e == cudaSuccess) e = set_smem_attr(k_fft_smem<T, 8, RS_, LAY_C2C, true, kMaxThreadsE8>, bytes);      \
    if (e == cudaSuccess) e = set_smem_attr(k_fft_smem<T, 8, RS_, LAY_R2HC, true, kMaxThreadsE8>, bytes);     \
    if (e == cudaSuccess) e = set_smem_attr(k_fft_smem<T, 8, RS_, LAY_PR2HC, true, kMaxThreadsE8>, bytes);    \
    if (e == cudaSuccess) e = set_smem_attr(k_fft_smem<T, 8, RS_, LAY_TW, true, kMaxThreadsE8>, bytes);       \
    if (e == cudaSuccess) e = set_smem_attr(k_fft_smem<T, 8, RS_, LAY_RC, true, kMaxThreadsE8>, bytes);
    IG_SW(RS_P235)
    IG_SW(RS_ALL)
    IG_SW(RS_FULL)
#undef IG_SW
    return e;
}

// the halfcomplex line variant (split pass; the other double-float line
// variants run at 128 registers, 512 threads at most)
template <class T> cudaError_t launch_line_wide(const CoreDesc &d, const IODesc &io, size_t smem, cudaStream_t st)
{
    const unsigned grid = (unsigned)((io.nlines + io.lpc - 1) / io.lpc), blk = (unsigned)(io.lpc * io.tpl);
    if (blk > (unsigned)kMaxThreadsE8 || io.lay != LAY_R2HC) return cudaErrorInvalidConfiguration;
    if (d.rs == RS_P2 || d.rs == RS_P235)
        k_fft_line<T, 8, RS_P235, LK_R2HC_S, true, kMaxThreadsE8><<<grid, blk, smem, st>>>(d, io);
    else if (d.rs == RS_ALL)
        k_fft_line<T, 8, RS_ALL, LK_R2HC_S, true, kMaxThreadsE8><<<grid, blk, smem, st>>>(d, io);
    else
        return cudaErrorNotSupported;
    return cudaGetLastError();
}

template <class T> cudaError_t set_smem_line_wide(int bytes)
{
    cudaError_t e = line_smem_attr(k_fft_line<T, 8, RS_P235, LK_R2HC_S, true, kMaxThreadsE8>, bytes);
    if (e == cudaSuccess) e = line_smem_attr(k_fft_line<T, 8, RS_ALL, LK_R2HC_S, true, kMaxThreadsE8>, bytes);
    return e;
}

template cudaError_t launch_fft_wide<df>(const CoreDesc &, const IODesc &, size_t, cudaStream_t);
template cudaError_t set_smem_wide<df>(int);
template cudaError_t launch_line_wide<df>(const CoreDesc &, const IODesc &, size_t, cudaStream_t);
template cudaError_t set_smem_line_wide<df>(int);

}  // namespace ig
