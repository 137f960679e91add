// ig_pair_f32.cu -- k_fft_pair (FP32 lines, two butterflies per thread in
// paired FP32 lanes): launchers and the pair twiddle tables.
#include "ig_inst.cuh"
#include "ig_pair.cuh"

namespace ig {

template <int RS, int K> static void pair_go(const CoreDesc &d, const IODesc &io, int GS, unsigned grid, unsigned blk,
                                             size_t smem, cudaStream_t st)
{
    k_fft_pair<RS, K><<<grid, blk, smem, st>>>(d, io, GS);
}

cudaError_t launch_pair(const CoreDesc &d, const IODesc &io, int GS, size_t smem, cudaStream_t st)
{
    const unsigned grid = (unsigned)((io.nlines + io.lpc - 1) / io.lpc), blk = (unsigned)(io.lpc * io.tpl);
    const int k = io.lay == LAY_R2HC ? PK_R2HC : io.lay == LAY_R2C ? PK_R2C : PK_C2C;
#define IG_PG(RS_)                                                                      \
    (k == PK_R2HC  ? pair_go<RS_, PK_R2HC>(d, io, GS, grid, blk, smem, st)              \
     : k == PK_R2C ? pair_go<RS_, PK_R2C>(d, io, GS, grid, blk, smem, st)               \
                   : pair_go<RS_, PK_C2C>(d, io, GS, grid, blk, smem, st))
    if (d.rs == RS_P2) IG_PG(RS_P2);
    else if (d.rs == RS_P235) IG_PG(RS_P235);
    else if (d.rs == RS_ALL) IG_PG(RS_ALL);
    else return cudaErrorNotSupported;
#undef IG_PG
    return cudaGetLastError();
}

template <class Kern> static cudaError_t pair_attr(Kern k, int bytes)
{
    cudaFuncAttributes fa;
    cudaError_t e = cudaFuncGetAttributes(&fa, k);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes - (int)fa.sharedSizeBytes);
}

cudaError_t set_smem_pair(int bytes)
{
    cudaError_t e = cudaSuccess;
#define IG_PA(RS_)                                                                     \
    if (e == cudaSuccess) e = pair_attr(k_fft_pair<RS_, PK_C2C>, bytes);               \
    if (e == cudaSuccess) e = pair_attr(k_fft_pair<RS_, PK_R2HC>, bytes);              \
    if (e == cudaSuccess) e = pair_attr(k_fft_pair<RS_, PK_R2C>, bytes);
    IG_PA(RS_P2)
    IG_PA(RS_P235)
    IG_PA(RS_ALL)
#undef IG_PA
    return e;
}

cudaError_t launch_stage_twp(void *tw, int R, int ns)
{
    const int n = (ns / 2) * (R - 1);
    if (n <= 0) return cudaSuccess;
    k_gen_stage_twp<<<(n + 255) / 256, 256>>>(reinterpret_cast<float4 *>(tw), R, ns);
    return cudaGetLastError();
}

}  // namespace ig
