// ig_inst.cuh -- launcher definitions, instantiated once per arithmetic.
#pragma once
#include <algorithm>

#include "ig_kernels.cuh"
#include "ig_launch.h"

namespace ig {

template <class Tag> struct TagType;
template <> struct TagType<TagF32> { using T = float; };
template <> struct TagType<TagDF> { using T = df; };
template <> struct TagType<TagF64> { using T = double; };

// k_fft_smem variants of one (arithmetic, elements-per-thread) pair live in
// their own translation unit (ig_inst_<arith>_e<E>.cu) to compile in parallel
// (16 elements per thread: in-place and double-buffered variants)
template <class T, int E, bool DB>
cudaError_t launch_fft_E(const CoreDesc &d, const IODesc &io, size_t smem, cudaStream_t st);
template <class T, int E, bool DB> cudaError_t set_smem_E(int bytes);
template <class T, int E, bool DB>
cudaError_t launch_worklist_E(int rs, int lay, const WorkGroup *groups, const long long *prefix, int ngroups,
                              unsigned long long total, unsigned long long *counter, const char *in, char *out,
                              char *scr, int grid, int block, size_t smem, cudaStream_t st, int *per_sm);
template <class T, int E, bool DB>
cudaError_t launch_line_E(const CoreDesc &d, const IODesc &io, size_t smem, cudaStream_t st);
template <class T, int E, bool DB> cudaError_t set_smem_line_E(int bytes);
template <class T, int E, bool DB>
cudaError_t launch_line_pipe_E(const CoreDesc &d, const IODesc &io, size_t work_bytes, int nslot, int sms,
                               cudaStream_t st);
template <class T, int E, bool DB> cudaError_t line_pipe_faults_E(unsigned *count);
// the wide double-float 8-element variants (more than 512 threads a CTA), in
// their own translation unit (ig_wide_df.cu)
template <class T> cudaError_t launch_fft_wide(const CoreDesc &d, const IODesc &io, size_t smem, cudaStream_t st);
template <class T> cudaError_t set_smem_wide(int bytes);
template <class T> cudaError_t launch_line_wide(const CoreDesc &d, const IODesc &io, size_t smem, cudaStream_t st);
template <class T> cudaError_t set_smem_line_wide(int bytes);

template <class Tag> cudaError_t Launch<Tag>::fft_smem(const CoreDesc &d, const IODesc &io, size_t smem, cudaStream_t st)
{
    using T = typename TagType<Tag>::T;
    return d.E == 8 ? launch_fft_E<T, 8, true>(d, io, smem, st)
         : d.db     ? launch_fft_E<T, 16, true>(d, io, smem, st)
                    : launch_fft_E<T, 16, false>(d, io, smem, st);
}
template <class Tag> cudaError_t Launch<Tag>::fft_line(const CoreDesc &d, const IODesc &io, size_t smem, cudaStream_t st)
{
    using T = typename TagType<Tag>::T;
    if constexpr (std::is_same<T, double>::value) {
        return cudaErrorNotSupported;  // native FP64 runs k_fft_smem only
    } else {
        return d.E == 8 ? launch_line_E<T, 8, true>(d, io, smem, st)
             : d.db     ? launch_line_E<T, 16, true>(d, io, smem, st)
                        : launch_line_E<T, 16, false>(d, io, smem, st);
    }
}
template <class Tag>
cudaError_t Launch<Tag>::fft_line_pipe(const CoreDesc &d, const IODesc &io, size_t work_bytes, int nslot, int sms,
                                       cudaStream_t st)
{
    using T = typename TagType<Tag>::T;
    if constexpr (!std::is_same<T, float>::value) {
        return cudaErrorNotSupported;  // FP32 only: double-float lines need the per-line range check
    } else {
        return d.E == 8 ? launch_line_pipe_E<T, 8, true>(d, io, work_bytes, nslot, sms, st)
             : d.db     ? launch_line_pipe_E<T, 16, true>(d, io, work_bytes, nslot, sms, st)
                        : launch_line_pipe_E<T, 16, false>(d, io, work_bytes, nslot, sms, st);
    }
}
template <class Tag> cudaError_t Launch<Tag>::pipe_faults(unsigned *count)
{
    using T = typename TagType<Tag>::T;
    if constexpr (!std::is_same<T, float>::value) {
        return cudaSuccess;
    } else {
        cudaError_t e = line_pipe_faults_E<T, 8, true>(count);
        if (e == cudaSuccess) e = line_pipe_faults_E<T, 16, true>(count);
        if (e == cudaSuccess) e = line_pipe_faults_E<T, 16, false>(count);
        return e;
    }
}
template <class K> static cudaError_t set_smem_attr(K kernel, int bytes)
{
    cudaFuncAttributes fa;
    cudaError_t e = cudaFuncGetAttributes(&fa, kernel);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes - (int)fa.sharedSizeBytes);
}
template <class Tag> cudaError_t Launch<Tag>::set_max_smem(int bytes)
{
    using T = typename TagType<Tag>::T;
    // the dynamic limit excludes each kernel's static shared memory
    cudaError_t e;
    if ((e = set_smem_E<T, 8, true>(bytes)) != cudaSuccess) return e;
    if constexpr (std::is_same<T, df>::value) {
        if ((e = set_smem_wide<T>(bytes)) != cudaSuccess) return e;
        if ((e = set_smem_line_wide<T>(bytes)) != cudaSuccess) return e;
    }
    if ((e = set_smem_E<T, 16, false>(bytes)) != cudaSuccess) return e;
    if ((e = set_smem_E<T, 16, true>(bytes)) != cudaSuccess) return e;
    if constexpr (!std::is_same<T, double>::value) {
        if ((e = set_smem_line_E<T, 8, true>(bytes)) != cudaSuccess) return e;
        if ((e = set_smem_line_E<T, 16, false>(bytes)) != cudaSuccess) return e;
        if ((e = set_smem_line_E<T, 16, true>(bytes)) != cudaSuccess) return e;
    }
    return cudaSuccess;
}
template <class Tag>
cudaError_t Launch<Tag>::fft_worklist(int E, int db, int rs, int lay, const WorkGroup *groups, const long long *prefix,
                                      int ngroups, unsigned long long total, unsigned long long *counter,
                                      const void *in, void *out, void *scr, int grid, int block, size_t smem,
                                      cudaStream_t st)
{
    using T = typename TagType<Tag>::T;
    auto f = E == 8 ? launch_worklist_E<T, 8, true> : db ? launch_worklist_E<T, 16, true> : launch_worklist_E<T, 16, false>;
    return f(rs, lay, groups, prefix, ngroups, total, counter, (const char *)in, (char *)out, (char *)scr, grid, block,
             smem, st, nullptr);
}
template <class Tag>
cudaError_t Launch<Tag>::worklist_occupancy(int E, int db, int rs, int lay, int block, size_t smem, int *per_sm)
{
    using T = typename TagType<Tag>::T;
    auto f = E == 8 ? launch_worklist_E<T, 8, true> : db ? launch_worklist_E<T, 16, true> : launch_worklist_E<T, 16, false>;
    return f(rs, lay, nullptr, nullptr, 0, 0, nullptr, nullptr, nullptr, nullptr, 0, block, smem, 0, per_sm);
}
template <class Tag> cudaError_t Launch<Tag>::stage_tw(void *tw, int R, int ns)
{
    using T = typename TagType<Tag>::T;
    int n = ns * (R - 1);
    if (!n) return cudaSuccess;
    k_gen_stage_tw<T><<<(n + 255) / 256, 256>>>((typename Bfly<T>::W *)tw, R, ns);
    return cudaGetLastError();
}
template <class Tag>
cudaError_t Launch<Tag>::roots(void *out, long long count, unsigned long long mult, unsigned long long D)
{
    using T = typename TagType<Tag>::T;
    if (!count) return cudaSuccess;
    k_gen_roots<T><<<(unsigned)((count + 255) / 256), 256>>>((cx<T> *)out, count, mult, D);
    return cudaGetLastError();
}
template <class Tag> cudaError_t Launch<Tag>::convert64(const void *in, void *out, long long n)
{
    using T = typename TagType<Tag>::T;
    if (!n) return cudaSuccess;
    k_convert64<T><<<(unsigned)((n + 255) / 256), 256>>>((const double2 *)in, (cx<T> *)out, n);
    return cudaGetLastError();
}

static inline unsigned map_grid(long long total)
{
    long long g = (total + 255) / 256;
    return (unsigned)(g < 152LL * 32 ? (g > 0 ? g : 1) : 152LL * 32);
}
template <class Tag> cudaError_t Launch<Tag>::gather(const IODesc &io, const MapDesc &mp, cudaStream_t st)
{
    using T = typename TagType<Tag>::T;
    k_gather<T><<<map_grid(io.nlines * mp.scr_len), 256, 0, st>>>(io, mp);
    return cudaGetLastError();
}
template <class Tag> cudaError_t Launch<Tag>::scatter(const IODesc &io, const MapDesc &mp, cudaStream_t st)
{
    using T = typename TagType<Tag>::T;
    k_scatter<T><<<map_grid(io.nlines * (long long)io.cnt_out), 256, 0, st>>>(io, mp);
    return cudaGetLastError();
}

template <class Tag> cudaError_t Launch<Tag>::line_exp(const IODesc &io, int *esc, cudaStream_t st)
{
    using T = typename TagType<Tag>::T;
    k_line_exp<T><<<(unsigned)io.nlines, 1024, 0, st>>>(io, esc);
    return cudaGetLastError();
}
template <class Tag>
cudaError_t Launch<Tag>::gather_pair(const IODesc &io, const MapDesc &mp, const int *esc, cudaStream_t st)
{
    using T = typename TagType<Tag>::T;
    k_gather_pair<T><<<map_grid(io.nlines * mp.scr_len), 256, 0, st>>>(io, mp, esc);
    return cudaGetLastError();
}
template <class Tag>
cudaError_t Launch<Tag>::scatter_pair(const IODesc &io, const MapDesc &mp, const int *esc, cudaStream_t st)
{
    using T = typename TagType<Tag>::T;
    k_scatter_pair<T><<<map_grid(io.nlines * (long long)io.cnt_out), 256, 0, st>>>(io, mp, esc);
    return cudaGetLastError();
}
template <class Tag>
cudaError_t Launch<Tag>::pad2d(const void *in, void *out, long long B, long long H, long long W, long long P0,
                               long long P1, long long r0, long long c0, cudaStream_t st)
{
    using S = typename Traits<typename TagType<Tag>::T>::S;
    const long long rows = B * P0;
    k_pad2d<S><<<(unsigned)std::min<long long>(std::max<long long>(rows, 1), 152LL * 16), 256, 0, st>>>(
        (const S *)in, (S *)out, B, H, W, P0, P1, r0, c0);
    return cudaGetLastError();
}
template <class Tag>
cudaError_t Launch<Tag>::crop2d(const void *in, void *out, long long B, long long H, long long W, long long P0,
                                long long P1, long long r0, long long c0, cudaStream_t st)
{
    using S = typename Traits<typename TagType<Tag>::T>::S;
    const long long rows = B * H;
    k_crop2d<S><<<(unsigned)std::min<long long>(std::max<long long>(rows, 1), 152LL * 16), 256, 0, st>>>(
        (const S *)in, (S *)out, B, H, W, P0, P1, r0, c0);
    return cudaGetLastError();
}
template <class Tag>
cudaError_t Launch<Tag>::spec_mul(const void *a, const void *f, void *out, long long B, long long nf, long long n,
                                  int mode, cudaStream_t st)
{
    using T = typename TagType<Tag>::T;
    using S2 = typename Traits<T>::S2;
    k_spec_mul<T><<<map_grid(mode == 2 ? n : B * n), 256, 0, st>>>((const S2 *)a, (const S2 *)f, (S2 *)out, B, nf, n,
                                                                    mode);
    return cudaGetLastError();
}
template <class Tag>
cudaError_t Launch<Tag>::half_weight(void *x, long long lines, long long n_half, long long nreal, double w,
                                     int drop_im, cudaStream_t st)
{
    using T = typename TagType<Tag>::T;
    using S = typename Traits<T>::S;
    using S2 = typename Traits<T>::S2;
    k_half_weight<T><<<map_grid(lines * n_half), 256, 0, st>>>((S2 *)x, lines, n_half, nreal, (S)w, drop_im);
    return cudaGetLastError();
}
template <class Tag> cudaError_t Launch<Tag>::r2r_pre(const IODesc &io, const R2RDesc &d, cudaStream_t st)
{
    using T = typename TagType<Tag>::T;
    k_r2r_pre<T><<<map_grid(io.nlines * d.L2), 256, 0, st>>>(io, d);
    return cudaGetLastError();
}
template <class Tag> cudaError_t Launch<Tag>::r2r_post(const IODesc &io, const R2RDesc &d, cudaStream_t st)
{
    using T = typename TagType<Tag>::T;
    k_r2r_post<T><<<map_grid(io.nlines * d.N), 256, 0, st>>>(io, d);
    return cudaGetLastError();
}
template <class Tag> cudaError_t Launch<Tag>::tw4_table(void *tab, long long N1, long long N2)
{
    using T = typename TagType<Tag>::T;
    const long long n = N1 * N2;
    k_gen_tw4<T><<<(unsigned)((n + 255) / 256), 256>>>((typename Bfly<T>::W *)tab, N1, N2);
    return cudaGetLastError();
}
template <class Tag> cudaError_t Launch<Tag>::r2r_tw(void *tw1, void *tw2, long long N)
{
    using T = typename TagType<Tag>::T;
    k_gen_r2r_tw<T><<<(unsigned)((N + 256) / 256), 256>>>((cx<T> *)tw1, (cx<T> *)tw2, N);
    return cudaGetLastError();
}
template <class Tag>
cudaError_t Launch<Tag>::upsample_pad(const void *x, long long dx, long long n, int up, void *U, long long P,
                                      long long B, cudaStream_t st)
{
    using S = typename Traits<typename TagType<Tag>::T>::S;
    k_upsample_pad<S><<<map_grid(B * P), 256, 0, st>>>((const S *)x, dx, n, up, (S *)U, P, B);
    return cudaGetLastError();
}
template <class Tag>
cudaError_t Launch<Tag>::decimate(const void *C, long long P, int down, void *y, long long dy, long long ny,
                                  long long B, cudaStream_t st)
{
    using S = typename Traits<typename TagType<Tag>::T>::S;
    k_decimate<S><<<map_grid(B * ny), 256, 0, st>>>((const S *)C, P, down, (S *)y, dy, ny, B);
    return cudaGetLastError();
}
template <class Tag>
cudaError_t Launch<Tag>::hartley_fold(const void *X, void *out, const HartleyDesc &h, cudaStream_t st)
{
    using T = typename TagType<Tag>::T;
    k_hartley_fold<T><<<map_grid(h.total), 256, 0, st>>>((const typename Traits<T>::S2 *)X, (char *)out, h);
    return cudaGetLastError();
}

}  // namespace ig
