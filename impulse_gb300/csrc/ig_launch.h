// ig_launch.h -- host entry points into the per-arithmetic kernel units
// (ig_inst_f32.cu, ig_inst_df.cu, ig_inst_f64.cu).  Each returns the CUDA
// launch status.
#pragma once
#include <cuda_runtime.h>

#include "ig_types.h"

namespace ig {

// tag types standing for the device arithmetic of each unit
struct TagF32 {};
struct TagDF {};
struct TagF64 {};

template <class Tag> struct Launch {
    // k_fft_smem with `lpc` lines of `tpl` threads per CTA and `smem` bytes
    static cudaError_t fft_smem(const CoreDesc &d, const IODesc &io, size_t smem, cudaStream_t st);
    // k_fft_line (first / last stages fused with the HBM reads / writes): the
    // same descriptors, for complex lines and even real lines to halfcomplex
    static cudaError_t fft_line(const CoreDesc &d, const IODesc &io, size_t smem, cudaStream_t st);
    // k_fft_line_pipe (FP32, contiguous lines): bulk-copy (TMA) staging of
    // `nslot` tiles ahead, persistent CTAs on `sms` SMs; `work_bytes` = the
    // line buffers of one CTA
    static cudaError_t fft_line_pipe(const CoreDesc &d, const IODesc &io, size_t work_bytes, int nslot, int sms,
                                     cudaStream_t st);
    // adds the pipelined kernels' bounded-wait give-ups since the last call
    static cudaError_t pipe_faults(unsigned *count);
    static cudaError_t set_max_smem(int bytes);
    // persistent work-list launch of the k_fft_smem variant (E, db, rs, lay):
    // `grid` CTAs of `block` threads; `occupancy` reports CTAs per SM for it
    static cudaError_t fft_worklist(int E, int db, int rs, int lay, const WorkGroup *groups, const long long *prefix,
                                    int ngroups, unsigned long long total, unsigned long long *counter, const void *in,
                                    void *out, void *scr, int grid, int block, size_t smem, cudaStream_t st);
    static cudaError_t worklist_occupancy(int E, int db, int rs, int lay, int block, size_t smem, int *per_sm);
    static cudaError_t stage_tw(void *tw, int R, int ns);
    static cudaError_t roots(void *out, long long count, unsigned long long mult, unsigned long long D);
    static cudaError_t convert64(const void *in, void *out, long long n);
    static cudaError_t gather(const IODesc &io, const MapDesc &mp, cudaStream_t st);
    static cudaError_t scatter(const IODesc &io, const MapDesc &mp, cudaStream_t st);
    // two real lines per complex line on the multi-pass paths
    static cudaError_t line_exp(const IODesc &io, int *esc, cudaStream_t st);
    static cudaError_t gather_pair(const IODesc &io, const MapDesc &mp, const int *esc, cudaStream_t st);
    static cudaError_t scatter_pair(const IODesc &io, const MapDesc &mp, const int *esc, cudaStream_t st);
    // FFT convolution helpers on the storage type of the arithmetic
    static cudaError_t pad2d(const void *in, void *out, long long B, long long H, long long W, long long P0,
                             long long P1, long long r0, long long c0, cudaStream_t st);
    static cudaError_t crop2d(const void *in, void *out, long long B, long long H, long long W, long long P0,
                              long long P1, long long r0, long long c0, cudaStream_t st);
    static cudaError_t spec_mul(const void *a, const void *f, void *out, long long B, long long nf, long long n,
                                int mode, cudaStream_t st);
    static cudaError_t half_weight(void *x, long long lines, long long n_half, long long nreal, double w,
                                   int drop_im, cudaStream_t st);
    // real-to-real transforms
    static cudaError_t r2r_pre(const IODesc &io, const R2RDesc &d, cudaStream_t st);
    static cudaError_t r2r_post(const IODesc &io, const R2RDesc &d, cudaStream_t st);
    static cudaError_t r2r_tw(void *tw1, void *tw2, long long N);
    // four-step inter-pass twiddles w_M^(n2 k1), row n2 < N2 of N1 entries (M = N1 N2)
    static cudaError_t tw4_table(void *tab, long long N1, long long N2);
    static cudaError_t hartley_fold(const void *X, void *out, const HartleyDesc &h, cudaStream_t st);
    // upfirdn
    static cudaError_t upsample_pad(const void *x, long long dx, long long n, int up, void *U, long long P,
                                    long long B, cudaStream_t st);
    static cudaError_t decimate(const void *C, long long P, int down, void *y, long long dy, long long ny, long long B,
                                cudaStream_t st);
};

// k_fft_pair (ig_pair_f32.cu): FP32 lines with two butterflies per thread in
// paired FP32 lanes; GS = padded 16-byte groups of one line buffer
cudaError_t launch_pair(const CoreDesc &d, const IODesc &io, int GS, size_t smem, cudaStream_t st);
cudaError_t set_smem_pair(int bytes);
// pair twiddle table of one stage (ns even)
cudaError_t launch_stage_twp(void *tw, int R, int ns);
// copy of `bytes` bytes by the SMs (grid of at most 8 CTAs per SM on `sms`
// SMs), for host memory the device addresses through the host page tables
cudaError_t launch_copy(const void *src, void *dst, size_t bytes, int sms, cudaStream_t st);

// FP64 helpers for Bluestein tables (built in ig_inst_df.cu)
cudaError_t launch_chirp64(void *bk, long long n);
cudaError_t launch_pad_chirp64(const void *bk, void *out, long long n, long long L);

}  // namespace ig
