// ig_inst_df.cu -- kernels and launchers for the double-float (FP64 data) arithmetic.
#include "ig_inst.cuh"

namespace ig {
template struct Launch<TagDF>;

cudaError_t launch_chirp64(void *bk, long long n)
{
    k_gen_chirp64<<<(unsigned)((n + 255) / 256), 256>>>((double2 *)bk, n);
    return cudaGetLastError();
}
cudaError_t launch_pad_chirp64(const void *bk, void *out, long long n, long long L)
{
    k_pad_chirp64<<<(unsigned)((L + 255) / 256), 256>>>((const double2 *)bk, (double2 *)out, n, L);
    return cudaGetLastError();
}
}  // namespace ig
