// ig_inst_f32_e16.cu -- shared-memory FFT kernel variants, float arithmetic, 16 elements per thread.
#include "ig_inst_e.cuh"

namespace ig {
template cudaError_t launch_fft_E<float, 16, false>(const CoreDesc &, const IODesc &, size_t, cudaStream_t);
template cudaError_t launch_worklist_E<float, 16, false>(int, int, const WorkGroup *, const long long *, int,
                                                    unsigned long long, unsigned long long *, const char *,
                                                    char *, char *, int, int, size_t, cudaStream_t, int *);
template cudaError_t set_smem_E<float, 16, false>(int);
}  // namespace ig
