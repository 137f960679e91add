// ig_inst_df_e16db.cu -- shared-memory FFT kernel variants, df arithmetic, 16 elements per thread,
// double-buffered stages.
#include "ig_inst_e.cuh"

namespace ig {
template cudaError_t launch_fft_E<df, 16, true>(const CoreDesc &, const IODesc &, size_t, cudaStream_t);
template cudaError_t launch_worklist_E<df, 16, true>(int, int, const WorkGroup *, const long long *, int,
                                                    unsigned long long, unsigned long long *, const char *,
                                                    char *, char *, int, int, size_t, cudaStream_t, int *);
template cudaError_t set_smem_E<df, 16, true>(int);
}  // namespace ig
