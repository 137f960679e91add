// ig_line_df_e16db.cu -- k_fft_line variants, double-float arithmetic, 16 elements per thread, double-buffered.
#include "ig_inst.cuh"
#include "ig_line.cuh"

namespace ig {
template cudaError_t launch_line_E<df, 16, true>(const CoreDesc &, const IODesc &, size_t, cudaStream_t);
template cudaError_t set_smem_line_E<df, 16, true>(int);
}  // namespace ig
