// ig_inst_f64_e8.cu -- shared-memory FFT kernel variants, double arithmetic, 8 elements per thread.
#include "ig_inst_e.cuh"

namespace ig {
template cudaError_t launch_fft_E<double, 8, true>(const CoreDesc &, const IODesc &, size_t, cudaStream_t);
template cudaError_t set_smem_E<double, 8, true>(int);
}  // namespace ig
