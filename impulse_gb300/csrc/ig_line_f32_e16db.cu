// ig_line_f32_e16db.cu -- k_fft_line variants, float arithmetic, 16 elements per thread, double-buffered.
#include "ig_inst.cuh"
#include "ig_line.cuh"

namespace ig {
template cudaError_t launch_line_E<float, 16, true>(const CoreDesc &, const IODesc &, size_t, cudaStream_t);
template cudaError_t set_smem_line_E<float, 16, true>(int);
template cudaError_t launch_line_pipe_E<float, 16, true>(const CoreDesc &, const IODesc &, size_t, int, int,
                                                         cudaStream_t);
template cudaError_t line_pipe_faults_E<float, 16, true>(unsigned *);
}  // namespace ig
