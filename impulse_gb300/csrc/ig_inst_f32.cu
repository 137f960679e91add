// ig_inst_f32.cu -- kernels and launchers for the FP32 arithmetic.
#include "ig_inst.cuh"

namespace ig {
template struct Launch<TagF32>;
}  // namespace ig
