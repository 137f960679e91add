// ig_inst_f64.cu -- kernels and launchers for the native FP64 arithmetic.
#include "ig_inst.cuh"

namespace ig {
template struct Launch<TagF64>;
}  // namespace ig
