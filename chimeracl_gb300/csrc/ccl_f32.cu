// FP32 instantiation of the particle, grid and elementwise kernels (FMA
// contraction on).
#include "ccl_ops.cuh"

namespace ccl {

template struct Ops<float>;

}  // namespace ccl
