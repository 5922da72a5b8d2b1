// FP64 instantiation of the particle, grid and elementwise kernels.  Built
// with -fmad=false: no multiply-add contraction, so each expression rounds
// as the reference's strict-IEEE arithmetic does and the plain FP64 drop-in
// matches the reference kernels bit for bit on the same inputs.
#include "ccl_ops.cuh"

namespace ccl {

template struct Ops<double>;

size_t index_sort_ws_bytes(long np, long ncells) {
  return sort_ws_bytes(np, ncells);
}

int iota_u32(uint32_t *a, long n, cudaStream_t s) {
  if (n == 0) return CCL_OK;
  k_iota<<<grid_for(n, 256), 256, 0, s>>>(a, n);
  CCL_LAUNCH_CHECK("iota");
  return CCL_OK;
}

}  // namespace ccl
