// Allocation-free form of the cell sort: the workspace of ccl_index_sort
// lives in a file-scope device array instead of caller-owned memory.
//
// The scratch's device address is looked up (cudaGetSymbolAddress, with the
// calling device current) on every call made outside a stream capture, so a
// new context after cudaDeviceReset is picked up; a call made while its
// stream is being captured reuses the address of the last uncaptured call on
// that device, and is refused (CCL_ERR_UNSUPPORTED) when there was none.
// Every call then runs the unchanged ccl_index_sort with it.  Nothing here allocates device
// or host memory.  ccl_index_sort clears what must start at zero (the
// per-cell counts and the scatter cursors) itself, on the stream, before
// use; the rest of the scratch is written before it is read.  One scratch
// array serves all calls on a device, so calls that overlap in time (two
// streams, or two host threads) race on it.
#include <cuda_runtime.h>

#include <mutex>

#include "ccl_common.cuh"

namespace {

constexpr size_t kSortScratchBytes = (size_t)9 << 20;  // 9 MiB
constexpr int kMaxDevices = 64;

__device__ __align__(256) unsigned char g_sort_scratch[kSortScratchBytes];

std::mutex g_mu;
void *g_scratch[kMaxDevices] = {};

// the scratch's device address for the current device
int scratch_for_current_device(cudaStream_t stream, void **out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    ccl::set_error("ccl_index_sort_noalloc: cudaGetDevice: %s", cudaGetErrorString(e));
    return CCL_ERR_CUDA;
  }
  if (dev < 0 || dev >= kMaxDevices) {
    ccl::set_error("ccl_index_sort_noalloc: device %d outside [0, %d)", dev, kMaxDevices);
    return CCL_ERR_UNSUPPORTED;
  }
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  e = cudaStreamIsCapturing(stream, &cap);
  if (e != cudaSuccess) {
    ccl::set_error("ccl_index_sort_noalloc: cudaStreamIsCapturing: %s", cudaGetErrorString(e));
    return CCL_ERR_CUDA;
  }
  std::lock_guard<std::mutex> lock(g_mu);
  if (cap != cudaStreamCaptureStatusNone) {
    if (!g_scratch[dev]) {
      ccl::set_error("ccl_index_sort_noalloc: first call on device %d inside a stream capture; "
                     "call it once outside the capture first", dev);
      return CCL_ERR_UNSUPPORTED;
    }
  } else {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_sort_scratch);
    if (e != cudaSuccess || !p) {
      ccl::set_error("ccl_index_sort_noalloc: cudaGetSymbolAddress: %s",
                     cudaGetErrorString(e));
      return CCL_ERR_CUDA;
    }
    g_scratch[dev] = p;
  }
  *out = g_scratch[dev];
  return CCL_OK;
}

}  // namespace

extern "C" int ccl_index_sort_noalloc(int dtype, long np, const void *x, const void *y,
                                      const void *z, int Nx, double xmin, double dx_inv,
                                      int Nr, double rmin, double dr_inv,
                                      uint32_t *indx_in_cell, uint32_t *sum_in_cell,
                                      uint32_t *cell_offset, uint32_t *sort_indx,
                                      uint32_t *np_stay, void *stream) {
  // argument checks are those of ccl_index_sort_workspace / ccl_index_sort
  const long ncells = (long)(Nx - 1) * (long)(Nr - 1);
  size_t need = 0;
  int rc = ccl_index_sort_workspace(np, ncells, &need);
  if (rc) return rc;
  if (need > kSortScratchBytes) {
    ccl::set_error(
        "ccl_index_sort_noalloc: np=%ld on %ld cells needs %zu bytes of workspace, more than "
        "the %zu-byte static scratch; use ccl_index_sort with a caller-owned workspace",
        np, ncells, need, kSortScratchBytes);
    return CCL_ERR_WORKSPACE;
  }
  void *ws = nullptr;
  if ((rc = scratch_for_current_device((cudaStream_t)stream, &ws))) return rc;
  return ccl_index_sort(dtype, np, x, y, z, Nx, xmin, dx_inv, Nr, rmin, dr_inv, indx_in_cell,
                        sum_in_cell, cell_offset, sort_indx, np_stay, ws, kSortScratchBytes,
                        stream);
}
