// Shared definitions for the chimeracl_gb300 CUDA kernels (sm_103a).
//
// Layout conventions (identical to the reference's device containers):
//  * particles: structure of arrays, one array per component (x, y, z, px,
//    py, pz, w, g_inv), index = particle number;
//  * real-space fields: row-major (Nr, Nx), node (ir, ix) at ix + ir*Nx, row 0
//    the ghost row at r = -dr/2; mode m=0 real, m>=1 complex interleaved;
//  * spectral fields: row-major complex (Nr-1, Nx), row = radial mode index,
//    column = longitudinal wavenumber index (numpy fftfreq order).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/chimeracl_gb300.h"

namespace ccl {

typedef uint32_t u32;

// Number of SMs on the GB300 (2 dies x 76); grid-stride kernels size their
// grids in multiples of it.
constexpr int kNumSM = 152;
constexpr int kMaxModes = 4;  // azimuthal modes m = 0..3 (M <= 3)

void set_error(const char *fmt, ...);
void count_launch();

#define CCL_REQUIRE(cond, code, ...)                                           \
  do {                                                                         \
    if (!(cond)) {                                                             \
      ::ccl::set_error(__VA_ARGS__);                                           \
      return (code);                                                           \
    }                                                                          \
  } while (0)

#define CCL_LAUNCH_CHECK(what)                                                 \
  do {                                                                         \
    ::ccl::count_launch();                                                     \
    cudaError_t e_ = cudaGetLastError();                                       \
    if (e_ != cudaSuccess) {                                                   \
      ::ccl::set_error("%s: %s", what, cudaGetErrorString(e_));                \
      return CCL_ERR_CUDA;                                                     \
    }                                                                          \
  } while (0)

static inline int grid_for(long n, int threads, int per_sm = 8) {
  long b = (n + threads - 1) / threads;
  long cap = (long)kNumSM * per_sm;
  if (b > cap) b = cap;
  if (b < 1) b = 1;
  return (int)b;
}

static inline cudaStream_t S(void *stream) { return (cudaStream_t)stream; }

// Programmatic dependent launch.  A kernel started by launch_pdl may be
// placed on the SMs while the kernel before it in the stream is finishing
// (the launch and set-up of the next grid overlap the last CTAs of this
// one).  Such a kernel calls pdl_wait() before it touches any memory an
// earlier kernel reads or writes: it returns once those kernels have
// completed and their writes are visible (in a kernel launched the ordinary
// way it returns at once).  In a CUDA graph the dependency becomes a
// programmatic edge.  (Releasing the next grid early, before this one's
// CTAs have all exited, measured slower on the step: its waiting CTAs take
// SM slots from this grid's last wave.)
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

template <typename... KArgs, typename... Args>
static inline cudaError_t launch_pdl(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem,
                                     cudaStream_t s, Args... args) {
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kern, static_cast<KArgs>(args)...);
}

// Row-chunked indexing of (nrows x nx) spectral arrays (the spectral
// combines and their transposes): block blockIdx.x takes row
// blockIdx.x / nch and RcCols<T> consecutive columns of it, each thread
// RcPer<T> of them RC_THREADS apart, with no division per element.  (The
// combines load all of a thread's columns before their first store: the
// field bundles may alias, so the compiler would not move the loads.)
constexpr int RC_THREADS = 256;
// (two columns per thread: four measured slower in FP32, fewer blocks per SM)
template <typename T> constexpr int RcPer = 2;
template <typename T> constexpr int RcCols = RC_THREADS * RcPer<T>;
template <typename T> inline dim3 row_chunk_grid(int nrows, int nx, int nz) {
  return dim3((unsigned)nrows * (unsigned)((nx + RcCols<T> - 1) / RcCols<T>), (unsigned)nz);
}
template <typename T> struct RowChunk {
  int ir, c0;
  __device__ __forceinline__ RowChunk(int nx) {
    const int nch = (nx + RcCols<T> - 1) / RcCols<T>;
    ir = blockIdx.x / nch;
    c0 = (blockIdx.x - ir * nch) * RcCols<T> + threadIdx.x;
  }
  __device__ __forceinline__ int col(int q) const { return c0 + q * RC_THREADS; }
};

// Complex number of real type T, laid out as (re, im).
template <typename T> struct cplx {
  T re, im;
};

template <typename T> struct vec2;
template <> struct vec2<double> { typedef double2 type; };
template <> struct vec2<float> { typedef float2 type; };

template <typename T> __device__ __forceinline__ cplx<T> ld_c(const T *p, long i) {
  typename vec2<T>::type v = reinterpret_cast<const typename vec2<T>::type *>(p)[i];
  cplx<T> r;
  r.re = v.x;
  r.im = v.y;
  return r;
}
template <typename T> __device__ __forceinline__ void st_c(T *p, long i, cplx<T> c) {
  typename vec2<T>::type v;
  v.x = c.re;
  v.y = c.im;
  reinterpret_cast<typename vec2<T>::type *>(p)[i] = v;
}

// Pointer bundles passed by value to kernels (kernel parameter space).
template <int N> struct ptrs {
  void *p[N];
};

// Element i of a bundle for an index known only at run time (a block
// coordinate, a count): a chain of selects over constant indices, so the
// bundle stays in parameter space.  Indexing it directly makes the compiler
// copy the whole bundle into every thread's local memory first.
template <int N> __device__ __forceinline__ void *pick(const ptrs<N> &a, int i) {
  void *r = a.p[0];
#pragma unroll
  for (int j = 1; j < N; j++) r = i == j ? a.p[j] : r;
  return r;
}

}  // namespace ccl
