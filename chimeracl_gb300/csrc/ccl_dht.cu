// Discrete Hankel transform (and the spectral radial-derivative matrices)
// as a batched dense GEMM: Y = beta*Y + alpha*(A X), A real (m x k), X real
// or complex-interleaved (k x ncols real columns).  This is the only dense
// contraction of the step (the reference's Reikna MatrixMul,
// transformer_methods_cl.py:458-480).
//
// This translation unit holds the SIMT form used by the plain FP64 drop-in
// (DFMA; GB300's FP64 rate is the same on the tensor pipe) and by FP32
// fallback shapes: 64x64 output tiles, 16-deep k slabs double-buffered
// through registers, 4x4 outputs per thread.
#include "ccl_common.cuh"
#include "ccl_launch.h"

namespace ccl {

constexpr int GB_M = 64, GB_N = 64, GB_K = 16, GB_THREADS = 256;
constexpr int GB_MAXBATCH = 32;

// Per-entry operands; ncols / ldx / ldy may differ between entries (the
// real m=0 and the complex m>=1 Hankel transforms of a field group share a
// launch: with a real alpha a complex GEMM is a real GEMM over 2*Nx columns).
struct GemmBatch {
  const void *A[GB_MAXBATCH];
  const void *X[GB_MAXBATCH];
  void *Y[GB_MAXBATCH];
  int ncols[GB_MAXBATCH];
  long ldx[GB_MAXBATCH], ldy[GB_MAXBATCH];
};

template <typename T, bool CPLX, bool ACC>
__global__ void __launch_bounds__(GB_THREADS)
    k_gemm(GemmBatch b, int M, int K, T are, T aim) {
  __shared__ T As[2][GB_K][GB_M + 1];
  __shared__ __align__(16) T Xs[2][GB_K][GB_N];
  const T *__restrict__ A = (const T *)b.A[blockIdx.z];
  const T *__restrict__ X = (const T *)b.X[blockIdx.z];
  T *__restrict__ Y = (T *)b.Y[blockIdx.z];
  const int N = b.ncols[blockIdx.z];
  const long ldx = b.ldx[blockIdx.z], ldy = b.ldy[blockIdx.z];
  const int m0 = blockIdx.y * GB_M, n0 = blockIdx.x * GB_N;
  if (n0 >= N) return;
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;

  // loader mapping: A tile 64x16 (4 per thread), X tile 16x64 (4 per thread)
  const int a_m = tid >> 2, a_k = (tid & 3) * 4;  // 4 consecutive k
  const int x_k = tid >> 4, x_n = (tid & 15) * 4; // 4 consecutive n
  T ra[4], rx[4];
  auto load = [&](int k0) {
#pragma unroll
    for (int q = 0; q < 4; q++) {
      int gm = m0 + a_m, gk = k0 + a_k + q;
      ra[q] = (gm < M && gk < K) ? A[(long)gm * K + gk] : T(0);
      int xk = k0 + x_k, xn = n0 + x_n + q;
      rx[q] = (xk < K && xn < N) ? X[(long)xk * ldx + xn] : T(0);
    }
  };
  auto store = [&](int buf) {
#pragma unroll
    for (int q = 0; q < 4; q++) {
      As[buf][a_k + q][a_m] = ra[q];
      Xs[buf][x_k][x_n + q] = rx[q];
    }
  };
  T acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int j = 0; j < 4; j++) acc[i][j] = T(0);

  const int nk = (K + GB_K - 1) / GB_K;
  load(0);
  store(0);
  __syncthreads();
  for (int t = 0; t < nk; t++) {
    const int buf = t & 1;
    if (t + 1 < nk) load((t + 1) * GB_K);
#pragma unroll
    for (int kk = 0; kk < GB_K; kk++) {
      T a[4], x[4];
#pragma unroll
      for (int i = 0; i < 4; i++) a[i] = As[buf][kk][ty * 4 + i];
#pragma unroll
      for (int j = 0; j < 4; j++) x[j] = Xs[buf][kk][tx * 4 + j];
#pragma unroll
      for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) acc[i][j] += a[i] * x[j];
    }
    if (t + 1 < nk) store(buf ^ 1);
    __syncthreads();
  }

#pragma unroll
  for (int i = 0; i < 4; i++) {
    const int gm = m0 + ty * 4 + i;
    if (gm >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; j += (CPLX ? 2 : 1)) {
      const int gn = n0 + tx * 4 + j;
      if (gn >= N) continue;
      T *y = Y + (long)gm * ldy + gn;
      if (CPLX) {
        T re = are * acc[i][j] - aim * acc[i][j + 1];
        T im = are * acc[i][j + 1] + aim * acc[i][j];
        if (ACC) {
          re += y[0];
          im += y[1];
        }
        y[0] = re;
        y[1] = im;
      } else {
        T v = are * acc[i][j];
        if (ACC) v += y[0];
        y[0] = v;
      }
    }
  }
}

template <typename T>
int dht_gemm_batch(int batch, int m, int k, const int *ncols, int cplx,
                   const void *const *A, const void *const *X, const long *ldx,
                   void *const *Y, const long *ldy, double are, double aim,
                   double beta, cudaStream_t s) {
  CCL_REQUIRE(batch >= 0 && batch <= GB_MAXBATCH, CCL_ERR_ARG,
              "dht_gemm: batch %d outside [0, %d]", batch, GB_MAXBATCH);
  CCL_REQUIRE(m > 0 && k > 0, CCL_ERR_ARG, "dht_gemm: sizes m=%d k=%d", m, k);
  CCL_REQUIRE(beta == 0.0 || beta == 1.0, CCL_ERR_ARG,
              "dht_gemm: beta must be 0 or 1");
  if (batch == 0) return CCL_OK;
  GemmBatch b;
  int nmax = 0;
  for (int i = 0; i < batch; i++) {
    CCL_REQUIRE(A[i] && X[i] && Y[i], CCL_ERR_ARG, "dht_gemm: null operand %d",
                i);
    CCL_REQUIRE(ncols[i] > 0 && (!cplx || ncols[i] % 2 == 0), CCL_ERR_ARG,
                "dht_gemm: entry %d ncols %d", i, ncols[i]);
    CCL_REQUIRE(ldx[i] >= ncols[i] && ldy[i] >= ncols[i], CCL_ERR_ARG,
                "dht_gemm: entry %d ldx %ld / ldy %ld < ncols %d", i, ldx[i],
                ldy[i], ncols[i]);
    b.A[i] = A[i];
    b.X[i] = X[i];
    b.Y[i] = Y[i];
    b.ncols[i] = ncols[i];
    b.ldx[i] = ldx[i];
    b.ldy[i] = ldy[i];
    if (ncols[i] > nmax) nmax = ncols[i];
  }
  dim3 grid((nmax + GB_N - 1) / GB_N, (m + GB_M - 1) / GB_M, batch);
  T ar = (T)are, ai = (T)aim;
  bool acc = beta == 1.0;
  if (cplx) {
    if (acc) k_gemm<T, true, true><<<grid, GB_THREADS, 0, s>>>(b, m, k, ar, ai);
    else k_gemm<T, true, false><<<grid, GB_THREADS, 0, s>>>(b, m, k, ar, ai);
  } else {
    if (acc) k_gemm<T, false, true><<<grid, GB_THREADS, 0, s>>>(b, m, k, ar, ai);
    else k_gemm<T, false, false><<<grid, GB_THREADS, 0, s>>>(b, m, k, ar, ai);
  }
  CCL_LAUNCH_CHECK("dht_gemm");
  return CCL_OK;
}

template <typename T>
int dht_gemm(int batch, int m, int k, int ncols, int cplx, const void *const *A,
             const void *const *X, long ldx, void *const *Y, long ldy,
             double are, double aim, double beta, cudaStream_t s) {
  CCL_REQUIRE(batch >= 0 && batch <= GB_MAXBATCH, CCL_ERR_ARG,
              "dht_gemm: batch %d outside [0, %d]", batch, GB_MAXBATCH);
  int nc[GB_MAXBATCH];
  long lx[GB_MAXBATCH], ly[GB_MAXBATCH];
  for (int i = 0; i < batch; i++) {
    nc[i] = ncols;
    lx[i] = ldx;
    ly[i] = ldy;
  }
  return dht_gemm_batch<T>(batch, m, k, nc, cplx, A, X, lx, Y, ly, are, aim,
                           beta, s);
}

#define CCL_INST_GEMM(T)                                                       \
  template int dht_gemm<T>(int, int, int, int, int, const void *const *,      \
                           const void *const *, long, void *const *, long,    \
                           double, double, double, cudaStream_t);              \
  template int dht_gemm_batch<T>(int, int, int, const int *, int,             \
                                 const void *const *, const void *const *,    \
                                 const long *, void *const *, const long *,   \
                                 double, double, double, cudaStream_t);
CCL_INST_GEMM(double)
CCL_INST_GEMM(float)

}  // namespace ccl
