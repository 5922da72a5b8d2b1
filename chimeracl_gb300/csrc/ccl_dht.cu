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

struct GemmBatch {
  const void *A[GB_MAXBATCH];
  const void *X[GB_MAXBATCH];
  void *Y[GB_MAXBATCH];
};

template <typename T, bool CPLX, bool ACC>
__global__ void __launch_bounds__(GB_THREADS)
    k_gemm(GemmBatch b, int M, int K, int N, long ldx, long ldy, T are,
           T aim) {
  __shared__ T As[2][GB_K][GB_M + 1];
  __shared__ __align__(16) T Xs[2][GB_K][GB_N];
  const T *__restrict__ A = (const T *)b.A[blockIdx.z];
  const T *__restrict__ X = (const T *)b.X[blockIdx.z];
  T *__restrict__ Y = (T *)b.Y[blockIdx.z];
  const int m0 = blockIdx.y * GB_M, n0 = blockIdx.x * GB_N;
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
int dht_gemm(int batch, int m, int k, int ncols, int cplx, const void *const *A,
             const void *const *X, long ldx, void *const *Y, long ldy,
             double are, double aim, double beta, cudaStream_t s) {
  CCL_REQUIRE(batch >= 0 && batch <= GB_MAXBATCH, CCL_ERR_ARG,
              "dht_gemm: batch %d outside [0, %d]", batch, GB_MAXBATCH);
  CCL_REQUIRE(m > 0 && k > 0 && ncols > 0, CCL_ERR_ARG,
              "dht_gemm: sizes m=%d k=%d ncols=%d", m, k, ncols);
  CCL_REQUIRE(!cplx || ncols % 2 == 0, CCL_ERR_ARG,
              "dht_gemm: complex ncols %d must be even", ncols);
  CCL_REQUIRE(ldx >= ncols && ldy >= ncols, CCL_ERR_ARG,
              "dht_gemm: ldx %ld / ldy %ld < ncols %d", ldx, ldy, ncols);
  CCL_REQUIRE(beta == 0.0 || beta == 1.0, CCL_ERR_ARG,
              "dht_gemm: beta must be 0 or 1");
  if (batch == 0) return CCL_OK;
  GemmBatch b;
  for (int i = 0; i < batch; i++) {
    CCL_REQUIRE(A[i] && X[i] && Y[i], CCL_ERR_ARG, "dht_gemm: null operand %d",
                i);
    b.A[i] = A[i];
    b.X[i] = X[i];
    b.Y[i] = Y[i];
  }
  dim3 grid((ncols + GB_N - 1) / GB_N, (m + GB_M - 1) / GB_M, batch);
  T ar = (T)are, ai = (T)aim;
  bool acc = beta == 1.0;
  if (cplx) {
    if (acc) k_gemm<T, true, true><<<grid, GB_THREADS, 0, s>>>(b, m, k, ncols, ldx, ldy, ar, ai);
    else k_gemm<T, true, false><<<grid, GB_THREADS, 0, s>>>(b, m, k, ncols, ldx, ldy, ar, ai);
  } else {
    if (acc) k_gemm<T, false, true><<<grid, GB_THREADS, 0, s>>>(b, m, k, ncols, ldx, ldy, ar, ai);
    else k_gemm<T, false, false><<<grid, GB_THREADS, 0, s>>>(b, m, k, ncols, ldx, ldy, ar, ai);
  }
  CCL_LAUNCH_CHECK("dht_gemm");
  return CCL_OK;
}

template int dht_gemm<double>(int, int, int, int, int, const void *const *,
                              const void *const *, long, void *const *, long,
                              double, double, double, cudaStream_t);
template int dht_gemm<float>(int, int, int, int, int, const void *const *,
                             const void *const *, long, void *const *, long,
                             double, double, double, cudaStream_t);

}  // namespace ccl
