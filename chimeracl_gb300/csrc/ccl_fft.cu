// Batched longitudinal FFT (along x, contiguous rows) for the spectral
// transforms: mixed-radix Stockham autosort in shared memory, one CTA per
// row, radices 8/4/2 for powers of two and a table-driven DFT for odd prime
// factors (3, 5, 7, 11, 13).  The row's phase factor, smoothing filter,
// real-part cast and absorbing-edge profile are applied on the way in/out
// so that every transform stage of the step reads and writes HBM once.
//
// Forward: X_k = sum_n x_n e^{-2 pi i nk/N} (unnormalised); inverse with
// e^{+2 pi i nk/N} and 1/N -- the conventions of the reference's Reikna FFT
// (transformer_methods_cl.py:507-509).
#include <math.h>

#include <map>
#include <mutex>
#include <utility>

#include "ccl_common.cuh"
#include "ccl_launch.h"

namespace ccl {

constexpr int FFT_THREADS = 256;
constexpr int FFT_MAXST = 16;

struct FftPlan {
  int n, nst;
  int rad[FFT_MAXST];
};

static bool make_plan(int n, FftPlan *p) {
  p->n = n;
  p->nst = 0;
  int m = n;
  while (m % 8 == 0) { p->rad[p->nst++] = 8; m /= 8; }
  while (m % 4 == 0) { p->rad[p->nst++] = 4; m /= 4; }
  while (m % 2 == 0) { p->rad[p->nst++] = 2; m /= 2; }
  const int odd[] = {3, 5, 7, 11, 13};
  for (int q : odd)
    while (m % q == 0) {
      if (p->nst >= FFT_MAXST) return false;
      p->rad[p->nst++] = q;
      m /= q;
    }
  return m == 1 && p->nst <= FFT_MAXST;
}

template <typename T> __device__ __forceinline__ cplx<T> cmul(cplx<T> a, cplx<T> b) {
  cplx<T> r = {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
  return r;
}
template <typename T> __device__ __forceinline__ cplx<T> cadd(cplx<T> a, cplx<T> b) {
  cplx<T> r = {a.re + b.re, a.im + b.im};
  return r;
}
template <typename T> __device__ __forceinline__ cplx<T> csub(cplx<T> a, cplx<T> b) {
  cplx<T> r = {a.re - b.re, a.im - b.im};
  return r;
}
// multiply by -i (forward) or +i (inverse)
template <typename T, bool INV> __device__ __forceinline__ cplx<T> mul_mi(cplx<T> a) {
  cplx<T> r;
  if (INV) { r.re = -a.im; r.im = a.re; }
  else { r.re = a.im; r.im = -a.re; }
  return r;
}

template <typename T, bool INV>
__device__ __forceinline__ void dft4(cplx<T> &a, cplx<T> &b, cplx<T> &c, cplx<T> &d) {
  cplx<T> t0 = cadd(a, c), t1 = csub(a, c), t2 = cadd(b, d), t3 = mul_mi<T, INV>(csub(b, d));
  a = cadd(t0, t2);
  c = csub(t0, t2);
  b = cadd(t1, t3);
  d = csub(t1, t3);
}

template <typename T, bool INV>
__device__ __forceinline__ void dft8(cplx<T> *v) {
  cplx<T> e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6];
  cplx<T> o0 = v[1], o1 = v[3], o2 = v[5], o3 = v[7];
  dft4<T, INV>(e0, e1, e2, e3);
  dft4<T, INV>(o0, o1, o2, o3);
  const T h = (T)0.70710678118654752440084436210485;
  // o_q *= W8^q, W8 = e^{-i pi/4} (forward) / e^{+i pi/4} (inverse)
  cplx<T> w1 = {h, INV ? h : -h}, w3 = {-h, INV ? h : -h};
  o1 = cmul(o1, w1);
  o2 = mul_mi<T, INV>(o2);
  o3 = cmul(o3, w3);
  v[0] = cadd(e0, o0); v[4] = csub(e0, o0);
  v[1] = cadd(e1, o1); v[5] = csub(e1, o1);
  v[2] = cadd(e2, o2); v[6] = csub(e2, o2);
  v[3] = cadd(e3, o3); v[7] = csub(e3, o3);
}

template <typename T> __device__ __forceinline__ cplx<T> twid(const cplx<T> *tw, long t, bool inv) {
  cplx<T> w = tw[t];
  if (inv) w.im = -w.im;
  return w;
}

// One Stockham stage of a power-of-two radix R (unrolled, in registers).
template <typename T, bool INV, int R>
__device__ __forceinline__ void stage_pow2(const cplx<T> *__restrict__ src,
                                           cplx<T> *__restrict__ dst, int N,
                                           int Ns,
                                           const cplx<T> *__restrict__ tw) {
  const int NR = N / R, tstride = N / (Ns * R);
  for (int j = threadIdx.x; j < NR; j += blockDim.x) {
    const int k = j % Ns;
    cplx<T> v[R];
#pragma unroll
    for (int r = 0; r < R; r++) v[r] = src[j + r * NR];
    if (Ns > 1) {
#pragma unroll
      for (int r = 1; r < R; r++)
        v[r] = cmul(v[r], twid(tw, (long)(r * k) * tstride, INV));
    }
    if (R == 8) {
      dft8<T, INV>(v);
    } else if (R == 4) {
      dft4<T, INV>(v[0], v[1], v[2], v[3]);
    } else {
      cplx<T> a = cadd(v[0], v[1]), b = csub(v[0], v[1]);
      v[0] = a;
      v[1] = b;
    }
    const int ob = (j / Ns) * Ns * R + k;
#pragma unroll
    for (int r = 0; r < R; r++) dst[ob + r * Ns] = v[r];
  }
}

// One Stockham stage of an odd prime radix R <= 13 (table-driven DFT).
template <typename T, bool INV>
__device__ void stage_odd(const cplx<T> *__restrict__ src,
                          cplx<T> *__restrict__ dst, int N, int Ns, int R,
                          const cplx<T> *__restrict__ tw) {
  const int NR = N / R, tstride = N / (Ns * R);
  for (int j = threadIdx.x; j < NR; j += blockDim.x) {
    const int k = j % Ns;
    cplx<T> v[13], y[13];
    for (int r = 0; r < R; r++) v[r] = src[j + r * NR];
    if (Ns > 1)
      for (int r = 1; r < R; r++)
        v[r] = cmul(v[r], twid(tw, (long)(r * k) * tstride, INV));
    // y_q = sum_r v_r W_R^{rq}, with W_R^t = W_N^{t N/R}
    for (int q = 0; q < R; q++) {
      cplx<T> acc = v[0];
      for (int r = 1; r < R; r++)
        acc = cadd(acc, cmul(v[r], twid(tw, (long)((r * q) % R) * NR, INV)));
      y[q] = acc;
    }
    const int ob = (j / Ns) * Ns * R + k;
    for (int r = 0; r < R; r++) dst[ob + r * Ns] = y[r];
  }
}

// One full transform of the row held in sA (result returned: sA or sB).
template <typename T, bool INV>
__device__ cplx<T> *fft_row(cplx<T> *sA, cplx<T> *sB, const FftPlan &pl,
                            const cplx<T> *__restrict__ tw) {
  const int N = pl.n;
  int Ns = 1;
  cplx<T> *src = sA, *dst = sB;
  for (int st = 0; st < pl.nst; st++) {
    const int R = pl.rad[st];
    if (R == 8) stage_pow2<T, INV, 8>(src, dst, N, Ns, tw);
    else if (R == 4) stage_pow2<T, INV, 4>(src, dst, N, Ns, tw);
    else if (R == 2) stage_pow2<T, INV, 2>(src, dst, N, Ns, tw);
    else stage_odd<T, INV>(src, dst, N, Ns, R, tw);
    __syncthreads();
    cplx<T> *t = src;
    src = dst;
    dst = t;
    Ns *= R;
  }
  return src;
}

constexpr int FFT_MAXBATCH = 32;

// Per-entry operands of a batched row transform (blockIdx.y = entry).
struct FftBatch {
  const void *in[FFT_MAXBATCH];
  void *out[FFT_MAXBATCH];
  const void *filt[FFT_MAXBATCH];
  long ld[FFT_MAXBATCH];   // leading dimension of the real-space side
  int real[FFT_MAXBATCH];  // real-space side is real (mode 0)
};

template <typename T>
__device__ __forceinline__ cplx<T> mul_phs(cplx<T> v, cplx<T> p) {
  cplx<T> r = {(v.re * p.re - v.im * p.im), (v.re * p.im + v.im * p.re)};
  return r;
}

// Forward stage: in -> FFT -> * phs (* filter) -> out (complex (nrows, N))
template <typename T>
__global__ void __launch_bounds__(FFT_THREADS)
    k_fft_fwd(FftPlan pl, FftBatch b, const T *__restrict__ phs,
              const cplx<T> *__restrict__ tw) {
  extern __shared__ __align__(16) unsigned char smraw[];
  cplx<T> *sA = (cplx<T> *)smraw, *sB = sA + pl.n;
  const int N = pl.n, e = blockIdx.y;
  const long row = blockIdx.x;
  const long ld = b.ld[e];
  const T *in = (const T *)b.in[e];
  if (b.real[e]) {
    for (int ix = threadIdx.x; ix < N; ix += blockDim.x) {
      cplx<T> v = {in[row * ld + ix], T(0)};
      sA[ix] = v;
    }
  } else {
    for (int ix = threadIdx.x; ix < N; ix += blockDim.x) sA[ix] = ld_c(in, row * ld + ix);
  }
  __syncthreads();
  cplx<T> *res = fft_row<T, false>(sA, sB, pl, tw);
  T *out = (T *)b.out[e];
  const T *filt = (const T *)b.filt[e];
  for (int ix = threadIdx.x; ix < N; ix += blockDim.x) {
    cplx<T> r = mul_phs(res[ix], ld_c(phs, ix));
    if (filt) {
      T f = filt[row * N + ix];
      r.re = f * r.re;
      r.im = f * r.im;
    }
    st_c(out, row * N + ix, r);
  }
}

// Backward stage: in * phs -> inverse FFT / N -> out (complex or real part)
template <typename T>
__global__ void __launch_bounds__(FFT_THREADS)
    k_fft_bwd(FftPlan pl, FftBatch b, const T *__restrict__ phs,
              const cplx<T> *__restrict__ tw) {
  extern __shared__ __align__(16) unsigned char smraw[];
  cplx<T> *sA = (cplx<T> *)smraw, *sB = sA + pl.n;
  const int N = pl.n, e = blockIdx.y;
  const long row = blockIdx.x;
  const T *in = (const T *)b.in[e];
  for (int ix = threadIdx.x; ix < N; ix += blockDim.x)
    sA[ix] = mul_phs(ld_c(in, row * N + ix), ld_c(phs, ix));
  __syncthreads();
  cplx<T> *res = fft_row<T, true>(sA, sB, pl, tw);
  const T inv_n = (T)(1.0 / (double)N);
  T *out = (T *)b.out[e];
  const long ld = b.ld[e];
  if (b.real[e]) {
    for (int ix = threadIdx.x; ix < N; ix += blockDim.x) out[row * ld + ix] = res[ix].re * inv_n;
  } else {
    for (int ix = threadIdx.x; ix < N; ix += blockDim.x) {
      cplx<T> r = {res[ix].re * inv_n, res[ix].im * inv_n};
      st_c(out, row * ld + ix, r);
    }
  }
}

// Edge damping of a row, f(x) x = x + (f(x) - 1) x.  In FP32 the damped
// spectrum is formed as that increment: the spectrum itself is kept and only
// FFT((f - 1) IFFT(x)) -- zero away from the edges -- goes through the
// rounded transforms and phase factors.  Damping the whole row instead sends
// it through a backward and a forward FFT every step, and the round trip's
// gain at each frequency (the product of its twiddles' and phase factors'
// rounded moduli) is a fixed number within a few units in the last place of
// 1: a pulse confined to a few frequencies gains or loses energy by that
// factor every step, about 1e-7 a step in FP32.  The FP64 form keeps the
// reference's order (backward, profile, forward).
template <typename T> constexpr bool DAMP_INCREMENT = sizeof(T) == 4;

template <typename T>
__device__ __forceinline__ T damp_factor(const T *__restrict__ prof, u32 ux, u32 un, u32 nf) {
  T f = T(1);
  if (ux < nf) f *= prof[ux];
  if (ux > un - nf) f *= prof[un - ux];
  return f;
}

// Absorbing-edge round trip, in place: b.in = b.out = spectral field,
// b.filt = real-space field (nrows+1, N), b.real = mode 0.
template <typename T>
__global__ void __launch_bounds__(FFT_THREADS)
    k_damp(FftPlan pl, FftBatch b, const T *__restrict__ phs_p,
           const T *__restrict__ phs_m, const T *__restrict__ prof, u32 nf,
           const cplx<T> *__restrict__ tw) {
  extern __shared__ __align__(16) unsigned char smraw[];
  cplx<T> *sA = (cplx<T> *)smraw, *sB = sA + pl.n;
  const int N = pl.n, e = blockIdx.y;
  const u32 un = (u32)N;
  const long row = blockIdx.x;
  T *spec = (T *)b.out[e];
  T *rs = (T *)b.filt[e];
  const bool rs_real = b.real[e] != 0;
  for (int ix = threadIdx.x; ix < N; ix += blockDim.x)
    sA[ix] = mul_phs(ld_c(spec, row * N + ix), ld_c(phs_p, ix));
  __syncthreads();
  cplx<T> *res = fft_row<T, true>(sA, sB, pl, tw);
  cplx<T> *other = (res == sA) ? sB : sA;
  const T inv_n = (T)(1.0 / (double)N);
  for (int ix = threadIdx.x; ix < N; ix += blockDim.x) {
    cplx<T> v = res[ix];
    v.re = v.re * inv_n;
    v.im = rs_real ? T(0) : v.im * inv_n;
    const u32 ux = (u32)ix;
    if constexpr (DAMP_INCREMENT<T>) {
      const T f = damp_factor(prof, ux, un, nf), fm1 = f - T(1);
      other[ix] = {v.re * fm1, v.im * fm1};
      v.re *= f;
      v.im *= f;
    } else {
      if (ux < nf) { v.re *= prof[ux]; v.im *= prof[ux]; }
      if (ux > un - nf) { v.re *= prof[un - ux]; v.im *= prof[un - ux]; }
      other[ix] = v;
    }
    if (rs_real) rs[(row + 1) * N + ix] = v.re;
    else st_c(rs, (row + 1) * N + ix, v);
    if (row == 0) {  // the ghost row is damped in place as well
      if (rs_real) {
        T g = rs[ix];
        if (ux < nf) g *= prof[ux];
        if (ux > un - nf) g *= prof[un - ux];
        rs[ix] = g;
      } else {
        cplx<T> g = ld_c(rs, ix);
        if (ux < nf) { g.re *= prof[ux]; g.im *= prof[ux]; }
        if (ux > un - nf) { g.re *= prof[un - ux]; g.im *= prof[un - ux]; }
        st_c(rs, ix, g);
      }
    }
  }
  __syncthreads();
  cplx<T> *tmp2 = (other == sA) ? sB : sA;
  cplx<T> *res2 = fft_row<T, false>(other, tmp2, pl, tw);
  for (int ix = threadIdx.x; ix < N; ix += blockDim.x) {
    cplx<T> o = mul_phs(res2[ix], ld_c(phs_m, ix));
    if constexpr (DAMP_INCREMENT<T>) {
      const cplx<T> x = ld_c(spec, row * N + ix);
      o.re = x.re + o.re;
      o.im = x.im + o.im;
    }
    st_c(spec, row * N + ix, o);
  }
}

// ---------------------------------------------------------------------
// Register-resident transform for N = 512, 1024, 2048, 4096: N/8 threads,
// 8 points each.  Radix-8 Stockham passes in registers (then one radix-4 or
// radix-2 pass for N = 8^a * 4 or * 2); between passes the row goes through
// shared memory once, padded by one point in eight so that the strided
// pass writes are free of bank conflicts.  Thread j reads its input points
// x[j + r N/8] straight from HBM and ends holding X[j + q N/8], q = 0..7, so
// the first and last passes touch global memory directly (and a backward
// transform's output is exactly the layout a forward transform starts from).
__device__ __forceinline__ int fpad(int i) { return i + (i >> 3); }

template <int N> struct RegFft {
  static constexpr int TH = N / 8;
  static constexpr int P8 = N == 4096 ? 4 : 3;             // radix-8 passes
  static constexpr int TAIL = N == 2048 ? 4 : (N == 1024 ? 2 : 1);  // last radix
  static constexpr int SMEM_PTS = N + N / 8;
};

template <typename T, bool INV, int N>
__device__ __forceinline__ void fft_reg(cplx<T> (&v)[8], cplx<T> *sm,
                                        const cplx<T> *__restrict__ tw) {
  using F = RegFft<N>;
  const int j = threadIdx.x;
  int Ns = 1;
#pragma unroll
  for (int p = 0; p < F::P8; p++) {
    const int k = j & (Ns - 1);
    if (p > 0) {
      // W^(r k) for r = 1..7 from one table entry: the powers by a product
      // tree at most three multiplications deep (one table read instead of
      // seven; the table reads were the kernel's L1 bottleneck)
      const int ts = N / (8 * Ns);
      cplx<T> w[8];
      w[1] = twid(tw, (long)k * ts, INV);
      w[2] = cmul(w[1], w[1]);
      w[3] = cmul(w[2], w[1]);
      w[4] = cmul(w[2], w[2]);
      w[5] = cmul(w[4], w[1]);
      w[6] = cmul(w[4], w[2]);
      w[7] = cmul(w[4], w[3]);
#pragma unroll
      for (int r = 1; r < 8; r++) v[r] = cmul(v[r], w[r]);
    }
    dft8<T, INV>(v);
    const bool last = (p == F::P8 - 1) && F::TAIL == 1;
    if (!last) {
      const int ob = (j / Ns) * Ns * 8 + k;
      __syncthreads();  // the previous pass's reads are done
#pragma unroll
      for (int r = 0; r < 8; r++) sm[fpad(ob + r * Ns)] = v[r];
      __syncthreads();
      if (p < F::P8 - 1) {
#pragma unroll
        for (int r = 0; r < 8; r++) v[r] = sm[fpad(j + r * F::TH)];
      }
    }
    Ns *= 8;
  }
  if (F::TAIL == 4) {
    // butterflies jj = j + t N/8 (t = 0, 1), points jj + r N/4; Ns = N/4
#pragma unroll
    for (int t = 0; t < 2; t++) {
      const int jj = j + t * F::TH;
      cplx<T> a[4];
#pragma unroll
      for (int r = 0; r < 4; r++) a[r] = sm[fpad(jj + r * (N / 4))];
      const cplx<T> w1 = twid(tw, (long)jj, INV), w2 = cmul(w1, w1), w3 = cmul(w2, w1);
      a[1] = cmul(a[1], w1);
      a[2] = cmul(a[2], w2);
      a[3] = cmul(a[3], w3);
      dft4<T, INV>(a[0], a[1], a[2], a[3]);
#pragma unroll
      for (int r = 0; r < 4; r++) v[t + 2 * r] = a[r];  // X[j + (t + 2r) N/8]
    }
  } else if (F::TAIL == 2) {
#pragma unroll
    for (int t = 0; t < 4; t++) {
      const int jj = j + t * F::TH;
      cplx<T> a0 = sm[fpad(jj)], a1 = sm[fpad(jj + N / 2)];
      a1 = cmul(a1, twid(tw, (long)jj, INV));
      v[t] = cadd(a0, a1);      // X[j + t N/8]
      v[t + 4] = csub(a0, a1);  // X[j + (t + 4) N/8]
    }
  }
}

template <typename T, int N>
__global__ void __launch_bounds__(N / 8)
    k_fft_fwd_reg(FftBatch b, const T *__restrict__ phs, const cplx<T> *__restrict__ tw) {
  pdl_wait();
  __shared__ cplx<T> sm[RegFft<N>::SMEM_PTS];
  constexpr int TH = N / 8;
  const int j = threadIdx.x, e = blockIdx.y;
  const long row = blockIdx.x;
  const T *in = (const T *)b.in[e] + row * b.ld[e] * (b.real[e] ? 1 : 2);
  cplx<T> v[8];
  if (b.real[e]) {
#pragma unroll
    for (int r = 0; r < 8; r++) v[r] = {in[j + r * TH], T(0)};
  } else {
#pragma unroll
    for (int r = 0; r < 8; r++) v[r] = ld_c(in, j + r * TH);
  }
  fft_reg<T, false, N>(v, sm, tw);
  T *out = (T *)b.out[e] + row * N * 2;
  const T *filt = b.filt[e] ? (const T *)b.filt[e] + row * N : nullptr;
#pragma unroll
  for (int q = 0; q < 8; q++) {
    const int ix = j + q * TH;
    cplx<T> r = mul_phs(v[q], ld_c(phs, ix));
    if (filt) {
      const T f = filt[ix];
      r.re = f * r.re;
      r.im = f * r.im;
    }
    st_c(out, ix, r);
  }
}

template <typename T, int N>
__global__ void __launch_bounds__(N / 8)
    k_fft_bwd_reg(FftBatch b, const T *__restrict__ phs, const cplx<T> *__restrict__ tw) {
  pdl_wait();
  __shared__ cplx<T> sm[RegFft<N>::SMEM_PTS];
  constexpr int TH = N / 8;
  const int j = threadIdx.x, e = blockIdx.y;
  const long row = blockIdx.x;
  const T *in = (const T *)b.in[e] + row * N * 2;
  cplx<T> v[8];
#pragma unroll
  for (int r = 0; r < 8; r++) v[r] = mul_phs(ld_c(in, j + r * TH), ld_c(phs, j + r * TH));
  fft_reg<T, true, N>(v, sm, tw);
  const T inv_n = (T)(1.0 / (double)N);
  T *out = (T *)b.out[e];
  const long ld = b.ld[e];
  if (b.real[e]) {
#pragma unroll
    for (int q = 0; q < 8; q++) out[row * ld + j + q * TH] = v[q].re * inv_n;
  } else {
#pragma unroll
    for (int q = 0; q < 8; q++) {
      cplx<T> r = {v[q].re * inv_n, v[q].im * inv_n};
      st_c(out, row * ld + j + q * TH, r);
    }
  }
}

template <typename T, int N>
__global__ void __launch_bounds__(N / 8, sizeof(T) == 4 && N <= 2048 ? 6144 / N : 1)
    k_damp_reg(FftBatch b, const T *__restrict__ phs_p, const T *__restrict__ phs_m,
               const T *__restrict__ prof, u32 nf, const cplx<T> *__restrict__ tw) {
  pdl_wait();
  __shared__ cplx<T> sm[RegFft<N>::SMEM_PTS];
  constexpr int TH = N / 8;
  const int j = threadIdx.x, e = blockIdx.y;
  const u32 un = (u32)N;
  const long row = blockIdx.x;
  T *spec = (T *)b.out[e] + row * N * 2;
  T *rs = (T *)b.filt[e];
  const bool rs_real = b.real[e] != 0;
  cplx<T> v[8];
#pragma unroll
  for (int r = 0; r < 8; r++) v[r] = mul_phs(ld_c(spec, j + r * TH), ld_c(phs_p, j + r * TH));
  fft_reg<T, true, N>(v, sm, tw);
  const T inv_n = (T)(1.0 / (double)N);
#pragma unroll
  for (int q = 0; q < 8; q++) {
    const u32 ux = (u32)(j + q * TH);
    cplx<T> w = v[q];
    w.re = w.re * inv_n;
    w.im = rs_real ? T(0) : w.im * inv_n;
    if constexpr (DAMP_INCREMENT<T>) {
      const T f = damp_factor(prof, ux, un, nf), fm1 = f - T(1);
      v[q] = {w.re * fm1, w.im * fm1};
      w.re *= f;
      w.im *= f;
    } else {
      if (ux < nf) { w.re *= prof[ux]; w.im *= prof[ux]; }
      if (ux > un - nf) { w.re *= prof[un - ux]; w.im *= prof[un - ux]; }
      v[q] = w;
    }
    if (rs_real) rs[(row + 1) * N + ux] = w.re;
    else st_c(rs, (row + 1) * N + ux, w);
    if (row == 0) {  // the ghost row is damped in place as well
      if (rs_real) {
        T g = rs[ux];
        if (ux < nf) g *= prof[ux];
        if (ux > un - nf) g *= prof[un - ux];
        rs[ux] = g;
      } else {
        cplx<T> g = ld_c(rs, ux);
        if (ux < nf) { g.re *= prof[ux]; g.im *= prof[ux]; }
        if (ux > un - nf) { g.re *= prof[un - ux]; g.im *= prof[un - ux]; }
        st_c(rs, ux, g);
      }
    }
  }
  fft_reg<T, false, N>(v, sm, tw);
#pragma unroll
  for (int q = 0; q < 8; q++) {
    cplx<T> o = mul_phs(v[q], ld_c(phs_m, j + q * TH));
    if constexpr (DAMP_INCREMENT<T>) {
      const cplx<T> x = ld_c(spec, j + q * TH);
      o.re = x.re + o.re;
      o.im = x.im + o.im;
    }
    st_c(spec, j + q * TH, o);
  }
}

// (double at N = 4096 would need more than the 48 KB of static shared memory)
template <typename T> static bool reg_size(int n) {
  return n == 512 || n == 1024 || n == 2048 || (n == 4096 && sizeof(T) == 4);
}

#define CCL_REG_DISPATCH(N_, LAUNCH)                     \
  switch (N_) {                                          \
    case 512: LAUNCH(512); break;                        \
    case 1024: LAUNCH(1024); break;                      \
    case 2048: LAUNCH(2048); break;                      \
    case 4096:                                           \
      if constexpr (sizeof(T) == 4) { LAUNCH(4096); }    \
      break;                                             \
  }

// ---------------------------------------------------------------------
// Twiddle tables W_N^t = e^{-2 pi i t/N}, built once per (device, N, type)
// by a device kernel (sincospi) and kept for the life of the process.
template <typename T> __global__ void k_twiddles(int n, cplx<T> *tw) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n;
       t += gridDim.x * blockDim.x) {
    double s, c;
    sincospi(2.0 * (double)t / (double)n, &s, &c);
    cplx<T> w = {(T)c, (T)(-s)};
    tw[t] = w;
  }
}

// A table enters the cache only once it is complete (the building stream
// is synchronised), so a call on another stream or host thread never reads
// a table still being written.  Building one inside a stream capture would
// only record the kernel (and cudaMalloc is not allowed there): the first
// transform of each length must run outside any capture, else *why is set
// and nullptr returned.
template <typename T>
static const cplx<T> *twiddles(int n, cudaStream_t s, const char **why) {
  static std::mutex mu;
  static std::map<std::pair<int, int>, void *> cache;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    *why = "cudaGetDevice failed";
    return nullptr;
  }
  std::lock_guard<std::mutex> lk(mu);
  auto key = std::make_pair(dev, n);
  auto it = cache.find(key);
  if (it != cache.end()) return (const cplx<T> *)it->second;
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &cap) != cudaSuccess || cap != cudaStreamCaptureStatusNone) {
    *why = "first transform of this length inside a stream capture (run one outside it first)";
    return nullptr;
  }
  void *p = nullptr;
  if (cudaMalloc(&p, sizeof(cplx<T>) * (size_t)n) != cudaSuccess) {
    *why = "cudaMalloc failed";
    return nullptr;
  }
  k_twiddles<T><<<(n + 255) / 256, 256, 0, s>>>(n, (cplx<T> *)p);
  if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(s) != cudaSuccess) {
    cudaFree(p);
    *why = "twiddle kernel failed";
    return nullptr;
  }
  cache[key] = p;
  return (const cplx<T> *)p;
}

template <typename T> static int fft_check(int nx, FftPlan *pl, size_t *smem) {
  const int nmax = sizeof(T) == 8 ? 4096 : 8192;
  CCL_REQUIRE(nx >= 2 && nx <= nmax, CCL_ERR_UNSUPPORTED,
              "fft: nx=%d outside [2, %d]", nx, nmax);
  CCL_REQUIRE(make_plan(nx, pl), CCL_ERR_UNSUPPORTED,
              "fft: nx=%d has prime factors above 13", nx);
  *smem = 2 * sizeof(cplx<T>) * (size_t)nx;
  return CCL_OK;
}

// Raise a kernel's dynamic shared-memory limit once per size (not on every
// launch, so that steady-state steps issue launches only).
template <typename K> static void allow_smem(K kernel, size_t smem) {
  if (smem <= 48 * 1024) return;
  static std::mutex mu;
  static std::map<const void *, size_t> done;
  std::lock_guard<std::mutex> lk(mu);
  size_t &v = done[(const void *)kernel];
  if (v < smem) {
    cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    v = smem;
  }
}

static int batch_check(int batch, int nrows) {
  CCL_REQUIRE(batch >= 0 && batch <= FFT_MAXBATCH, CCL_ERR_ARG,
              "fft: batch %d outside [0, %d]", batch, FFT_MAXBATCH);
  CCL_REQUIRE(nrows >= 0 && nrows <= 65535 * 32, CCL_ERR_ARG, "fft: nrows %d",
              nrows);
  return CCL_OK;
}

template <typename T>
int fft_forward_batch(int batch, int nrows, int nx, const void *const *in,
                      const long *in_ld, const int *in_real, void *const *out,
                      const void *phs, const void *const *filt,
                      cudaStream_t s) {
  FftPlan pl;
  size_t smem;
  int rc = fft_check<T>(nx, &pl, &smem);
  if (rc) return rc;
  if ((rc = batch_check(batch, nrows))) return rc;
  if (nrows == 0 || batch == 0) return CCL_OK;
  FftBatch b;
  for (int i = 0; i < batch; i++) {
    CCL_REQUIRE(in[i] && out[i], CCL_ERR_ARG, "fft: null operand %d", i);
    CCL_REQUIRE(in_ld[i] >= nx, CCL_ERR_ARG, "fft: entry %d ld %ld < nx", i,
                in_ld[i]);
    b.in[i] = in[i];
    b.out[i] = out[i];
    b.filt[i] = filt ? filt[i] : nullptr;
    b.ld[i] = in_ld[i];
    b.real[i] = in_real[i];
  }
  const char *why = "";
  const cplx<T> *tw = twiddles<T>(nx, s, &why);
  CCL_REQUIRE(tw, CCL_ERR_CUDA, "fft: twiddle table for nx=%d: %s", nx, why);
  if (reg_size<T>(nx)) {
#define CCL_L(NN) \
  launch_pdl(k_fft_fwd_reg<T, NN>, dim3(nrows, batch), NN / 8, 0, s, b, (const T *)phs, tw)
    CCL_REG_DISPATCH(nx, CCL_L)
#undef CCL_L
  } else {
    auto kern = k_fft_fwd<T>;
    allow_smem(kern, smem);
    kern<<<dim3(nrows, batch), FFT_THREADS, smem, s>>>(pl, b, (const T *)phs, tw);
  }
  CCL_LAUNCH_CHECK("fft_forward");
  return CCL_OK;
}

template <typename T>
int fft_backward_batch(int batch, int nrows, int nx, const void *const *in,
                       void *const *out, const long *out_ld,
                       const int *out_real, const void *phs, cudaStream_t s) {
  FftPlan pl;
  size_t smem;
  int rc = fft_check<T>(nx, &pl, &smem);
  if (rc) return rc;
  if ((rc = batch_check(batch, nrows))) return rc;
  if (nrows == 0 || batch == 0) return CCL_OK;
  FftBatch b;
  for (int i = 0; i < batch; i++) {
    CCL_REQUIRE(in[i] && out[i], CCL_ERR_ARG, "fft: null operand %d", i);
    CCL_REQUIRE(out_ld[i] >= nx, CCL_ERR_ARG, "fft: entry %d ld %ld < nx", i,
                out_ld[i]);
    b.in[i] = in[i];
    b.out[i] = out[i];
    b.filt[i] = nullptr;
    b.ld[i] = out_ld[i];
    b.real[i] = out_real[i];
  }
  const char *why = "";
  const cplx<T> *tw = twiddles<T>(nx, s, &why);
  CCL_REQUIRE(tw, CCL_ERR_CUDA, "fft: twiddle table for nx=%d: %s", nx, why);
  if (reg_size<T>(nx)) {
#define CCL_L(NN) \
  launch_pdl(k_fft_bwd_reg<T, NN>, dim3(nrows, batch), NN / 8, 0, s, b, (const T *)phs, tw)
    CCL_REG_DISPATCH(nx, CCL_L)
#undef CCL_L
  } else {
    auto kern = k_fft_bwd<T>;
    allow_smem(kern, smem);
    kern<<<dim3(nrows, batch), FFT_THREADS, smem, s>>>(pl, b, (const T *)phs, tw);
  }
  CCL_LAUNCH_CHECK("fft_backward");
  return CCL_OK;
}

template <typename T>
int damp_batch(int batch, int nrows, int nx, void *const *spec,
               void *const *rs, const int *rs_real, const void *phs_p,
               const void *phs_m, const void *prof, int nf, cudaStream_t s) {
  FftPlan pl;
  size_t smem;
  int rc = fft_check<T>(nx, &pl, &smem);
  if (rc) return rc;
  if ((rc = batch_check(batch, nrows))) return rc;
  CCL_REQUIRE(nf >= 0, CCL_ERR_ARG, "damp: nf=%d", nf);
  if (nrows == 0 || batch == 0) return CCL_OK;
  FftBatch b;
  for (int i = 0; i < batch; i++) {
    CCL_REQUIRE(spec[i] && rs[i], CCL_ERR_ARG, "damp: null operand %d", i);
    b.in[i] = spec[i];
    b.out[i] = spec[i];
    b.filt[i] = rs[i];
    b.ld[i] = nx;
    b.real[i] = rs_real[i];
  }
  const char *why = "";
  const cplx<T> *tw = twiddles<T>(nx, s, &why);
  CCL_REQUIRE(tw, CCL_ERR_CUDA, "fft: twiddle table for nx=%d: %s", nx, why);
  if (reg_size<T>(nx)) {
#define CCL_L(NN)                                                                           \
  launch_pdl(k_damp_reg<T, NN>, dim3(nrows, batch), NN / 8, 0, s, b, (const T *)phs_p,        \
             (const T *)phs_m, (const T *)prof, (u32)nf, tw)
    CCL_REG_DISPATCH(nx, CCL_L)
#undef CCL_L
  } else {
    auto kern = k_damp<T>;
    allow_smem(kern, smem);
    kern<<<dim3(nrows, batch), FFT_THREADS, smem, s>>>(
        pl, b, (const T *)phs_p, (const T *)phs_m, (const T *)prof, (u32)nf, tw);
  }
  CCL_LAUNCH_CHECK("damp");
  return CCL_OK;
}

template <typename T>
int fft_forward_rows(int nrows, int nx, const T *in, long in_ld, int in_real,
                     T *out, const T *phs, const T *filt, cudaStream_t s) {
  const void *i[1] = {in};
  void *o[1] = {out};
  const void *f[1] = {filt};
  long ld[1] = {in_ld};
  int r[1] = {in_real};
  return fft_forward_batch<T>(1, nrows, nx, i, ld, r, o, phs, f, s);
}

template <typename T>
int fft_backward_rows(int nrows, int nx, const T *in, T *out, long out_ld,
                      int out_real, const T *phs, cudaStream_t s) {
  const void *i[1] = {in};
  void *o[1] = {out};
  long ld[1] = {out_ld};
  int r[1] = {out_real};
  return fft_backward_batch<T>(1, nrows, nx, i, o, ld, r, phs, s);
}

template <typename T>
int damp_rows(int nrows, int nx, T *spec, T *rs, int rs_real, const T *phs_p,
              const T *phs_m, const T *prof, int nf, cudaStream_t s) {
  void *sp[1] = {spec}, *r[1] = {rs};
  int re[1] = {rs_real};
  return damp_batch<T>(1, nrows, nx, sp, r, re, phs_p, phs_m, prof, nf, s);
}

#define CCL_INST_FFT(T)                                                        \
  template int fft_forward_rows<T>(int, int, const T *, long, int, T *,       \
                                   const T *, const T *, cudaStream_t);        \
  template int fft_backward_rows<T>(int, int, const T *, T *, long, int,      \
                                    const T *, cudaStream_t);                  \
  template int damp_rows<T>(int, int, T *, T *, int, const T *, const T *,    \
                            const T *, int, cudaStream_t);                     \
  template int fft_forward_batch<T>(int, int, int, const void *const *,       \
                                    const long *, const int *, void *const *, \
                                    const void *, const void *const *,        \
                                    cudaStream_t);                             \
  template int fft_backward_batch<T>(int, int, int, const void *const *,      \
                                     void *const *, const long *, const int *,\
                                     const void *, cudaStream_t);              \
  template int damp_batch<T>(int, int, int, void *const *, void *const *,     \
                             const int *, const void *, const void *,         \
                             const void *, int, cudaStream_t);
CCL_INST_FFT(double)
CCL_INST_FFT(float)

}  // namespace ccl
