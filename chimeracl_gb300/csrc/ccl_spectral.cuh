// Streaming spectral-space kernels: PSATD update, phase factors, m=-1
// mirror, edge profile and the complex BLAS-1 set of the reference's
// generic.cl.  All HBM-bound; grid-stride loops over whole arrays.  Each
// expression keeps the reference's operation order (the FP64 instantiation is
// compiled without FMA contraction).
#pragma once
#include "ccl_common.cuh"

namespace ccl {

#define CCL_GRID_STRIDE(i, n)                                                  \
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < (n);         \
       i += (long)gridDim.x * blockDim.x)

// advance_e_g_m (solver_ms_pic.cl:57-143); f: E xyz, G xyz, J xyz, N0 xyz,
// N1 xyz.
template <typename T>
__global__ void __launch_bounds__(256)
    k_psatd(long n, T dt_inv, const T *__restrict__ c1m,
            const T *__restrict__ c2m, const T *__restrict__ c3m,
            ptrs<15> f) {
  pdl_wait();
  const T pi2 = T(2) * T(M_PI);
  CCL_GRID_STRIDE(i, n) {
    const T c1 = c1m[i], c2 = c2m[i], c3 = c3m[i];
#pragma unroll
    for (int k = 0; k < 3; k++) {
      cplx<T> E0 = ld_c((const T *)f.p[k], i), G0 = ld_c((const T *)f.p[3 + k], i);
      cplx<T> J0 = ld_c((const T *)f.p[6 + k], i);
      cplx<T> A0 = ld_c((const T *)f.p[9 + k], i), A1 = ld_c((const T *)f.p[12 + k], i);
      T e0[2] = {E0.re, E0.im}, g0[2] = {G0.re, G0.im};
      T j0[2] = {J0.re * pi2, J0.im * pi2};
      T n0[2] = {A0.re * pi2, A0.im * pi2}, n1[2] = {A1.re * pi2, A1.im * pi2};
      T e1[2], g1[2];
#pragma unroll
      for (int q = 0; q < 2; q++) {
        e1[q] = c1 * e0[q] + c2 * c3 * (g0[q] - j0[q]) +
                c3 * (c1 * n0[q] - n1[q] - (n0[q] - n1[q]) * dt_inv * c2 * c3);
        g1[q] = -c2 * e0[q] + c1 * (g0[q] - j0[q]) + j0[q] +
                c3 * (dt_inv * (T(1) - c1) * (n0[q] - n1[q]) - c2 * n0[q]);
      }
      cplx<T> E1 = {e1[0], e1[1]}, G1 = {g1[0], g1[1]};
      st_c((T *)f.p[k], i, E1);
      st_c((T *)f.p[3 + k], i, G1);
    }
  }
}

// The same update written with coefficients that carry no cancellation
// (formed in double on the host, x = w dt, 2 pi folded in):
//   e1 = c1 e0 + s g0 - s2 j0 + a2 n0 + b2 n1
//   g1 = -c2 e0 + c1 g0 + q2 j0 + d2 (n0 - n1) - s2 n0
// with c1 = cos x, c2 = w sin x, s = sin x / w, s2 = 2 pi s,
// q2 = 2 pi (1 - cos x), a2 = 2 pi (cos x - sin x / x) / w^2,
// b2 = 2 pi (sin x / x - 1) / w^2, d2 = 2 pi (1 - cos x) / (w^2 dt).
// Algebraically the reference's expressions; but where those form the small
// terms of the long-wavelength modes (x ~ 1e-3: O(x^2) results from O(1)
// differences, c1 (g0 - j0) + j0 for (1 - cos x) j0) they lose
// log10(1/x^2) digits, which FP32 cannot spare: at a plasma wake's x the
// charge and current terms would keep 1 to 2 digits.  coef holds the eight
// values per element, in that order.
template <typename T>
__global__ void __launch_bounds__(256)
    k_psatd_split(long n, const T *__restrict__ coef, ptrs<15> f) {
  pdl_wait();
  CCL_GRID_STRIDE(i, n) {
    T c[8];
    if constexpr (sizeof(T) == 4) {  // two 16-byte loads (the array is 32-byte aligned)
      const float4 a = ((const float4 *)coef)[2 * i], b = ((const float4 *)coef)[2 * i + 1];
      c[0] = a.x, c[1] = a.y, c[2] = a.z, c[3] = a.w, c[4] = b.x, c[5] = b.y, c[6] = b.z,
      c[7] = b.w;
    } else {
#pragma unroll
      for (int k = 0; k < 8; k++) c[k] = coef[8 * i + k];
    }
    const T c1 = c[0], c2 = c[1], s = c[2], s2 = c[3], q2 = c[4], a2 = c[5], b2 = c[6],
            d2 = c[7];
#pragma unroll
    for (int k = 0; k < 3; k++) {
      const cplx<T> E0 = ld_c((const T *)f.p[k], i), G0 = ld_c((const T *)f.p[3 + k], i);
      const cplx<T> J0 = ld_c((const T *)f.p[6 + k], i);
      const cplx<T> N0 = ld_c((const T *)f.p[9 + k], i), N1 = ld_c((const T *)f.p[12 + k], i);
      const T e0[2] = {E0.re, E0.im}, g0[2] = {G0.re, G0.im}, j0[2] = {J0.re, J0.im};
      const T n0[2] = {N0.re, N0.im}, n1[2] = {N1.re, N1.im};
      T e1[2], g1[2];
#pragma unroll
      for (int q = 0; q < 2; q++) {
        e1[q] = c1 * e0[q] + s * g0[q] - s2 * j0[q] + a2 * n0[q] + b2 * n1[q];
        g1[q] = -c2 * e0[q] + c1 * g0[q] + q2 * j0[q] + d2 * (n0[q] - n1[q]) - s2 * n0[q];
      }
      st_c((T *)f.p[k], i, cplx<T>{e1[0], e1[1]});
      st_c((T *)f.p[3 + k], i, cplx<T>{g1[0], g1[1]});
    }
  }
}

// get_phase_plus / get_phase_minus (transformer_generic.cl:28-55); computed
// in double whatever T is.
template <typename T>
__global__ void k_phase(int nx, T *phs, const double *kx, double x0,
                        int sign) {
  CCL_GRID_STRIDE(i, nx) {
    double a = x0 * kx[i];
    double s = sin(a), c = cos(a);
    phs[2 * i] = (T)c;
    phs[2 * i + 1] = (T)(sign > 0 ? s : -s);
  }
}

// multiply_by_phase (transformer_generic.cl:58-80)
template <typename T>
__global__ void k_mul_phase(long n, int nx, T *a, const T *phs) {
  CCL_GRID_STRIDE(i, n) {
    long ix = i % nx;
    cplx<T> v = ld_c(a, i), p = ld_c(phs, ix);
    cplx<T> r = {(v.re * p.re - v.im * p.im), (v.re * p.im + v.im * p.re)};
    st_c(a, i, r);
  }
}

// get_m1 (transformer_generic.cl:3-24)
template <typename T>
__global__ void k_get_m1(long n, int nx, T *out, const T *in) {
  CCL_GRID_STRIDE(i, n) {
    long ir = i / nx, ix = i - ir * nx;
    long io = ix == 0 ? 0 : nx - ix;
    cplx<T> v = ld_c(in, io + ir * nx);
    cplx<T> r = {-v.re, v.im};
    st_c(out, i, r);
  }
}

// profile_edges_c / _d (solver_ms_pic.cl:5-55), unsigned index arithmetic
template <typename T>
__global__ void k_profile_edges(long n, u32 nx, int cplxf, T *a,
                                const T *f, u32 nf) {
  CCL_GRID_STRIDE(i, n) {
    u32 ir = (u32)(i / nx), ix = (u32)i - ir * nx;
    const int nc = cplxf ? 2 : 1;
    if (ix < nf)
      for (int c = 0; c < nc; c++) a[nc * i + c] *= f[ix];
    if (ix > nx - nf)
      for (int c = 0; c < nc; c++) a[nc * i + c] *= f[nx - ix];
  }
}

template <typename T>
__global__ void k_set(long n, int cplxf, T *a, T re, T im) {
  CCL_GRID_STRIDE(i, n) {
    if (cplxf) {
      a[2 * i] = re;
      a[2 * i + 1] = im;
    } else {
      a[i] = re;
    }
  }
}

// set over a batch of arrays: blockIdx.y = array
struct SetBatch {
  void *a[32];
  long n[32];
  int cplx[32];
};
template <typename T>
__global__ void k_set_batch(SetBatch b, T re, T im) {
  pdl_wait();
  const int e = blockIdx.y;
  T *a = (T *)b.a[e];
  const long n = b.n[e];
  if (b.cplx[e]) {
    CCL_GRID_STRIDE(i, n) {
      a[2 * i] = re;
      a[2 * i + 1] = im;
    }
  } else {
    CCL_GRID_STRIDE(i, n) a[i] = re;
  }
}

// append_c2c (generic.cl:18-29)
template <typename T>
__global__ void k_append(long n, T *base, const T *add) {
  CCL_GRID_STRIDE(i, n) {
    cplx<T> b = ld_c(base, i), d = ld_c(add, i);
    cplx<T> r = {b.re + d.re, b.im + d.im};
    st_c(base, i, r);
  }
}

// zpaxz_c2c (generic.cl:32-44)
template <typename T>
__global__ void k_zpaxz(long n, T *z, T are, T aim, const T *x) {
  CCL_GRID_STRIDE(i, n) {
    cplx<T> v = ld_c(x, i), w = ld_c(z, i);
    cplx<T> r = {w.re + are * v.re - aim * v.im, w.im + are * v.im + aim * v.re};
    st_c(z, i, r);
  }
}

// axpbyz_c2c (generic.cl:61-77)
template <typename T>
__global__ void k_axpbyz(long n, T are, T aim, const T *x, T bre, T bim,
                         const T *y, T *z) {
  CCL_GRID_STRIDE(i, n) {
    cplx<T> u = ld_c(x, i), v = ld_c(y, i);
    cplx<T> r = {are * u.re - aim * u.im + bre * v.re - bim * v.im,
                 are * u.im + aim * u.re + bre * v.im + bim * v.re};
    st_c(z, i, r);
  }
}

// mult_elementwise_d2c (generic.cl:47-58)
template <typename T>
__global__ void k_mult_elem(long n, const T *x, T *z) {
  CCL_GRID_STRIDE(i, n) {
    cplx<T> v = ld_c(z, i);
    T s = x[i];
    cplx<T> r = {s * v.re, s * v.im};
    st_c(z, i, r);
  }
}

// ab_dot_x (generic.cl:82-99)
template <typename T>
__global__ void k_ab_dot_x(long n, int nx, T are, T aim, const T *b,
                           const T *x, T *z) {
  CCL_GRID_STRIDE(i, n) {
    long ix = i % nx;
    cplx<T> v = ld_c(x, i);
    T bb = b[ix];
    cplx<T> r = {bb * (are * v.re - aim * v.im), bb * (are * v.im + aim * v.re)};
    st_c(z, i, r);
  }
}

// cast_array_d2c (generic.cl:102-112): real part
template <typename T>
__global__ void k_cast_c2d(long n, const T *in, T *out) {
  CCL_GRID_STRIDE(i, n) out[i] = in[2 * i];
}

// ---------------------------------------------------------------------
// Spectral gradient and curl, combine step.  The radial derivative matrix
// products arrive precomputed (one batched GEMM launch): for mode m,
//   Pm[m] = dDHT_minus_m . f_{m-1}  (for m = 0: dDHT_minus_0 . f_{+1}, read
//           here through the m=-1 mirror (-Re, +Im) at column (nx-ix) mod nx,
//           which commutes with the real radial matrix), Pp[m] = dDHT_plus_m .
//           f_{m+1}; NULL where the reference has no such term.
// Gradient (transformer_methods_cl.py:87-133):
//   Nx = i kx rho_m,  Ny = -T- + T+,  Nz = -i (T- + T+).
template <typename T>
__device__ __forceinline__ cplx<T> ld_mode(const T *p, long i, long ir, long ix, int nx,
                                           bool mirror) {
  if (!p) {
    cplx<T> z = {T(0), T(0)};
    return z;
  }
  if (!mirror) return ld_c(p, i);
  const long io = ix == 0 ? 0 : nx - ix;
  cplx<T> q = ld_c(p, ir * nx + io);
  q.re = -q.re;
  return q;
}

template <typename T>
__global__ void __launch_bounds__(RC_THREADS)
    k_grad_combine(int nx, const T *__restrict__ kx, ptrs<4> rho, ptrs<4> Pm, ptrs<4> Pp,
                   ptrs<12> dN) {
  pdl_wait();
  constexpr int RP = RcPer<T>;
  const int m = blockIdx.y;
  const RowChunk<T> rc(nx);
  const T *rh = (const T *)pick(rho, m), *pmm = (const T *)pick(Pm, m),
          *ppm = (const T *)pick(Pp, m);
  T *ox = (T *)pick(dN, 3 * m), *oy = (T *)pick(dN, 3 * m + 1), *oz = (T *)pick(dN, 3 * m + 2);
  cplx<T> r[RP], tm[RP], tp[RP];
#pragma unroll
  for (int q = 0; q < RP; q++) {
    const int ix = rc.col(q);
    if (ix < nx) {
      const long i = (long)rc.ir * nx + ix;
      r[q] = ld_c(rh, i);
      tm[q] = ld_mode(pmm, i, rc.ir, ix, nx, m == 0);
      tp[q] = ld_mode(ppm, i, rc.ir, ix, nx, false);
    }
  }
#pragma unroll
  for (int q = 0; q < RP; q++) {
    const int ix = rc.col(q);
    if (ix < nx) {
      const long i = (long)rc.ir * nx + ix;
      const T k = kx[ix];
      const cplx<T> gx = {k * (-r[q].im), k * r[q].re};
      const cplx<T> gy = {-tm[q].re + tp[q].re, -tm[q].im + tp[q].im};
      const cplx<T> gz = {tm[q].im + tp[q].im, -(tm[q].re + tp[q].re)};
      st_c(ox, i, gx);
      st_c(oy, i, gy);
      st_c(oz, i, gz);
    }
  }
}

// Curl (transformer_methods_cl.py:185-263), with U-_c, U+_c the products of
// component c (same mirror rule), times the Poisson factor 1/w^2 of
// field_poiss_vec when `poiss` is given:
//   Bx = (-U-_z + i U-_y) + (U+_z + i U+_y)
//   By = -i (kx Gz + U-_x + U+_x)
//   Bz = i kx Gy + U-_x - U+_x
template <typename T>
__global__ void __launch_bounds__(RC_THREADS)
    k_rot_combine(int nx, const T *__restrict__ kx, ptrs<12> G, ptrs<12> Qm, ptrs<12> Qp,
                  ptrs<4> poiss, ptrs<12> B) {
  pdl_wait();
  constexpr int RP = RcPer<T>;
  const int m = blockIdx.y;
  const RowChunk<T> rc(nx);
  const T *po = (const T *)pick(poiss, m);
  const T *gyp = (const T *)pick(G, 3 * m + 1), *gzp = (const T *)pick(G, 3 * m + 2);
  const T *qmp[3], *qpp[3];
  T *bp[3];
#pragma unroll
  for (int c = 0; c < 3; c++) {
    qmp[c] = (const T *)pick(Qm, 3 * m + c);
    qpp[c] = (const T *)pick(Qp, 3 * m + c);
    bp[c] = (T *)pick(B, 3 * m + c);
  }
  cplx<T> gy[RP], gz[RP], um[RP][3], up[RP][3];
  T f[RP];
#pragma unroll
  for (int q = 0; q < RP; q++) {
    const int ix = rc.col(q);
    if (ix < nx) {
      const long i = (long)rc.ir * nx + ix;
      gy[q] = ld_c(gyp, i);
      gz[q] = ld_c(gzp, i);
#pragma unroll
      for (int c = 0; c < 3; c++) {
        um[q][c] = ld_mode(qmp[c], i, rc.ir, ix, nx, m == 0);
        up[q][c] = ld_mode(qpp[c], i, rc.ir, ix, nx, false);
      }
      f[q] = po ? po[i] : T(1);
    }
  }
#pragma unroll
  for (int q = 0; q < RP; q++) {
    const int ix = rc.col(q);
    if (ix < nx) {
      const long i = (long)rc.ir * nx + ix;
      const T k = kx[ix];
      cplx<T> bx = {-um[q][2].re - um[q][1].im + up[q][2].re - up[q][1].im,
                    -um[q][2].im + um[q][1].re + up[q][2].im + up[q][1].re};
      const cplx<T> sy = {k * gz[q].re + um[q][0].re + up[q][0].re,
                          k * gz[q].im + um[q][0].im + up[q][0].im};
      cplx<T> by = {sy.im, -sy.re};
      cplx<T> bz = {-k * gy[q].im + um[q][0].re - up[q][0].re,
                    k * gy[q].re + um[q][0].im - up[q][0].im};
      if (po) {
        bx.re *= f[q]; bx.im *= f[q];
        by.re *= f[q]; by.im *= f[q];
        bz.re *= f[q]; bz.im *= f[q];
      }
      st_c(bp[0], i, bx);
      st_c(bp[1], i, by);
      st_c(bp[2], i, bz);
    }
  }
}

}  // namespace ccl
