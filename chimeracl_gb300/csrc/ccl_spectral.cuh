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

}  // namespace ccl
