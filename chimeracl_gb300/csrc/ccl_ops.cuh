// Ops<T>: launch wrappers of the particle, grid and elementwise kernels for
// one real type.  Included by ccl_f64.cu (compiled without FMA contraction:
// the plain FP64 drop-in reproduces the reference's rounding) and by
// ccl_f32.cu (FMA on).
#pragma once
#include "ccl_grid.cuh"
#include "ccl_launch.h"
#include "ccl_particles.cuh"
#include "ccl_spectral.cuh"

namespace ccl {

template <typename T>
int Ops<T>::push_x(long np, void *x, void *y, void *z, const void *px,
                   const void *py, const void *pz, const void *g_inv, double dt,
                   cudaStream_t s) {
  return ccl::push_x<T>(np, (T *)x, (T *)y, (T *)z, (const T *)px,
                        (const T *)py, (const T *)pz, (const T *)g_inv, dt, s);
}

template <typename T>
int Ops<T>::push_x_comp(long np, void *x, void *y, void *z, void *xl, void *yl, void *zl,
                        const void *px, const void *py, const void *pz, const void *g_inv,
                        double dt, cudaStream_t s) {
  return ccl::push_x_comp<T>(np, (T *)x, (T *)y, (T *)z, (T *)xl, (T *)yl, (T *)zl,
                             (const T *)px, (const T *)py, (const T *)pz, (const T *)g_inv,
                             dt, s);
}

template <typename T>
int Ops<T>::index_sort(long np, const void *x, const void *y, const void *z,
                       int Nx, double xmin, double dx_inv, int Nr, double rmin,
                       double dr_inv, uint32_t *indx, uint32_t *counts,
                       uint32_t *cell_offset, uint32_t *sort_indx,
                       uint32_t *np_stay, void *ws, size_t ws_bytes,
                       cudaStream_t s) {
  const GridP<T> g = make_gridp<T>(Nx, Nr, xmin, dx_inv, rmin, dr_inv);
  return ccl::index_sort<T>(np, (const T *)x, (const T *)y, (const T *)z, g,
                            indx, counts, cell_offset, sort_indx, np_stay, ws,
                            ws_bytes, s);
}

template <typename T>
int Ops<T>::push_x_keys(long np, void *x, void *y, void *z, void *xl, void *yl, void *zl,
                        const void *px, const void *py, const void *pz, const void *g_inv,
                        double dt, int Nx, double xmin, double dx_inv, int Nr, double rmin,
                        double dr_inv, uint32_t *indx, uint32_t *counts, void *ws,
                        size_t ws_bytes, cudaStream_t s) {
  const GridP<T> g = make_gridp<T>(Nx, Nr, xmin, dx_inv, rmin, dr_inv);
  return ccl::push_keys<T>(np, (T *)x, (T *)y, (T *)z, (T *)xl, (T *)yl, (T *)zl,
                           (const T *)px, (const T *)py, (const T *)pz, (const T *)g_inv, dt,
                           g, indx, counts, ws, ws_bytes, s);
}

template <typename T>
int Ops<T>::align(long n, int ncomp, void *const *src, void *const *dst,
                  const uint32_t *idx, cudaStream_t s) {
  return ccl::align<T>(n, ncomp, src, dst, idx, s);
}

template <typename T>
int Ops<T>::fill_grid(long ncells, void *x, void *y, void *z, void *w,
                      const double *theta, const double *xgrid,
                      const double *rgrid, uint32_t Nx, uint32_t npx,
                      uint32_t npr, uint32_t npth, cudaStream_t s) {
  if (ncells == 0) return CCL_OK;
  k_fill_grid<T><<<grid_for(ncells, 128), 128, 0, s>>>(
      ncells, (T *)x, (T *)y, (T *)z, (T *)w, theta, xgrid, rgrid, Nx, npx,
      npr, npth);
  CCL_LAUNCH_CHECK("fill_grid");
  return CCL_OK;
}

template <typename T>
int Ops<T>::dens_profile(long np, const void *x, void *w, const double *xx,
                         const double *ff, const double *dxm1, uint32_t nloc,
                         cudaStream_t s) {
  if (np == 0) return CCL_OK;
  k_dens_profile<T><<<grid_for(np, 256), 256, 0, s>>>(np, (const T *)x,
                                                       (T *)w, xx, ff, dxm1,
                                                       nloc);
  CCL_LAUNCH_CHECK("dens_profile");
  return CCL_OK;
}

template <typename T>
int Ops<T>::gamma_inv(long np, const void *px, const void *py, const void *pz,
                      void *g, cudaStream_t s) {
  if (np == 0) return CCL_OK;
  k_gamma_inv<T><<<grid_for(np, 256), 256, 0, s>>>(
      np, (const T *)px, (const T *)py, (const T *)pz, (T *)g);
  CCL_LAUNCH_CHECK("gamma_inv");
  return CCL_OK;
}

template <typename T>
int Ops<T>::deposit(int vec, int M, const uint32_t *sort_indx,
                    const uint32_t *cell_off, const void *x, const void *y,
                    const void *z, const void *ux, const void *uy,
                    const void *uz, const void *g_inv, const void *w,
                    int charge, int Nx, double xmin, double dx_inv, int Nr,
                    double rmin, double dr_inv, void *const *flds,
                    cudaStream_t s, const void *const *lo) {
  const GridP<T> g = make_gridp<T>(Nx, Nr, xmin, dx_inv, rmin, dr_inv);
  const T *const *lt = (const T *const *)lo;
  if (vec)
    return ccl::deposit<T, true>(M, sort_indx, cell_off, (const T *)x,
                                 (const T *)y, (const T *)z, (const T *)ux,
                                 (const T *)uy, (const T *)uz,
                                 (const T *)g_inv, (const T *)w, charge, g,
                                 flds, s, lt);
  return ccl::deposit<T, false>(M, sort_indx, cell_off, (const T *)x,
                                (const T *)y, (const T *)z, nullptr, nullptr,
                                nullptr, nullptr, (const T *)w, charge, g,
                                flds, s, lt);
}

template <typename T>
int Ops<T>::postproc(int M, int nfld, void *const *flds, int Nx, int Nr,
                     const void *dv, cudaStream_t s) {
  int n = nfld * (M + 1);
  CCL_REQUIRE(n > 0 && n <= 32, CCL_ERR_ARG, "postproc: %d fields", n);
  ptrs<32> f;
  for (int i = 0; i < n; i++) {
    CCL_REQUIRE(flds[i], CCL_ERR_ARG, "postproc: null field %d", i);
    f.p[i] = flds[i];
  }
  if (Nr < 2) return CCL_OK;
  dim3 grid((Nx + 127) / 128, Nr - 1, n);
  launch_pdl(k_postproc<T>, grid, 128, 0, s, f, M + 1, Nx, Nr, (const T *)dv);
  CCL_LAUNCH_CHECK("postproc");
  return CCL_OK;
}

template <typename T>
int Ops<T>::warp_axis(int M, int nfld, void *const *flds, int Nx,
                      cudaStream_t s) {
  int n = nfld * (M + 1);
  CCL_REQUIRE(n > 0 && n <= 32, CCL_ERR_ARG, "warp_axis: %d fields", n);
  ptrs<32> f;
  for (int i = 0; i < n; i++) {
    CCL_REQUIRE(flds[i], CCL_ERR_ARG, "warp_axis: null field %d", i);
    f.p[i] = flds[i];
  }
  dim3 grid((Nx + 127) / 128, n);
  launch_pdl(k_warp_axis<T>, grid, 128, 0, s, f, M + 1, Nx);
  CCL_LAUNCH_CHECK("warp_axis");
  return CCL_OK;
}

template <typename T>
int Ops<T>::gather_push(int M, long np, const void *x, const void *y,
                        const void *z, void *px, void *py, void *pz,
                        void *g_inv, const uint32_t *sort_indx,
                        const uint32_t *np_stay, double factor_push, int Nx,
                        double xmin, double dx_inv, int Nr, double rmin,
                        double dr_inv, const void *const *flds,
                        cudaStream_t s) {
  const GridP<T> g = make_gridp<T>(Nx, Nr, xmin, dx_inv, rmin, dr_inv);
  return ccl::gather_push<T>(M, np, (const T *)x, (const T *)y, (const T *)z,
                             (T *)px, (T *)py, (T *)pz, (T *)g_inv, sort_indx,
                             np_stay, factor_push, g, flds, s);
}

template <typename T>
int Ops<T>::gather_push_cells(int M, long np, const void *x, const void *y,
                              const void *z, void *px, void *py, void *pz,
                              void *g_inv, const uint32_t *sort_indx,
                              const uint32_t *cell_offset, const uint32_t *np_stay,
                              double factor_push, int Nx, double xmin,
                              double dx_inv, int Nr, double rmin, double dr_inv,
                              const void *const *flds, cudaStream_t s,
                              const void *const *lo) {
  const GridP<T> g = make_gridp<T>(Nx, Nr, xmin, dx_inv, rmin, dr_inv);
  return ccl::gather_push_cells<T>(M, np, (const T *)x, (const T *)y, (const T *)z,
                                   (T *)px, (T *)py, (T *)pz, (T *)g_inv, sort_indx,
                                   cell_offset, np_stay, factor_push, g, flds, s,
                                   (const T *const *)lo);
}

template <typename T>
int Ops<T>::psatd(long n, double dt_inv, const void *c1, const void *c2,
                  const void *c3, void *const *flds, cudaStream_t s) {
  ptrs<15> f;
  for (int i = 0; i < 15; i++) {
    CCL_REQUIRE(flds[i], CCL_ERR_ARG, "psatd: null field %d", i);
    f.p[i] = flds[i];
  }
  if (n == 0) return CCL_OK;
  launch_pdl(k_psatd<T>, grid_for(n, 256), 256, 0, s, n, (T)dt_inv, (const T *)c1, (const T *)c2,
             (const T *)c3, f);
  CCL_LAUNCH_CHECK("psatd");
  return CCL_OK;
}

template <typename T>
int Ops<T>::psatd_split(long n, const void *coef, void *const *flds, cudaStream_t s) {
  ptrs<15> f;
  for (int i = 0; i < 15; i++) {
    CCL_REQUIRE(flds[i], CCL_ERR_ARG, "psatd_split: null field %d", i);
    f.p[i] = flds[i];
  }
  CCL_REQUIRE(((uintptr_t)coef & 15) == 0, CCL_ERR_ARG,
              "psatd_split: coefficient array not 16-byte aligned");
  if (n == 0) return CCL_OK;
  launch_pdl(k_psatd_split<T>, grid_for(n, 256), 256, 0, s, n, (const T *)coef, f);
  CCL_LAUNCH_CHECK("psatd_split");
  return CCL_OK;
}

template <typename T>
int Ops<T>::phase(int nx, void *phs, const double *kx, double x0, int sign,
                  cudaStream_t s) {
  k_phase<T><<<grid_for(nx, 256), 256, 0, s>>>(nx, (T *)phs, kx, x0, sign);
  CCL_LAUNCH_CHECK("phase");
  return CCL_OK;
}

template <typename T>
int Ops<T>::get_m1(int nrows, int nx, void *out, const void *in,
                   cudaStream_t s) {
  long n = (long)nrows * nx;
  if (n == 0) return CCL_OK;
  k_get_m1<T><<<grid_for(n, 256), 256, 0, s>>>(n, nx, (T *)out, (const T *)in);
  CCL_LAUNCH_CHECK("get_m1");
  return CCL_OK;
}

template <typename T>
int Ops<T>::set(int cplx, long n, void *a, double re, double im,
                cudaStream_t s) {
  if (n == 0) return CCL_OK;
  k_set<T><<<grid_for(n, 256), 256, 0, s>>>(n, cplx, (T *)a, (T)re, (T)im);
  CCL_LAUNCH_CHECK("set");
  return CCL_OK;
}

template <typename T>
int Ops<T>::set_batch(int narr, const int *cplx, const long *n, void *const *a, double re,
                      double im, cudaStream_t s) {
  SetBatch b;
  long nmax = 0;
  for (int i = 0; i < narr; i++) {
    b.a[i] = a[i];
    b.n[i] = n[i];
    b.cplx[i] = cplx[i];
    if (n[i] > nmax) nmax = n[i];
  }
  if (nmax == 0) return CCL_OK;
  dim3 grid((unsigned)((grid_for(nmax, 256) + narr - 1) / narr), (unsigned)narr);
  launch_pdl(k_set_batch<T>, grid, 256, 0, s, b, (T)re, (T)im);
  CCL_LAUNCH_CHECK("set_batch");
  return CCL_OK;
}

template <typename T>
int Ops<T>::append(long n, void *base, const void *add, cudaStream_t s) {
  if (n == 0) return CCL_OK;
  k_append<T><<<grid_for(n, 256), 256, 0, s>>>(n, (T *)base, (const T *)add);
  CCL_LAUNCH_CHECK("append_c2c");
  return CCL_OK;
}

template <typename T>
int Ops<T>::zpaxz(long n, void *z, double are, double aim, const void *x,
                  cudaStream_t s) {
  if (n == 0) return CCL_OK;
  k_zpaxz<T><<<grid_for(n, 256), 256, 0, s>>>(n, (T *)z, (T)are, (T)aim,
                                               (const T *)x);
  CCL_LAUNCH_CHECK("zpaxz");
  return CCL_OK;
}

template <typename T>
int Ops<T>::axpbyz(long n, double are, double aim, const void *x, double bre,
                   double bim, const void *y, void *z, cudaStream_t s) {
  if (n == 0) return CCL_OK;
  k_axpbyz<T><<<grid_for(n, 256), 256, 0, s>>>(n, (T)are, (T)aim, (const T *)x,
                                                (T)bre, (T)bim, (const T *)y,
                                                (T *)z);
  CCL_LAUNCH_CHECK("axpbyz");
  return CCL_OK;
}

template <typename T>
int Ops<T>::mult_elem(long n, const void *x, void *z, cudaStream_t s) {
  if (n == 0) return CCL_OK;
  k_mult_elem<T><<<grid_for(n, 256), 256, 0, s>>>(n, (const T *)x, (T *)z);
  CCL_LAUNCH_CHECK("mult_elementwise");
  return CCL_OK;
}

template <typename T>
int Ops<T>::ab_dot_x(int nrows, int nx, double are, double aim, const void *b,
                     const void *x, void *z, cudaStream_t s) {
  long n = (long)nrows * nx;
  if (n == 0) return CCL_OK;
  k_ab_dot_x<T><<<grid_for(n, 256), 256, 0, s>>>(n, nx, (T)are, (T)aim,
                                                  (const T *)b, (const T *)x,
                                                  (T *)z);
  CCL_LAUNCH_CHECK("ab_dot_x");
  return CCL_OK;
}

template <typename T>
int Ops<T>::cast_c2d(long n, const void *in, void *out, cudaStream_t s) {
  if (n == 0) return CCL_OK;
  k_cast_c2d<T><<<grid_for(n, 256), 256, 0, s>>>(n, (const T *)in, (T *)out);
  CCL_LAUNCH_CHECK("cast_c2d");
  return CCL_OK;
}

template <typename T>
int Ops<T>::profile_edges(int cplx, int nrows, int nx, void *a, const void *f,
                          int nf, cudaStream_t s) {
  long n = (long)nrows * nx;
  if (n == 0) return CCL_OK;
  k_profile_edges<T><<<grid_for(n, 256), 256, 0, s>>>(n, (u32)nx, cplx, (T *)a,
                                                       (const T *)f, (u32)nf);
  CCL_LAUNCH_CHECK("profile_edges");
  return CCL_OK;
}

template <typename T>
int Ops<T>::mul_phase(int nrows, int nx, void *a, const void *phs,
                      cudaStream_t s) {
  long n = (long)nrows * nx;
  if (n == 0) return CCL_OK;
  k_mul_phase<T><<<grid_for(n, 256), 256, 0, s>>>(n, nx, (T *)a,
                                                   (const T *)phs);
  CCL_LAUNCH_CHECK("multiply_by_phase");
  return CCL_OK;
}

template <typename T>
int Ops<T>::grad_combine(int M, int nrows, int nx, const void *kx, const void *const *rho,
                         const void *const *Pm, const void *const *Pp, void *const *dN,
                         cudaStream_t s) {
  CCL_REQUIRE(M >= 0 && M < kMaxModes, CCL_ERR_UNSUPPORTED, "grad_combine: M=%d", M);
  ptrs<4> r, pm, pp;
  ptrs<12> d;
  for (int m = 0; m <= M; m++) {
    CCL_REQUIRE(rho[m], CCL_ERR_ARG, "grad_combine: null rho %d", m);
    r.p[m] = (void *)rho[m];
    pm.p[m] = Pm ? (void *)Pm[m] : nullptr;
    pp.p[m] = Pp ? (void *)Pp[m] : nullptr;
    for (int c = 0; c < 3; c++) {
      CCL_REQUIRE(dN[3 * m + c], CCL_ERR_ARG, "grad_combine: null output %d", 3 * m + c);
      d.p[3 * m + c] = dN[3 * m + c];
    }
  }
  if ((long)nrows * nx == 0) return CCL_OK;
  launch_pdl(k_grad_combine<T>, row_chunk_grid<T>(nrows, nx, M + 1), RC_THREADS, 0, s, nx,
             (const T *)kx, r, pm, pp, d);
  CCL_LAUNCH_CHECK("grad_combine");
  return CCL_OK;
}

template <typename T>
int Ops<T>::rot_combine(int M, int nrows, int nx, const void *kx, const void *const *G,
                        const void *const *Qm, const void *const *Qp, const void *const *poiss,
                        void *const *B, cudaStream_t s) {
  CCL_REQUIRE(M >= 0 && M < kMaxModes, CCL_ERR_UNSUPPORTED, "rot_combine: M=%d", M);
  ptrs<12> g, qm, qp, b;
  ptrs<4> po;
  for (int m = 0; m <= M; m++) {
    po.p[m] = poiss ? (void *)poiss[m] : nullptr;
    for (int c = 0; c < 3; c++) {
      const int j = 3 * m + c;
      CCL_REQUIRE(G[j] && B[j], CCL_ERR_ARG, "rot_combine: null field %d", j);
      g.p[j] = (void *)G[j];
      b.p[j] = B[j];
      qm.p[j] = Qm ? (void *)Qm[j] : nullptr;
      qp.p[j] = Qp ? (void *)Qp[j] : nullptr;
    }
  }
  if ((long)nrows * nx == 0) return CCL_OK;
  launch_pdl(k_rot_combine<T>, row_chunk_grid<T>(nrows, nx, M + 1), RC_THREADS, 0, s, nx,
             (const T *)kx, g, qm, qp, po, b);
  CCL_LAUNCH_CHECK("rot_combine");
  return CCL_OK;
}

}  // namespace ccl
