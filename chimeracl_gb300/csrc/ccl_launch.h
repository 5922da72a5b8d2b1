// Internal launch functions shared by the translation units of the library.
// The C ABI (ccl_capi.cu) validates arguments and dispatches on dtype to
// these templates; each is explicitly instantiated for double and float in
// the translation unit named beside it.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace ccl {

template <typename T>
struct GridP;

// ccl_fft.cu
template <typename T>
int fft_forward_rows(int nrows, int nx, const T *in, long in_ld, int in_real,
                     T *out, const T *phs, const T *filt, cudaStream_t s);
template <typename T>
int fft_backward_rows(int nrows, int nx, const T *in, T *out, long out_ld,
                      int out_real, const T *phs, cudaStream_t s);
template <typename T>
int damp_rows(int nrows, int nx, T *spec, T *rs, int rs_real, const T *phs_p,
              const T *phs_m, const T *prof, int nf, cudaStream_t s);
template <typename T>
int fft_forward_batch(int batch, int nrows, int nx, const void *const *in,
                      const long *in_ld, const int *in_real, void *const *out,
                      const void *phs, const void *const *filt, cudaStream_t s);
template <typename T>
int fft_backward_batch(int batch, int nrows, int nx, const void *const *in,
                       void *const *out, const long *out_ld,
                       const int *out_real, const void *phs, cudaStream_t s);
template <typename T>
int damp_batch(int batch, int nrows, int nx, void *const *spec,
               void *const *rs, const int *rs_real, const void *phs_p,
               const void *phs_m, const void *prof, int nf, cudaStream_t s);

// ccl_dht.cu
template <typename T>
int dht_gemm_batch(int batch, int m, int k, const int *ncols, int cplx,
                   const void *const *A, const void *const *X, const long *ldx,
                   void *const *Y, const long *ldy, double are, double aim,
                   double beta, cudaStream_t s);
template <typename T>
int dht_gemm(int batch, int m, int k, int ncols, int cplx, const void *const *A,
             const void *const *X, long ldx, void *const *Y, long ldy,
             double are, double aim, double beta, cudaStream_t s);

// ccl_f64.cu / ccl_f32.cu (particles, grid, elementwise)
template <typename T> struct Ops {
  static int push_x(long np, void *x, void *y, void *z, const void *px,
                    const void *py, const void *pz, const void *g_inv,
                    double dt, cudaStream_t s);
  static int push_x_comp(long np, void *x, void *y, void *z, void *xl, void *yl, void *zl,
                         const void *px, const void *py, const void *pz,
                         const void *g_inv, double dt, cudaStream_t s);
  static int index_sort(long np, const void *x, const void *y, const void *z,
                        int Nx, double xmin, double dx_inv, int Nr,
                        double rmin, double dr_inv, uint32_t *indx,
                        uint32_t *counts, uint32_t *cell_offset,
                        uint32_t *sort_indx, uint32_t *np_stay, void *ws,
                        size_t ws_bytes, cudaStream_t s);
  static int push_x_keys(long np, void *x, void *y, void *z, void *xl, void *yl, void *zl,
                         const void *px, const void *py, const void *pz, const void *g_inv,
                         double dt, int Nx, double xmin, double dx_inv, int Nr, double rmin,
                         double dr_inv, uint32_t *indx, uint32_t *counts, void *ws,
                         size_t ws_bytes, cudaStream_t s);
  static int align(long n, int ncomp, void *const *src, void *const *dst,
                   const uint32_t *idx, cudaStream_t s);
  static int fill_grid(long ncells, void *x, void *y, void *z, void *w,
                       const double *theta, const double *xgrid,
                       const double *rgrid, uint32_t Nx, uint32_t npx,
                       uint32_t npr, uint32_t npth, cudaStream_t s);
  static int dens_profile(long np, const void *x, void *w, const double *xx,
                          const double *ff, const double *dxm1, uint32_t nloc,
                          cudaStream_t s);
  static int gamma_inv(long np, const void *px, const void *py,
                       const void *pz, void *g, cudaStream_t s);
  static int deposit(int vec, int M, const uint32_t *sort_indx,
                     const uint32_t *cell_off, const void *x, const void *y,
                     const void *z, const void *ux, const void *uy,
                     const void *uz, const void *g_inv, const void *w,
                     int charge, int Nx, double xmin, double dx_inv, int Nr,
                     double rmin, double dr_inv, void *const *flds,
                     cudaStream_t s, const void *const *lo = nullptr);
  static int postproc(int M, int nfld, void *const *flds, int Nx, int Nr,
                      const void *dv, cudaStream_t s);
  static int warp_axis(int M, int nfld, void *const *flds, int Nx,
                       cudaStream_t s);
  static int gather_push(int M, long np, const void *x, const void *y,
                         const void *z, void *px, void *py, void *pz,
                         void *g_inv, const uint32_t *sort_indx,
                         const uint32_t *np_stay, double factor_push, int Nx,
                         double xmin, double dx_inv, int Nr, double rmin,
                         double dr_inv, const void *const *flds,
                         cudaStream_t s);
  static int gather_push_cells(int M, long np, const void *x, const void *y,
                               const void *z, void *px, void *py, void *pz,
                               void *g_inv, const uint32_t *sort_indx,
                               const uint32_t *cell_offset, const uint32_t *np_stay,
                               double factor_push, int Nx, double xmin,
                               double dx_inv, int Nr, double rmin, double dr_inv,
                               const void *const *flds, cudaStream_t s,
                               const void *const *lo = nullptr);
  static int psatd(long n, double dt_inv, const void *c1, const void *c2,
                   const void *c3, void *const *flds, cudaStream_t s);
  static int psatd_split(long n, const void *coef, void *const *flds, cudaStream_t s);
  static int phase(int nx, void *phs, const double *kx, double x0, int sign,
                   cudaStream_t s);
  static int get_m1(int nrows, int nx, void *out, const void *in,
                    cudaStream_t s);
  static int set(int cplx, long n, void *a, double re, double im,
                 cudaStream_t s);
  static int set_batch(int narr, const int *cplx, const long *n, void *const *a, double re,
                       double im, cudaStream_t s);
  static int append(long n, void *base, const void *add, cudaStream_t s);
  static int zpaxz(long n, void *z, double are, double aim, const void *x,
                   cudaStream_t s);
  static int axpbyz(long n, double are, double aim, const void *x, double bre,
                    double bim, const void *y, void *z, cudaStream_t s);
  static int mult_elem(long n, const void *x, void *z, cudaStream_t s);
  static int ab_dot_x(int nrows, int nx, double are, double aim,
                      const void *b, const void *x, void *z, cudaStream_t s);
  static int cast_c2d(long n, const void *in, void *out, cudaStream_t s);
  static int profile_edges(int cplx, int nrows, int nx, void *a, const void *f,
                           int nf, cudaStream_t s);
  static int mul_phase(int nrows, int nx, void *a, const void *phs,
                       cudaStream_t s);
  static int grad_combine(int M, int nrows, int nx, const void *kx,
                          const void *const *rho, const void *const *Pm,
                          const void *const *Pp, void *const *dN, cudaStream_t s);
  static int rot_combine(int M, int nrows, int nx, const void *kx,
                         const void *const *G, const void *const *Qm,
                         const void *const *Qp, const void *const *poiss,
                         void *const *B, cudaStream_t s);
};

// ccl_umma.cu (BF16x3 tensor-core Hankel GEMM, FP32 operands)
size_t umma_split_bytes(int m, int k);
template <typename TA>
int umma_split_a(const TA *A, int m, int k, void *out, size_t bytes, cudaStream_t s);
int umma_gemm_batch(int batch, int m, int k, const int *ncols, int cplx, const void *const *Ap,
                    const void *const *X, const long *ldx, void *const *Y, const long *ldy,
                    double are, double aim, double beta, cudaStream_t s);
int umma_status(int reset);
int umma_wait_probe(long spins, int arrive, int *gave_up, cudaStream_t s);

size_t index_sort_ws_bytes(long np, long ncells);
int index_sort_keyed_launch(long np, long ncells, const uint32_t *indx, uint32_t *counts,
                            uint32_t *cell_offset, uint32_t *sort_indx, uint32_t *np_stay,
                            void *ws, size_t ws_bytes, cudaStream_t s);
int iota_u32(uint32_t *a, long n, cudaStream_t s);
int sort_status(int reset);
int scan_wait_probe(long spins, int publish, int *gave_up, uint32_t *scratch, cudaStream_t s);

}  // namespace ccl
