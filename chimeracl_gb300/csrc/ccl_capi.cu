// The C ABI (include/chimeracl_gb300.h): argument validation, dtype
// dispatch, error reporting.  No entry point synchronises the host.
#include <stdarg.h>
#include <stdio.h>

#include <atomic>

#include "ccl_common.cuh"
#include "ccl_launch.h"

namespace ccl {

static thread_local char g_err[512] = "";
static std::atomic<unsigned long long> g_launches{0};

void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

void set_error(const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

}  // namespace ccl

using namespace ccl;

#define DTYPE_CHECK(dt)                                                        \
  CCL_REQUIRE((dt) == CCL_F64 || (dt) == CCL_F32, CCL_ERR_ARG,                 \
              "%s: dtype %d is neither CCL_F64 nor CCL_F32", __func__, (dt))
#define NONNULL(p)                                                             \
  CCL_REQUIRE((p) != nullptr, CCL_ERR_ARG, "%s: %s is NULL", __func__, #p)
#define NONNEG(n)                                                              \
  CCL_REQUIRE((n) >= 0, CCL_ERR_ARG, "%s: %s = %ld < 0", __func__, #n,         \
              (long)(n))
#define DISPATCH(dt, call)                                                     \
  ((dt) == CCL_F64 ? Ops<double>::call : Ops<float>::call)

static int grid_check(const char *fn, int Nx, int Nr) {
  CCL_REQUIRE(Nx >= 4 && Nr >= 3, CCL_ERR_ARG, "%s: grid Nx=%d Nr=%d too small",
              fn, Nx, Nr);
  CCL_REQUIRE((long)(Nx - 1) * (Nr - 1) < 0x7fffffffL, CCL_ERR_UNSUPPORTED,
              "%s: grid too large for 32-bit cell keys", fn);
  return CCL_OK;
}

extern "C" {

int ccl_version(void) { return 100; }

const char *ccl_last_error(void) { return g_err; }

unsigned long long ccl_launch_count(void) { return g_launches.load(); }

// ---------------------------------------------------------------- particles
int ccl_push_x(int dtype, long np, void *x, void *y, void *z, const void *px,
               const void *py, const void *pz, const void *g_inv, double dt,
               void *stream) {
  DTYPE_CHECK(dtype);
  NONNEG(np);
  if (np == 0) return CCL_OK;
  NONNULL(x); NONNULL(y); NONNULL(z); NONNULL(px); NONNULL(py); NONNULL(pz);
  NONNULL(g_inv);
  return DISPATCH(dtype, push_x(np, x, y, z, px, py, pz, g_inv, dt, S(stream)));
}

int ccl_push_x_compensated(int dtype, long np, void *x, void *y, void *z, void *x_lo,
                           void *y_lo, void *z_lo, const void *px, const void *py,
                           const void *pz, const void *g_inv, double dt, void *stream) {
  DTYPE_CHECK(dtype);
  NONNEG(np);
  if (np == 0) return CCL_OK;
  NONNULL(x); NONNULL(y); NONNULL(z); NONNULL(x_lo); NONNULL(y_lo); NONNULL(z_lo);
  NONNULL(px); NONNULL(py); NONNULL(pz); NONNULL(g_inv);
  return DISPATCH(dtype, push_x_comp(np, x, y, z, x_lo, y_lo, z_lo, px, py, pz, g_inv, dt,
                                     S(stream)));
}

int ccl_push_x_keys(int dtype, long np, void *x, void *y, void *z, void *x_lo, void *y_lo,
                    void *z_lo, const void *px, const void *py, const void *pz,
                    const void *g_inv, double dt, int Nx, double xmin, double dx_inv, int Nr,
                    double rmin, double dr_inv, uint32_t *indx_in_cell, uint32_t *sum_in_cell,
                    void *workspace, size_t workspace_bytes, void *stream) {
  DTYPE_CHECK(dtype);
  NONNEG(np);
  CCL_REQUIRE(np < 0xffffffffL, CCL_ERR_UNSUPPORTED,
              "%s: np %ld exceeds 32-bit particle numbers", __func__, np);
  int rc = grid_check(__func__, Nx, Nr);
  if (rc) return rc;
  NONNULL(sum_in_cell); NONNULL(workspace);
  CCL_REQUIRE((x_lo == nullptr) == (y_lo == nullptr) && (x_lo == nullptr) == (z_lo == nullptr),
              CCL_ERR_ARG, "%s: give all three low parts or none", __func__);
  if (np > 0) {
    NONNULL(x); NONNULL(y); NONNULL(z); NONNULL(px); NONNULL(py); NONNULL(pz);
    NONNULL(g_inv); NONNULL(indx_in_cell);
  }
  return DISPATCH(dtype, push_x_keys(np, x, y, z, x_lo, y_lo, z_lo, px, py, pz, g_inv, dt, Nx,
                                     xmin, dx_inv, Nr, rmin, dr_inv, indx_in_cell, sum_in_cell,
                                     workspace, workspace_bytes, S(stream)));
}

int ccl_index_sort_keyed(long np, int Nx, int Nr, const uint32_t *indx_in_cell,
                         uint32_t *sum_in_cell, uint32_t *cell_offset, uint32_t *sort_indx,
                         uint32_t *np_stay, void *workspace, size_t workspace_bytes,
                         void *stream) {
  NONNEG(np);
  CCL_REQUIRE(np < 0xffffffffL, CCL_ERR_UNSUPPORTED,
              "%s: np %ld exceeds 32-bit particle numbers", __func__, np);
  int rc = grid_check(__func__, Nx, Nr);
  if (rc) return rc;
  NONNULL(sum_in_cell); NONNULL(cell_offset); NONNULL(np_stay); NONNULL(workspace);
  if (np > 0) {
    NONNULL(indx_in_cell); NONNULL(sort_indx);
  }
  return index_sort_keyed_launch(np, (long)(Nx - 1) * (Nr - 1), indx_in_cell, sum_in_cell,
                                 cell_offset, sort_indx, np_stay, workspace, workspace_bytes,
                                 S(stream));
}

int ccl_index_sort_workspace(long np, long ncells, size_t *bytes) {
  NONNEG(np);
  CCL_REQUIRE(ncells > 0, CCL_ERR_ARG, "%s: ncells %ld", __func__, ncells);
  NONNULL(bytes);
  *bytes = index_sort_ws_bytes(np, ncells);
  return CCL_OK;
}

int ccl_index_sort(int dtype, long np, const void *x, const void *y,
                   const void *z, int Nx, double xmin, double dx_inv, int Nr,
                   double rmin, double dr_inv, uint32_t *indx_in_cell,
                   uint32_t *sum_in_cell, uint32_t *cell_offset,
                   uint32_t *sort_indx, uint32_t *np_stay, void *workspace,
                   size_t workspace_bytes, void *stream) {
  DTYPE_CHECK(dtype);
  NONNEG(np);
  CCL_REQUIRE(np < 0xffffffffL, CCL_ERR_UNSUPPORTED,
              "%s: np %ld exceeds 32-bit particle numbers", __func__, np);
  int rc = grid_check(__func__, Nx, Nr);
  if (rc) return rc;
  NONNULL(sum_in_cell); NONNULL(cell_offset); NONNULL(np_stay);
  NONNULL(workspace);
  if (np > 0) {
    NONNULL(x); NONNULL(y); NONNULL(z); NONNULL(indx_in_cell);
    NONNULL(sort_indx);
  }
  return DISPATCH(dtype, index_sort(np, x, y, z, Nx, xmin, dx_inv, Nr, rmin,
                                    dr_inv, indx_in_cell, sum_in_cell,
                                    cell_offset, sort_indx, np_stay, workspace,
                                    workspace_bytes, S(stream)));
}

int ccl_align(int dtype, long n, int ncomp, void *const *src, void *const *dst,
              const uint32_t *sort_indx, void *stream) {
  DTYPE_CHECK(dtype);
  NONNEG(n);
  if (n == 0) return CCL_OK;
  NONNULL(src); NONNULL(dst); NONNULL(sort_indx);
  return DISPATCH(dtype, align(n, ncomp, src, dst, sort_indx, S(stream)));
}

int ccl_iota_u32(uint32_t *a, long n, void *stream) {
  NONNEG(n);
  if (n == 0) return CCL_OK;
  NONNULL(a);
  return iota_u32(a, n, S(stream));
}

int ccl_fill_grid(int dtype, long ncells, void *x, void *y, void *z, void *w,
                  const double *theta, const double *xgrid,
                  const double *rgrid, uint32_t Nx_loc, uint32_t npx,
                  uint32_t npr, uint32_t npth, void *stream) {
  DTYPE_CHECK(dtype);
  NONNEG(ncells);
  if (ncells == 0) return CCL_OK;
  NONNULL(x); NONNULL(y); NONNULL(z); NONNULL(w); NONNULL(theta);
  NONNULL(xgrid); NONNULL(rgrid);
  CCL_REQUIRE(Nx_loc >= 2 && npx > 0 && npr > 0 && npth > 0, CCL_ERR_ARG,
              "%s: Nx_loc=%u Nppc=(%u,%u,%u)", __func__, Nx_loc, npx, npr, npth);
  return DISPATCH(dtype, fill_grid(ncells, x, y, z, w, theta, xgrid, rgrid,
                                   Nx_loc, npx, npr, npth, S(stream)));
}

int ccl_dens_profile(int dtype, long np, const void *x, void *w,
                     const double *xx, const double *ff, const double *dxm1,
                     uint32_t nloc, void *stream) {
  DTYPE_CHECK(dtype);
  NONNEG(np);
  CCL_REQUIRE(nloc >= 2, CCL_ERR_ARG, "%s: %u knots, need >= 2", __func__, nloc);
  if (np == 0) return CCL_OK;
  NONNULL(x); NONNULL(w); NONNULL(xx); NONNULL(ff); NONNULL(dxm1);
  return DISPATCH(dtype, dens_profile(np, x, w, xx, ff, dxm1, nloc, S(stream)));
}

int ccl_gamma_inv(int dtype, long np, const void *px, const void *py,
                  const void *pz, void *g_inv, void *stream) {
  DTYPE_CHECK(dtype);
  NONNEG(np);
  if (np == 0) return CCL_OK;
  NONNULL(px); NONNULL(py); NONNULL(pz); NONNULL(g_inv);
  return DISPATCH(dtype, gamma_inv(np, px, py, pz, g_inv, S(stream)));
}

// --------------------------------------------------------------------- grid
int ccl_deposit_scalar(int dtype, int M, const uint32_t *sort_indx,
                       const uint32_t *cell_offset, const void *x,
                       const void *y, const void *z, const void *w, int charge,
                       int Nx, double xmin, double dx_inv, int Nr, double rmin,
                       double dr_inv, void *const *rho, void *stream) {
  DTYPE_CHECK(dtype);
  CCL_REQUIRE(M >= 0 && M < kMaxModes, CCL_ERR_UNSUPPORTED, "%s: M=%d", __func__, M);
  int rc = grid_check(__func__, Nx, Nr);
  if (rc) return rc;
  NONNULL(sort_indx); NONNULL(cell_offset); NONNULL(x); NONNULL(y); NONNULL(z);
  NONNULL(w); NONNULL(rho);
  return DISPATCH(dtype, deposit(0, M, sort_indx, cell_offset, x, y, z, nullptr,
                                 nullptr, nullptr, nullptr, w, charge, Nx, xmin,
                                 dx_inv, Nr, rmin, dr_inv, rho, S(stream)));
}

int ccl_deposit_vector(int dtype, int M, const uint32_t *sort_indx,
                       const uint32_t *cell_offset, const void *x,
                       const void *y, const void *z, const void *ux,
                       const void *uy, const void *uz, const void *g_inv,
                       const void *w, int charge, int Nx, double xmin,
                       double dx_inv, int Nr, double rmin, double dr_inv,
                       void *const *J, void *stream) {
  DTYPE_CHECK(dtype);
  CCL_REQUIRE(M >= 0 && M < kMaxModes, CCL_ERR_UNSUPPORTED, "%s: M=%d", __func__, M);
  int rc = grid_check(__func__, Nx, Nr);
  if (rc) return rc;
  NONNULL(sort_indx); NONNULL(cell_offset); NONNULL(x); NONNULL(y); NONNULL(z);
  NONNULL(ux); NONNULL(uy); NONNULL(uz); NONNULL(g_inv); NONNULL(w); NONNULL(J);
  return DISPATCH(dtype, deposit(1, M, sort_indx, cell_offset, x, y, z, ux, uy,
                                 uz, g_inv, w, charge, Nx, xmin, dx_inv, Nr,
                                 rmin, dr_inv, J, S(stream)));
}

#define LO_CHECK()                                                              \
  CCL_REQUIRE(dtype == CCL_F32, CCL_ERR_UNSUPPORTED,                             \
              "%s: low coordinate parts are for FP32 particles", __func__);      \
  NONNULL(x_lo); NONNULL(y_lo); NONNULL(z_lo)

int ccl_deposit_scalar_lo(int dtype, int M, const uint32_t *sort_indx,
                          const uint32_t *cell_offset, const void *x, const void *y,
                          const void *z, const void *w, int charge, int Nx, double xmin,
                          double dx_inv, int Nr, double rmin, double dr_inv, void *const *rho,
                          const void *x_lo, const void *y_lo, const void *z_lo, void *stream) {
  DTYPE_CHECK(dtype);
  LO_CHECK();
  CCL_REQUIRE(M >= 0 && M < kMaxModes, CCL_ERR_UNSUPPORTED, "%s: M=%d", __func__, M);
  int rc = grid_check(__func__, Nx, Nr);
  if (rc) return rc;
  NONNULL(sort_indx); NONNULL(cell_offset); NONNULL(x); NONNULL(y); NONNULL(z);
  NONNULL(w); NONNULL(rho);
  const void *lo[3] = {x_lo, y_lo, z_lo};
  return DISPATCH(dtype, deposit(0, M, sort_indx, cell_offset, x, y, z, nullptr, nullptr,
                                 nullptr, nullptr, w, charge, Nx, xmin, dx_inv, Nr, rmin,
                                 dr_inv, rho, S(stream), lo));
}

int ccl_deposit_vector_lo(int dtype, int M, const uint32_t *sort_indx,
                          const uint32_t *cell_offset, const void *x, const void *y,
                          const void *z, const void *ux, const void *uy, const void *uz,
                          const void *g_inv, const void *w, int charge, int Nx, double xmin,
                          double dx_inv, int Nr, double rmin, double dr_inv, void *const *J,
                          const void *x_lo, const void *y_lo, const void *z_lo, void *stream) {
  DTYPE_CHECK(dtype);
  LO_CHECK();
  CCL_REQUIRE(M >= 0 && M < kMaxModes, CCL_ERR_UNSUPPORTED, "%s: M=%d", __func__, M);
  int rc = grid_check(__func__, Nx, Nr);
  if (rc) return rc;
  NONNULL(sort_indx); NONNULL(cell_offset); NONNULL(x); NONNULL(y); NONNULL(z);
  NONNULL(ux); NONNULL(uy); NONNULL(uz); NONNULL(g_inv); NONNULL(w); NONNULL(J);
  const void *lo[3] = {x_lo, y_lo, z_lo};
  return DISPATCH(dtype, deposit(1, M, sort_indx, cell_offset, x, y, z, ux, uy, uz, g_inv, w,
                                 charge, Nx, xmin, dx_inv, Nr, rmin, dr_inv, J, S(stream), lo));
}

int ccl_deposit_postproc(int dtype, int M, int nfld, void *const *flds,
                         int Nx, int Nr, const void *dV_inv, void *stream) {
  DTYPE_CHECK(dtype);
  CCL_REQUIRE(M >= 0 && M < kMaxModes, CCL_ERR_UNSUPPORTED, "%s: M=%d", __func__, M);
  NONNULL(flds); NONNULL(dV_inv);
  CCL_REQUIRE(Nx > 0 && Nr >= 2, CCL_ERR_ARG, "%s: Nx=%d Nr=%d", __func__, Nx, Nr);
  return DISPATCH(dtype, postproc(M, nfld, flds, Nx, Nr, dV_inv, S(stream)));
}

int ccl_warp_axis(int dtype, int M, int nfld, void *const *flds, int Nx,
                  void *stream) {
  DTYPE_CHECK(dtype);
  CCL_REQUIRE(M >= 0 && M < kMaxModes, CCL_ERR_UNSUPPORTED, "%s: M=%d", __func__, M);
  NONNULL(flds);
  CCL_REQUIRE(Nx > 0, CCL_ERR_ARG, "%s: Nx=%d", __func__, Nx);
  return DISPATCH(dtype, warp_axis(M, nfld, flds, Nx, S(stream)));
}

int ccl_gather_push(int dtype, int M, long np, const void *x, const void *y,
                    const void *z, void *px, void *py, void *pz, void *g_inv,
                    const uint32_t *sort_indx, const uint32_t *np_stay,
                    double factor_push, int Nx, double xmin, double dx_inv,
                    int Nr, double rmin, double dr_inv,
                    const void *const *flds, void *stream) {
  DTYPE_CHECK(dtype);
  CCL_REQUIRE(M >= 0 && M < kMaxModes, CCL_ERR_UNSUPPORTED, "%s: M=%d", __func__, M);
  NONNEG(np);
  int rc = grid_check(__func__, Nx, Nr);
  if (rc) return rc;
  if (np == 0) return CCL_OK;
  NONNULL(x); NONNULL(y); NONNULL(z); NONNULL(px); NONNULL(py); NONNULL(pz);
  NONNULL(g_inv); NONNULL(sort_indx); NONNULL(np_stay); NONNULL(flds);
  return DISPATCH(dtype, gather_push(M, np, x, y, z, px, py, pz, g_inv,
                                     sort_indx, np_stay, factor_push, Nx, xmin,
                                     dx_inv, Nr, rmin, dr_inv, flds,
                                     S(stream)));
}

int ccl_gather_push_cells(int dtype, int M, long np, const void *x, const void *y,
                          const void *z, void *px, void *py, void *pz, void *g_inv,
                          const uint32_t *sort_indx, const uint32_t *cell_offset,
                          const uint32_t *np_stay, double factor_push, int Nx,
                          double xmin, double dx_inv, int Nr, double rmin,
                          double dr_inv, const void *const *flds, void *stream) {
  DTYPE_CHECK(dtype);
  CCL_REQUIRE(M >= 0 && M < kMaxModes, CCL_ERR_UNSUPPORTED, "%s: M=%d", __func__, M);
  NONNEG(np);
  int rc = grid_check(__func__, Nx, Nr);
  if (rc) return rc;
  if (np == 0) return CCL_OK;
  NONNULL(x); NONNULL(y); NONNULL(z); NONNULL(px); NONNULL(py); NONNULL(pz);
  NONNULL(g_inv); NONNULL(sort_indx); NONNULL(cell_offset); NONNULL(np_stay);
  NONNULL(flds);
  return DISPATCH(dtype, gather_push_cells(M, np, x, y, z, px, py, pz, g_inv, sort_indx,
                                           cell_offset, np_stay, factor_push, Nx, xmin,
                                           dx_inv, Nr, rmin, dr_inv, flds, S(stream)));
}

int ccl_gather_push_cells_lo(int dtype, int M, long np, const void *x, const void *y,
                             const void *z, void *px, void *py, void *pz, void *g_inv,
                             const uint32_t *sort_indx, const uint32_t *cell_offset,
                             const uint32_t *np_stay, double factor_push, int Nx, double xmin,
                             double dx_inv, int Nr, double rmin, double dr_inv,
                             const void *const *flds, const void *x_lo, const void *y_lo,
                             const void *z_lo, void *stream) {
  DTYPE_CHECK(dtype);
  CCL_REQUIRE(M >= 0 && M < kMaxModes, CCL_ERR_UNSUPPORTED, "%s: M=%d", __func__, M);
  NONNEG(np);
  int rc = grid_check(__func__, Nx, Nr);
  if (rc) return rc;
  if (np == 0) return CCL_OK;
  LO_CHECK();
  NONNULL(x); NONNULL(y); NONNULL(z); NONNULL(px); NONNULL(py); NONNULL(pz);
  NONNULL(g_inv); NONNULL(sort_indx); NONNULL(cell_offset); NONNULL(np_stay);
  NONNULL(flds);
  const void *lo[3] = {x_lo, y_lo, z_lo};
  return DISPATCH(dtype, gather_push_cells(M, np, x, y, z, px, py, pz, g_inv, sort_indx,
                                           cell_offset, np_stay, factor_push, Nx, xmin,
                                           dx_inv, Nr, rmin, dr_inv, flds, S(stream), lo));
}

// ----------------------------------------------------------------- spectral
int ccl_phase(int dtype, int nx, void *phs, const double *kx, double x0,
              int sign, void *stream) {
  DTYPE_CHECK(dtype);
  CCL_REQUIRE(nx > 0, CCL_ERR_ARG, "%s: nx=%d", __func__, nx);
  NONNULL(phs); NONNULL(kx);
  return DISPATCH(dtype, phase(nx, phs, kx, x0, sign, S(stream)));
}

int ccl_fft_forward_rows(int dtype, int nrows, int nx, const void *in,
                         long in_ld, int in_real, void *out, const void *phs,
                         const void *filter, void *stream) {
  DTYPE_CHECK(dtype);
  NONNEG(nrows);
  if (nrows == 0) return CCL_OK;
  NONNULL(in); NONNULL(out); NONNULL(phs);
  CCL_REQUIRE(in_ld >= nx, CCL_ERR_ARG, "%s: in_ld %ld < nx %d", __func__, in_ld, nx);
  if (dtype == CCL_F64)
    return fft_forward_rows<double>(nrows, nx, (const double *)in, in_ld,
                                    in_real, (double *)out, (const double *)phs,
                                    (const double *)filter, S(stream));
  return fft_forward_rows<float>(nrows, nx, (const float *)in, in_ld, in_real,
                                 (float *)out, (const float *)phs,
                                 (const float *)filter, S(stream));
}

int ccl_fft_backward_rows(int dtype, int nrows, int nx, const void *in,
                          void *out, long out_ld, int out_real,
                          const void *phs, void *stream) {
  DTYPE_CHECK(dtype);
  NONNEG(nrows);
  if (nrows == 0) return CCL_OK;
  NONNULL(in); NONNULL(out); NONNULL(phs);
  CCL_REQUIRE(out_ld >= nx, CCL_ERR_ARG, "%s: out_ld %ld < nx %d", __func__, out_ld, nx);
  if (dtype == CCL_F64)
    return fft_backward_rows<double>(nrows, nx, (const double *)in,
                                     (double *)out, out_ld, out_real,
                                     (const double *)phs, S(stream));
  return fft_backward_rows<float>(nrows, nx, (const float *)in, (float *)out,
                                  out_ld, out_real, (const float *)phs,
                                  S(stream));
}

int ccl_damp_rows(int dtype, int nrows, int nx, void *spec, void *rs,
                  int rs_real, const void *phs_plus, const void *phs_minus,
                  const void *profile, int nf, void *stream) {
  DTYPE_CHECK(dtype);
  NONNEG(nrows);
  if (nrows == 0) return CCL_OK;
  NONNULL(spec); NONNULL(rs); NONNULL(phs_plus); NONNULL(phs_minus);
  NONNULL(profile);
  if (dtype == CCL_F64)
    return damp_rows<double>(nrows, nx, (double *)spec, (double *)rs, rs_real,
                             (const double *)phs_plus,
                             (const double *)phs_minus,
                             (const double *)profile, nf, S(stream));
  return damp_rows<float>(nrows, nx, (float *)spec, (float *)rs, rs_real,
                          (const float *)phs_plus, (const float *)phs_minus,
                          (const float *)profile, nf, S(stream));
}

int ccl_fft_forward_batch(int dtype, int batch, int nrows, int nx,
                          const void *const *in, const long *in_ld,
                          const int *in_real, void *const *out,
                          const void *phs, const void *const *filter,
                          void *stream) {
  DTYPE_CHECK(dtype);
  NONNULL(in); NONNULL(in_ld); NONNULL(in_real); NONNULL(out); NONNULL(phs);
  if (dtype == CCL_F64)
    return fft_forward_batch<double>(batch, nrows, nx, in, in_ld, in_real, out,
                                     phs, filter, S(stream));
  return fft_forward_batch<float>(batch, nrows, nx, in, in_ld, in_real, out,
                                  phs, filter, S(stream));
}

int ccl_fft_backward_batch(int dtype, int batch, int nrows, int nx,
                           const void *const *in, void *const *out,
                           const long *out_ld, const int *out_real,
                           const void *phs, void *stream) {
  DTYPE_CHECK(dtype);
  NONNULL(in); NONNULL(out); NONNULL(out_ld); NONNULL(out_real); NONNULL(phs);
  if (dtype == CCL_F64)
    return fft_backward_batch<double>(batch, nrows, nx, in, out, out_ld,
                                      out_real, phs, S(stream));
  return fft_backward_batch<float>(batch, nrows, nx, in, out, out_ld, out_real,
                                   phs, S(stream));
}

int ccl_damp_batch(int dtype, int batch, int nrows, int nx, void *const *spec,
                   void *const *rs, const int *rs_real, const void *phs_plus,
                   const void *phs_minus, const void *profile, int nf,
                   void *stream) {
  DTYPE_CHECK(dtype);
  NONNULL(spec); NONNULL(rs); NONNULL(rs_real); NONNULL(phs_plus);
  NONNULL(phs_minus); NONNULL(profile);
  if (dtype == CCL_F64)
    return damp_batch<double>(batch, nrows, nx, spec, rs, rs_real, phs_plus,
                              phs_minus, profile, nf, S(stream));
  return damp_batch<float>(batch, nrows, nx, spec, rs, rs_real, phs_plus,
                           phs_minus, profile, nf, S(stream));
}

int ccl_dht_gemm_batch(int dtype, int batch, int m, int k, const int *ncols,
                       int cplx, const void *const *A, const void *const *X,
                       const long *ldx, void *const *Y, const long *ldy,
                       double alpha_re, double alpha_im, double beta,
                       void *stream) {
  DTYPE_CHECK(dtype);
  NONNULL(ncols); NONNULL(A); NONNULL(X); NONNULL(ldx); NONNULL(Y); NONNULL(ldy);
  if (dtype == CCL_F64)
    return dht_gemm_batch<double>(batch, m, k, ncols, cplx, A, X, ldx, Y, ldy,
                                  alpha_re, alpha_im, beta, S(stream));
  return dht_gemm_batch<float>(batch, m, k, ncols, cplx, A, X, ldx, Y, ldy,
                               alpha_re, alpha_im, beta, S(stream));
}

int ccl_dht_gemm(int dtype, int batch, int m, int k, int ncols, int cplx,
                 const void *const *A, const void *const *X, long ldx,
                 void *const *Y, long ldy, double alpha_re, double alpha_im,
                 double beta, void *stream) {
  DTYPE_CHECK(dtype);
  NONNULL(A); NONNULL(X); NONNULL(Y);
  if (dtype == CCL_F64)
    return dht_gemm<double>(batch, m, k, ncols, cplx, A, X, ldx, Y, ldy,
                            alpha_re, alpha_im, beta, S(stream));
  return dht_gemm<float>(batch, m, k, ncols, cplx, A, X, ldx, Y, ldy, alpha_re,
                         alpha_im, beta, S(stream));
}

int ccl_dht_bf16x3_prepare_bytes(int m, int k, size_t *bytes) {
  NONNULL(bytes);
  CCL_REQUIRE(m > 0 && k > 0 && k <= 512 && m <= 512, CCL_ERR_UNSUPPORTED,
              "%s: m=%d k=%d (m, k <= 512)", __func__, m, k);
  *bytes = umma_split_bytes(m, k);
  return CCL_OK;
}

int ccl_dht_bf16x3_prepare(int dtype, const void *A, int m, int k, void *out,
                           size_t bytes, void *stream) {
  DTYPE_CHECK(dtype);
  NONNULL(A); NONNULL(out);
  if (dtype == CCL_F64)
    return umma_split_a<double>((const double *)A, m, k, out, bytes, S(stream));
  return umma_split_a<float>((const float *)A, m, k, out, bytes, S(stream));
}

int ccl_dht_bf16x3_gemm_batch(int batch, int m, int k, const int *ncols,
                              int cplx, const void *const *A_prepared,
                              const void *const *X, const long *ldx,
                              void *const *Y, const long *ldy, double alpha_re,
                              double alpha_im, double beta, void *stream) {
  NONNULL(ncols); NONNULL(A_prepared); NONNULL(X); NONNULL(ldx); NONNULL(Y);
  NONNULL(ldy);
  return umma_gemm_batch(batch, m, k, ncols, cplx, A_prepared, X, ldx, Y, ldy,
                         alpha_re, alpha_im, beta, S(stream));
}

int ccl_dht_bf16x3_status(int reset) { return umma_status(reset); }

int ccl_wait_probe(long spins, int arrive, int *gave_up, void *stream) {
  NONNULL(gave_up);
  return umma_wait_probe(spins, arrive, gave_up, S(stream));
}

int ccl_sort_status(int reset) { return sort_status(reset); }

int ccl_scan_wait_probe(long spins, int publish, int *gave_up, uint32_t *scratch, void *stream) {
  NONNULL(gave_up); NONNULL(scratch);
  return scan_wait_probe(spins, publish, gave_up, scratch, S(stream));
}

int ccl_psatd_advance(int dtype, long ncells, double dt_inv, const void *c1,
                      const void *c2, const void *c3, void *const *flds,
                      void *stream) {
  DTYPE_CHECK(dtype);
  NONNEG(ncells);
  NONNULL(c1); NONNULL(c2); NONNULL(c3); NONNULL(flds);
  return DISPATCH(dtype, psatd(ncells, dt_inv, c1, c2, c3, flds, S(stream)));
}

int ccl_psatd_advance_split(int dtype, long ncells, const void *coef, void *const *flds,
                            void *stream) {
  DTYPE_CHECK(dtype);
  NONNEG(ncells);
  NONNULL(coef); NONNULL(flds);
  return DISPATCH(dtype, psatd_split(ncells, coef, flds, S(stream)));
}

int ccl_get_m1(int dtype, int nrows, int nx, void *out, const void *in,
               void *stream) {
  DTYPE_CHECK(dtype);
  CCL_REQUIRE(nrows >= 0 && nx > 0, CCL_ERR_ARG, "%s: nrows=%d nx=%d", __func__, nrows, nx);
  NONNULL(out); NONNULL(in);
  return DISPATCH(dtype, get_m1(nrows, nx, out, in, S(stream)));
}

int ccl_grad_combine(int dtype, int M, int nrows, int nx, const void *kx,
                     const void *const *rho, const void *const *Pm,
                     const void *const *Pp, void *const *dN, void *stream) {
  DTYPE_CHECK(dtype);
  CCL_REQUIRE(nrows >= 0 && nx > 0, CCL_ERR_ARG, "%s: nrows=%d nx=%d", __func__, nrows, nx);
  NONNULL(kx); NONNULL(rho); NONNULL(dN);
  return DISPATCH(dtype, grad_combine(M, nrows, nx, kx, rho, Pm, Pp, dN, S(stream)));
}

int ccl_rot_combine(int dtype, int M, int nrows, int nx, const void *kx,
                    const void *const *G, const void *const *Qm,
                    const void *const *Qp, const void *const *poiss,
                    void *const *B, void *stream) {
  DTYPE_CHECK(dtype);
  CCL_REQUIRE(nrows >= 0 && nx > 0, CCL_ERR_ARG, "%s: nrows=%d nx=%d", __func__, nrows, nx);
  NONNULL(kx); NONNULL(G); NONNULL(B);
  return DISPATCH(dtype, rot_combine(M, nrows, nx, kx, G, Qm, Qp, poiss, B, S(stream)));
}

// -------------------------------------------------------------- elementwise
int ccl_set(int dtype, int cplx, long n, void *a, double re, double im,
            void *stream) {
  DTYPE_CHECK(dtype);
  NONNEG(n);
  if (n == 0) return CCL_OK;
  NONNULL(a);
  return DISPATCH(dtype, set(cplx, n, a, re, im, S(stream)));
}

int ccl_set_batch(int dtype, int narr, const int *cplx, const long *n,
                  void *const *a, double re, double im, void *stream) {
  DTYPE_CHECK(dtype);
  CCL_REQUIRE(narr >= 0 && narr <= 32, CCL_ERR_ARG, "%s: narr %d outside [0, 32]", __func__,
              narr);
  if (narr == 0) return CCL_OK;
  NONNULL(cplx); NONNULL(n); NONNULL(a);
  for (int i = 0; i < narr; i++) {
    CCL_REQUIRE(n[i] >= 0, CCL_ERR_ARG, "%s: n[%d] = %ld", __func__, i, n[i]);
    CCL_REQUIRE(n[i] == 0 || a[i], CCL_ERR_ARG, "%s: a[%d] is NULL", __func__, i);
  }
  return DISPATCH(dtype, set_batch(narr, cplx, n, a, re, im, S(stream)));
}

int ccl_append_c2c(int dtype, long n, void *base, const void *add,
                   void *stream) {
  DTYPE_CHECK(dtype);
  NONNEG(n);
  if (n == 0) return CCL_OK;
  NONNULL(base); NONNULL(add);
  return DISPATCH(dtype, append(n, base, add, S(stream)));
}

int ccl_zpaxz(int dtype, long n, void *z, double are, double aim,
              const void *x, void *stream) {
  DTYPE_CHECK(dtype);
  NONNEG(n);
  if (n == 0) return CCL_OK;
  NONNULL(z); NONNULL(x);
  return DISPATCH(dtype, zpaxz(n, z, are, aim, x, S(stream)));
}

int ccl_axpbyz(int dtype, long n, double are, double aim, const void *x,
               double bre, double bim, const void *y, void *z, void *stream) {
  DTYPE_CHECK(dtype);
  NONNEG(n);
  if (n == 0) return CCL_OK;
  NONNULL(x); NONNULL(y); NONNULL(z);
  return DISPATCH(dtype, axpbyz(n, are, aim, x, bre, bim, y, z, S(stream)));
}

int ccl_mult_elementwise(int dtype, long n, const void *x, void *z,
                         void *stream) {
  DTYPE_CHECK(dtype);
  NONNEG(n);
  if (n == 0) return CCL_OK;
  NONNULL(x); NONNULL(z);
  return DISPATCH(dtype, mult_elem(n, x, z, S(stream)));
}

int ccl_ab_dot_x(int dtype, int nrows, int nx, double are, double aim,
                 const void *b, const void *x, void *z, void *stream) {
  DTYPE_CHECK(dtype);
  CCL_REQUIRE(nrows >= 0 && nx > 0, CCL_ERR_ARG, "%s: nrows=%d nx=%d", __func__, nrows, nx);
  NONNULL(b); NONNULL(x); NONNULL(z);
  return DISPATCH(dtype, ab_dot_x(nrows, nx, are, aim, b, x, z, S(stream)));
}

int ccl_cast_c2d(int dtype, long n, const void *in, void *out, void *stream) {
  DTYPE_CHECK(dtype);
  NONNEG(n);
  if (n == 0) return CCL_OK;
  NONNULL(in); NONNULL(out);
  return DISPATCH(dtype, cast_c2d(n, in, out, S(stream)));
}

int ccl_profile_edges(int dtype, int cplx, int nrows, int nx, void *a,
                      const void *f, int nf, void *stream) {
  DTYPE_CHECK(dtype);
  CCL_REQUIRE(nrows >= 0 && nx > 0 && nf >= 0, CCL_ERR_ARG,
              "%s: nrows=%d nx=%d nf=%d", __func__, nrows, nx, nf);
  NONNULL(a); NONNULL(f);
  return DISPATCH(dtype, profile_edges(cplx, nrows, nx, a, f, nf, S(stream)));
}

int ccl_multiply_by_phase(int dtype, int nrows, int nx, void *a,
                          const void *phs, void *stream) {
  DTYPE_CHECK(dtype);
  CCL_REQUIRE(nrows >= 0 && nx > 0, CCL_ERR_ARG, "%s: nrows=%d nx=%d", __func__, nrows, nx);
  NONNULL(a); NONNULL(phs);
  return DISPATCH(dtype, mul_phase(nrows, nx, a, phs, S(stream)));
}

}  // extern "C"
