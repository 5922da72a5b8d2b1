// Test infrastructure only (the oracle). Never linked into the product.
//
// Serial NDRange launchers for the reference's own OpenCL kernels, compiled
// from the reference sources where they lie (the recipe in oracle/Makefile
// puts the reference's chimeraCL/kernels directory on the include path).  One exported
// ref_<kernel>(n, ...) per reference __kernel runs work-items 0..n-1 in order.
// Scalars that the reference passes through __constant pointers are taken by
// value here and passed by address; double2 values arrive as two doubles.
//
// Built as three shared objects because the m0 and m1 deposit sources define
// kernels of the same names:
//   -DREF_COMMON  generic.cl grid_generic.cl particles_generic.cl
//                 solver_ms_pic.cl transformer_generic.cl
//   -DREF_GRID_M0 grid_deposit_m0.cl
//   -DREF_GRID_M1 grid_deposit_m1.cl
#include "cl_shim.hpp"

thread_local size_t ccl_ref_gid;

template <typename F> static void ndrange(size_t n, F f) {
  for (size_t i = 0; i < n; i++) {
    ccl_ref_gid = i;
    f();
  }
}

static inline double2 d2(double a, double b) {
  double2 r;
  r.s0 = a;
  r.s1 = b;
  return r;
}

#ifdef REF_COMMON
#include "generic.cl"
#include "grid_generic.cl"
#include "particles_generic.cl"
#include "solver_ms_pic.cl"
#include "transformer_generic.cl"

// ---- generic.cl
extern "C" void ref_set_cdouble_to(size_t n, double2 *x, double re, double im,
                                   uint sz) {
  ndrange(n, [&] { set_cdouble_to(x, d2(re, im), sz); });
}
extern "C" void ref_append_c2c(size_t n, double2 *a, double2 *b, uint sz) {
  ndrange(n, [&] { append_c2c(a, b, sz); });
}
extern "C" void ref_zpaxz_c2c(size_t n, double are, double aim, double2 *x,
                              double2 *z, uint sz) {
  ndrange(n, [&] { zpaxz_c2c(d2(are, aim), x, z, sz); });
}
extern "C" void ref_mult_elementwise_d2c(size_t n, double *x, double2 *z,
                                         uint sz) {
  ndrange(n, [&] { mult_elementwise_d2c(x, z, sz); });
}
extern "C" void ref_axpbyz_c2c(size_t n, double are, double aim, double2 *x,
                               double bre, double bim, double2 *y, double2 *z,
                               uint sz) {
  ndrange(n, [&] { axpbyz_c2c(d2(are, aim), x, d2(bre, bim), y, z, sz); });
}
extern "C" void ref_ab_dot_x(size_t n, double are, double aim, double *b,
                             double2 *x, double2 *z, uint NxNr, uint Nx) {
  ndrange(n, [&] { ab_dot_x(d2(are, aim), b, x, z, NxNr, Nx); });
}
extern "C" void ref_cast_array_d2c(size_t n, double2 *in, double *out,
                                   uint sz) {
  ndrange(n, [&] { cast_array_d2c(in, out, sz); });
}

// ---- grid_generic.cl
extern "C" void ref_divide_by_dv_d(size_t n, double *arr, uint NxNr, uint Nx,
                                   double *dv_inv) {
  ndrange(n, [&] { divide_by_dv_d(arr, &NxNr, &Nx, dv_inv); });
}
extern "C" void ref_divide_by_dv_c(size_t n, double2 *arr, uint NxNr, uint Nx,
                                   double *dv_inv) {
  ndrange(n, [&] { divide_by_dv_c(arr, &NxNr, &Nx, dv_inv); });
}
extern "C" void ref_treat_axis_d(size_t n, double *arr, uint Nx) {
  ndrange(n, [&] { treat_axis_d(arr, Nx); });
}
extern "C" void ref_treat_axis_c(size_t n, double2 *arr, uint Nx) {
  ndrange(n, [&] { treat_axis_c(arr, Nx); });
}
extern "C" void ref_warp_axis_m0_d(size_t n, double *arr, uint Nx) {
  ndrange(n, [&] { warp_axis_m0_d(arr, Nx); });
}
extern "C" void ref_warp_axis_m1plus_c(size_t n, double2 *arr, uint Nx) {
  ndrange(n, [&] { warp_axis_m1plus_c(arr, Nx); });
}

// ---- particles_generic.cl
extern "C" void ref_profile_by_interpolant(size_t n, double *x, double *w,
                                           uint Np, double *xx, double *ff,
                                           double *dxm1, uint Nx_loc) {
  ndrange(n, [&] { profile_by_interpolant(x, w, Np, xx, ff, dxm1, Nx_loc); });
}
extern "C" void ref_fill_grid(size_t n, double *x, double *y, double *z,
                              double *w, double *theta_var, double *xgrid,
                              double *rgrid, uint Nx, uint ncells, uint npx,
                              uint npr, uint npth) {
  ndrange(n, [&] {
    fill_grid(x, y, z, w, theta_var, xgrid, rgrid, Nx, ncells, npx, npr,
              npth);
  });
}
extern "C" void ref_index_and_sum_in_cell(size_t n, double *x, double *y,
                                          double *z, uint *sum_in_cell,
                                          uint num_p, uint *indx_in_cell,
                                          uint Nx, double xmin, double dx_inv,
                                          uint Nr, double rmin,
                                          double dr_inv) {
  ndrange(n, [&] {
    index_and_sum_in_cell(x, y, z, sum_in_cell, &num_p, indx_in_cell, &Nx,
                          &xmin, &dx_inv, &Nr, &rmin, &dr_inv);
  });
}
extern "C" void ref_push_xyz(size_t n, double *x, double *y, double *z,
                             double *px, double *py, double *pz, double *g_inv,
                             double dt, uint num_p) {
  ndrange(n, [&] { push_xyz(x, y, z, px, py, pz, g_inv, &dt, &num_p); });
}
extern "C" void ref_data_align_dbl(size_t n, double *x, double *x_new,
                                   uint *sorted_indx, uint num_p) {
  ndrange(n, [&] { data_align_dbl(x, x_new, sorted_indx, num_p); });
}
extern "C" void ref_sort(size_t n, uint *cell_offset, uint *indx_in_cell,
                         uint *new_sum_in_cell, uint *sorted_indx,
                         uint num_p) {
  ndrange(n, [&] {
    sort(cell_offset, indx_in_cell, new_sum_in_cell, sorted_indx, num_p);
  });
}

// ---- solver_ms_pic.cl
extern "C" void ref_profile_edges_c(size_t n, double2 *x, double *f, uint NxNr,
                                    uint Nx, uint Nf) {
  ndrange(n, [&] { profile_edges_c(x, f, NxNr, Nx, Nf); });
}
extern "C" void ref_profile_edges_d(size_t n, double *x, double *f, uint NxNr,
                                    uint Nx, uint Nf) {
  ndrange(n, [&] { profile_edges_d(x, f, NxNr, Nx, Nf); });
}
extern "C" void ref_advance_e_g_m(size_t n, uint NxNr, double dt_inv,
                                  double *c1, double *c2, double *c3,
                                  double2 **f /* e,g,j,n0,n1 x 3 comps */) {
  ndrange(n, [&] {
    advance_e_g_m(&NxNr, &dt_inv, c1, c2, c3, f[0], f[1], f[2], f[3], f[4],
                  f[5], f[6], f[7], f[8], f[9], f[10], f[11], f[12], f[13],
                  f[14]);
  });
}

// ---- transformer_generic.cl
extern "C" void ref_get_m1(size_t n, double2 *out, double2 *in, uint Nx,
                           uint NxNrm1) {
  ndrange(n, [&] { get_m1(out, in, &Nx, &NxNrm1); });
}
extern "C" void ref_get_phase_plus(size_t n, double2 *phs, double *kx,
                                   double x0, uint Nx) {
  ndrange(n, [&] { get_phase_plus(phs, kx, x0, Nx); });
}
extern "C" void ref_get_phase_minus(size_t n, double2 *phs, double *kx,
                                    double x0, uint Nx) {
  ndrange(n, [&] { get_phase_minus(phs, kx, x0, Nx); });
}
extern "C" void ref_multiply_by_phase(size_t n, double2 *arr, uint NxNr,
                                      uint Nx, double2 *phs) {
  ndrange(n, [&] { multiply_by_phase(arr, &NxNr, &Nx, phs); });
}
#endif // REF_COMMON

#if defined(REF_GRID_M0) || defined(REF_GRID_M1)
#ifdef REF_GRID_M0
#include "grid_deposit_m0.cl"
#define SCL_ARGS(f) f[0]
#define VEC_ARGS(f) f[0], f[1], f[2]
#define GATHER_ARGS(f) f[0], f[1], f[2], f[3], f[4], f[5]
#else
#include "grid_deposit_m1.cl"
#define SCL_ARGS(f) f[0], (double2 *)f[1]
#define VEC_ARGS(f)                                                            \
  f[0], f[1], f[2], (double2 *)f[3], (double2 *)f[4], (double2 *)f[5]
#define GATHER_ARGS(f)                                                         \
  f[0], f[1], f[2], f[3], f[4], f[5], (double2 *)f[6], (double2 *)f[7],        \
      (double2 *)f[8], (double2 *)f[9], (double2 *)f[10], (double2 *)f[11]
#endif

// grid scalars: Nx, xmin, dx_inv, Nr, rmin, dr_inv, then NxNr_4 / Nxm1Nrm1
extern "C" void ref_depose_scalar(size_t n, uint off, uint *sort_indx,
                                  double *x, double *y, double *z, double *w,
                                  uint *cell_off, int charge, uint Nx,
                                  double xmin, double dx_inv, uint Nr,
                                  double rmin, double dr_inv, uint NxNr_4,
                                  double **fld) {
  char q = (char)charge;
  ndrange(n, [&] {
    depose_scalar(off, sort_indx, x, y, z, w, cell_off, q, &Nx, &xmin,
                  &dx_inv, &Nr, &rmin, &dr_inv, &NxNr_4, SCL_ARGS(fld));
  });
}
extern "C" void ref_depose_vector(size_t n, uint off, uint *sort_indx,
                                  double *x, double *y, double *z, double *ux,
                                  double *uy, double *uz, double *g_inv,
                                  double *w, uint *cell_off, int charge,
                                  uint Nx, double xmin, double dx_inv, uint Nr,
                                  double rmin, double dr_inv, uint NxNr_4,
                                  double **fld) {
  char q = (char)charge;
  ndrange(n, [&] {
    depose_vector(off, sort_indx, x, y, z, ux, uy, uz, g_inv, w, cell_off, q,
                  &Nx, &xmin, &dx_inv, &Nr, &rmin, &dr_inv, &NxNr_4,
                  VEC_ARGS(fld));
  });
}
extern "C" void ref_gather_and_push(size_t n, double *x, double *y, double *z,
                                    double *px, double *py, double *pz,
                                    double *g_inv, uint *sort_indx,
                                    uint *cell_off, double dt, uint Np,
                                    uint Np_stay, uint Nx, double xmin,
                                    double dx_inv, uint Nr, double rmin,
                                    double dr_inv, uint Nxm1Nrm1,
                                    double **fld) {
  ndrange(n, [&] {
    gather_and_push(x, y, z, px, py, pz, g_inv, sort_indx, cell_off, &dt, Np,
                    Np_stay, &Nx, &xmin, &dx_inv, &Nr, &rmin, &dr_inv,
                    &Nxm1Nrm1, GATHER_ARGS(fld));
  });
}
#endif
