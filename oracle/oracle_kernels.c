/*
 * THE ORACLE -- test infrastructure only.  Nothing in the product imports,
 * links or calls this file; tests, __graft_entry__.smoke() and bench.py's CPU
 * baseline use it to check the product and as the timed CPU baseline.
 *
 * A plain-C restatement of the arithmetic of chimeraCL's OpenCL kernels
 * (chimeraCL/kernels/*.cl), one function per reference kernel, taking host
 * scalars by value and looping over the reference's NDRange internally.
 * Every floating-point expression keeps the reference's operation order, and
 * the library is built with -ffp-contract=off, so on the same inputs it agrees
 * bit for bit with the reference kernels compiled unchanged (oracle/_ref).
 *
 * Two generalisations, both labelled where they occur:
 *  - deposit and gather take the number of azimuthal modes M as an argument;
 *    for M <= 1 they reduce exactly to grid_deposit_m0.cl / grid_deposit_m1.cl,
 *    for M >= 2 they apply the m=1 formulas with e^{i m phi} built by complex
 *    recurrence (the reference ships no m>=2 kernels);
 *  - profile_by_interpolant clamps its knot search to the last interval where
 *    the reference would read past the knot arrays (undefined there).
 *
 * Complex arrays are interleaved (re, im) doubles.  OpenMP parallelises the
 * loops whose iterations are independent in the reference (one work-item
 * each); the counting-sort scatter stays serial so that the within-cell order
 * is ascending particle index, which is what the serial reference build gives.
 */
#include <math.h>
#include <stdint.h>
#include <stddef.h>

typedef uint32_t u32;
#define MMAX 4

/* ------------------------------------------------------------------ */
/* particles_generic.cl                                                 */
/* ------------------------------------------------------------------ */

/* push_xyz: particles_generic.cl:129-153 */
void port_push_xyz(long np, double *x, double *y, double *z, const double *px,
                   const double *py, const double *pz, const double *g_inv,
                   double dt) {
#pragma omp parallel for schedule(static)
  for (long ip = 0; ip < np; ip++) {
    double dt_g = dt * g_inv[ip];
    double ddx = px[ip] * dt_g;
    double ddy = py[ip] * dt_g;
    double ddz = pz[ip] * dt_g;
    x[ip] = x[ip] + ddx;
    y[ip] = y[ip] + ddy;
    z[ip] = z[ip] + ddz;
  }
}

/* cell key of one particle: particles_generic.cl:106-125 */
static inline u32 cell_key(double xp, double yp, double zp, int Nx, double xmin,
                           double dx_inv, int Nr, double rmin, double dr_inv) {
  int nxc = Nx - 1, nrc = Nr - 1;
  double r = sqrt(yp * yp + zp * zp);
  double fx = floor((xp - xmin) * dx_inv);
  double fr = floor((r - rmin) * dr_inv);
  /* (int) of an out-of-range double is undefined in C; such particles are
   * outside the window on every platform, so they take the overflow key. */
  int ix = (fx > -2147483648.0 && fx < 2147483647.0) ? (int)fx : -1;
  int ir = (fr > -2147483648.0 && fr < 2147483647.0) ? (int)fr : -1;
  if (ix > 0 && ix < nxc - 1 && ir < nrc - 1 && ir >= 0)
    return (u32)(ix + ir * nxc);
  return (u32)(nrc * nxc);
}

/* index_and_sum_in_cell: particles_generic.cl:88-126 */
void port_index_and_sum(long np, const double *x, const double *y,
                        const double *z, u32 *sum_in_cell, u32 *indx_in_cell,
                        int Nx, double xmin, double dx_inv, int Nr, double rmin,
                        double dr_inv) {
#pragma omp parallel for schedule(static)
  for (long ip = 0; ip < np; ip++) {
    u32 k = cell_key(x[ip], y[ip], z[ip], Nx, xmin, dx_inv, Nr, rmin, dr_inv);
    indx_in_cell[ip] = k;
#pragma omp atomic
    sum_in_cell[k] += 1u;
  }
}

/* sort: particles_generic.cl:186-201 (serial: ascending order in a cell) */
void port_sort(long np, const u32 *cell_offset, const u32 *indx_in_cell,
               u32 *new_sum_in_cell, u32 *sorted_indx) {
  for (long ip = 0; ip < np; ip++) {
    u32 c = indx_in_cell[ip];
    u32 loc = new_sum_in_cell[c]++;
    sorted_indx[cell_offset[c] + loc] = (u32)ip;
  }
}

/* data_align_dbl: particles_generic.cl:156-169 */
void port_data_align(long n, const double *x, double *x_new,
                     const u32 *sorted_indx) {
#pragma omp parallel for schedule(static)
  for (long ip = 0; ip < n; ip++)
    x_new[ip] = x[sorted_indx[ip]];
}

/* fill_grid: particles_generic.cl:33-84 */
void port_fill_grid(long ncells, double *x, double *y, double *z, double *w,
                    const double *theta_var, const double *xgrid,
                    const double *rgrid, u32 Nx, u32 npx, u32 npr, u32 npth) {
  u32 nxc = Nx - 1;
  u32 nppc = npx * npr * npth;
#pragma omp parallel for schedule(static)
  for (long ic = 0; ic < ncells; ic++) {
    u32 icell = (u32)ic;
    u32 ir = icell / nxc;
    u32 ix = icell - nxc * ir;
    u32 ip = icell * nppc;
    double xmin = xgrid[ix], rmin = rgrid[ir], thmin = theta_var[icell];
    double Lx = xgrid[ix + 1] - xgrid[ix];
    double Lr = rgrid[ir + 1] - rgrid[ir];
    double ddx = 1. / ((double)npx);
    double ddr = 1. / ((double)npr);
    double dth = 2 * M_PI / ((double)npth);
    for (u32 ith = 0; ith < npth; ith++) {
      double th = thmin + ith * dth;
      double s = sin(th), c = cos(th);
      for (int irr = 0; irr < (int)npr; irr++) {
        double rp = rmin + (0.5 + irr) * ddr * Lr;
        double rps = rp * s, rpc = rp * c;
        for (int ixx = 0; ixx < (int)npx; ixx++) {
          x[ip] = xmin + (0.5 + ixx) * ddx * Lx;
          y[ip] = rps;
          z[ip] = rpc;
          w[ip] = rp;
          ip += 1;
        }
      }
    }
  }
}

/* profile_by_interpolant: particles_generic.cl:6-30 (search clamped) */
void port_profile_by_interpolant(long np, const double *x, double *w,
                                 const double *xx, const double *ff,
                                 const double *dxm1, u32 nloc) {
#pragma omp parallel for schedule(static)
  for (long ip = 0; ip < np; ip++) {
    double xp = x[ip];
    u32 ix;
    for (ix = 0; ix < nloc - 1; ix++)
      if (xp > xx[ix] && xp <= xx[ix + 1])
        break;
    if (ix > nloc - 2)
      ix = nloc - 2;
    double fm = ff[ix] * dxm1[ix];
    double fp = ff[ix + 1] * dxm1[ix];
    w[ip] *= fm * (xx[ix + 1] - x[ip]) + fp * (x[ip] - xx[ix]);
  }
}

/* ------------------------------------------------------------------ */
/* grid_deposit_m0.cl / grid_deposit_m1.cl                              */
/* ------------------------------------------------------------------ */

/* The reference visits cells in four colours: a 2x2 block origin (2i, 2j)
 * plus an offset (0,0),(1,0),(0,1),(1,1) per launch, so that no two cells of
 * one launch share a node (grid_deposit_m0.cl:3-19, grid_methods_cl.py:61-64).
 * nxnr_4 is the reference's launch size, (Nr//2 * Nx)//2 in Python. */
static inline int colour_cell(u32 off, u32 ic, u32 Nx, u32 Nr, u32 *ix,
                              u32 *ir) {
  u32 nx2 = Nx / 2;
  u32 a = ic / nx2, b = ic - a * nx2;
  b *= 2;
  a *= 2;
  if (off == 1) b += 1;
  else if (off == 2) a += 1;
  else if (off == 3) { b += 1; a += 1; }
  *ix = b;
  *ir = a;
  return (b > 0 && b < Nx - 2 && a < Nr - 2);
}

/* depose_scalar: grid_deposit_m1.cl:20-152 (M=1), grid_deposit_m0.cl:20-129
 * (M=0); fld[m] is rho_m (m=0 real, m>=1 complex). */
void port_depose_scalar(int M, u32 nxnr_4, const u32 *sort_indx,
                        const double *x, const double *y, const double *z,
                        const double *w, const u32 *cell_off, int charge,
                        u32 Nx, double xmin, double dx_inv, u32 Nr, double rmin,
                        double dr_inv, double **fld) {
  double q = (double)(signed char)charge;
  for (u32 off = 0; off < 4; off++) {
#pragma omp parallel for schedule(dynamic, 64)
    for (long icl = 0; icl < (long)nxnr_4; icl++) {
      u32 ix, ir;
      if (!colour_cell(off, (u32)icl, Nx, Nr, &ix, &ir))
        continue;
      u32 cg = ix + ir * (Nx - 1), ng = ix + ir * Nx;
      u32 p0 = cell_off[cg], p1 = cell_off[cg + 1];
      if (p0 == p1)
        continue;
      double s0[2][2] = {{0, 0}, {0, 0}};
      double sm[MMAX][2][2][2] = {{{{0}}}};
      for (u32 ip = p0; ip < p1; ip++) {
        u32 p = sort_indx[ip];
        double xp = x[p], yp = y[p], zp = z[p], wp = w[p] * q;
        double rp = sqrt(yp * yp + zp * zp);
        double rinv = 1. / rp;
        double e1[2] = {yp * rinv, zp * rinv};
        double sX1 = (xp - xmin) * dx_inv - ix, sX0 = 1.0 - sX1;
        double sR1 = (rp - rmin) * dr_inv - ir, sR0 = 1.0 - sR1;
        sX0 *= wp;
        sX1 *= wp;
        double C[2][2] = {{sR0 * sX0, sR0 * sX1}, {sR1 * sX0, sR1 * sX1}};
        double em[2] = {e1[0], e1[1]};
        for (int i = 0; i < 2; i++)
          for (int j = 0; j < 2; j++)
            s0[i][j] += C[i][j];
        for (int m = 1; m <= M; m++) {
          if (m > 1) { /* generalisation: e^{i m phi} = e^{i(m-1)phi} e^{i phi} */
            double re = em[0] * e1[0] - em[1] * e1[1];
            double im = em[0] * e1[1] + em[1] * e1[0];
            em[0] = re;
            em[1] = im;
          }
          for (int i = 0; i < 2; i++)
            for (int j = 0; j < 2; j++) {
              sm[m - 1][i][j][0] += C[i][j] * em[0];
              sm[m - 1][i][j][1] += C[i][j] * em[1];
            }
        }
      }
      for (int i = 0; i < 2; i++)
        for (int j = 0; j < 2; j++) {
          u32 d = ng + j + Nx * i;
          fld[0][d] = fld[0][d] + s0[i][j];
          for (int m = 1; m <= M; m++) {
            fld[m][2 * d] = fld[m][2 * d] + sm[m - 1][i][j][0];
            fld[m][2 * d + 1] = fld[m][2 * d + 1] + sm[m - 1][i][j][1];
          }
        }
    }
  }
}

/* depose_vector: grid_deposit_m1.cl:171-327 (M=1), grid_deposit_m0.cl:148-277
 * (M=0); fld[3*m + k] is J_k of mode m, k = x,y,z. */
void port_depose_vector(int M, u32 nxnr_4, const u32 *sort_indx,
                        const double *x, const double *y, const double *z,
                        const double *ux, const double *uy, const double *uz,
                        const double *g_inv, const double *w,
                        const u32 *cell_off, int charge, u32 Nx, double xmin,
                        double dx_inv, u32 Nr, double rmin, double dr_inv,
                        double **fld) {
  double q = (double)(signed char)charge;
  for (u32 off = 0; off < 4; off++) {
#pragma omp parallel for schedule(dynamic, 64)
    for (long icl = 0; icl < (long)nxnr_4; icl++) {
      u32 ix, ir;
      if (!colour_cell(off, (u32)icl, Nx, Nr, &ix, &ir))
        continue;
      u32 cg = ix + ir * (Nx - 1), ng = ix + ir * Nx;
      u32 p0 = cell_off[cg], p1 = cell_off[cg + 1];
      if (p0 == p1)
        continue;
      double v0[3][2][2] = {{{0}}};
      double vm[MMAX][3][2][2][2] = {{{{{0}}}}};
      for (u32 ip = p0; ip < p1; ip++) {
        u32 p = sort_indx[ip];
        double xp = x[p], yp = y[p], zp = z[p];
        double jp[3] = {ux[p], uy[p], uz[p]};
        double wp = w[p] * g_inv[p] * q;
        double rp = sqrt(yp * yp + zp * zp);
        double rinv = 0;
        if (rp > 0)
          rinv = 1. / rp;
        double e1[2] = {yp * rinv, zp * rinv};
        double sX1 = (xp - xmin) * dx_inv - ix, sX0 = 1.0 - sX1;
        double sR1 = (rp - rmin) * dr_inv - ir, sR0 = 1.0 - sR1;
        sX0 *= wp;
        sX1 *= wp;
        double C[2][2] = {{sR0 * sX0, sR0 * sX1}, {sR1 * sX0, sR1 * sX1}};
        double em[MMAX][2];
        em[0][0] = e1[0];
        em[0][1] = e1[1];
        for (int m = 2; m <= M; m++) { /* generalisation for m >= 2 */
          em[m - 1][0] = em[m - 2][0] * e1[0] - em[m - 2][1] * e1[1];
          em[m - 1][1] = em[m - 2][0] * e1[1] + em[m - 2][1] * e1[0];
        }
        for (int k = 0; k < 3; k++)
          for (int i = 0; i < 2; i++)
            for (int j = 0; j < 2; j++) {
              double jproj = C[i][j] * jp[k];
              v0[k][i][j] += C[i][j] * jp[k];
              for (int m = 1; m <= M; m++) {
                vm[m - 1][k][i][j][0] += jproj * em[m - 1][0];
                vm[m - 1][k][i][j][1] += jproj * em[m - 1][1];
              }
            }
      }
      for (int i = 0; i < 2; i++)
        for (int j = 0; j < 2; j++) {
          u32 d = ng + j + Nx * i;
          for (int k = 0; k < 3; k++)
            fld[k][d] = fld[k][d] + v0[k][i][j];
          for (int m = 1; m <= M; m++)
            for (int k = 0; k < 3; k++) {
              double *f = fld[3 * m + k];
              f[2 * d] = f[2 * d] + vm[m - 1][k][i][j][0];
              f[2 * d + 1] = f[2 * d + 1] + vm[m - 1][k][i][j][1];
            }
        }
    }
  }
}

/* gather_and_push: grid_deposit_m1.cl:330-511 (M=1), grid_deposit_m0.cl:280-427
 * (M=0); fld[6*m + c] with c = ex,ey,ez,bx,by,bz. dt is FactorPush. */
void port_gather_and_push(int M, long np, const double *x, const double *y,
                          const double *z, double *px, double *py, double *pz,
                          double *g_inv, const u32 *sort_indx, double dt,
                          u32 np_stay, u32 Nx, double xmin, double dx_inv,
                          u32 Nr, double rmin, double dr_inv,
                          double *const *fld) {
  int nxg = (int)Nx, nxc = nxg - 1, nrc = (int)Nr - 1;
#pragma omp parallel for schedule(static)
  for (long i = 0; i < np; i++) {
    u32 p = sort_indx[i];
    if (p >= np_stay)
      continue;
    double xp = x[p], yp = y[p], zp = z[p];
    double rp = sqrt(yp * yp + zp * zp);
    double fx = floor((xp - xmin) * dx_inv), fr = floor((rp - rmin) * dr_inv);
    int ix = (fx > -2147483648.0 && fx < 2147483647.0) ? (int)fx : -1;
    int ir = (fr > -2147483648.0 && fr < 2147483647.0) ? (int)fr : 2147483647;
    if (!(ix > 0 && ix < nxc - 1 && ir < nrc - 1))
      continue;
    u32 ig = (u32)(ix + ir * nxg);
    double u[3] = {px[p], py[p], pz[p]};
    double dt_2 = 0.5 * dt;
    double rinv = 1. / rp;
    double sX1 = (xp - xmin) * dx_inv - ix, sX0 = 1.0 - sX1;
    double sR1 = (rp - rmin) * dr_inv - ir, sR0 = 1.0 - sR1;
    double e1[2] = {yp * rinv, -zp * rinv};
    double em[MMAX][2];
    em[0][0] = e1[0];
    em[0][1] = e1[1];
    for (int m = 2; m <= M; m++) { /* generalisation: e^{-i m phi} */
      em[m - 1][0] = em[m - 2][0] * e1[0] - em[m - 2][1] * e1[1];
      em[m - 1][1] = em[m - 2][0] * e1[1] + em[m - 2][1] * e1[0];
    }
    double C[2][2] = {{sR0 * sX0, sR0 * sX1}, {sR1 * sX0, sR1 * sX1}};
    double ep[3] = {0, 0, 0}, bp[3] = {0, 0, 0};
    for (int k = 0; k < 3; k++)
      for (int a = 0; a < 2; a++)
        for (int b = 0; b < 2; b++) {
          u32 l = ig + b + Nx * a;
          double c = C[a][b];
          ep[k] += c * fld[k][l];
          bp[k] += c * fld[3 + k][l];
          for (int m = 1; m <= M; m++) {
            const double *fe = fld[6 * m + k], *fb = fld[6 * m + 3 + k];
            double er = 2 * fe[2 * l], ei = 2 * fe[2 * l + 1];
            double br = 2 * fb[2 * l], bi = 2 * fb[2 * l + 1];
            ep[k] += c * er * em[m - 1][0];
            ep[k] -= c * ei * em[m - 1][1];
            bp[k] += c * br * em[m - 1][0];
            bp[k] -= c * bi * em[m - 1][1];
          }
        }
    double um[3], up[3], u0[3], t[3], s[3];
    for (int k = 0; k < 3; k++)
      um[k] = u[k] + dt_2 * ep[k];
    double gi = 1. / sqrt(1. + um[0] * um[0] + um[1] * um[1] + um[2] * um[2]);
    for (int k = 0; k < 3; k++)
      t[k] = dt_2 * bp[k] * gi;
    double f2 = 2. / (1. + t[0] * t[0] + t[1] * t[1] + t[2] * t[2]);
    for (int k = 0; k < 3; k++)
      s[k] = t[k] * f2;
    u0[0] = um[0] + um[1] * t[2] - um[2] * t[1];
    u0[1] = um[1] - um[0] * t[2] + um[2] * t[0];
    u0[2] = um[2] + um[0] * t[1] - um[1] * t[0];
    up[0] = um[0] + u0[1] * s[2] - u0[2] * s[1];
    up[1] = um[1] - u0[0] * s[2] + u0[2] * s[0];
    up[2] = um[2] + u0[0] * s[1] - u0[1] * s[0];
    for (int k = 0; k < 3; k++)
      u[k] = up[k] + dt_2 * ep[k];
    gi = 1. / sqrt(1. + u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
    px[p] = u[0];
    py[p] = u[1];
    pz[p] = u[2];
    g_inv[p] = gi;
  }
}

/* ------------------------------------------------------------------ */
/* grid_generic.cl                                                      */
/* ------------------------------------------------------------------ */

/* treat_axis_d/_c: grid_generic.cl:37-59; ncomp = 1 real, 2 complex */
void port_treat_axis(double *a, u32 Nx, int ncomp) {
  for (long i = 0; i < (long)Nx * ncomp; i++)
    a[Nx * ncomp + i] -= a[i];
}

/* divide_by_dv_d/_c: grid_generic.cl:4-34 */
void port_divide_by_dv(double *a, u32 NxNr, u32 Nx, const double *dv_inv,
                       int ncomp) {
#pragma omp parallel for schedule(static)
  for (long i = 0; i < (long)NxNr; i++) {
    u32 ir = (u32)i / Nx;
    for (int c = 0; c < ncomp; c++)
      a[i * ncomp + c] *= dv_inv[ir];
  }
}

/* warp_axis_m0_d / warp_axis_m1plus_c: grid_generic.cl:63-86 */
void port_warp_axis(double *a, u32 Nx, int m) {
  if (m == 0) {
    for (u32 i = 0; i < Nx; i++)
      a[i] = a[i + Nx];
  } else {
    for (u32 i = 0; i < Nx; i++) {
      a[2 * i] = -a[2 * (i + Nx)];
      a[2 * i + 1] = -a[2 * (i + Nx) + 1];
    }
  }
}

/* ------------------------------------------------------------------ */
/* solver_ms_pic.cl                                                     */
/* ------------------------------------------------------------------ */

/* profile_edges_c/_d: solver_ms_pic.cl:5-55 (unsigned arithmetic kept) */
void port_profile_edges(double *a, const double *f, u32 NxNr, u32 Nx, u32 Nf,
                        int ncomp) {
#pragma omp parallel for schedule(static)
  for (long i = 0; i < (long)NxNr; i++) {
    u32 ir = (u32)i / Nx, ix = (u32)i - ir * Nx;
    if (ix < Nf)
      for (int c = 0; c < ncomp; c++)
        a[i * ncomp + c] *= f[ix];
    if (ix > Nx - Nf)
      for (int c = 0; c < ncomp; c++)
        a[i * ncomp + c] *= f[Nx - ix];
  }
}

/* advance_e_g_m: solver_ms_pic.cl:57-143.  f[0..14] = e_x,e_y,e_z, g_x,g_y,
 * g_z, j_x,j_y,j_z, n0_x,n0_y,n0_z, n1_x,n1_y,n1_z (complex). */
void port_advance_e_g_m(long n, double dt_inv, const double *c1m,
                        const double *c2m, const double *c3m,
                        double *const *f) {
  const double pi2 = 2 * M_PI;
#pragma omp parallel for schedule(static)
  for (long i = 0; i < n; i++) {
    double c1 = c1m[i], c2 = c2m[i], c3 = c3m[i];
    for (int k = 0; k < 3; k++)
      for (int q = 0; q < 2; q++) {
        double e0 = f[k][2 * i + q], g0 = f[3 + k][2 * i + q];
        double j0 = f[6 + k][2 * i + q] * pi2;
        double n0 = f[9 + k][2 * i + q] * pi2;
        double n1 = f[12 + k][2 * i + q] * pi2;
        double e1 = c1 * e0 + c2 * c3 * (g0 - j0) +
                    c3 * (c1 * n0 - n1 - (n0 - n1) * dt_inv * c2 * c3);
        double g1 = -c2 * e0 + c1 * (g0 - j0) + j0 +
                    c3 * (dt_inv * (1. - c1) * (n0 - n1) - c2 * n0);
        f[k][2 * i + q] = e1;
        f[3 + k][2 * i + q] = g1;
      }
  }
}

/* ------------------------------------------------------------------ */
/* transformer_generic.cl                                               */
/* ------------------------------------------------------------------ */

/* get_m1: transformer_generic.cl:3-24 -- the m=-1 mirror of an m=+1 field */
void port_get_m1(double *out, const double *in, u32 Nx, u32 NxNrm1) {
#pragma omp parallel for schedule(static)
  for (long i = 0; i < (long)NxNrm1; i++) {
    u32 ir = (u32)i / Nx, ix = (u32)i - ir * Nx;
    u32 io = (ix == 0) ? 0 : Nx - ix;
    u32 g = io + ir * Nx;
    out[2 * i] = -in[2 * g];
    out[2 * i + 1] = in[2 * g + 1];
  }
}

/* get_phase_plus / get_phase_minus: transformer_generic.cl:28-55 */
void port_get_phase(double *phs, const double *kx, double x0, u32 Nx,
                    int sign) {
  for (u32 i = 0; i < Nx; i++) {
    phs[2 * i] = cos(x0 * kx[i]);
    phs[2 * i + 1] = sign > 0 ? sin(x0 * kx[i]) : -sin(x0 * kx[i]);
  }
}

/* multiply_by_phase: transformer_generic.cl:58-80 */
void port_multiply_by_phase(double *a, u32 NxNr, u32 Nx, const double *phs) {
#pragma omp parallel for schedule(static)
  for (long i = 0; i < (long)NxNr; i++) {
    u32 ir = (u32)i / Nx, ix = (u32)i - ir * Nx;
    double ar = a[2 * i], ai = a[2 * i + 1];
    double pr = phs[2 * ix], pi = phs[2 * ix + 1];
    a[2 * i] = (ar * pr - ai * pi);
    a[2 * i + 1] = (ar * pi + ai * pr);
  }
}

/* ------------------------------------------------------------------ */
/* generic.cl                                                           */
/* ------------------------------------------------------------------ */

/* append_c2c: generic.cl:18-29 */
void port_append_c2c(double *base, const double *add, long n) {
#pragma omp parallel for schedule(static)
  for (long i = 0; i < n; i++) {
    base[2 * i] = base[2 * i] + add[2 * i];
    base[2 * i + 1] = base[2 * i + 1] + add[2 * i + 1];
  }
}

/* zpaxz_c2c: generic.cl:32-44 */
void port_zpaxz(double are, double aim, const double *x, double *z, long n) {
#pragma omp parallel for schedule(static)
  for (long i = 0; i < n; i++) {
    double x0 = x[2 * i], x1 = x[2 * i + 1];
    z[2 * i] = z[2 * i] + are * x0 - aim * x1;
    z[2 * i + 1] = z[2 * i + 1] + are * x1 + aim * x0;
  }
}

/* mult_elementwise_d2c: generic.cl:47-58 */
void port_mult_elementwise(const double *x, double *z, long n) {
#pragma omp parallel for schedule(static)
  for (long i = 0; i < n; i++) {
    z[2 * i] = x[i] * z[2 * i];
    z[2 * i + 1] = x[i] * z[2 * i + 1];
  }
}

/* axpbyz_c2c: generic.cl:61-77 */
void port_axpbyz(double are, double aim, const double *x, double bre,
                 double bim, const double *y, double *z, long n) {
#pragma omp parallel for schedule(static)
  for (long i = 0; i < n; i++) {
    double x0 = x[2 * i], x1 = x[2 * i + 1], y0 = y[2 * i], y1 = y[2 * i + 1];
    z[2 * i] = are * x0 - aim * x1 + bre * y0 - bim * y1;
    z[2 * i + 1] = are * x1 + aim * x0 + bre * y1 + bim * y0;
  }
}

/* ab_dot_x: generic.cl:82-99 -- z = b[ix] * (a x) */
void port_ab_dot_x(double are, double aim, const double *b, const double *x,
                   double *z, u32 NxNr, u32 Nx) {
#pragma omp parallel for schedule(static)
  for (long i = 0; i < (long)NxNr; i++) {
    u32 ir = (u32)i / Nx, ix = (u32)i - ir * Nx;
    double x0 = x[2 * i], x1 = x[2 * i + 1];
    z[2 * i] = b[ix] * (are * x0 - aim * x1);
    z[2 * i + 1] = b[ix] * (are * x1 + aim * x0);
  }
}

/* cast_array_d2c (which takes the real part of a complex array): generic.cl:102-112 */
void port_cast_c2d(const double *in, double *out, long n) {
#pragma omp parallel for schedule(static)
  for (long i = 0; i < n; i++)
    out[i] = in[2 * i];
}

int port_num_threads(void) {
#ifdef _OPENMP
  extern int omp_get_max_threads(void);
  return omp_get_max_threads();
#else
  return 1;
#endif
}
