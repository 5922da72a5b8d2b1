// Adjoint (reverse-mode) kernels of the PIC step, for gradients of a loss
// of the final fields with respect to the laser and the plasma density.
// Each kernel is the transpose of one forward operation of the step, for
// the same particles and cells (the forward's cell sort is reused):
//
//  * k_deposit_adj  -- charge / current deposit (grid_deposit_m1.cl:20-327)
//    transposed: a gather of the node adjoints with the shape functions and
//    their derivatives, giving each particle's position, momentum, Lorentz
//    factor and weight adjoints;
//  * k_gather_push_adj -- field gather + Boris push (grid_deposit_m1.cl:
//    330-511) transposed: the push reversed by hand, the field adjoints at
//    the particle scattered onto the nodes (shared-memory tile, atomics on
//    the tile's nodes only once per CTA), the position adjoint from the
//    shape-function and angle derivatives of the gathered fields;
//  * k_push_x_adj   -- push_xyz (particles_generic.cl:129-153) transposed;
//  * spectral ones: PSATD update (solver_ms_pic.cl:57-143), the combine
//    steps of the spectral gradient and curl (transformer_methods_cl.py:
//    87-133, 185-263), deposit post-processing and ghost rows
//    (grid_generic.cl:4-86), the align permutation
//    (particles_generic.cl:156-169) and the density profile
//    (particles_generic.cl:6-30).
//
// Complex adjoints are stored like the fields: (dL/dRe, dL/dIm).  A complex
// linear map z' = a z has the adjoint conj(a) z'.  Shape functions are
// differentiated as the piecewise-linear functions they are (inside a cell).
#include <cuda_runtime.h>

#include "ccl_common.cuh"
#include "ccl_particles.cuh"

namespace ccl {

constexpr int AT_TX = 32, AT_TR = 8, AT_THREADS = 256;
constexpr int AT_NX = AT_TX + 1, AT_NR = AT_TR + 1;

template <typename T> struct AdjEdge;
template <> struct AdjEdge<float> { typedef CellEdge type; };
template <> struct AdjEdge<double> { typedef double type; };

// cell edge of column / row i: an exact float pair in FP32 (as the FP32
// deposit and gather take their fractions), the plain formula in FP64
__device__ __forceinline__ CellEdge adj_x_edge(const GridP<float> &g, int i) {
  return x_edge(g, i);
}
__device__ __forceinline__ CellEdge adj_r_edge(const GridP<float> &g, int i) {
  return r_edge(g, i);
}
__device__ __forceinline__ double adj_x_edge(const GridP<double> &, int i) { return (double)i; }
__device__ __forceinline__ double adj_r_edge(const GridP<double> &, int i) { return (double)i; }
__device__ __forceinline__ float adj_frac(float v, CellEdge e, float o, float h_inv) {
  (void)o;
  return edge_frac(v, e, h_inv);
}
__device__ __forceinline__ double adj_frac(double v, double e, double o, double h_inv) {
  return (v - o) * h_inv - e;
}

// Geometry of one particle in its cell: shape fractions, their derivative
// weights, e^{i m phi} and the radius.
template <typename T, int M>
struct PGeom {
  T C[4], Cx[4], Cr[4];  // shape weights, d/dx, d/dr
  T cs[M + 1], sn[M + 1];
  T c1, s1, rinv;
};

template <typename T, int M>
__device__ __forceinline__ void pgeom(PGeom<T, M> &p, T xp, T yp, T zp, T sX1, T sR1,
                                      T dx_inv, T dr_inv) {
  const T r2 = yp * yp + zp * zp;
  const T rp = sqrt(r2);
  p.rinv = rp > T(0) ? T(1) / rp : T(0);
  p.c1 = yp * p.rinv;
  p.s1 = zp * p.rinv;
  p.cs[0] = T(1);
  p.sn[0] = T(0);
#pragma unroll
  for (int m = 1; m <= M; m++) {
    p.cs[m] = p.cs[m - 1] * p.c1 - p.sn[m - 1] * p.s1;
    p.sn[m] = p.cs[m - 1] * p.s1 + p.sn[m - 1] * p.c1;
  }
  const T sX0 = T(1) - sX1, sR0 = T(1) - sR1;
  p.C[0] = sR0 * sX0;
  p.C[1] = sR0 * sX1;
  p.C[2] = sR1 * sX0;
  p.C[3] = sR1 * sX1;
  p.Cx[0] = -sR0 * dx_inv;
  p.Cx[1] = sR0 * dx_inv;
  p.Cx[2] = -sR1 * dx_inv;
  p.Cx[3] = sR1 * dx_inv;
  p.Cr[0] = -sX0 * dr_inv;
  p.Cr[1] = -sX1 * dr_inv;
  p.Cr[2] = sX0 * dr_inv;
  p.Cr[3] = sX1 * dr_inv;
}

// (lr, lphi) -> (ly, lz): r = |(y, z)|, phi = atan2(z, y)
template <typename T, int M>
__device__ __forceinline__ void polar_to_yz(const PGeom<T, M> &p, T lr, T lphi, T &ly, T &lz) {
  ly = lr * p.c1 - lphi * p.s1 * p.rinv;
  lz = lr * p.s1 + lphi * p.c1 * p.rinv;
}

// The tile's particles: rows ir = nr0 .. nr0+AT_TR-1 of valid cells
// 0 < ix < Nx-2, 0 <= ir < Nr-2, one contiguous range of sort_indx per row.
struct TileRows {
  u32 a[AT_TR], pre[AT_TR + 1];
  int ixl, ixh;
};

__device__ __forceinline__ void tile_rows(TileRows &tr, const u32 *__restrict__ cell_off,
                                          int Nx, int Nr, int nx0, int nr0) {
  const int nxc = Nx - 1;
  const int ixl = nx0 > 1 ? nx0 : 1, ixh = nx0 + AT_TX - 1 < Nx - 3 ? nx0 + AT_TX - 1 : Nx - 3;
  if (threadIdx.x == 0) {
    tr.ixl = ixl;
    tr.ixh = ixh;
  }
  if (threadIdx.x < AT_TR) {
    const int ir = nr0 + threadIdx.x;
    u32 a = 0, b = 0;
    if (ir < Nr - 2 && ixl <= ixh) {
      a = cell_off[(long)ixl + (long)ir * nxc];
      b = cell_off[(long)ixh + (long)ir * nxc + 1];
    }
    tr.a[threadIdx.x] = a;
    tr.pre[threadIdx.x + 1] = b - a;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    tr.pre[0] = 0;
    for (int r = 0; r < AT_TR; r++) tr.pre[r + 1] += tr.pre[r];
  }
  __syncthreads();
}

__device__ __forceinline__ void tile_item(const TileRows &tr, u32 idx, int &row, u32 &pos) {
  int r = 0;
#pragma unroll
  for (int q = 1; q < AT_TR; q++) r += idx >= tr.pre[q];
  row = r;
  pos = tr.a[r] + (idx - tr.pre[r]);
}

// ---------------------------------------------------------------------
// Deposit adjoint.  lam: node adjoints of the deposit targets before the
// post-processing (VEC: 3(M+1) pointers m-major then x, y, z; else M+1),
// mode 0 real, modes >= 1 complex.  Adds to the particle adjoints
// lx, ly, lz (may be null: positions held fixed), lw, and for VEC lu*, lg.
template <typename T, int M, bool VEC>
__global__ void __launch_bounds__(AT_THREADS)
    k_deposit_adj(const u32 *__restrict__ sort_indx, const u32 *__restrict__ cell_off,
                  const T *__restrict__ x, const T *__restrict__ y, const T *__restrict__ z,
                  const T *__restrict__ ux, const T *__restrict__ uy,
                  const T *__restrict__ uz, const T *__restrict__ g_inv,
                  const T *__restrict__ w, T q, GridP<T> g, ptrs<12> lam,
                  T *__restrict__ lx, T *__restrict__ ly, T *__restrict__ lz,
                  T *__restrict__ lw, T *__restrict__ lux, T *__restrict__ luy,
                  T *__restrict__ luz, T *__restrict__ lg) {
  pdl_wait();
  constexpr int NK = VEC ? 3 : 1, B = 1 + 2 * M, NS = NK * B;
  extern __shared__ __align__(16) unsigned char adj_sm[];
  T *nsm = (T *)adj_sm;  // [AT_NR][AT_NX][NS]
  __shared__ TileRows tr;
  __shared__ typename AdjEdge<T>::type xedge[AT_TX], redge[AT_TR];
  const int Nx = g.Nx, Nr = g.Nr;
  const int nx0 = blockIdx.x * AT_TX, nr0 = blockIdx.y * AT_TR;
  if (threadIdx.x < AT_TX) xedge[threadIdx.x] = adj_x_edge(g, nx0 + threadIdx.x);
  else if (threadIdx.x < AT_TX + AT_TR)
    redge[threadIdx.x - AT_TX] = adj_r_edge(g, nr0 + threadIdx.x - AT_TX);
  for (int t = threadIdx.x; t < AT_NR * AT_NX; t += AT_THREADS) {
    const int lr = t / AT_NX, lc = t - lr * AT_NX;
    const int nr = nr0 + lr, nx = nx0 + lc;
    T *d = nsm + t * NS;
    const bool in = nr < Nr && nx < Nx;
    const long node = (long)nr * Nx + nx;
#pragma unroll
    for (int k = 0; k < NK; k++) {
      d[k * B] = in ? ((const T *)lam.p[k])[node] : T(0);
#pragma unroll
      for (int m = 1; m <= M; m++) {
        const T *fm = (const T *)lam.p[m * NK + k];
        d[k * B + 2 * m - 1] = in ? fm[2 * node] : T(0);
        d[k * B + 2 * m] = in ? fm[2 * node + 1] : T(0);
      }
    }
  }
  tile_rows(tr, cell_off, Nx, Nr, nx0, nr0);
  const u32 total = tr.pre[AT_TR];
  for (u32 idx = threadIdx.x; idx < total; idx += AT_THREADS) {
    int row;
    u32 pos;
    tile_item(tr, idx, row, pos);
    const u32 p = sort_indx[pos];
    const T xp = x[p], yp = y[p], zp = z[p];
    const T rp = sqrt(yp * yp + zp * zp);
    int ix = (int)floor((xp - g.xmin) * g.dx_inv);
    ix = ix < tr.ixl ? tr.ixl : (ix > tr.ixh ? tr.ixh : ix);
    const T sX1 = adj_frac(xp, xedge[ix - nx0], g.xmin, g.dx_inv);
    const T sR1 = adj_frac(rp, redge[row], g.rmin, g.dr_inv);
    PGeom<T, M> pg;
    pgeom<T, M>(pg, xp, yp, zp, sX1, sR1, g.dx_inv, g.dr_inv);
    const int l0 = (row * AT_NX + (ix - nx0)) * NS;
    const int loff[4] = {l0, l0 + NS, l0 + AT_NX * NS, l0 + (AT_NX + 1) * NS};
    T SA[NK], SAx[NK], SAr[NK], SB[NK];
#pragma unroll
    for (int k = 0; k < NK; k++) {
      SA[k] = SAx[k] = SAr[k] = SB[k] = T(0);
#pragma unroll
      for (int c = 0; c < 4; c++) {
        const T *d = nsm + loff[c] + k * B;
        T A = d[0], Bp = T(0);
#pragma unroll
        for (int m = 1; m <= M; m++) {
          const T re = d[2 * m - 1], im = d[2 * m];
          A += re * pg.cs[m] + im * pg.sn[m];
          Bp += T(m) * (im * pg.cs[m] - re * pg.sn[m]);
        }
        SA[k] += pg.C[c] * A;
        SAx[k] += pg.Cx[c] * A;
        SAr[k] += pg.Cr[c] * A;
        SB[k] += pg.C[c] * Bp;
      }
    }
    const T wp = w[p];
    T fw, fx, fr, fphi;  // d/dw and the position derivatives' common factors
    if (VEC) {
      const T gi = g_inv[p];
      const T u[3] = {ux[p], uy[p], uz[p]};
      T su = T(0), sux = T(0), sur = T(0), sub = T(0);
#pragma unroll
      for (int k = 0; k < NK; k++) {
        su += u[k] * SA[k];
        sux += u[k] * SAx[k];
        sur += u[k] * SAr[k];
        sub += u[k] * SB[k];
      }
      const T qwg = q * wp * gi;
      lux[p] += qwg * SA[0];
      luy[p] += qwg * SA[NK > 1 ? 1 : 0];
      luz[p] += qwg * SA[NK > 2 ? 2 : 0];
      lg[p] += q * wp * su;
      fw = q * gi * su;
      fx = qwg * sux;
      fr = qwg * sur;
      fphi = qwg * sub;
    } else {
      fw = q * SA[0];
      fx = q * wp * SAx[0];
      fr = q * wp * SAr[0];
      fphi = q * wp * SB[0];
    }
    lw[p] += fw;
    if (lx) {
      T a, b;
      polar_to_yz<T, M>(pg, fr, fphi, a, b);
      lx[p] += fx;
      ly[p] += a;
      lz[p] += b;
    }
  }
}

// ---------------------------------------------------------------------
// Gather + Boris push adjoint.  F: the real-space E, B the forward gathered
// (6(M+1) pointers, m-major then ex, ey, ez, bx, by, bz, after the ghost
// rows); lF: their adjoints, added to (same layout).  u_old: the momenta
// before the push.  On entry lu*, lg hold the adjoints of the pushed u and
// g_inv; for every pushed particle they are replaced by the adjoint of the
// momenta before the push (lg by 0: the push overwrites g_inv), and lx, ly,
// lz are added to.  Particles the forward skipped (number >= *np_stay, the
// reference's quirk, or outside the window's cells) keep theirs.
template <typename T>
__device__ __forceinline__ void cross3(const T a[3], const T b[3], T o[3]) {
  o[0] = a[1] * b[2] - a[2] * b[1];
  o[1] = a[2] * b[0] - a[0] * b[2];
  o[2] = a[0] * b[1] - a[1] * b[0];
}

// One thread per cell of a 32 x 8-cell tile (the forward deposit's
// decomposition): the thread walks its cell's particles in sort order,
// reverses each particle's push, and sums the particle's field adjoints on
// the cell's 4 corner nodes in registers; the sums are added to the tile's
// node accumulators in shared memory in four phases, one per cell colour
// (ix & 1) + 2 (ir & 1) -- cells of one colour share no node, so no atomics --
// and the tile's nodes go to the global adjoints with one atomic each (the
// border nodes are shared with the neighbouring tiles).
template <typename T, int M>
__global__ void __launch_bounds__(AT_THREADS)
    k_gather_push_adj(const T *__restrict__ x, const T *__restrict__ y,
                      const T *__restrict__ z, const T *__restrict__ uxo,
                      const T *__restrict__ uyo, const T *__restrict__ uzo,
                      const u32 *__restrict__ sort_indx, const u32 *__restrict__ cell_off,
                      const u32 *__restrict__ np_stay_p, T dt, GridP<T> g, ptrs<24> F,
                      ptrs<24> lF, T *__restrict__ lx, T *__restrict__ ly, T *__restrict__ lz,
                      T *__restrict__ lux, T *__restrict__ luy, T *__restrict__ luz,
                      T *__restrict__ lg) {
  pdl_wait();
  constexpr int NS = 6 * (1 + 2 * M);
  extern __shared__ __align__(16) unsigned char adj_sm[];
  T *fsm = (T *)adj_sm;                     // [AT_NR][AT_NX][NS] fields (m >= 1 doubled)
  T *asm_ = fsm + AT_NR * AT_NX * NS;       // the same layout: adjoint accumulators
  const int Nx = g.Nx, Nr = g.Nr, nxc = Nx - 1;
  const int nx0 = blockIdx.x * AT_TX, nr0 = blockIdx.y * AT_TR;
  const u32 np_stay = *np_stay_p;
  for (int t = threadIdx.x; t < AT_NR * AT_NX; t += AT_THREADS) {
    const int lr = t / AT_NX, lc = t - lr * AT_NX;
    const int nr = nr0 + lr, nx = nx0 + lc;
    T *d = fsm + t * NS;
    T *a = asm_ + t * NS;
    const bool in = nr < Nr && nx < Nx;
    const long node = (long)nr * Nx + nx;
#pragma unroll
    for (int k = 0; k < 6; k++) d[k] = in ? ((const T *)F.p[k])[node] : T(0);
#pragma unroll
    for (int m = 1; m <= M; m++)
#pragma unroll
      for (int k = 0; k < 6; k++) {
        const T *fm = (const T *)F.p[6 * m + k];
        d[6 + 12 * (m - 1) + 2 * k] = in ? T(2) * fm[2 * node] : T(0);
        d[6 + 12 * (m - 1) + 2 * k + 1] = in ? T(2) * fm[2 * node + 1] : T(0);
      }
#pragma unroll
    for (int q = 0; q < NS; q++) a[q] = T(0);
  }
  __syncthreads();
  const int tx = threadIdx.x % AT_TX, ty = threadIdx.x / AT_TX;
  const int ix = nx0 + tx, ir = nr0 + ty;
  const bool valid = ix > 0 && ix < Nx - 2 && ir >= 0 && ir < Nr - 2;
  T acc[4][NS];
#pragma unroll
  for (int c = 0; c < 4; c++)
#pragma unroll
    for (int q = 0; q < NS; q++) acc[c][q] = T(0);
  const int l0 = (ty * AT_NX + tx) * NS;
  const int loff[4] = {l0, l0 + NS, l0 + AT_NX * NS, l0 + (AT_NX + 1) * NS};
  const T h = T(0.5) * dt;
  if (valid) {
    const long cg = (long)ix + (long)ir * nxc;
    const u32 q0 = cell_off[cg], q1 = cell_off[cg + 1];
    const typename AdjEdge<T>::type ex = adj_x_edge(g, ix), er = adj_r_edge(g, ir);
    for (u32 q = q0; q < q1; q++) {
      const u32 p = sort_indx[q];
      if (p >= np_stay) continue;  // not pushed by the forward
      const T xp = x[p], yp = y[p], zp = z[p];
      const T rp = sqrt(yp * yp + zp * zp);
      const T sX1 = adj_frac(xp, ex, g.xmin, g.dx_inv);
      const T sR1 = adj_frac(rp, er, g.rmin, g.dr_inv);
      PGeom<T, M> pg;
      pgeom<T, M>(pg, xp, yp, zp, sX1, sR1, g.dx_inv, g.dr_inv);
      // fields at the particle, their x, r and phi derivatives
      T fld[6], fx[6], fr[6], fph[6];
#pragma unroll
      for (int k = 0; k < 6; k++) {
        fld[k] = fx[k] = fr[k] = fph[k] = T(0);
#pragma unroll
        for (int c = 0; c < 4; c++) {
          const T *d = fsm + loff[c];
          T Fv = d[k], Dv = T(0);
#pragma unroll
          for (int m = 1; m <= M; m++) {
            const T re = d[6 + 12 * (m - 1) + 2 * k], im = d[6 + 12 * (m - 1) + 2 * k + 1];
            Fv += re * pg.cs[m] + im * pg.sn[m];
            Dv += T(m) * (im * pg.cs[m] - re * pg.sn[m]);
          }
          fld[k] += pg.C[c] * Fv;
          fx[k] += pg.Cx[c] * Fv;
          fr[k] += pg.Cr[c] * Fv;
          fph[k] += pg.C[c] * Dv;
        }
      }
      // Boris push, forward (its intermediates)
      const T u[3] = {uxo[p], uyo[p], uzo[p]};
      T um[3], t[3], sv[3], u0[3], up[3], un[3];
#pragma unroll
      for (int k = 0; k < 3; k++) um[k] = u[k] + h * fld[k];
      const T gi0 = T(1) / sqrt(T(1) + um[0] * um[0] + um[1] * um[1] + um[2] * um[2]);
#pragma unroll
      for (int k = 0; k < 3; k++) t[k] = h * fld[3 + k] * gi0;
      const T f2 = T(2) / (T(1) + t[0] * t[0] + t[1] * t[1] + t[2] * t[2]);
#pragma unroll
      for (int k = 0; k < 3; k++) sv[k] = t[k] * f2;
      cross3(um, t, u0);
#pragma unroll
      for (int k = 0; k < 3; k++) u0[k] += um[k];
      cross3(u0, sv, up);
#pragma unroll
      for (int k = 0; k < 3; k++) up[k] += um[k];
#pragma unroll
      for (int k = 0; k < 3; k++) un[k] = up[k] + h * fld[k];
      const T gn = T(1) / sqrt(T(1) + un[0] * un[0] + un[1] * un[1] + un[2] * un[2]);
      // ... and reversed
      T lun[3] = {lux[p], luy[p], luz[p]};
      const T lgn = lg[p];
      const T gg3 = -lgn * gn * gn * gn;
#pragma unroll
      for (int k = 0; k < 3; k++) lun[k] += gg3 * un[k];
      T lE[3], lB[3], lum[3], lu0[3], lsv[3], lt[3], tmp[3];
#pragma unroll
      for (int k = 0; k < 3; k++) {
        lE[k] = h * lun[k];
        lum[k] = lun[k];  // up = um + u0 x sv
      }
      cross3(sv, lun, lu0);
      cross3(lun, u0, lsv);
      cross3(t, lu0, tmp);  // u0 = um + um x t
#pragma unroll
      for (int k = 0; k < 3; k++) lum[k] += lu0[k] + tmp[k];
      cross3(lu0, um, lt);
      T lf2 = T(0);
#pragma unroll
      for (int k = 0; k < 3; k++) {
        lt[k] += f2 * lsv[k];  // sv = t f2
        lf2 += t[k] * lsv[k];
      }
      const T cf = -lf2 * f2 * f2;  // f2 = 2 / (1 + |t|^2)
      T lgi0 = T(0);
#pragma unroll
      for (int k = 0; k < 3; k++) {
        lt[k] += cf * t[k];
        lB[k] = h * gi0 * lt[k];  // t = h B gi0
        lgi0 += h * fld[3 + k] * lt[k];
      }
      const T cg0 = -lgi0 * gi0 * gi0 * gi0;  // gi0 = (1 + |um|^2)^-1/2
#pragma unroll
      for (int k = 0; k < 3; k++) {
        lum[k] += cg0 * um[k];
        lE[k] += h * lum[k];  // um = u + h E
      }
      lux[p] = lum[0];
      luy[p] = lum[1];
      luz[p] = lum[2];
      lg[p] = T(0);
      // position adjoint from the gathered fields' derivatives
      const T lf[6] = {lE[0], lE[1], lE[2], lB[0], lB[1], lB[2]};
      T sx = T(0), sr = T(0), sphi = T(0);
#pragma unroll
      for (int k = 0; k < 6; k++) {
        sx += lf[k] * fx[k];
        sr += lf[k] * fr[k];
        sphi += lf[k] * fph[k];
      }
      T a, b;
      polar_to_yz<T, M>(pg, sr, sphi, a, b);
      lx[p] += sx;
      ly[p] += a;
      lz[p] += b;
      // the field adjoints on the cell's corners (mode m >= 1: 2 C (cos, sin))
#pragma unroll
      for (int c = 0; c < 4; c++)
#pragma unroll
        for (int k = 0; k < 6; k++) {
          const T v = pg.C[c] * lf[k];
          acc[c][k] += v;
#pragma unroll
          for (int m = 1; m <= M; m++) {
            acc[c][6 + 12 * (m - 1) + 2 * k] += T(2) * v * pg.cs[m];
            acc[c][6 + 12 * (m - 1) + 2 * k + 1] += T(2) * v * pg.sn[m];
          }
        }
    }
  }
  // the corner sums onto the tile's nodes, colour by colour
  const int colour = (ix & 1) + 2 * (ir & 1);
#pragma unroll
  for (int col = 0; col < 4; col++) {
    __syncthreads();
    if (valid && colour == col) {
#pragma unroll
      for (int c = 0; c < 4; c++) {
        T *a = asm_ + loff[c];
#pragma unroll
        for (int q = 0; q < NS; q++) a[q] += acc[c][q];
      }
    }
  }
  __syncthreads();
  // flush the tile's node adjoints (border nodes are shared with the
  // neighbouring tiles)
  for (int tt = threadIdx.x; tt < AT_NR * AT_NX; tt += AT_THREADS) {
    const int lr = tt / AT_NX, lc = tt - lr * AT_NX;
    const int nr = nr0 + lr, nx = nx0 + lc;
    if (nr >= Nr || nx >= Nx) continue;
    const long node = (long)nr * Nx + nx;
    const T *a = asm_ + tt * NS;
#pragma unroll
    for (int k = 0; k < 6; k++)
      if (a[k] != T(0)) atomicAdd((T *)lF.p[k] + node, a[k]);
#pragma unroll
    for (int m = 1; m <= M; m++)
#pragma unroll
      for (int k = 0; k < 6; k++) {
        T *fm = (T *)lF.p[6 * m + k];
        const T re = a[6 + 12 * (m - 1) + 2 * k], im = a[6 + 12 * (m - 1) + 2 * k + 1];
        if (re != T(0)) atomicAdd(fm + 2 * node, re);
        if (im != T(0)) atomicAdd(fm + 2 * node + 1, im);
      }
  }
}

// push_xyz transposed: x += dt g u  =>  lu += dt g lx, lg += dt (lx . u)
template <typename T>
__global__ void k_push_x_adj(long np, const T *__restrict__ ux, const T *__restrict__ uy,
                             const T *__restrict__ uz, const T *__restrict__ g_inv,
                             const T *__restrict__ lx, const T *__restrict__ ly,
                             const T *__restrict__ lz, T *__restrict__ lux,
                             T *__restrict__ luy, T *__restrict__ luz, T *__restrict__ lg,
                             T dt) {
  pdl_wait();
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < np;
       i += (long)gridDim.x * blockDim.x) {
    const T gd = g_inv[i] * dt;
    const T a = lx[i], b = ly[i], c = lz[i];
    lux[i] += gd * a;
    luy[i] += gd * b;
    luz[i] += gd * c;
    lg[i] += dt * (a * ux[i] + b * uy[i] + c * uz[i]);
  }
}

// ---------------------------------------------------------------------
// Spectral and grid-side adjoints (grid-stride, HBM-bound).
#define CCL_GS(i, n)                                                           \
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < (n);         \
       i += (long)gridDim.x * blockDim.x)

// PSATD update transposed (the split form's coefficients, per cell:
// c1, c2, s, s2, q2, a2, b2, d2).  f: lE xyz, lG xyz (in: of the updated
// fields; out: of the old ones), lJ xyz (written; times filt when given:
// the smoothing filter of the current's forward transform, transposed in
// the same pass), lN0 xyz (written), lN1 xyz (added to).
template <typename T>
__global__ void __launch_bounds__(256)
    k_psatd_adj(long n, const T *__restrict__ coef, const T *__restrict__ filt, ptrs<15> f) {
  pdl_wait();
  CCL_GS(i, n) {
    const T fj = filt ? filt[i] : T(1);
    T c[8];
#pragma unroll
    for (int k = 0; k < 8; k++) c[k] = coef[8 * i + k];
    const T c1 = c[0], c2 = c[1], s = c[2], s2 = c[3], q2 = c[4], a2 = c[5], b2 = c[6],
            d2 = c[7];
#pragma unroll
    for (int k = 0; k < 3; k++) {
      const cplx<T> e1 = ld_c((const T *)f.p[k], i), g1 = ld_c((const T *)f.p[3 + k], i);
      const cplx<T> n1 = ld_c((const T *)f.p[12 + k], i);
      st_c((T *)f.p[k], i, cplx<T>{c1 * e1.re - c2 * g1.re, c1 * e1.im - c2 * g1.im});
      st_c((T *)f.p[3 + k], i, cplx<T>{s * e1.re + c1 * g1.re, s * e1.im + c1 * g1.im});
      st_c((T *)f.p[6 + k], i,
           cplx<T>{fj * (-s2 * e1.re + q2 * g1.re), fj * (-s2 * e1.im + q2 * g1.im)});
      st_c((T *)f.p[9 + k], i,
           cplx<T>{a2 * e1.re + (d2 - s2) * g1.re, a2 * e1.im + (d2 - s2) * g1.im});
      st_c((T *)f.p[12 + k], i,
           cplx<T>{n1.re + b2 * e1.re - d2 * g1.re, n1.im + b2 * e1.im - d2 * g1.im});
    }
  }
}

// m = -1 mirror (-Re, +Im) at column (nx - ix) mod nx: its own transpose
template <typename T>
__device__ __forceinline__ cplx<T> mirror_at(const T *p, long ir, long ix, int nx) {
  const long io = ix == 0 ? 0 : nx - ix;
  cplx<T> q = ld_c(p, ir * nx + io);
  q.re = -q.re;
  return q;
}

// Gradient combine transposed, first half.  ldN: 3(M+1) adjoints of the
// gradient (m-major, x y z).  Writes lrho[m] = -i kx ldN_x (the direct
// term), Pm[m] = -ldN_y + i ldN_z (mirrored for m = 0) and
// Pp[m] = ldN_y + i ldN_z, for the radial products' transposes.
template <typename T>
__global__ void __launch_bounds__(RC_THREADS)
    k_grad_adj_pre(int nx, int M, const T *__restrict__ kx, ptrs<12> ldN, ptrs<4> lrho,
                   ptrs<4> Pm, ptrs<4> Pp) {
  pdl_wait();
  const int m = blockIdx.y;
  const RowChunk<T> rc(nx);
  const T *lx = (const T *)pick(ldN, 3 * m), *ly = (const T *)pick(ldN, 3 * m + 1),
          *lz = (const T *)pick(ldN, 3 * m + 2);
  T *lr = (T *)pick(lrho, m), *pmp = (T *)pick(Pm, m), *ppp = (T *)pick(Pp, m);
#pragma unroll
  for (int q = 0; q < RcPer<T>; q++) {
    const long ir = rc.ir, ix = rc.col(q);
    if (ix >= nx) continue;
    const long i = ir * nx + ix;
    const T k = kx[ix];
    const cplx<T> ax = ld_c(lx, i);
    st_c(lr, i, cplx<T>{k * ax.im, -k * ax.re});
    if (pmp) {
      // -ly + i lz, at the mirrored column for m = 0
      cplx<T> ay, az;
      if (m == 0) {
        const long io = ix == 0 ? 0 : nx - ix;
        ay = ld_c((const T *)ldN.p[1], ir * nx + io);
        az = ld_c((const T *)ldN.p[2], ir * nx + io);
        const cplx<T> v = {-ay.re - az.im, -ay.im + az.re};
        st_c(pmp, i, cplx<T>{-v.re, v.im});
      } else {
        ay = ld_c(ly, i);
        az = ld_c(lz, i);
        st_c(pmp, i, cplx<T>{-ay.re - az.im, -ay.im + az.re});
      }
    }
    if (ppp) {
      const cplx<T> ay = ld_c(ly, i);
      const cplx<T> az = ld_c(lz, i);
      st_c(ppp, i, cplx<T>{ay.re - az.im, ay.im + az.re});
    }
  }
}

// Second half: lrho[j] += Rm[j+1] + Rp[j-1] (+ Rm[0] for j = 1), where
// Rm[m] = dDHT_minus_m^T Pm[m], Rp[m] = dDHT_plus_m^T Pp[m] (null where
// absent); ncomp arrays per mode (1 for the gradient, 3 for the curl); the
// sums times filt[j] where given.
template <typename T>
__global__ void k_modes_adj_post(long n, int M, int ncomp, ptrs<12> lo, ptrs<12> Rm,
                                 ptrs<12> Rp, ptrs<4> filt) {
  pdl_wait();
  const int j = blockIdx.y / ncomp, c = blockIdx.y - j * ncomp;
  const T *fl = (const T *)pick(filt, j);
  T *lop = (T *)pick(lo, j * ncomp + c);
  const T *srcs[3] = {j + 1 <= M ? (const T *)pick(Rm, (j + 1) * ncomp + c) : nullptr,
                      j >= 1 ? (const T *)pick(Rp, (j - 1) * ncomp + c) : nullptr,
                      j == 1 ? (const T *)pick(Rm, c) : nullptr};
  CCL_GS(i, n) {
    cplx<T> v = ld_c(lop, i);
#pragma unroll
    for (int q = 0; q < 3; q++)
      if (srcs[q]) {
        const cplx<T> a = ld_c(srcs[q], i);
        v.re += a.re;
        v.im += a.im;
      }
    if (fl) {
      v.re *= fl[i];
      v.im *= fl[i];
    }
    st_c(lop, i, v);
  }
}

// Curl combine transposed, first half.  lB: 3(M+1) adjoints of B (after
// the Poisson factor, which is applied here first).  Adds the direct terms
// to lG (lGy -= i kx lBz, lGz += i kx lBy) and writes
//   Qm_x = i lBy + lBz, Qm_y = -i lBx, Qm_z = -lBx  (mirrored for m = 0),
//   Qp_x = i lBy - lBz, Qp_y = -i lBx, Qp_z = lBx.
template <typename T>
__global__ void __launch_bounds__(RC_THREADS)
    k_rot_adj_pre(int nx, int M, const T *__restrict__ kx, ptrs<4> poiss, ptrs<12> lB,
                  ptrs<12> lG, ptrs<12> Qm, ptrs<12> Qp) {
  pdl_wait();
  const int m = blockIdx.y;
  const RowChunk<T> rc(nx);
  const T *pf = (const T *)pick(poiss, m);
  const T *lbp[3];
  T *qmp[3], *qpp[3];
#pragma unroll
  for (int c = 0; c < 3; c++) {
    lbp[c] = (const T *)pick(lB, 3 * m + c);
    qmp[c] = (T *)pick(Qm, 3 * m + c);
    qpp[c] = (T *)pick(Qp, 3 * m + c);
  }
  T *lgy = (T *)pick(lG, 3 * m + 1), *lgz = (T *)pick(lG, 3 * m + 2);
#pragma unroll
  for (int q = 0; q < RcPer<T>; q++) {
    const long ir = rc.ir, ix = rc.col(q);
    if (ix >= nx) continue;
    const long i = ir * nx + ix;
    const T k = kx[ix];
    auto lb = [&](int c, long at) {
      cplx<T> v = ld_c(lbp[c], at);
      if (pf) {
        const T f = pf[at];
        v.re *= f;
        v.im *= f;
      }
      return v;
    };
    const cplx<T> bx = lb(0, i), by = lb(1, i), bz = lb(2, i);
    cplx<T> gy = ld_c(lgy, i), gz = ld_c(lgz, i);
    gy.re += k * bz.im;   // -i k bz
    gy.im -= k * bz.re;
    gz.re -= k * by.im;   // +i k by
    gz.im += k * by.re;
    st_c(lgy, i, gy);
    st_c(lgz, i, gz);
    if (qmp[0]) {
      cplx<T> ax = bx, ay = by, az = bz;
      if (m == 0) {
        const long io = ix == 0 ? 0 : nx - ix;
        ax = lb(0, ir * nx + io);
        ay = lb(1, ir * nx + io);
        az = lb(2, ir * nx + io);
      }
      cplx<T> qx = {-ay.im + az.re, ay.re + az.im};
      cplx<T> qy = {ax.im, -ax.re};
      cplx<T> qz = {-ax.re, -ax.im};
      if (m == 0) {
        qx.re = -qx.re;
        qy.re = -qy.re;
        qz.re = -qz.re;
      }
      st_c(qmp[0], i, qx);
      st_c(qmp[1], i, qy);
      st_c(qmp[2], i, qz);
    }
    if (qpp[0]) {
      st_c(qpp[0], i, cplx<T>{-by.im - bz.re, by.re - bz.im});
      st_c(qpp[1], i, cplx<T>{bx.im, -bx.re});
      st_c(qpp[2], i, cplx<T>{bx.re, bx.im});
    }
  }
}

// Deposit post-processing transposed (k_postproc: row 1 -= row 0, then
// x dV_inv per row): in place, row 0 <- row 0 dv[0] - row 1 dv[1], others
// x dv[ir].
template <typename T>
__global__ void k_postproc_adj(ptrs<32> f, int Mp1, int Nx, int Nr, const T *__restrict__ dv) {
  pdl_wait();
  const int pidx = blockIdx.z, m = pidx % Mp1;
  const int ir = blockIdx.y + 1;
  const int ix = blockIdx.x * blockDim.x + threadIdx.x;
  if (ix >= Nx) return;
  T *a = (T *)f.p[pidx];
  const int nc = m == 0 ? 1 : 2;
  for (int c = 0; c < nc; c++) {
    const long i = ((long)ir * Nx + ix) * nc + c;
    if (ir == 1) {
      const long i0 = (long)ix * nc + c;
      const T l1 = a[i], l0 = a[i0];
      a[i] = l1 * dv[1];
      a[i0] = l0 * dv[0] - l1 * dv[1];
    } else {
      a[i] = a[i] * dv[ir];
    }
  }
}

// ghost rows transposed: row 0 = +row 1 (m = 0) or -row 1 (m >= 1)
template <typename T>
__global__ void k_warp_axis_adj(ptrs<32> f, int Mp1, int Nx) {
  pdl_wait();
  const int pidx = blockIdx.y, m = pidx % Mp1;
  const int ix = blockIdx.x * blockDim.x + threadIdx.x;
  if (ix >= Nx) return;
  T *a = (T *)f.p[pidx];
  if (m == 0) {
    a[ix + Nx] += a[ix];
    a[ix] = T(0);
  } else {
    a[2 * (ix + Nx)] -= a[2 * ix];
    a[2 * (ix + Nx) + 1] -= a[2 * ix + 1];
    a[2 * ix] = T(0);
    a[2 * ix + 1] = T(0);
  }
}

// dst[a] += src[a] over `narr` arrays of n[a] reals (blockIdx.y = array)
struct AddBatch {
  void *dst[32];
  const void *src[32];
  long n[32];
};
template <typename T>
__global__ void k_add_batch(AddBatch b) {
  pdl_wait();
  const int a = blockIdx.y;
  T *d = (T *)b.dst[a];
  const T *s = (const T *)b.src[a];
  CCL_GS(i, b.n[a]) d[i] += s[i];
}

// dst[a][i] = src[a][i] for i < n[a] 32-bit words, a < narr (blockIdx.y);
// 16 bytes per access where both arrays are 16-byte aligned (the recording's
// snapshots and the checkpoints' restores move ~100 MB a step), the
// remainder word by word
template <typename W>
__global__ void k_copy_batch(AddBatch b) {
  pdl_wait();
  const int a = blockIdx.y;
  W *d = (W *)b.dst[a];
  const W *s = (const W *)b.src[a];
  const long n = b.n[a];
  long head = 0;
  if ((((uintptr_t)d | (uintptr_t)s) & 15) == 0) {
    const long n4 = n / 4;
    CCL_GS(i, n4) reinterpret_cast<uint4 *>(d)[i] = reinterpret_cast<const uint4 *>(s)[i];
    head = n4 * 4;
  }
  for (long i = head + blockIdx.x * (long)blockDim.x + threadIdx.x; i < n;
       i += (long)gridDim.x * blockDim.x)
    d[i] = s[i];
}

// align transposed: dst[c][idx[i]] = src[c][i], i < n
template <typename T>
__global__ void k_scatter(long n, int ncomp, ptrs<16> src, ptrs<16> dst,
                          const u32 *__restrict__ idx) {
  pdl_wait();
  CCL_GS(i, n) {
    const u32 j = idx[i];
#pragma unroll
    for (int c = 0; c < 16; c++)
      if (c < ncomp) ((T *)dst.p[c])[j] = ((const T *)src.p[c])[i];
  }
}

// density profile transposed: w = w0 f(x), f piecewise linear through
// (xx[k], ff[k]); lff[k] += sum_i lw[i] w[i] / f(x_i) df/dff[k](x_i), in
// double, per block in shared memory then one atomic per knot per block.
constexpr int DP_MAXK = 256;
template <typename T>
__global__ void k_dens_profile_adj(long np, const T *__restrict__ x, const T *__restrict__ w,
                                   const T *__restrict__ lw, const double *__restrict__ xx,
                                   const double *__restrict__ ff,
                                   const double *__restrict__ dxm1, u32 nloc,
                                   double *__restrict__ lff) {
  pdl_wait();
  __shared__ double acc[DP_MAXK];
  for (u32 k = threadIdx.x; k < nloc; k += blockDim.x) acc[k] = 0.0;
  __syncthreads();
  CCL_GS(i, np) {
    const double xp = (double)x[i];
    u32 k;
    for (k = 0; k < nloc - 1; k++)
      if (xp > xx[k] && xp <= xx[k + 1]) break;
    if (k > nloc - 2) k = nloc - 2;
    const double am = dxm1[k] * (xx[k + 1] - xp), ap = dxm1[k] * (xp - xx[k]);
    const double f = ff[k] * am + ff[k + 1] * ap;
    if (f != 0.0) {
      const double s = (double)lw[i] * (double)w[i] / f;
      atomicAdd(&acc[k], s * am);
      atomicAdd(&acc[k + 1], s * ap);
    }
  }
  __syncthreads();
  for (u32 k = threadIdx.x; k < nloc; k += blockDim.x)
    if (acc[k] != 0.0) atomicAdd(&lff[k], acc[k]);
}

#undef CCL_GS

// ---------------------------------------------------------------------
// launchers
template <typename T, bool VEC, int M>
static int deposit_adj_m(const u32 *si, const u32 *co, const T *x, const T *y, const T *z,
                         const T *ux, const T *uy, const T *uz, const T *gi, const T *w, int q,
                         GridP<T> g, void *const *lam, T *lx, T *ly, T *lz, T *lw, T *lux,
                         T *luy, T *luz, T *lg, cudaStream_t s) {
  constexpr int NK = VEC ? 3 : 1;
  ptrs<12> L;
  for (int i = 0; i < NK * (M + 1); i++) {
    CCL_REQUIRE(lam[i], CCL_ERR_ARG, "deposit_adjoint: null adjoint field %d", i);
    L.p[i] = lam[i];
  }
  const size_t smem = (size_t)AT_NR * AT_NX * NK * (1 + 2 * M) * sizeof(T);
  auto kern = k_deposit_adj<T, M, VEC>;
  static bool set = false;
  if (!set) {
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    set = true;
  }
  dim3 grid((g.Nx + AT_TX - 1) / AT_TX, (g.Nr + AT_TR - 1) / AT_TR);
  launch_pdl(kern, grid, AT_THREADS, smem, s, si, co, x, y, z, ux, uy, uz, gi, w, (T)(signed char)q,
             g, L, lx, ly, lz, lw, lux, luy, luz, lg);
  CCL_LAUNCH_CHECK("deposit_adjoint");
  return CCL_OK;
}

template <typename T, int M>
static int gather_push_adj_m(const T *x, const T *y, const T *z, const T *ux, const T *uy,
                             const T *uz, const u32 *si, const u32 *co, const u32 *np_stay,
                             double factor, GridP<T> g, const void *const *F, void *const *lF,
                             T *lx, T *ly, T *lz, T *lux, T *luy, T *luz, T *lg,
                             cudaStream_t s) {
  ptrs<24> f, lf;
  for (int i = 0; i < 6 * (M + 1); i++) {
    CCL_REQUIRE(F[i] && lF[i], CCL_ERR_ARG, "gather_push_adjoint: null field %d", i);
    f.p[i] = (void *)F[i];
    lf.p[i] = lF[i];
  }
  const size_t smem = 2 * (size_t)AT_NR * AT_NX * 6 * (1 + 2 * M) * sizeof(T);
  auto kern = k_gather_push_adj<T, M>;
  static bool set = false;
  if (!set) {
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    set = true;
  }
  dim3 grid((g.Nx + AT_TX - 1) / AT_TX, (g.Nr + AT_TR - 1) / AT_TR);
  launch_pdl(kern, grid, AT_THREADS, smem, s, x, y, z, ux, uy, uz, si, co, np_stay, (T)factor, g, f,
             lf, lx, ly, lz, lux, luy, luz, lg);
  CCL_LAUNCH_CHECK("gather_push_adjoint");
  return CCL_OK;
}

template <typename T>
static GridP<T> adj_gridp(int Nx, int Nr, double xmin, double dx_inv, double rmin,
                          double dr_inv) {
  return make_gridp<T>(Nx, Nr, xmin, dx_inv, rmin, dr_inv);
}

}  // namespace ccl

using namespace ccl;

#define ADJ_DTYPE(dt)                                                          \
  CCL_REQUIRE((dt) == CCL_F64 || (dt) == CCL_F32, CCL_ERR_ARG,                 \
              "%s: dtype %d is neither CCL_F64 nor CCL_F32", __func__, (dt))
#define ADJ_NONNULL(p)                                                         \
  CCL_REQUIRE((p) != nullptr, CCL_ERR_ARG, "%s: %s is NULL", __func__, #p)

template <typename T>
static int deposit_adj_t(int vec, int M, const u32 *si, const u32 *co, const void *x,
                         const void *y, const void *z, const void *ux, const void *uy,
                         const void *uz, const void *gi, const void *w, int q, GridP<T> g,
                         void *const *lam, void *lx, void *ly, void *lz, void *lw, void *lux,
                         void *luy, void *luz, void *lg, cudaStream_t s) {
#define ARGS_(V, MM)                                                                       \
  deposit_adj_m<T, V, MM>(si, co, (const T *)x, (const T *)y, (const T *)z, (const T *)ux, \
                          (const T *)uy, (const T *)uz, (const T *)gi, (const T *)w, q, g, lam, \
                          (T *)lx, (T *)ly, (T *)lz, (T *)lw, (T *)lux, (T *)luy, (T *)luz,  \
                          (T *)lg, s)
  switch (M) {
    case 0: return vec ? ARGS_(true, 0) : ARGS_(false, 0);
    case 1: return vec ? ARGS_(true, 1) : ARGS_(false, 1);
    case 2: return vec ? ARGS_(true, 2) : ARGS_(false, 2);
    case 3: return vec ? ARGS_(true, 3) : ARGS_(false, 3);
  }
#undef ARGS_
  set_error("deposit_adjoint: M=%d not supported (0..3)", M);
  return CCL_ERR_UNSUPPORTED;
}

template <typename T>
static int gather_adj_t(int M, const void *x, const void *y, const void *z, const void *ux,
                        const void *uy, const void *uz, const u32 *si, const u32 *co,
                        const u32 *ns, double factor, GridP<T> g, const void *const *F,
                        void *const *lF, void *lx, void *ly, void *lz, void *lux, void *luy,
                        void *luz, void *lg, cudaStream_t s) {
#define ARGS_(MM)                                                                          \
  gather_push_adj_m<T, MM>((const T *)x, (const T *)y, (const T *)z, (const T *)ux,         \
                           (const T *)uy, (const T *)uz, si, co, ns, factor, g, F, lF,      \
                           (T *)lx, (T *)ly, (T *)lz, (T *)lux, (T *)luy, (T *)luz, (T *)lg, s)
  switch (M) {
    case 0: return ARGS_(0);
    case 1: return ARGS_(1);
    case 2: return ARGS_(2);
    case 3: return ARGS_(3);
  }
#undef ARGS_
  set_error("gather_push_adjoint: M=%d not supported (0..3)", M);
  return CCL_ERR_UNSUPPORTED;
}

extern "C" {

int ccl_deposit_adjoint(int dtype, int vec, int M, const uint32_t *sort_indx,
                        const uint32_t *cell_offset, const void *x, const void *y,
                        const void *z, const void *ux, const void *uy, const void *uz,
                        const void *g_inv, const void *w, int charge, int Nx, double xmin,
                        double dx_inv, int Nr, double rmin, double dr_inv, void *const *lam,
                        void *lx, void *ly, void *lz, void *lw, void *lux, void *luy,
                        void *luz, void *lg, void *stream) {
  ADJ_DTYPE(dtype);
  CCL_REQUIRE(Nx >= 4 && Nr >= 3, CCL_ERR_ARG, "%s: grid %d x %d too small", __func__, Nx, Nr);
  ADJ_NONNULL(sort_indx); ADJ_NONNULL(cell_offset); ADJ_NONNULL(x); ADJ_NONNULL(y);
  ADJ_NONNULL(z); ADJ_NONNULL(w); ADJ_NONNULL(lam); ADJ_NONNULL(lw);
  CCL_REQUIRE((lx && ly && lz) || (!lx && !ly && !lz), CCL_ERR_ARG,
              "%s: lx, ly, lz must be all given or all NULL", __func__);
  if (vec) {
    ADJ_NONNULL(ux); ADJ_NONNULL(uy); ADJ_NONNULL(uz); ADJ_NONNULL(g_inv);
    ADJ_NONNULL(lux); ADJ_NONNULL(luy); ADJ_NONNULL(luz); ADJ_NONNULL(lg);
  }
  if (dtype == CCL_F64)
    return deposit_adj_t<double>(vec, M, sort_indx, cell_offset, x, y, z, ux, uy, uz, g_inv, w,
                                 charge, adj_gridp<double>(Nx, Nr, xmin, dx_inv, rmin, dr_inv),
                                 lam, lx, ly, lz, lw, lux, luy, luz, lg, S(stream));
  return deposit_adj_t<float>(vec, M, sort_indx, cell_offset, x, y, z, ux, uy, uz, g_inv, w,
                              charge, adj_gridp<float>(Nx, Nr, xmin, dx_inv, rmin, dr_inv), lam,
                              lx, ly, lz, lw, lux, luy, luz, lg, S(stream));
}

int ccl_gather_push_adjoint(int dtype, int M, const void *x, const void *y, const void *z,
                            const void *ux_old, const void *uy_old, const void *uz_old,
                            const uint32_t *sort_indx, const uint32_t *cell_offset,
                            const uint32_t *np_stay, double factor_push, int Nx, double xmin,
                            double dx_inv, int Nr, double rmin, double dr_inv,
                            const void *const *flds, void *const *lflds, void *lx, void *ly,
                            void *lz, void *lux, void *luy, void *luz, void *lg,
                            void *stream) {
  ADJ_DTYPE(dtype);
  CCL_REQUIRE(Nx >= 4 && Nr >= 3, CCL_ERR_ARG, "%s: grid %d x %d too small", __func__, Nx, Nr);
  ADJ_NONNULL(x); ADJ_NONNULL(y); ADJ_NONNULL(z); ADJ_NONNULL(ux_old); ADJ_NONNULL(uy_old);
  ADJ_NONNULL(uz_old); ADJ_NONNULL(sort_indx); ADJ_NONNULL(cell_offset); ADJ_NONNULL(np_stay);
  ADJ_NONNULL(flds); ADJ_NONNULL(lflds); ADJ_NONNULL(lx); ADJ_NONNULL(ly); ADJ_NONNULL(lz);
  ADJ_NONNULL(lux); ADJ_NONNULL(luy); ADJ_NONNULL(luz); ADJ_NONNULL(lg);
  if (dtype == CCL_F64)
    return gather_adj_t<double>(M, x, y, z, ux_old, uy_old, uz_old, sort_indx, cell_offset,
                                np_stay, factor_push,
                                adj_gridp<double>(Nx, Nr, xmin, dx_inv, rmin, dr_inv), flds,
                                lflds, lx, ly, lz, lux, luy, luz, lg, S(stream));
  return gather_adj_t<float>(M, x, y, z, ux_old, uy_old, uz_old, sort_indx, cell_offset,
                             np_stay, factor_push,
                             adj_gridp<float>(Nx, Nr, xmin, dx_inv, rmin, dr_inv), flds, lflds,
                             lx, ly, lz, lux, luy, luz, lg, S(stream));
}

int ccl_push_x_adjoint(int dtype, long np, const void *ux, const void *uy, const void *uz,
                       const void *g_inv, const void *lx, const void *ly, const void *lz,
                       void *lux, void *luy, void *luz, void *lg, double dt, void *stream) {
  ADJ_DTYPE(dtype);
  CCL_REQUIRE(np >= 0, CCL_ERR_ARG, "%s: np = %ld < 0", __func__, np);
  if (np == 0) return CCL_OK;
  ADJ_NONNULL(ux); ADJ_NONNULL(uy); ADJ_NONNULL(uz); ADJ_NONNULL(g_inv); ADJ_NONNULL(lx);
  ADJ_NONNULL(ly); ADJ_NONNULL(lz); ADJ_NONNULL(lux); ADJ_NONNULL(luy); ADJ_NONNULL(luz);
  ADJ_NONNULL(lg);
  const int nb = grid_for(np, 256);
  if (dtype == CCL_F64)
    launch_pdl(k_push_x_adj<double>, nb, 256, 0, S(stream), np, (const double *)ux,
               (const double *)uy, (const double *)uz, (const double *)g_inv, (const double *)lx,
               (const double *)ly, (const double *)lz, (double *)lux, (double *)luy, (double *)luz,
               (double *)lg, dt);
  else
    launch_pdl(k_push_x_adj<float>, nb, 256, 0, S(stream), np, (const float *)ux, (const float *)uy,
               (const float *)uz, (const float *)g_inv, (const float *)lx, (const float *)ly,
               (const float *)lz, (float *)lux, (float *)luy, (float *)luz, (float *)lg, (float)dt);
  CCL_LAUNCH_CHECK("push_x_adjoint");
  return CCL_OK;
}

int ccl_psatd_adjoint(int dtype, long ncells, const void *coef, const void *filter,
                      void *const *flds, void *stream) {
  ADJ_DTYPE(dtype);
  CCL_REQUIRE(ncells >= 0, CCL_ERR_ARG, "%s: ncells = %ld < 0", __func__, ncells);
  if (ncells == 0) return CCL_OK;
  ADJ_NONNULL(coef); ADJ_NONNULL(flds);
  ptrs<15> f;
  for (int i = 0; i < 15; i++) {
    CCL_REQUIRE(flds[i], CCL_ERR_ARG, "%s: null field %d", __func__, i);
    f.p[i] = flds[i];
  }
  const int nb = grid_for(ncells, 256);
  if (dtype == CCL_F64)
    launch_pdl(k_psatd_adj<double>, nb, 256, 0, S(stream), ncells, (const double *)coef,
               (const double *)filter, f);
  else
    launch_pdl(k_psatd_adj<float>, nb, 256, 0, S(stream), ncells, (const float *)coef,
               (const float *)filter, f);
  CCL_LAUNCH_CHECK("psatd_adjoint");
  return CCL_OK;
}

int ccl_grad_combine_adjoint(int dtype, int M, int nrows, int nx, const void *kx,
                             const void *const *ldN, void *const *lrho, void *const *Pm,
                             void *const *Pp, void *stream) {
  ADJ_DTYPE(dtype);
  CCL_REQUIRE(M >= 0 && M <= 3, CCL_ERR_UNSUPPORTED, "%s: M=%d", __func__, M);
  ADJ_NONNULL(kx); ADJ_NONNULL(ldN); ADJ_NONNULL(lrho);
  ptrs<12> a;
  ptrs<4> r, pm, pp;
  for (int m = 0; m <= M; m++) {
    for (int c = 0; c < 3; c++) {
      CCL_REQUIRE(ldN[3 * m + c], CCL_ERR_ARG, "%s: null ldN %d", __func__, 3 * m + c);
      a.p[3 * m + c] = (void *)ldN[3 * m + c];
    }
    CCL_REQUIRE(lrho[m], CCL_ERR_ARG, "%s: null lrho %d", __func__, m);
    r.p[m] = lrho[m];
    pm.p[m] = Pm ? Pm[m] : nullptr;
    pp.p[m] = Pp ? Pp[m] : nullptr;
  }
  if ((long)nrows * nx == 0) return CCL_OK;
  if (dtype == CCL_F64)
    launch_pdl(k_grad_adj_pre<double>, row_chunk_grid<double>(nrows, nx, M + 1), RC_THREADS, 0,
               S(stream), nx, M, (const double *)kx, a, r, pm, pp);
  else
    launch_pdl(k_grad_adj_pre<float>, row_chunk_grid<float>(nrows, nx, M + 1), RC_THREADS, 0,
               S(stream), nx, M, (const float *)kx, a, r, pm, pp);
  CCL_LAUNCH_CHECK("grad_combine_adjoint");
  return CCL_OK;
}

int ccl_rot_combine_adjoint(int dtype, int M, int nrows, int nx, const void *kx,
                            const void *const *poiss, const void *const *lB, void *const *lG,
                            void *const *Qm, void *const *Qp, void *stream) {
  ADJ_DTYPE(dtype);
  CCL_REQUIRE(M >= 0 && M <= 3, CCL_ERR_UNSUPPORTED, "%s: M=%d", __func__, M);
  ADJ_NONNULL(kx); ADJ_NONNULL(lB); ADJ_NONNULL(lG);
  ptrs<12> b, g, qm, qp;
  ptrs<4> po;
  for (int m = 0; m <= M; m++) {
    po.p[m] = poiss ? (void *)poiss[m] : nullptr;
    for (int c = 0; c < 3; c++) {
      const int i = 3 * m + c;
      CCL_REQUIRE(lB[i] && lG[i], CCL_ERR_ARG, "%s: null lB/lG %d", __func__, i);
      b.p[i] = (void *)lB[i];
      g.p[i] = lG[i];
      qm.p[i] = Qm ? Qm[i] : nullptr;
      qp.p[i] = Qp ? Qp[i] : nullptr;
    }
    CCL_REQUIRE((qm.p[3 * m] && qm.p[3 * m + 1] && qm.p[3 * m + 2]) ||
                    (!qm.p[3 * m] && !qm.p[3 * m + 1] && !qm.p[3 * m + 2]),
                CCL_ERR_ARG, "%s: Qm of mode %d partly NULL", __func__, m);
    CCL_REQUIRE((qp.p[3 * m] && qp.p[3 * m + 1] && qp.p[3 * m + 2]) ||
                    (!qp.p[3 * m] && !qp.p[3 * m + 1] && !qp.p[3 * m + 2]),
                CCL_ERR_ARG, "%s: Qp of mode %d partly NULL", __func__, m);
  }
  if ((long)nrows * nx == 0) return CCL_OK;
  if (dtype == CCL_F64)
    launch_pdl(k_rot_adj_pre<double>, row_chunk_grid<double>(nrows, nx, M + 1), RC_THREADS, 0,
               S(stream), nx, M, (const double *)kx, po, b, g, qm, qp);
  else
    launch_pdl(k_rot_adj_pre<float>, row_chunk_grid<float>(nrows, nx, M + 1), RC_THREADS, 0,
               S(stream), nx, M, (const float *)kx, po, b, g, qm, qp);
  CCL_LAUNCH_CHECK("rot_combine_adjoint");
  return CCL_OK;
}

int ccl_modes_adjoint_accumulate(int dtype, int M, int ncomp, int nrows, int nx,
                                 void *const *lo, const void *const *Rm,
                                 const void *const *Rp, const void *const *filt,
                                 void *stream) {
  ADJ_DTYPE(dtype);
  CCL_REQUIRE(M >= 0 && M <= 3 && (ncomp == 1 || ncomp == 3), CCL_ERR_ARG,
              "%s: M=%d ncomp=%d", __func__, M, ncomp);
  ADJ_NONNULL(lo);
  ptrs<12> o, rm, rp;
  ptrs<4> fl;
  for (int m = 0; m <= M; m++) fl.p[m] = filt ? (void *)filt[m] : nullptr;
  for (int i = 0; i < ncomp * (M + 1); i++) {
    CCL_REQUIRE(lo[i], CCL_ERR_ARG, "%s: null lo %d", __func__, i);
    o.p[i] = lo[i];
    rm.p[i] = Rm ? (void *)Rm[i] : nullptr;
    rp.p[i] = Rp ? (void *)Rp[i] : nullptr;
  }
  const long n = (long)nrows * nx;
  if (n == 0) return CCL_OK;
  dim3 grid(grid_for(n, 256, 2), ncomp * (M + 1));
  if (dtype == CCL_F64)
    launch_pdl(k_modes_adj_post<double>, grid, 256, 0, S(stream), n, M, ncomp, o, rm, rp, fl);
  else
    launch_pdl(k_modes_adj_post<float>, grid, 256, 0, S(stream), n, M, ncomp, o, rm, rp, fl);
  CCL_LAUNCH_CHECK("modes_adjoint_accumulate");
  return CCL_OK;
}

int ccl_add_batch(int dtype, int narr, const long *n, void *const *dst, const void *const *src,
                  void *stream) {
  ADJ_DTYPE(dtype);
  CCL_REQUIRE(narr >= 0 && narr <= 32, CCL_ERR_ARG, "%s: narr %d outside [0, 32]", __func__,
              narr);
  if (narr == 0) return CCL_OK;
  ADJ_NONNULL(n); ADJ_NONNULL(dst); ADJ_NONNULL(src);
  AddBatch b;
  long nmax = 0;
  for (int a = 0; a < narr; a++) {
    CCL_REQUIRE(n[a] >= 0 && (n[a] == 0 || (dst[a] && src[a])), CCL_ERR_ARG,
                "%s: array %d (n = %ld) has a NULL pointer", __func__, a, n[a]);
    b.dst[a] = dst[a];
    b.src[a] = src[a];
    b.n[a] = n[a];
    nmax = n[a] > nmax ? n[a] : nmax;
  }
  if (nmax == 0) return CCL_OK;
  dim3 grid(grid_for(nmax, 256, 2), narr);
  if (dtype == CCL_F64)
    launch_pdl(k_add_batch<double>, grid, 256, 0, S(stream), b);
  else
    launch_pdl(k_add_batch<float>, grid, 256, 0, S(stream), b);
  CCL_LAUNCH_CHECK("add_batch");
  return CCL_OK;
}

int ccl_copy_batch(int narr, const long *nbytes, void *const *dst, const void *const *src,
                   void *stream) {
  CCL_REQUIRE(narr >= 0 && narr <= 32, CCL_ERR_ARG, "%s: narr %d outside [0, 32]", __func__,
              narr);
  if (narr == 0) return CCL_OK;
  ADJ_NONNULL(nbytes); ADJ_NONNULL(dst); ADJ_NONNULL(src);
  AddBatch b;
  long nmax = 0;
  for (int a = 0; a < narr; a++) {
    CCL_REQUIRE(nbytes[a] >= 0 && nbytes[a] % 4 == 0, CCL_ERR_ARG,
                "%s: array %d: %ld bytes (a multiple of 4 expected)", __func__, a, nbytes[a]);
    CCL_REQUIRE(nbytes[a] == 0 || (dst[a] && src[a] && ((uintptr_t)dst[a] % 4) == 0 &&
                                   ((uintptr_t)src[a] % 4) == 0),
                CCL_ERR_ARG, "%s: array %d: NULL or misaligned pointer", __func__, a);
    b.dst[a] = dst[a];
    b.src[a] = src[a];
    b.n[a] = nbytes[a] / 4;
    nmax = b.n[a] > nmax ? b.n[a] : nmax;
  }
  if (nmax == 0) return CCL_OK;
  dim3 grid(grid_for((nmax + 3) / 4, 256, 4), narr);
  launch_pdl(k_copy_batch<uint32_t>, grid, 256, 0, S(stream), b);
  CCL_LAUNCH_CHECK("copy_batch");
  return CCL_OK;
}

int ccl_deposit_postproc_adjoint(int dtype, int M, int nfld, void *const *flds, int Nx, int Nr,
                                 const void *dV_inv, void *stream) {
  ADJ_DTYPE(dtype);
  CCL_REQUIRE(nfld >= 1 && nfld * (M + 1) <= 32 && M >= 0, CCL_ERR_ARG, "%s: nfld=%d M=%d",
              __func__, nfld, M);
  ADJ_NONNULL(flds); ADJ_NONNULL(dV_inv);
  ptrs<32> f;
  for (int i = 0; i < nfld * (M + 1); i++) {
    CCL_REQUIRE(flds[i], CCL_ERR_ARG, "%s: null field %d", __func__, i);
    f.p[i] = flds[i];
  }
  dim3 grid((Nx + 127) / 128, Nr - 1, nfld * (M + 1));
  if (dtype == CCL_F64)
    launch_pdl(k_postproc_adj<double>, grid, 128, 0, S(stream), f, M + 1, Nx, Nr,
               (const double *)dV_inv);
  else
    launch_pdl(k_postproc_adj<float>, grid, 128, 0, S(stream), f, M + 1, Nx, Nr,
               (const float *)dV_inv);
  CCL_LAUNCH_CHECK("postproc_adjoint");
  return CCL_OK;
}

int ccl_warp_axis_adjoint(int dtype, int M, int nfld, void *const *flds, int Nx, void *stream) {
  ADJ_DTYPE(dtype);
  CCL_REQUIRE(nfld >= 1 && nfld * (M + 1) <= 32 && M >= 0, CCL_ERR_ARG, "%s: nfld=%d M=%d",
              __func__, nfld, M);
  ADJ_NONNULL(flds);
  ptrs<32> f;
  for (int i = 0; i < nfld * (M + 1); i++) {
    CCL_REQUIRE(flds[i], CCL_ERR_ARG, "%s: null field %d", __func__, i);
    f.p[i] = flds[i];
  }
  dim3 grid((Nx + 127) / 128, nfld * (M + 1));
  if (dtype == CCL_F64)
    launch_pdl(k_warp_axis_adj<double>, grid, 128, 0, S(stream), f, M + 1, Nx);
  else
    launch_pdl(k_warp_axis_adj<float>, grid, 128, 0, S(stream), f, M + 1, Nx);
  CCL_LAUNCH_CHECK("warp_axis_adjoint");
  return CCL_OK;
}

int ccl_align_adjoint(int dtype, long n, int ncomp, void *const *src, void *const *dst,
                      const uint32_t *sort_indx, void *stream) {
  ADJ_DTYPE(dtype);
  CCL_REQUIRE(n >= 0 && ncomp >= 0 && ncomp <= 16, CCL_ERR_ARG, "%s: n=%ld ncomp=%d", __func__,
              n, ncomp);
  if (n == 0 || ncomp == 0) return CCL_OK;
  ADJ_NONNULL(src); ADJ_NONNULL(dst); ADJ_NONNULL(sort_indx);
  ptrs<16> a, b;
  for (int c = 0; c < ncomp; c++) {
    CCL_REQUIRE(src[c] && dst[c], CCL_ERR_ARG, "%s: null component %d", __func__, c);
    a.p[c] = src[c];
    b.p[c] = dst[c];
  }
  const int nb = grid_for(n, 256);
  if (dtype == CCL_F64)
    launch_pdl(k_scatter<double>, nb, 256, 0, S(stream), n, ncomp, a, b, sort_indx);
  else
    launch_pdl(k_scatter<float>, nb, 256, 0, S(stream), n, ncomp, a, b, sort_indx);
  CCL_LAUNCH_CHECK("align_adjoint");
  return CCL_OK;
}

int ccl_dens_profile_adjoint(int dtype, long np, const void *x, const void *w, const void *lw,
                             const double *xx, const double *ff, const double *dxm1,
                             uint32_t nloc, double *lff, void *stream) {
  ADJ_DTYPE(dtype);
  CCL_REQUIRE(np >= 0, CCL_ERR_ARG, "%s: np = %ld < 0", __func__, np);
  CCL_REQUIRE(nloc >= 2 && nloc <= (uint32_t)DP_MAXK, CCL_ERR_ARG, "%s: %u knots (2..%d)",
              __func__, nloc, DP_MAXK);
  if (np == 0) return CCL_OK;
  ADJ_NONNULL(x); ADJ_NONNULL(w); ADJ_NONNULL(lw); ADJ_NONNULL(xx); ADJ_NONNULL(ff);
  ADJ_NONNULL(dxm1); ADJ_NONNULL(lff);
  const int nb = grid_for(np, 256, 2);
  if (dtype == CCL_F64)
    launch_pdl(k_dens_profile_adj<double>, nb, 256, 0, S(stream), np, (const double *)x,
               (const double *)w, (const double *)lw, xx, ff, dxm1, nloc, lff);
  else
    launch_pdl(k_dens_profile_adj<float>, nb, 256, 0, S(stream), np, (const float *)x,
               (const float *)w, (const float *)lw, xx, ff, dxm1, nloc, lff);
  CCL_LAUNCH_CHECK("dens_profile_adjoint");
  return CCL_OK;
}

}  // extern "C"
