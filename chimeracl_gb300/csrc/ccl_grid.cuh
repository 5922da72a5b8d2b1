// Grid kernels: charge/current deposit, deposit post-processing, ghost-row
// fill, field gather + Boris push.  Templated on the real type T and the
// highest azimuthal mode M.
//
// Deposit design.  One CTA owns a tile of (DEP_TR-1) x (DEP_TX-1) grid nodes
// and runs one thread per cell of the DEP_TR x DEP_TX cells that touch them
// (cells on the tile border are also computed by the neighbouring CTA, so no
// node is written by two CTAs and no atomics are needed).  Each thread sums
// its cell's cell-sorted particles into 2x2 corner accumulators in registers,
// in the order of sort_indx, exactly as the reference's per-cell loop does
// (grid_deposit_m1.cl:105-138).  The corner sums are then added to the node
// tile in shared memory in four phases, one per cell colour
// (ix&1) + 2(ir&1): the order in which the reference's four colour launches
// add them (grid_methods_cl.py:66-69).  The result is the reference's sum,
// term by term and in the same order, without its four launches.
#pragma once
#include "ccl_common.cuh"
#include "ccl_particles.cuh"

namespace ccl {

constexpr int DEP_TX = 32, DEP_TR = 8, DEP_THREADS = DEP_TX * DEP_TR;
constexpr int DEP_NTX = DEP_TX - 1, DEP_NTR = DEP_TR - 1;
constexpr int DEP_CARVEOUT = 10;  // percent of the unified L1 / shared memory

// One particle's contribution to the 2x2 corner sums of its cell, in the
// reference's operation order (grid_deposit_m1.cl:105-138 scalar,
// 259-316 vector).
template <typename T, int M, bool VEC>
__device__ __forceinline__ void dep_particle(T (&s)[4][(VEC ? 3 : 1) * (1 + 2 * M)], T xp,
                                             T yp, T zp, T wraw, T ux, T uy, T uz, T gi, T q,
                                             const GridP<T> &g, T fix, T fir) {
  constexpr int NK = VEC ? 3 : 1;
  T wp;
  if (VEC)
    wp = wraw * gi * q;
  else
    wp = wraw * q;
  const T rp = sqrt(yp * yp + zp * zp);
  T rinv;
  if (VEC)
    rinv = rp > T(0) ? T(1) / rp : T(0);  // grid_deposit_m1.cl:280-281
  else
    rinv = T(1) / rp;                     // grid_deposit_m1.cl:115
  T e[M + 1][2];
  if (M >= 1) {
    e[1][0] = yp * rinv;
    e[1][1] = zp * rinv;
  }
#pragma unroll
  for (int m = 2; m <= M; m++) {  // e^{i m phi} by recurrence (m >= 2)
    e[m][0] = e[m - 1][0] * e[1][0] - e[m - 1][1] * e[1][1];
    e[m][1] = e[m - 1][0] * e[1][1] + e[m - 1][1] * e[1][0];
  }
  T sX1 = (xp - g.xmin) * g.dx_inv - fix;
  T sX0 = T(1) - sX1;
  T sR1 = (rp - g.rmin) * g.dr_inv - fir;
  T sR0 = T(1) - sR1;
  sX0 *= wp;
  sX1 *= wp;
  const T C[4] = {sR0 * sX0, sR0 * sX1, sR1 * sX0, sR1 * sX1};
  const T jp[3] = {ux, uy, uz};
#pragma unroll
  for (int c = 0; c < 4; c++) {
#pragma unroll
    for (int k = 0; k < NK; k++) {
      constexpr int B = 1 + 2 * M;
      if (VEC) {
        T jproj = C[c] * jp[k];
        s[c][k * B] += C[c] * jp[k];
#pragma unroll
        for (int m = 1; m <= M; m++) {
          s[c][k * B + 2 * m - 1] += jproj * e[m][0];
          s[c][k * B + 2 * m] += jproj * e[m][1];
        }
      } else {
        s[c][0] += C[c];
#pragma unroll
        for (int m = 1; m <= M; m++) {
          s[c][2 * m - 1] += C[c] * e[m][0];
          s[c][2 * m] += C[c] * e[m][1];
        }
      }
    }
  }
}

// FP32 form (the mixed-precision step; no bit-exact counterpart): the same
// corner sums with 1/r from rsqrt and the per-particle moments (1, e^{im phi}
// per component) formed once, then one FMA per (corner, moment).  LO: the
// coordinates are hi + lo (compensated), and the shape fractions take the
// low parts in.
template <int M, bool VEC, bool LO = false>
__device__ __forceinline__ void dep_particle_f32(float (&s)[4][(VEC ? 3 : 1) * (1 + 2 * M)],
                                             float xp, float yp, float zp, float wraw, float ux,
                                             float uy, float uz, float gi, float q,
                                             const GridP<float> &g, CellEdge ex, CellEdge er,
                                             float xl = 0.f, float yl = 0.f, float zl = 0.f) {
  constexpr int NK = VEC ? 3 : 1, B = 1 + 2 * M;
  const float wp = VEC ? wraw * gi * q : wraw * q;
  const float r2 = yp * yp + zp * zp;
  const float rinv = r2 > 0.f ? rsqrtf(r2) : (VEC ? 0.f : __int_as_float(0x7f800000));
  const float rp = radius_from_rsqrt(r2, rinv);
  float e[M + 1][2];
  e[0][0] = 1.f;
  e[0][1] = 0.f;
  if (M >= 1) {
    e[1][0] = yp * rinv;
    e[1][1] = zp * rinv;
  }
#pragma unroll
  for (int m = 2; m <= M; m++) {
    e[m][0] = e[m - 1][0] * e[1][0] - e[m - 1][1] * e[1][1];
    e[m][1] = e[m - 1][0] * e[1][1] + e[m - 1][1] * e[1][0];
  }
  float sX1, sR1;
  if constexpr (LO) {
    float rr, rrl;
    radius_pair(yp, zp, yl, zl, rinv, rr, rrl);
    sX1 = edge_frac_lo(xp, xl, ex, g.dx_inv);
    sR1 = edge_frac_lo(rr, rrl, er, g.dr_inv);
  } else {
    sX1 = edge_frac(xp, ex, g.dx_inv);
    sR1 = edge_frac(rp, er, g.dr_inv);
  }
  const float sX0 = 1.f - sX1, sR0 = 1.f - sR1;
  const float wX0 = sX0 * wp, wX1 = sX1 * wp;
  const float C[4] = {sR0 * wX0, sR0 * wX1, sR1 * wX0, sR1 * wX1};
  const float jp[3] = {VEC ? ux : 1.f, uy, uz};
  float mom[NK * B];
#pragma unroll
  for (int k = 0; k < NK; k++) {
    mom[k * B] = jp[k];
#pragma unroll
    for (int m = 1; m <= M; m++) {
      mom[k * B + 2 * m - 1] = jp[k] * e[m][0];
      mom[k * B + 2 * m] = jp[k] * e[m][1];
    }
  }
#pragma unroll
  for (int c = 0; c < 4; c++)
#pragma unroll
    for (int qq = 0; qq < NK * B; qq++) s[c][qq] = fmaf(C[c], mom[qq], s[c][qq]);
}

// Field pointer bundle: for a scalar deposit f[m] (m = 0..M); for a vector
// deposit f[3m + k].  Mode 0 is real, modes >= 1 complex.
template <typename T, int M, bool VEC, bool LO = false>
__global__ void __launch_bounds__(DEP_THREADS)
    k_deposit(const u32 *__restrict__ sort_indx,
              const u32 *__restrict__ cell_off, const T *__restrict__ x,
              const T *__restrict__ y, const T *__restrict__ z,
              const T *__restrict__ ux, const T *__restrict__ uy,
              const T *__restrict__ uz, const T *__restrict__ g_inv,
              const T *__restrict__ w, T q, GridP<T> g, ptrs<12> f,
              const T *__restrict__ xl = nullptr, const T *__restrict__ yl = nullptr,
              const T *__restrict__ zl = nullptr) {
  pdl_wait();
  constexpr int NK = VEC ? 3 : 1;       // vector components
  constexpr int NQ = NK * (1 + 2 * M);  // reals per node
  __shared__ T acc[NQ][DEP_NTR][DEP_NTX];
  const int Nx = g.Nx, Nr = g.Nr;
  const int nx0 = blockIdx.x * DEP_NTX, nr0 = blockIdx.y * DEP_NTR;
  const int tx = threadIdx.x % DEP_TX, tr = threadIdx.x / DEP_TX;

  // 1. node tile <- current field values
  for (int t = threadIdx.x; t < DEP_NTR * DEP_NTX; t += DEP_THREADS) {
    int r = t / DEP_NTX, c = t - r * DEP_NTX;
    int nr = nr0 + r, nx = nx0 + c;
    bool in = nr < Nr && nx < Nx;
    long node = (long)nr * Nx + nx;
#pragma unroll
    for (int k = 0; k < NK; k++) {
      acc[k * (1 + 2 * M)][r][c] = in ? ((const T *)f.p[k])[node] : T(0);
#pragma unroll
      for (int m = 1; m <= M; m++) {
        const T *fm = (const T *)f.p[m * NK + k];
        acc[k * (1 + 2 * M) + 2 * m - 1][r][c] = in ? fm[2 * node] : T(0);
        acc[k * (1 + 2 * M) + 2 * m][r][c] = in ? fm[2 * node + 1] : T(0);
      }
    }
  }

  // 2. this thread's cell: per-corner sums over its particles
  const int ix = nx0 - 1 + tx, ir = nr0 - 1 + tr;
  const bool valid = ix > 0 && ix < Nx - 2 && ir >= 0 && ir < Nr - 2;
  T s[4][NQ];
#pragma unroll
  for (int c = 0; c < 4; c++)
#pragma unroll
    for (int qq = 0; qq < NQ; qq++) s[c][qq] = T(0);
  if (valid) {
    const long cg = (long)ix + (long)ir * (Nx - 1);
    const u32 p0 = cell_off[cg], p1 = cell_off[cg + 1];
    const T fix = (T)ix, fir = (T)ir;
    CellEdge ex{}, er{};  // FP32: this thread's cell edges, formed once
    if constexpr (sizeof(T) == 4) {
      ex = x_edge(g, ix);
      er = r_edge(g, ir);
    }
    // two particles in flight (their dependent loads overlap); the
    // accumulation order is unchanged
#pragma unroll 2
    for (u32 ip = p0; ip < p1; ip++) {
      const u32 p = sort_indx[ip];
      const T a = VEC ? ux[p] : T(0), b = VEC ? uy[p] : T(0), c = VEC ? uz[p] : T(0),
              d = VEC ? g_inv[p] : T(0);
      if constexpr (sizeof(T) == 4 && LO)
        dep_particle_f32<M, VEC, true>(s, x[p], y[p], z[p], w[p], a, b, c, d, q, g, ex, er,
                                       xl[p], yl[p], zl[p]);
      else if constexpr (sizeof(T) == 4)
        dep_particle_f32<M, VEC>(s, x[p], y[p], z[p], w[p], a, b, c, d, q, g, ex, er);
      else
        dep_particle<T, M, VEC>(s, x[p], y[p], z[p], w[p], a, b, c, d, q, g, fix, fir);
    }
  }

  // 3. add to the node tile colour by colour (the reference's launch order)
  const int colour = (ix & 1) + 2 * (ir & 1);
#pragma unroll
  for (int col = 0; col < 4; col++) {
    __syncthreads();
    if (valid && colour == col) {
#pragma unroll
      for (int c = 0; c < 4; c++) {
        int lr = ir + (c >> 1) - nr0, lc = ix + (c & 1) - nx0;
        if (lr >= 0 && lr < DEP_NTR && lc >= 0 && lc < DEP_NTX) {
#pragma unroll
          for (int qq = 0; qq < NQ; qq++) acc[qq][lr][lc] += s[c][qq];
        }
      }
    }
  }
  __syncthreads();

  // 4. node tile -> global
  for (int t = threadIdx.x; t < DEP_NTR * DEP_NTX; t += DEP_THREADS) {
    int r = t / DEP_NTX, c = t - r * DEP_NTX;
    int nr = nr0 + r, nx = nx0 + c;
    if (nr >= Nr || nx >= Nx) continue;
    long node = (long)nr * Nx + nx;
#pragma unroll
    for (int k = 0; k < NK; k++) {
      ((T *)f.p[k])[node] = acc[k * (1 + 2 * M)][r][c];
#pragma unroll
      for (int m = 1; m <= M; m++) {
        T *fm = (T *)f.p[m * NK + k];
        fm[2 * node] = acc[k * (1 + 2 * M) + 2 * m - 1][r][c];
        fm[2 * node + 1] = acc[k * (1 + 2 * M) + 2 * m][r][c];
      }
    }
  }
}

template <typename T, int M, bool VEC, bool LO>
void deposit_launch(dim3 grid, const u32 *sort_indx, const u32 *cell_off, const T *x,
                    const T *y, const T *z, const T *ux, const T *uy, const T *uz,
                    const T *g_inv, const T *w, T q, GridP<T> g, ptrs<12> f,
                    const T *const *lo, cudaStream_t s) {
  // the per-lane particle streams are re-read from L1 across a cell's
  // particles: ask for the smallest shared-memory carve-out (largest L1)
  static bool set = false;  // per instantiation, once
  if (!set) {
    cudaFuncSetAttribute(k_deposit<T, M, VEC, LO>,
                         cudaFuncAttributePreferredSharedMemoryCarveout, DEP_CARVEOUT);
    set = true;
  }
  launch_pdl(k_deposit<T, M, VEC, LO>, grid, DEP_THREADS, 0, s, sort_indx, cell_off, x, y, z, ux,
             uy, uz, g_inv, w, q, g, f, LO ? lo[0] : nullptr, LO ? lo[1] : nullptr,
             LO ? lo[2] : nullptr);
}

// lo: nullptr, or the low parts {x_lo, y_lo, z_lo} of compensated FP32
// coordinates
template <typename T, int M, bool VEC>
int deposit_m(const u32 *sort_indx, const u32 *cell_off, const T *x,
              const T *y, const T *z, const T *ux, const T *uy, const T *uz,
              const T *g_inv, const T *w, int charge, GridP<T> g,
              void *const *flds, cudaStream_t s, const T *const *lo = nullptr) {
  ptrs<12> f;
  const int nptr = (VEC ? 3 : 1) * (M + 1);
  for (int i = 0; i < nptr; i++) {
    CCL_REQUIRE(flds[i], CCL_ERR_ARG, "deposit: null field pointer %d", i);
    f.p[i] = flds[i];
  }
  dim3 grid((g.Nx + DEP_NTX - 1) / DEP_NTX, (g.Nr + DEP_NTR - 1) / DEP_NTR);
  // the reference passes the charge as a signed char (grid_methods_cl.py:61)
  T q = (T)(signed char)charge;
  if constexpr (sizeof(T) == 4) {
    if (lo) {
      deposit_launch<T, M, VEC, true>(grid, sort_indx, cell_off, x, y, z, ux, uy, uz, g_inv, w,
                                      q, g, f, lo, s);
      CCL_LAUNCH_CHECK("deposit");
      return CCL_OK;
    }
  }
  deposit_launch<T, M, VEC, false>(grid, sort_indx, cell_off, x, y, z, ux, uy, uz, g_inv, w, q,
                                   g, f, lo, s);
  CCL_LAUNCH_CHECK("deposit");
  return CCL_OK;
}

template <typename T, bool VEC>
int deposit(int M, const u32 *sort_indx, const u32 *cell_off, const T *x,
            const T *y, const T *z, const T *ux, const T *uy, const T *uz,
            const T *g_inv, const T *w, int charge, GridP<T> g,
            void *const *flds, cudaStream_t s, const T *const *lo = nullptr) {
  switch (M) {
    case 0:
      return deposit_m<T, 0, VEC>(sort_indx, cell_off, x, y, z, ux, uy, uz,
                                  g_inv, w, charge, g, flds, s, lo);
    case 1:
      return deposit_m<T, 1, VEC>(sort_indx, cell_off, x, y, z, ux, uy, uz,
                                  g_inv, w, charge, g, flds, s, lo);
    case 2:
      return deposit_m<T, 2, VEC>(sort_indx, cell_off, x, y, z, ux, uy, uz,
                                  g_inv, w, charge, g, flds, s, lo);
    case 3:
      return deposit_m<T, 3, VEC>(sort_indx, cell_off, x, y, z, ux, uy, uz,
                                  g_inv, w, charge, g, flds, s, lo);
  }
  set_error("deposit: M=%d not supported (0..3)", M);
  return CCL_ERR_UNSUPPORTED;
}

// ---------------------------------------------------------------------
// treat_axis + divide_by_dv (grid_generic.cl:4-59) fused: the thread of row 1
// also writes row 0 so that row 0 is read before it is scaled.
template <typename T>
__global__ void k_postproc(ptrs<32> f, int Mp1, int Nx, int Nr,
                           const T *__restrict__ dv) {
  pdl_wait();
  const int pidx = blockIdx.z, m = pidx % Mp1;
  const int ir = blockIdx.y + 1;
  const int ix = blockIdx.x * blockDim.x + threadIdx.x;
  if (ix >= Nx) return;
  T *a = (T *)f.p[pidx];
  if (m == 0) {
    long i = (long)ir * Nx + ix;
    if (ir == 1) {
      T r0 = a[ix];
      a[i] = (a[i] - r0) * dv[1];
      a[ix] = r0 * dv[0];
    } else {
      a[i] = a[i] * dv[ir];
    }
  } else {
    // complex values as one 8- or 16-byte vector each (same arithmetic)
    using V2 = typename std::conditional<sizeof(T) == 4, float2, double2>::type;
    V2 *c = (V2 *)a;
    long i = (long)ir * Nx + ix;
    V2 v = c[i];
    if (ir == 1) {
      V2 z = c[ix];
      v.x = (v.x - z.x) * dv[1];
      v.y = (v.y - z.y) * dv[1];
      z.x = z.x * dv[0];
      z.y = z.y * dv[0];
      c[ix] = z;
    } else {
      v.x = v.x * dv[ir];
      v.y = v.y * dv[ir];
    }
    c[i] = v;
  }
}

// warp_axis_m0_d / warp_axis_m1plus_c (grid_generic.cl:63-86)
template <typename T>
__global__ void k_warp_axis(ptrs<32> f, int Mp1, int Nx) {
  pdl_wait();
  const int pidx = blockIdx.y, m = pidx % Mp1;
  const int ix = blockIdx.x * blockDim.x + threadIdx.x;
  if (ix >= Nx) return;
  T *a = (T *)f.p[pidx];
  if (m == 0) {
    a[ix] = a[ix + Nx];
  } else {
    a[2 * ix] = -a[2 * (ix + Nx)];
    a[2 * ix + 1] = -a[2 * (ix + Nx) + 1];
  }
}

// ---------------------------------------------------------------------
// gather_and_push (grid_deposit_m1.cl:330-511): bilinear gather of E, B over
// modes 0..M (factor 2 for m >= 1, Hermitian symmetry) and Boris push.
// f.p[6m + c], c = ex, ey, ez, bx, by, bz.
template <typename T, int M>
__global__ void __launch_bounds__(256)
    k_gather_push(long np, const T *__restrict__ x, const T *__restrict__ y,
                  const T *__restrict__ z, T *__restrict__ px,
                  T *__restrict__ py, T *__restrict__ pz,
                  T *__restrict__ g_inv, const u32 *__restrict__ sort_indx,
                  const u32 *__restrict__ np_stay_p, T dt, GridP<T> g,
                  ptrs<24> f) {
  pdl_wait();
  const u32 np_stay = *np_stay_p;
  const int Nx = g.Nx, nxc = Nx - 1, nrc = g.Nr - 1;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < np;
       i += (long)gridDim.x * blockDim.x) {
    const u32 p = sort_indx[i];
    if (p >= np_stay) continue;  // grid_deposit_m1.cl:367-368
    const T xp = x[p], yp = y[p], zp = z[p];
    const T rp = sqrt(yp * yp + zp * zp);
    const T xmin = g.xmin, dx_inv = g.dx_inv, rmin = g.rmin, dr_inv = g.dr_inv;
    const int ix = floor_to_int<T>(floor((xp - xmin) * dx_inv), -1);
    const int ir = floor_to_int<T>(floor((rp - rmin) * dr_inv), 1 << 30);
    if (!(ix > 0 && ix < nxc - 1 && ir < nrc - 1)) continue;
    const long ig = (long)ix + (long)ir * Nx;
    T u[3] = {px[p], py[p], pz[p]};
    const T dt_2 = T(0.5) * dt;
    const T rinv = T(1) / rp;
    const T sX1 = (xp - xmin) * dx_inv - (T)ix, sX0 = T(1) - sX1;
    const T sR1 = (rp - rmin) * dr_inv - (T)ir, sR0 = T(1) - sR1;
    T e[M + 1][2];
    if (M >= 1) {
      e[1][0] = yp * rinv;
      e[1][1] = -zp * rinv;
    }
#pragma unroll
    for (int m = 2; m <= M; m++) {  // e^{-i m phi} by recurrence (m >= 2)
      e[m][0] = e[m - 1][0] * e[1][0] - e[m - 1][1] * e[1][1];
      e[m][1] = e[m - 1][0] * e[1][1] + e[m - 1][1] * e[1][0];
    }
    const T C[4] = {sR0 * sX0, sR0 * sX1, sR1 * sX0, sR1 * sX1};
    T ep[3] = {T(0), T(0), T(0)}, bp[3] = {T(0), T(0), T(0)};
#pragma unroll
    for (int k = 0; k < 3; k++) {
#pragma unroll
      for (int c = 0; c < 4; c++) {
        const long l = ig + (c & 1) + (long)Nx * (c >> 1);
        const T cc = C[c];
        ep[k] += cc * ((const T *)f.p[k])[l];
        bp[k] += cc * ((const T *)f.p[3 + k])[l];
#pragma unroll
        for (int m = 1; m <= M; m++) {
          cplx<T> fe = ld_c((const T *)f.p[6 * m + k], l);
          cplx<T> fb = ld_c((const T *)f.p[6 * m + 3 + k], l);
          T er = T(2) * fe.re, ei = T(2) * fe.im;
          T br = T(2) * fb.re, bi = T(2) * fb.im;
          ep[k] += cc * er * e[m][0];
          ep[k] -= cc * ei * e[m][1];
          bp[k] += cc * br * e[m][0];
          bp[k] -= cc * bi * e[m][1];
        }
      }
    }
    T um[3], up[3], u0[3], t[3], sv[3];
#pragma unroll
    for (int k = 0; k < 3; k++) um[k] = u[k] + dt_2 * ep[k];
    T gi = T(1) / sqrt(T(1) + um[0] * um[0] + um[1] * um[1] + um[2] * um[2]);
#pragma unroll
    for (int k = 0; k < 3; k++) t[k] = dt_2 * bp[k] * gi;
    const T f2 = T(2) / (T(1) + t[0] * t[0] + t[1] * t[1] + t[2] * t[2]);
#pragma unroll
    for (int k = 0; k < 3; k++) sv[k] = t[k] * f2;
    u0[0] = um[0] + um[1] * t[2] - um[2] * t[1];
    u0[1] = um[1] - um[0] * t[2] + um[2] * t[0];
    u0[2] = um[2] + um[0] * t[1] - um[1] * t[0];
    up[0] = um[0] + u0[1] * sv[2] - u0[2] * sv[1];
    up[1] = um[1] - u0[0] * sv[2] + u0[2] * sv[0];
    up[2] = um[2] + u0[0] * sv[1] - u0[1] * sv[0];
#pragma unroll
    for (int k = 0; k < 3; k++) u[k] = up[k] + dt_2 * ep[k];
    gi = T(1) / sqrt(T(1) + u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
    px[p] = u[0];
    py[p] = u[1];
    pz[p] = u[2];
    g_inv[p] = gi;
  }
}

// FP32 form of the gather + push (the mixed-precision step; no bit-exact
// counterpart): per field component the mode-0 and mode-m node sums are
// formed first and combined once with e^{-i m phi}; 1/r and the Lorentz
// factors from rsqrt.  The physics and the node weights are those of the
// exact kernel above.
template <int M>
__global__ void __launch_bounds__(256)
    k_gather_push_f32(long np, const float *__restrict__ x, const float *__restrict__ y,
                      const float *__restrict__ z, float *__restrict__ px,
                      float *__restrict__ py, float *__restrict__ pz,
                      float *__restrict__ g_inv, const u32 *__restrict__ sort_indx,
                      const u32 *__restrict__ np_stay_p, float dt, GridP<float> g,
                      ptrs<24> f) {
  pdl_wait();
  const u32 np_stay = *np_stay_p;
  const int Nx = g.Nx, nxc = Nx - 1, nrc = g.Nr - 1;
  const float dt_2 = 0.5f * dt;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < np;
       i += (long)gridDim.x * blockDim.x) {
    const u32 p = sort_indx[i];
    if (p >= np_stay) continue;
    const float xp = x[p], yp = y[p], zp = z[p];
    const float r2 = yp * yp + zp * zp;
    const float rinv = r2 > 0.f ? rsqrtf(r2) : __int_as_float(0x7f800000);
    const float rp = radius_from_rsqrt(r2, rinv);
    const float fx = (xp - g.xmin) * g.dx_inv, fr = (rp - g.rmin) * g.dr_inv;
    const int ix = floor_to_int<float>(floorf(fx), -1);
    const int ir = floor_to_int<float>(floorf(fr), 1 << 30);
    if (!(ix > 0 && ix < nxc - 1 && ir < nrc - 1)) continue;
    const unsigned ig = (unsigned)ix + (unsigned)ir * (unsigned)Nx;
    const float sX1 = frac_x(xp, ix, g), sX0 = 1.f - sX1;
    const float sR1 = frac_r(rp, ir, g), sR0 = 1.f - sR1;
    const float C[4] = {sR0 * sX0, sR0 * sX1, sR1 * sX0, sR1 * sX1};
    const unsigned nodes[4] = {ig, ig + 1, ig + (unsigned)Nx, ig + (unsigned)Nx + 1};
    float e[M + 1][2];
    if (M >= 1) {
      e[1][0] = yp * rinv;
      e[1][1] = -zp * rinv;
    }
#pragma unroll
    for (int m = 2; m <= M; m++) {
      e[m][0] = e[m - 1][0] * e[1][0] - e[m - 1][1] * e[1][1];
      e[m][1] = e[m - 1][0] * e[1][1] + e[m - 1][1] * e[1][0];
    }
    float fld[6];  // ex ey ez bx by bz at the particle
#pragma unroll
    for (int k = 0; k < 6; k++) {
      const float *f0 = (const float *)f.p[k];
      float a = 0.f;
#pragma unroll
      for (int c = 0; c < 4; c++) a = fmaf(C[c], __ldg(f0 + nodes[c]), a);
#pragma unroll
      for (int m = 1; m <= M; m++) {
        const float2 *fm = (const float2 *)f.p[6 * m + k];
        float re = 0.f, im = 0.f;
#pragma unroll
        for (int c = 0; c < 4; c++) {
          const float2 v = __ldg(fm + nodes[c]);
          re = fmaf(C[c], v.x, re);
          im = fmaf(C[c], v.y, im);
        }
        a = fmaf(2.f * re, e[m][0], a);
        a = fmaf(-2.f * im, e[m][1], a);
      }
      fld[k] = a;
    }
    // Boris push (grid_deposit_m1.cl:440-505)
    float um[3];
    um[0] = px[p] + dt_2 * fld[0];
    um[1] = py[p] + dt_2 * fld[1];
    um[2] = pz[p] + dt_2 * fld[2];
    const float gi0 = rsqrtf(1.f + um[0] * um[0] + um[1] * um[1] + um[2] * um[2]);
    float t[3], sv[3], u0[3], up[3];
#pragma unroll
    for (int k = 0; k < 3; k++) t[k] = dt_2 * fld[3 + k] * gi0;
    const float f2 = __fdividef(2.f, 1.f + t[0] * t[0] + t[1] * t[1] + t[2] * t[2]);
#pragma unroll
    for (int k = 0; k < 3; k++) sv[k] = t[k] * f2;
    u0[0] = um[0] + um[1] * t[2] - um[2] * t[1];
    u0[1] = um[1] - um[0] * t[2] + um[2] * t[0];
    u0[2] = um[2] + um[0] * t[1] - um[1] * t[0];
    up[0] = um[0] + u0[1] * sv[2] - u0[2] * sv[1];
    up[1] = um[1] - u0[0] * sv[2] + u0[2] * sv[0];
    up[2] = um[2] + u0[0] * sv[1] - u0[1] * sv[0];
    const float u[3] = {up[0] + dt_2 * fld[0], up[1] + dt_2 * fld[1], up[2] + dt_2 * fld[2]};
    px[p] = u[0];
    py[p] = u[1];
    pz[p] = u[2];
    g_inv[p] = rsqrtf(1.f + u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
  }
}

// FP32 form, cell tile by cell tile: one CTA per tile of 32 x 8 cells (the
// deposit's tiling without its halo).  The 33 x 9 nodes' E and B over all
// modes are staged in shared memory once (mode m >= 1 already doubled); the
// tile's particles -- one contiguous range of sort_indx per tile row, from
// cell_offset -- are then taken by consecutive threads (coalesced), and each
// interpolates from shared memory.  The row comes from the sort; the column
// from the particle's x with the sort's own formula, clamped to the tile.
constexpr int GT_TX = 32, GT_TR = 8, GT_THREADS = 256;
constexpr int GT_NX = GT_TX + 1, GT_NR = GT_TR + 1;
__host__ __device__ constexpr int gt_stride(int M) {  // floats per staged node, 16-B multiple
  return ((6 * (1 + 2 * M)) + 3) & ~3;
}

// LO: coordinates held as hi + lo (compensated); the shape fractions take
// the low parts in (xl, yl, zl), the cell and angle come from hi.
template <int M, bool LO = false>
__global__ void __launch_bounds__(GT_THREADS)
    k_gather_push_tiled(const float *__restrict__ x, const float *__restrict__ y,
                        const float *__restrict__ z, float *__restrict__ px,
                        float *__restrict__ py, float *__restrict__ pz,
                        float *__restrict__ g_inv, const u32 *__restrict__ sort_indx,
                        const u32 *__restrict__ cell_off, const u32 *__restrict__ np_stay_p,
                        float dt, GridP<float> g, ptrs<24> f,
                        const float *__restrict__ xl = nullptr,
                        const float *__restrict__ yl = nullptr,
                        const float *__restrict__ zl = nullptr) {
  pdl_wait();
  constexpr int NS = gt_stride(M);
  extern __shared__ __align__(16) float gsm[];  // [GT_NR][GT_NX][NS]
  __shared__ u32 row_a[GT_TR], row_pre[GT_TR + 1];
  __shared__ CellEdge xedge[GT_TX], redge[GT_TR];  // the tile's cell edges
  const int Nx = g.Nx, Nr = g.Nr, nxc = Nx - 1;
  const int nx0 = blockIdx.x * GT_TX, nr0 = blockIdx.y * GT_TR;
  const u32 np_stay = *np_stay_p;
  if (threadIdx.x < GT_TX) xedge[threadIdx.x] = x_edge(g, nx0 + threadIdx.x);
  else if (threadIdx.x < GT_TX + GT_TR) redge[threadIdx.x - GT_TX] = r_edge(g, nr0 + threadIdx.x - GT_TX);
  // 1. node tile: [ex ey ez bx by bz] (m = 0), then per mode m >= 1 the same
  //    six as 2*(re, im)
  for (int t = threadIdx.x; t < GT_NR * GT_NX; t += GT_THREADS) {
    const int lr = t / GT_NX, lc = t - lr * GT_NX;
    const int nr = nr0 + lr, nx = nx0 + lc;
    float *d = gsm + t * NS;
    const bool in = nr < Nr && nx < Nx;
    const long node = (long)nr * Nx + nx;
#pragma unroll
    for (int k = 0; k < 6; k++) d[k] = in ? __ldg((const float *)f.p[k] + node) : 0.f;
#pragma unroll
    for (int m = 1; m <= M; m++)
#pragma unroll
      for (int k = 0; k < 6; k++) {
        const float2 v = in ? __ldg((const float2 *)f.p[6 * m + k] + node) : make_float2(0.f, 0.f);
        d[6 + 12 * (m - 1) + 2 * k] = 2.f * v.x;
        d[6 + 12 * (m - 1) + 2 * k + 1] = 2.f * v.y;
      }
  }
  // 2. the tile's valid cells per row: 0 < ix < Nx-2, 0 <= ir < Nr-2
  const int ixl = nx0 > 1 ? nx0 : 1, ixh = nx0 + GT_TX - 1 < Nx - 3 ? nx0 + GT_TX - 1 : Nx - 3;
  if (threadIdx.x < GT_TR) {
    const int ir = nr0 + threadIdx.x;
    u32 a = 0, b = 0;
    if (ir < Nr - 2 && ixl <= ixh) {
      a = cell_off[(long)ixl + (long)ir * nxc];
      b = cell_off[(long)ixh + (long)ir * nxc + 1];
    }
    row_a[threadIdx.x] = a;
    row_pre[threadIdx.x + 1] = b - a;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    row_pre[0] = 0;
    for (int r = 0; r < GT_TR; r++) row_pre[r + 1] += row_pre[r];
  }
  __syncthreads();
  const u32 total = row_pre[GT_TR];
  const float dt_2 = 0.5f * dt;
  // two particles per thread and pass: both particles' loads are issued
  // before either's results are stored (a store to px[p] would otherwise
  // keep the next particle's loads from being hoisted above it)
  constexpr int GP = 2;
  for (u32 i0 = threadIdx.x; i0 < total; i0 += GP * GT_THREADS) {
    u32 pp[GP];
    int rr_[GP];
    bool ok[GP];
#pragma unroll
    for (int j = 0; j < GP; j++) {
      const u32 idx = i0 + (u32)j * GT_THREADS;
      ok[j] = idx < total;
      pp[j] = 0;
      rr_[j] = 0;
      if (ok[j]) {
        int r = 0;
#pragma unroll
        for (int q = 1; q < GT_TR; q++) r += idx >= row_pre[q];
        pp[j] = __ldg(sort_indx + row_a[r] + (idx - row_pre[r]));
        rr_[j] = r;
        ok[j] = pp[j] < np_stay;  // grid_deposit_m1.cl:367-368
      }
    }
    float vx[GP], vy[GP], vz[GP], vpx[GP], vpy[GP], vpz[GP], vxl[GP], vyl[GP], vzl[GP];
#pragma unroll
    for (int j = 0; j < GP; j++) {
      vxl[j] = vyl[j] = vzl[j] = 0.f;
      if (ok[j]) {
        const u32 p = pp[j];
        vx[j] = x[p];
        vy[j] = y[p];
        vz[j] = z[p];
        vpx[j] = px[p];
        vpy[j] = py[p];
        vpz[j] = pz[p];
        if constexpr (LO) {
          vxl[j] = xl[p];
          vyl[j] = yl[p];
          vzl[j] = zl[p];
        }
      }
    }
#pragma unroll
    for (int j = 0; j < GP; j++) {
      if (!ok[j]) continue;
      const u32 p = pp[j];
      const int r = rr_[j];
      const float xp = vx[j], yp = vy[j], zp = vz[j];
      const float pxp = vpx[j], pyp = vpy[j], pzp = vpz[j];
      const float xlp = vxl[j], ylp = vyl[j], zlp = vzl[j];
      const float r2 = yp * yp + zp * zp;
      const float rp = sqrtf(r2);
      const float rinv = r2 > 0.f ? 1.f / rp : __int_as_float(0x7f800000);
      const float fx = (xp - g.xmin) * g.dx_inv;
      int ix = (int)floorf(fx);
      ix = ix < ixl ? ixl : (ix > ixh ? ixh : ix);
      float sX1, sR1;
      if constexpr (LO) {
        float rr, rrl;
        radius_pair(yp, zp, ylp, zlp, rinv, rr, rrl);
        sX1 = edge_frac_lo(xp, xlp, xedge[ix - nx0], g.dx_inv);
        // the index from hi can be one off within an FP32 spacing of a face:
        // the cell of the full coordinate (within the tile's cells)
        if (sX1 < 0.f && ix > ixl) {
          ix--;
          sX1 = edge_frac_lo(xp, xlp, xedge[ix - nx0], g.dx_inv);
        } else if (sX1 >= 1.f && ix < ixh) {
          ix++;
          sX1 = edge_frac_lo(xp, xlp, xedge[ix - nx0], g.dx_inv);
        }
        sR1 = edge_frac_lo(rr, rrl, redge[r], g.dr_inv);
      } else {
        sX1 = edge_frac(xp, xedge[ix - nx0], g.dx_inv);
        sR1 = edge_frac(rp, redge[r], g.dr_inv);
      }
      const float sX0 = 1.f - sX1, sR0 = 1.f - sR1;
      const float C[4] = {sR0 * sX0, sR0 * sX1, sR1 * sX0, sR1 * sX1};
      const int l0 = (r * GT_NX + (ix - nx0)) * NS;
      const int loff[4] = {l0, l0 + NS, l0 + GT_NX * NS, l0 + (GT_NX + 1) * NS};
      float e[M + 1][2];
      if (M >= 1) {
        e[1][0] = yp * rinv;
        e[1][1] = -zp * rinv;
      }
  #pragma unroll
      for (int m = 2; m <= M; m++) {
        e[m][0] = e[m - 1][0] * e[1][0] - e[m - 1][1] * e[1][1];
        e[m][1] = e[m - 1][0] * e[1][1] + e[m - 1][1] * e[1][0];
      }
      float fld[6];
  #pragma unroll
      for (int k = 0; k < 6; k++) {
        float a = 0.f;
  #pragma unroll
        for (int c = 0; c < 4; c++) a = fmaf(C[c], gsm[loff[c] + k], a);
  #pragma unroll
        for (int m = 1; m <= M; m++) {
          float re = 0.f, im = 0.f;
  #pragma unroll
          for (int c = 0; c < 4; c++) {
            re = fmaf(C[c], gsm[loff[c] + 6 + 12 * (m - 1) + 2 * k], re);
            im = fmaf(C[c], gsm[loff[c] + 6 + 12 * (m - 1) + 2 * k + 1], im);
          }
          a = fmaf(re, e[m][0], a);
          a = fmaf(-im, e[m][1], a);
        }
        fld[k] = a;
      }
      // Boris push (grid_deposit_m1.cl:440-505)
      float um[3];
      um[0] = pxp + dt_2 * fld[0];
      um[1] = pyp + dt_2 * fld[1];
      um[2] = pzp + dt_2 * fld[2];
      const float gi0 = rsqrtf(1.f + um[0] * um[0] + um[1] * um[1] + um[2] * um[2]);
      float t[3], sv[3], u0[3], up[3];
  #pragma unroll
      for (int k = 0; k < 3; k++) t[k] = dt_2 * fld[3 + k] * gi0;
      const float f2 = __fdividef(2.f, 1.f + t[0] * t[0] + t[1] * t[1] + t[2] * t[2]);
  #pragma unroll
      for (int k = 0; k < 3; k++) sv[k] = t[k] * f2;
      u0[0] = um[0] + um[1] * t[2] - um[2] * t[1];
      u0[1] = um[1] - um[0] * t[2] + um[2] * t[0];
      u0[2] = um[2] + um[0] * t[1] - um[1] * t[0];
      up[0] = um[0] + u0[1] * sv[2] - u0[2] * sv[1];
      up[1] = um[1] - u0[0] * sv[2] + u0[2] * sv[0];
      up[2] = um[2] + u0[0] * sv[1] - u0[1] * sv[0];
      const float u[3] = {up[0] + dt_2 * fld[0], up[1] + dt_2 * fld[1], up[2] + dt_2 * fld[2]};
      px[p] = u[0];
      py[p] = u[1];
      pz[p] = u[2];
      g_inv[p] = rsqrtf(1.f + u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);

    }
  }
}

// with the sort's cell offsets: the FP32 form runs tile by tile, the FP64
// form is the exact kernel above
template <typename T>
int gather_push_cells(int M, long np, const T *x, const T *y, const T *z, T *px, T *py, T *pz,
                      T *g_inv, const u32 *sort_indx, const u32 *cell_off, const u32 *np_stay,
                      double factor_push, GridP<T> g, const void *const *flds, cudaStream_t s);

template <typename T>
int gather_push(int M, long np, const T *x, const T *y, const T *z, T *px,
                T *py, T *pz, T *g_inv, const u32 *sort_indx,
                const u32 *np_stay, double factor_push, GridP<T> g,
                const void *const *flds, cudaStream_t s) {
  if (np == 0) return CCL_OK;
  ptrs<24> f;
  for (int i = 0; i < 6 * (M + 1); i++) {
    CCL_REQUIRE(flds[i], CCL_ERR_ARG, "gather: null field pointer %d", i);
    f.p[i] = (void *)flds[i];
  }
  int nb = grid_for(np, 256, 16);
  T dt = (T)factor_push;
#define CCL_GP(MM)                                                                     \
  if constexpr (sizeof(T) == 4) {                                                      \
    static bool set = false; /* no shared memory: all of it as L1, set once */          \
    if (!set) {                                                                        \
      cudaFuncSetAttribute(k_gather_push_f32<MM>,                                      \
                           cudaFuncAttributePreferredSharedMemoryCarveout, 0);         \
      set = true;                                                                      \
    }                                                                                  \
    launch_pdl(k_gather_push_f32<MM>, nb, 256, 0, s, np, x, y, z, px, py, pz, g_inv, sort_indx, \
                                             np_stay, dt, g, f);                       \
  } else                                                                               \
    launch_pdl(k_gather_push<T, MM>, nb, 256, 0, s, np, x, y, z, px, py, pz, g_inv, sort_indx,  \
                                            np_stay, dt, g, f)
  switch (M) {
    case 0: CCL_GP(0); break;
    case 1: CCL_GP(1); break;
    case 2: CCL_GP(2); break;
    case 3: CCL_GP(3); break;
    default:
      set_error("gather: M=%d not supported (0..3)", M);
      return CCL_ERR_UNSUPPORTED;
  }
#undef CCL_GP
  CCL_LAUNCH_CHECK("gather_push");
  return CCL_OK;
}

// lo: nullptr, or the low parts {x_lo, y_lo, z_lo} of compensated FP32
// coordinates
template <typename T>
int gather_push_cells(int M, long np, const T *x, const T *y, const T *z, T *px, T *py, T *pz,
                      T *g_inv, const u32 *sort_indx, const u32 *cell_off, const u32 *np_stay,
                      double factor_push, GridP<T> g, const void *const *flds, cudaStream_t s,
                      const T *const *lo = nullptr) {
  if constexpr (sizeof(T) == 8) {
    (void)cell_off;
    return gather_push<T>(M, np, x, y, z, px, py, pz, g_inv, sort_indx, np_stay, factor_push, g,
                          flds, s);
  } else {
    if (np == 0) return CCL_OK;
    CCL_REQUIRE(M >= 0 && M <= 3, CCL_ERR_UNSUPPORTED, "gather: M=%d not supported (0..3)", M);
    ptrs<24> f;
    for (int i = 0; i < 6 * (M + 1); i++) {
      CCL_REQUIRE(flds[i], CCL_ERR_ARG, "gather: null field pointer %d", i);
      f.p[i] = (void *)flds[i];
    }
    dim3 grid((g.Nx + GT_TX - 1) / GT_TX, (g.Nr + GT_TR - 1) / GT_TR);
    const float dt = (float)factor_push;
#define CCL_GT(MM)                                                                         \
  {                                                                                        \
    const size_t smem = (size_t)GT_NR * GT_NX * gt_stride(MM) * sizeof(float);            \
    auto kern = lo ? k_gather_push_tiled<MM, true> : k_gather_push_tiled<MM, false>;     \
    static bool set[2] = {false, false}; /* once per instantiation */                     \
    if (!set[lo != nullptr]) {                                                             \
      cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);  \
      set[lo != nullptr] = true;                                                           \
    }                                                                                      \
    launch_pdl(kern, grid, GT_THREADS, smem, s, x, y, z, px, py, pz, g_inv, sort_indx,      \
               cell_off, np_stay, dt, g, f, lo ? lo[0] : nullptr, lo ? lo[1] : nullptr,    \
               lo ? lo[2] : nullptr);                                                      \
  }
    switch (M) {
      case 0: CCL_GT(0); break;
      case 1: CCL_GT(1); break;
      case 2: CCL_GT(2); break;
      default: CCL_GT(3); break;
    }
#undef CCL_GT
    CCL_LAUNCH_CHECK("gather_push_tiled");
    return CCL_OK;
  }
}

}  // namespace ccl
