// Particle kernels: coordinate push, cell index + stable cell sort, align,
// plasma injector.  Templated on the real type T; the FP64 instantiation is
// compiled with -fmad=false so that every expression rounds exactly as the
// reference kernels written in strict IEEE arithmetic do.
#pragma once
#include <type_traits>
#include "ccl_common.cuh"

namespace ccl {

// ---------------------------------------------------------------------
// push_xyz (particles_generic.cl:129-153): one particle's arithmetic
template <typename T>
__device__ __forceinline__ void push_one(T &xo, T &yo, T &zo, T a, T b, T c, T gi, T dt) {
  T dt_g = dt * gi;
  T ddx = a * dt_g, ddy = b * dt_g, ddz = c * dt_g;
  xo = xo + ddx;
  yo = yo + ddy;
  zo = zo + ddz;
}

template <typename T>
__global__ void k_push_x(long np, T *__restrict__ x, T *__restrict__ y,
                         T *__restrict__ z, const T *__restrict__ px,
                         const T *__restrict__ py, const T *__restrict__ pz,
                         const T *__restrict__ g_inv, T dt, int vec) {
  pdl_wait();
  // 16-byte vectors of VW particles when every array is 16-byte aligned, the
  // per-particle arithmetic of push_xyz unchanged; the tail one by one
  constexpr int VW = 16 / sizeof(T);
  using V = typename std::conditional<sizeof(T) == 4, float4, double2>::type;
  const long nv = vec ? np / VW : 0;
  for (long v = blockIdx.x * (long)blockDim.x + threadIdx.x; v < nv;
       v += (long)gridDim.x * blockDim.x) {
    V gx = ((const V *)g_inv)[v], ux = ((const V *)px)[v], uy = ((const V *)py)[v],
      uz = ((const V *)pz)[v];
    V xx = ((V *)x)[v], yy = ((V *)y)[v], zz = ((V *)z)[v];
    T *g = (T *)&gx, *a = (T *)&ux, *b = (T *)&uy, *c = (T *)&uz;
    T *xo = (T *)&xx, *yo = (T *)&yy, *zo = (T *)&zz;
#pragma unroll
    for (int q = 0; q < VW; q++) push_one(xo[q], yo[q], zo[q], a[q], b[q], c[q], g[q], dt);
    ((V *)x)[v] = xx;
    ((V *)y)[v] = yy;
    ((V *)z)[v] = zz;
  }
  for (long i = nv * VW + blockIdx.x * (long)blockDim.x + threadIdx.x; i < np;
       i += (long)gridDim.x * blockDim.x) {
    T xo = x[i], yo = y[i], zo = z[i];
    push_one(xo, yo, zo, px[i], py[i], pz[i], g_inv[i], dt);
    x[i] = xo;
    y[i] = yo;
    z[i] = zo;
  }
}

template <typename T>
int push_x(long np, T *x, T *y, T *z, const T *px, const T *py, const T *pz,
           const T *g_inv, double dt, cudaStream_t s) {
  // the vector path needs 16-byte aligned arrays (device allocations are)
  const uintptr_t mis = ((uintptr_t)x | (uintptr_t)y | (uintptr_t)z | (uintptr_t)px |
                         (uintptr_t)py | (uintptr_t)pz | (uintptr_t)g_inv) & 15;
  if (np == 0) return CCL_OK;
  launch_pdl(k_push_x<T>, grid_for(np, 256), 256, 0, s, np, x, y, z, px, py, pz, g_inv, (T)dt,
             mis == 0);
  CCL_LAUNCH_CHECK("push_x");
  return CCL_OK;
}

// ---------------------------------------------------------------------
// Compensated form of push_xyz: each coordinate is the unevaluated sum
// hi + lo of two values of the particles' type, hi the nearest value to the
// sum (what the sort, deposits and gather read).  The displacement is the
// one push_xyz forms; it is added by Knuth's two-sum (the rounding error of
// hi + d, exactly) into lo, and the pair renormalised by Dekker's fast
// two-sum.  A coordinate then drifts by no more than a few units in the last
// place of lo over a run, where a plain FP32 sum loses up to half a unit of
// hi per push (and a displacement below that is lost whole).
template <typename T>
__device__ __forceinline__ T add_rn(T a, T b) {
  if constexpr (sizeof(T) == 4) return __fadd_rn(a, b);
  else return __dadd_rn(a, b);
}
template <typename T>
__device__ __forceinline__ T sub_rn(T a, T b) {
  if constexpr (sizeof(T) == 4) return __fsub_rn(a, b);
  else return __dsub_rn(a, b);
}
template <typename T>
__device__ __forceinline__ void comp_add(T &hi, T &lo, T d) {
  const T s = add_rn(hi, d);
  const T bp = sub_rn(s, hi);
  const T e = add_rn(sub_rn(hi, sub_rn(s, bp)), sub_rn(d, bp));  // hi + d - s, exact
  const T l = add_rn(lo, e);
  const T h2 = add_rn(s, l);
  lo = sub_rn(l, sub_rn(h2, s));
  hi = h2;
}

template <typename T>
__device__ __forceinline__ void push_one_comp(T &xo, T &yo, T &zo, T &xs, T &ys, T &zs, T a,
                                              T b, T c, T gi, T dt) {
  T dt_g = dt * gi;
  comp_add(xo, xs, a * dt_g);
  comp_add(yo, ys, b * dt_g);
  comp_add(zo, zs, c * dt_g);
}

template <typename T>
__global__ void k_push_x_comp(long np, T *__restrict__ x, T *__restrict__ y,
                              T *__restrict__ z, T *__restrict__ xl, T *__restrict__ yl,
                              T *__restrict__ zl, const T *__restrict__ px,
                              const T *__restrict__ py, const T *__restrict__ pz,
                              const T *__restrict__ g_inv, T dt, int vec) {
  pdl_wait();
  constexpr int VW = 16 / sizeof(T);
  using V = typename std::conditional<sizeof(T) == 4, float4, double2>::type;
  const long nv = vec ? np / VW : 0;
  for (long v = blockIdx.x * (long)blockDim.x + threadIdx.x; v < nv;
       v += (long)gridDim.x * blockDim.x) {
    V gx = ((const V *)g_inv)[v], ux = ((const V *)px)[v], uy = ((const V *)py)[v],
      uz = ((const V *)pz)[v];
    V xx = ((V *)x)[v], yy = ((V *)y)[v], zz = ((V *)z)[v];
    V xe = ((V *)xl)[v], ye = ((V *)yl)[v], ze = ((V *)zl)[v];
    T *g = (T *)&gx, *a = (T *)&ux, *b = (T *)&uy, *c = (T *)&uz;
    T *xo = (T *)&xx, *yo = (T *)&yy, *zo = (T *)&zz;
    T *xs = (T *)&xe, *ys = (T *)&ye, *zs = (T *)&ze;
#pragma unroll
    for (int q = 0; q < VW; q++)
      push_one_comp(xo[q], yo[q], zo[q], xs[q], ys[q], zs[q], a[q], b[q], c[q], g[q], dt);
    ((V *)x)[v] = xx;
    ((V *)y)[v] = yy;
    ((V *)z)[v] = zz;
    ((V *)xl)[v] = xe;
    ((V *)yl)[v] = ye;
    ((V *)zl)[v] = ze;
  }
  for (long i = nv * VW + blockIdx.x * (long)blockDim.x + threadIdx.x; i < np;
       i += (long)gridDim.x * blockDim.x) {
    T xo = x[i], yo = y[i], zo = z[i], xs = xl[i], ys = yl[i], zs = zl[i];
    push_one_comp(xo, yo, zo, xs, ys, zs, px[i], py[i], pz[i], g_inv[i], dt);
    x[i] = xo;
    y[i] = yo;
    z[i] = zo;
    xl[i] = xs;
    yl[i] = ys;
    zl[i] = zs;
  }
}

template <typename T>
int push_x_comp(long np, T *x, T *y, T *z, T *xl, T *yl, T *zl, const T *px, const T *py,
                const T *pz, const T *g_inv, double dt, cudaStream_t s) {
  const uintptr_t mis = ((uintptr_t)x | (uintptr_t)y | (uintptr_t)z | (uintptr_t)xl |
                         (uintptr_t)yl | (uintptr_t)zl | (uintptr_t)px | (uintptr_t)py |
                         (uintptr_t)pz | (uintptr_t)g_inv) & 15;
  if (np == 0) return CCL_OK;
  launch_pdl(k_push_x_comp<T>, grid_for(np, 256), 256, 0, s, np, x, y, z, xl, yl, zl, px, py, pz,
             g_inv, (T)dt, mis == 0);
  CCL_LAUNCH_CHECK("push_x_compensated");
  return CCL_OK;
}

// ---------------------------------------------------------------------
// Cell key of a particle (particles_generic.cl:106-125).
// Grid geometry in the particles' own precision (converted once on the
// host: the FP32 kernels then never touch the FP64 pipe)
template <typename T>
struct GridP {
  int Nx, Nr;
  T xmin, dx_inv, rmin, dr_inv;
  // the FP32 kernels' cell edges xmin + i dx, rmin + i dr: origin and step as
  // unevaluated pairs hi + lo of the double values (dx = 1/dx_inv)
  T xmin_lo, dx, dx_lo, rmin_lo, dr, dr_lo;
};

template <typename T>
inline GridP<T> make_gridp(int Nx, int Nr, double xmin, double dx_inv, double rmin,
                           double dr_inv) {
  auto lo = [](double v) { return (T)(v - (double)(T)v); };
  const double dx = 1.0 / dx_inv, dr = 1.0 / dr_inv;
  return GridP<T>{Nx, Nr, (T)xmin, (T)dx_inv, (T)rmin, (T)dr_inv,
                  lo(xmin), (T)dx, lo(dx), lo(rmin), (T)dr, lo(dr)};
}

// Fraction of coordinate v in cell i of an FP32 axis with edges o + i h
// (o = o_hi + o_lo, h = h_hi + h_lo): the edge is formed as a float pair
// (two-product of i h, two-sum with o) and v - edge is exact, so the
// fraction keeps v's own precision.  The plain (v - o) / h - i rounds at
// the magnitude of the cell count: at ~2000 cells an FP32 unit in the last
// place is 1.2e-4 of a cell, which every shape-function weight then carries.
// (A kernel whose cell is fixed per thread or per tile forms the edge once.)
struct CellEdge {
  float hi, lo;
};
__device__ __forceinline__ CellEdge cell_edge(int i, float o_hi, float o_lo, float h_hi,
                                              float h_lo) {
  const float fi = (float)i;
  const float p = __fmul_rn(fi, h_hi);
  const float pe = __fmaf_rn(fi, h_hi, -p);  // fi h_hi - p, exactly
  const float c = __fadd_rn(o_hi, p);
  const float bp = __fsub_rn(c, o_hi);
  const float ce = __fadd_rn(__fsub_rn(o_hi, __fsub_rn(c, bp)), __fsub_rn(p, bp));  // o_hi + p - c
  return CellEdge{c, __fadd_rn(__fadd_rn(ce, pe), __fmaf_rn(fi, h_lo, o_lo))};
}
__device__ __forceinline__ float edge_frac(float v, CellEdge e, float h_inv) {
  return __fmul_rn(__fsub_rn(__fsub_rn(v, e.hi), e.lo), h_inv);
}
__device__ __forceinline__ CellEdge x_edge(const GridP<float> &g, int ix) {
  return cell_edge(ix, g.xmin, g.xmin_lo, g.dx, g.dx_lo);
}
__device__ __forceinline__ CellEdge r_edge(const GridP<float> &g, int ir) {
  return cell_edge(ir, g.rmin, g.rmin_lo, g.dr, g.dr_lo);
}
// r = sqrt(r2) from rinv = rsqrt(r2) (which the kernels need for e^{i m phi}
// anyway) with one Newton correction: within a unit in the last place, where
// r2 * rinv alone carries rsqrt's approximation error.  0 for r2 = 0.
__device__ __forceinline__ float radius_from_rsqrt(float r2, float rinv) {
  if (!(r2 > 0.f)) return 0.f;
  const float r = r2 * rinv;
  return fmaf(fmaf(-r, r, r2), 0.5f * rinv, r);
}
// Coordinates held as hi + lo (compensated): the in-cell fraction of v + vl
// from the edge pair, (v - e.hi) exact, the low parts added after it.
__device__ __forceinline__ float edge_frac_lo(float v, float vl, CellEdge e, float h_inv) {
  return __fmul_rn(__fadd_rn(__fsub_rn(v, e.hi), __fsub_rn(vl, e.lo)), h_inv);
}
// |(y + yl, z + zl)| as r + rl: y^2 + z^2 with its rounding errors kept
// (two-products by fma, a two-sum), the low parts to first order, then the
// Newton residual of r (exact by fma) carried into rl.  rinv ~ 1/r.
__device__ __forceinline__ void radius_pair(float y, float z, float yl, float zl, float rinv,
                                            float &r, float &rl) {
  const float p1 = __fmul_rn(y, y), p2 = __fmul_rn(z, z);
  const float e1 = __fmaf_rn(y, y, -p1), e2 = __fmaf_rn(z, z, -p2);
  const float s = __fadd_rn(p1, p2);
  const float bp = __fsub_rn(s, p1);
  const float es = __fadd_rn(__fsub_rn(p1, __fsub_rn(s, bp)), __fsub_rn(p2, bp));
  if (!(s > 0.f)) {
    r = 0.f;
    rl = 0.f;
    return;
  }
  const float slo = __fadd_rn(__fadd_rn(e1, e2), __fadd_rn(es, 2.f * (y * yl + z * zl)));
  r = radius_from_rsqrt(s, rinv);
  rl = __fmul_rn(__fadd_rn(__fmaf_rn(-r, r, s), slo), 0.5f * rinv);
}
__device__ __forceinline__ float frac_x(float xp, int ix, const GridP<float> &g) {
  return edge_frac(xp, x_edge(g, ix), g.dx_inv);
}
__device__ __forceinline__ float frac_r(float rp, int ir, const GridP<float> &g) {
  return edge_frac(rp, r_edge(g, ir), g.dr_inv);
}

template <typename T>
__device__ __forceinline__ int floor_to_int(T f, int bad) {
  // (int) of an out-of-range or NaN value: such particles are outside the
  // window; give them an index that fails the window test.  (For float the
  // upper bound rounds to 2^31, still a valid strict bound.)
  return (f > T(-2147483648.0) && f < T(2147483647.0)) ? (int)f : bad;
}

// In the particles' own precision: the FP32 form must not touch the FP64
// pipe (a few FP64 instructions per particle cost more than the whole
// kernel's memory traffic on this part).
template <typename T>
__device__ __forceinline__ u32 cell_key(T xp, T yp, T zp, const GridP<T> &g) {
  int nxc = g.Nx - 1, nrc = g.Nr - 1;
  T r = sqrt(yp * yp + zp * zp);
  int ix = floor_to_int<T>(floor((xp - g.xmin) * g.dx_inv), -1);
  int ir = floor_to_int<T>(floor((r - g.rmin) * g.dr_inv), -1);
  if (ix > 0 && ix < nxc - 1 && ir < nrc - 1 && ir >= 0)
    return (u32)(ix + ir * nxc);
  return (u32)(nrc * nxc);
}

// ---------------------------------------------------------------------
// Exclusive scan of u32 (device-wide, reduce-then-scan).
constexpr int SCAN_THREADS = 512, SCAN_ITEMS = 8,
              SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

__device__ __forceinline__ u32 block_exclusive_scan(u32 v, u32 *sh,
                                                    u32 *total) {
  // sh: SCAN_THREADS/32 words
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  u32 inc = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    u32 t = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += t;
  }
  if (lane == 31) sh[warp] = inc;
  __syncthreads();
  if (warp == 0) {
    const int nw = blockDim.x >> 5;
    u32 s = lane < nw ? sh[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      u32 t = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += t;
    }
    if (lane < nw) sh[lane] = s;
  }
  __syncthreads();
  u32 wpre = warp ? sh[warp - 1] : 0;
  if (total) *total = sh[(blockDim.x >> 5) - 1];
  __syncthreads();
  return wpre + inc - v;
}

// The sort's first pass also zeroes the workspace region that the rest of
// the sort expects at zero (scatter cursors, multi-claim bits, the scan's
// tile status words and ticket), spread over its blocks: the previous sort
// on the workspace has finished when a dependent launch passes pdl_wait.
__device__ __forceinline__ void clear_sort_region(uint4 *__restrict__ clr, long n4) {
  const long stride = (long)gridDim.x * blockDim.x;
  for (long q = (long)blockIdx.x * blockDim.x + threadIdx.x; q < n4; q += stride)
    clr[q] = make_uint4(0u, 0u, 0u, 0u);
}

// Keys + per-cell counts over tiles of ST_TILE consecutive particles; cell
// counts are aggregated per warp with match_any (a warp of cell-sorted
// particles issues one atomic per distinct cell); the particles outside the
// window (overflow key) are counted per tile.
constexpr int ST_THREADS = 256, ST_ITEMS = 8, ST_TILE = ST_THREADS * ST_ITEMS;

template <typename T>
__global__ void __launch_bounds__(ST_THREADS)
    k_keys(long np, const T *__restrict__ x, const T *__restrict__ y,
           const T *__restrict__ z, GridP<T> g, u32 *__restrict__ keys,
           u32 *__restrict__ counts, u32 *__restrict__ tile_ovf, uint4 *__restrict__ clr,
           long nclr4) {
  pdl_wait();
  clear_sort_region(clr, nclr4);
  __shared__ u32 sh[32];
  const int lane = threadIdx.x & 31;
  const u32 C = (u32)(g.Nx - 1) * (u32)(g.Nr - 1);
  const long base = (long)blockIdx.x * ST_TILE;
  u32 novf = 0;
#pragma unroll
  for (int it = 0; it < ST_ITEMS; it++) {
    const long i = base + it * ST_THREADS + threadIdx.x;
    const bool valid = i < np;
    u32 k = 0xffffffffu;
    if (valid) {
      k = cell_key<T>(x[i], y[i], z[i], g);
      keys[i] = k;
    }
    novf += (valid && k == C) ? 1u : 0u;
    const unsigned peers = __match_any_sync(0xffffffffu, k);
    if (valid && k != C && lane == __ffs(peers) - 1) atomicAdd(&counts[k], __popc(peers));
  }
  u32 tot;
  block_exclusive_scan(novf, sh, &tot);
  if (threadIdx.x == 0) {
    tile_ovf[blockIdx.x] = tot;
    if (tot) atomicAdd(&counts[C], tot);
  }
}

// The coordinate push fused with the sort's first pass: one block per tile
// of ST_TILE particles pushes them (the arithmetic of k_push_x, or of
// k_push_x_comp when COMP, 16-byte vectors when every array is 16-byte
// aligned), and writes the cell keys of the coordinates it has just formed,
// the per-cell counts and the tile's overflow count exactly as k_keys does
// from those coordinates -- without reading them back.
template <typename T, bool COMP>
__global__ void __launch_bounds__(ST_THREADS)
    k_push_keys(long np, T *__restrict__ x, T *__restrict__ y, T *__restrict__ z,
                T *__restrict__ xl, T *__restrict__ yl, T *__restrict__ zl,
                const T *__restrict__ px, const T *__restrict__ py, const T *__restrict__ pz,
                const T *__restrict__ g_inv, T dt, int vec, GridP<T> g,
                u32 *__restrict__ keys, u32 *__restrict__ counts,
                u32 *__restrict__ tile_ovf, uint4 *__restrict__ clr, long nclr4) {
  pdl_wait();
  clear_sort_region(clr, nclr4);
  constexpr int VW = 16 / sizeof(T);
  constexpr int NVT = ST_TILE / VW / ST_THREADS;  // vectors per thread
  using V = typename std::conditional<sizeof(T) == 4, float4, double2>::type;
  __shared__ u32 sh[32];
  const int lane = threadIdx.x & 31;
  const u32 C = (u32)(g.Nx - 1) * (u32)(g.Nr - 1);
  u32 novf = 0;
#pragma unroll
  for (int it = 0; it < NVT; it++) {
    const long v = (long)blockIdx.x * (ST_TILE / VW) + it * ST_THREADS + threadIdx.x;
    const long i0 = v * VW;
    u32 k[VW];
    if (vec && i0 + VW <= np) {
      V gx = ((const V *)g_inv)[v], ux = ((const V *)px)[v], uy = ((const V *)py)[v],
        uz = ((const V *)pz)[v];
      V xx = ((V *)x)[v], yy = ((V *)y)[v], zz = ((V *)z)[v];
      T *gg = (T *)&gx, *a = (T *)&ux, *b = (T *)&uy, *c = (T *)&uz;
      T *xo = (T *)&xx, *yo = (T *)&yy, *zo = (T *)&zz;
      if constexpr (COMP) {
        V xe = ((V *)xl)[v], ye = ((V *)yl)[v], ze = ((V *)zl)[v];
        T *xs = (T *)&xe, *ys = (T *)&ye, *zs = (T *)&ze;
#pragma unroll
        for (int q = 0; q < VW; q++)
          push_one_comp(xo[q], yo[q], zo[q], xs[q], ys[q], zs[q], a[q], b[q], c[q], gg[q], dt);
        ((V *)xl)[v] = xe;
        ((V *)yl)[v] = ye;
        ((V *)zl)[v] = ze;
      } else {
#pragma unroll
        for (int q = 0; q < VW; q++) push_one(xo[q], yo[q], zo[q], a[q], b[q], c[q], gg[q], dt);
      }
      ((V *)x)[v] = xx;
      ((V *)y)[v] = yy;
      ((V *)z)[v] = zz;
#pragma unroll
      for (int q = 0; q < VW; q++) {
        k[q] = cell_key<T>(xo[q], yo[q], zo[q], g);
        keys[i0 + q] = k[q];
      }
    } else {
#pragma unroll
      for (int q = 0; q < VW; q++) {
        const long i = i0 + q;
        k[q] = 0xffffffffu;
        if (i < np) {
          T xo = x[i], yo = y[i], zo = z[i];
          if constexpr (COMP) {
            T xs = xl[i], ys = yl[i], zs = zl[i];
            push_one_comp(xo, yo, zo, xs, ys, zs, px[i], py[i], pz[i], g_inv[i], dt);
            xl[i] = xs;
            yl[i] = ys;
            zl[i] = zs;
          } else {
            push_one(xo, yo, zo, px[i], py[i], pz[i], g_inv[i], dt);
          }
          x[i] = xo;
          y[i] = yo;
          z[i] = zo;
          k[q] = cell_key<T>(xo, yo, zo, g);
          keys[i] = k[q];
        }
      }
    }
#pragma unroll
    for (int q = 0; q < VW; q++) {
      const bool valid = k[q] != 0xffffffffu;
      novf += (valid && k[q] == C) ? 1u : 0u;
      const unsigned peers = __match_any_sync(0xffffffffu, k[q]);
      if (valid && k[q] != C && lane == __ffs(peers) - 1) atomicAdd(&counts[k[q]], __popc(peers));
    }
  }
  u32 tot;
  block_exclusive_scan(novf, sh, &tot);
  if (threadIdx.x == 0) {
    tile_ovf[blockIdx.x] = tot;
    if (tot) atomicAdd(&counts[C], tot);
  }
}

static inline long scan_ws_words(long L) {
  long w = 0;
  while (L > SCAN_TILE) {
    L = (L + SCAN_TILE - 1) / SCAN_TILE;
    w += L;
  }
  return w + 1;
}

// workspace: scatter cursors (C + 1 words), multi-claim bits (one per
// cell), the single-pass scan's tile status words and ticket -- together
// the region the key pass clears, a whole number of 16-byte words -- then
// per-tile overflow counts and scan partials
struct SortWs {
  u32 *cursor, *multi, *ticket, *tile_ovf, *scan;
  unsigned long long *status;
  long nclear4;  // 16-byte words cleared by the key pass, from cursor on
};

static inline long sort_multi_words(long ncells) { return (ncells + 31) / 32; }

long scan_lookback_tiles(long L);

static inline long sort_clear_words(long ncells) {
  long w = (ncells + 1 + sort_multi_words(ncells) + 1) & ~1L;  // status: 8-byte aligned
  w += 2 * scan_lookback_tiles(ncells + 1) + 2;                 // status words, ticket
  return (w + 3) & ~3L;
}

static inline size_t sort_ws_bytes(long np, long ncells) {
  long ntiles = (np + ST_TILE - 1) / ST_TILE;
  long scanw = scan_ws_words(ncells + 1 > ntiles ? ncells + 1 : ntiles);
  long words = sort_clear_words(ncells) + ntiles + 1 + scanw + 64;
  return (size_t)words * 4 + 256;
}

static inline SortWs carve_sort_ws(void *ws, long np, long ncells) {
  long ntiles = (np + ST_TILE - 1) / ST_TILE;
  uintptr_t p = ((uintptr_t)ws + 255) & ~(uintptr_t)255;
  u32 *w = (u32 *)p;
  SortWs s;
  s.cursor = w;
  s.multi = w + ncells + 1;
  const long st = (ncells + 1 + sort_multi_words(ncells) + 1) & ~1L;
  s.status = (unsigned long long *)(w + st);
  s.ticket = w + st + 2 * scan_lookback_tiles(ncells + 1);
  const long cw = sort_clear_words(ncells);
  s.nclear4 = cw / 4;
  s.tile_ovf = w + cw;
  s.scan = s.tile_ovf + ntiles + 1;
  return s;
}

// The sort after its first pass (ccl_sort.cu): offsets, scatter, fix-up.
int index_sort_keyed(long np, long C, const u32 *indx, u32 *counts, u32 *cell_offset,
                     u32 *sort_indx, u32 *np_stay, void *ws, size_t ws_bytes, cudaStream_t s);

template <typename T>
int index_sort(long np, const T *x, const T *y, const T *z, GridP<T> g,
               u32 *indx, u32 *counts, u32 *cell_offset, u32 *sort_indx,
               u32 *np_stay, void *ws, size_t ws_bytes, cudaStream_t s) {
  long C = (long)(g.Nx - 1) * (g.Nr - 1);
  CCL_REQUIRE(ws_bytes >= sort_ws_bytes(np, C), CCL_ERR_WORKSPACE,
              "index_sort: workspace %zu < %zu bytes", ws_bytes,
              sort_ws_bytes(np, C));
  SortWs w = carve_sort_ws(ws, np, C);
  const long ntiles = (np + ST_TILE - 1) / ST_TILE;
  cudaError_t me = cudaMemsetAsync(counts, 0, (C + 1) * sizeof(u32), s);
  CCL_REQUIRE(me == cudaSuccess, CCL_ERR_CUDA, "index_sort: clearing the counts: %s",
              cudaGetErrorString(me));
  if (np > 0) {
    launch_pdl(k_keys<T>, (unsigned)ntiles, ST_THREADS, 0, s, np, x, y, z, g, indx, counts,
               w.tile_ovf, (uint4 *)w.cursor, w.nclear4);
    CCL_LAUNCH_CHECK("keys");
  }
  return index_sort_keyed(np, C, indx, counts, cell_offset, sort_indx, np_stay, ws, ws_bytes,
                          s);
}

// push_xyz (compensated when xl != nullptr) + the sort's first pass; the
// sort then completes with index_sort_keyed on the same workspace
template <typename T>
int push_keys(long np, T *x, T *y, T *z, T *xl, T *yl, T *zl, const T *px, const T *py,
              const T *pz, const T *g_inv, double dt, GridP<T> g, u32 *indx, u32 *counts,
              void *ws, size_t ws_bytes, cudaStream_t s) {
  long C = (long)(g.Nx - 1) * (g.Nr - 1);
  CCL_REQUIRE(ws_bytes >= sort_ws_bytes(np, C), CCL_ERR_WORKSPACE,
              "push_x_keys: workspace %zu < %zu bytes", ws_bytes, sort_ws_bytes(np, C));
  SortWs w = carve_sort_ws(ws, np, C);
  const long ntiles = (np + ST_TILE - 1) / ST_TILE;
  cudaError_t me = cudaMemsetAsync(counts, 0, (C + 1) * sizeof(u32), s);
  CCL_REQUIRE(me == cudaSuccess, CCL_ERR_CUDA, "push_x_keys: clearing the counts: %s",
              cudaGetErrorString(me));
  if (np == 0) return CCL_OK;
  uintptr_t mis = ((uintptr_t)x | (uintptr_t)y | (uintptr_t)z | (uintptr_t)px |
                   (uintptr_t)py | (uintptr_t)pz | (uintptr_t)g_inv) & 15;
  if (xl) {
    mis |= ((uintptr_t)xl | (uintptr_t)yl | (uintptr_t)zl) & 15;
    launch_pdl(k_push_keys<T, true>, (unsigned)ntiles, ST_THREADS, 0, s, np, x, y, z, xl, yl, zl,
               px, py, pz, g_inv, (T)dt, mis == 0, g, indx, counts, w.tile_ovf,
               (uint4 *)w.cursor, w.nclear4);
  } else {
    launch_pdl(k_push_keys<T, false>, (unsigned)ntiles, ST_THREADS, 0, s, np, x, y, z, nullptr,
               nullptr, nullptr, px, py, pz, g_inv, (T)dt, mis == 0, g, indx, counts, w.tile_ovf,
               (uint4 *)w.cursor, w.nclear4);
  }
  CCL_LAUNCH_CHECK("push_x_keys");
  return CCL_OK;
}

// ---------------------------------------------------------------------
// data_align_dbl (particles_generic.cl:156-169) over up to 16 components
template <typename T>
__global__ void k_align(long n, int ncomp, ptrs<16> src, ptrs<16> dst,
                        const u32 *__restrict__ idx) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n;
       i += (long)gridDim.x * blockDim.x) {
    u32 j = idx[i];
#pragma unroll
    for (int c = 0; c < 16; c++)
      if (c < ncomp) ((T *)dst.p[c])[i] = ((const T *)src.p[c])[j];
  }
}

template <typename T>
int align(long n, int ncomp, void *const *src, void *const *dst,
          const u32 *idx, cudaStream_t s) {
  CCL_REQUIRE(ncomp >= 0 && ncomp <= 16, CCL_ERR_ARG, "align: ncomp %d", ncomp);
  if (n == 0 || ncomp == 0) return CCL_OK;
  ptrs<16> a, b;
  for (int c = 0; c < ncomp; c++) {
    CCL_REQUIRE(src[c] && dst[c], CCL_ERR_ARG, "align: null component %d", c);
    a.p[c] = src[c];
    b.p[c] = dst[c];
  }
  k_align<T><<<grid_for(n, 256), 256, 0, s>>>(n, ncomp, a, b, idx);
  CCL_LAUNCH_CHECK("align");
  return CCL_OK;
}

static __global__ void k_iota(u32 *a, long n) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n;
       i += (long)gridDim.x * blockDim.x)
    a[i] = (u32)i;
}

// ---------------------------------------------------------------------
// fill_grid (particles_generic.cl:33-84): one thread per cell
template <typename T>
__global__ void k_fill_grid(long ncells, T *x, T *y, T *z, T *w,
                            const double *theta, const double *xgrid,
                            const double *rgrid, u32 Nx, u32 npx, u32 npr,
                            u32 npth) {
  const u32 nxc = Nx - 1, nppc = npx * npr * npth;
  for (long ic = blockIdx.x * (long)blockDim.x + threadIdx.x; ic < ncells;
       ic += (long)gridDim.x * blockDim.x) {
    u32 icell = (u32)ic, ir = icell / nxc, ix = icell - nxc * ir;
    long ip = (long)icell * nppc;
    double xmin = xgrid[ix], rmin = rgrid[ir], thmin = theta[icell];
    double Lx = xgrid[ix + 1] - xgrid[ix], Lr = rgrid[ir + 1] - rgrid[ir];
    double ddx = 1. / ((double)npx), ddr = 1. / ((double)npr);
    double dth = 2 * M_PI / ((double)npth);
    for (u32 ith = 0; ith < npth; ith++) {
      double th = thmin + ith * dth;
      double sn, cs;
      sincos(th, &sn, &cs);
      for (u32 irr = 0; irr < npr; irr++) {
        double rp = rmin + (0.5 + (int)irr) * ddr * Lr;
        double rps = rp * sn, rpc = rp * cs;
        for (u32 ixx = 0; ixx < npx; ixx++) {
          x[ip] = (T)(xmin + (0.5 + (int)ixx) * ddx * Lx);
          y[ip] = (T)rps;
          z[ip] = (T)rpc;
          w[ip] = (T)rp;
          ip++;
        }
      }
    }
  }
}

// profile_by_interpolant (particles_generic.cl:6-30); the knot search is
// clamped to the last interval where the reference reads past its arrays.
template <typename T>
__global__ void k_dens_profile(long np, const T *x, T *w, const double *xx,
                               const double *ff, const double *dxm1,
                               u32 nloc) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < np;
       i += (long)gridDim.x * blockDim.x) {
    double xp = (double)x[i];
    u32 k;
    for (k = 0; k < nloc - 1; k++)
      if (xp > xx[k] && xp <= xx[k + 1]) break;
    if (k > nloc - 2) k = nloc - 2;
    double fm = ff[k] * dxm1[k], fp = ff[k + 1] * dxm1[k];
    double f = fm * (xx[k + 1] - xp) + fp * (xp - xx[k]);
    w[i] = (T)((double)w[i] * f);
  }
}

template <typename T>
__global__ void k_gamma_inv(long np, const T *px, const T *py, const T *pz,
                            T *g) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < np;
       i += (long)gridDim.x * blockDim.x)
    g[i] = (T)1 / sqrt((T)1 + px[i] * px[i] + py[i] * py[i] + pz[i] * pz[i]);
}

}  // namespace ccl
