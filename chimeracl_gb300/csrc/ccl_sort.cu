// The cell sort after its first pass (the key pass, k_keys / k_push_keys in
// ccl_particles.cuh): the cell offsets by a single-pass scan, the counting
// scatter and the fix-up of cells whose claims may be out of order -- and
// the sort's device status word.  Compiled once (no template on the
// particles' type: everything here works on keys and indices).
#include "ccl_launch.h"
#include "ccl_particles.cuh"

namespace ccl {

// the sort's status word: set when a bounded wait of the scan gave up, or
// when the scan found its ticket not cleared (a workspace on which no key
// pass ran since its last sort)
__device__ int g_sort_error = 0;

// ---------------------------------------------------------------------
// Exclusive scan of u32 (device-wide, reduce-then-scan): the per-tile
// overflow counts of very large particle sets, and the cell offsets when
// there are no particles (no key pass ran).
static __global__ void k_scan_reduce(const u32 *__restrict__ in, long L,
                              u32 *__restrict__ part) {
  pdl_wait();
  __shared__ u32 sh[32];
  long base = (long)blockIdx.x * SCAN_TILE;
  u32 s = 0;
#pragma unroll
  for (int it = 0; it < SCAN_ITEMS; it++) {
    long i = base + it * SCAN_THREADS + threadIdx.x;
    if (i < L) s += in[i];
  }
  u32 tot;
  block_exclusive_scan(s, sh, &tot);
  if (threadIdx.x == 0) part[blockIdx.x] = tot;
}

// exclusive scan of one tile per block, offset by the tile's prefix: with
// sum_parts the block adds up the raw tile sums part[0 .. blockIdx) itself
// (few tiles), else part holds them scanned.  Optionally copies out[tap_i]
// to *tap (the in-window count of the cell sort).
static __global__ void k_scan_tile(const u32 *__restrict__ in, long L,
                            const u32 *__restrict__ part, int sum_parts,
                            u32 *__restrict__ out, u32 *__restrict__ total_out,
                            u32 *__restrict__ tap, long tap_i) {
  pdl_wait();
  __shared__ u32 sh[32];
  __shared__ u32 tile_pre;
  if (threadIdx.x == 0) tile_pre = 0;
  if (part && sum_parts) {
    u32 ps = 0;
    for (long t = threadIdx.x; t < blockIdx.x; t += blockDim.x) ps += part[t];
    u32 ptot;
    __syncthreads();
    block_exclusive_scan(ps, sh, &ptot);
    if (threadIdx.x == 0) tile_pre = ptot;
  } else if (part && threadIdx.x == 0) {
    tile_pre = part[blockIdx.x];
  }
  __syncthreads();
  long base = (long)blockIdx.x * SCAN_TILE + (long)threadIdx.x * SCAN_ITEMS;
  u32 v[SCAN_ITEMS];
  u32 s = 0;
#pragma unroll
  for (int it = 0; it < SCAN_ITEMS; it++) {
    long i = base + it;
    v[it] = i < L ? in[i] : 0;
    s += v[it];
  }
  u32 tot;
  const u32 tp = tile_pre;
  u32 pre = block_exclusive_scan(s, sh, &tot) + tp;
#pragma unroll
  for (int it = 0; it < SCAN_ITEMS; it++) {
    long i = base + it;
    if (i < L) out[i] = pre;
    if (tap && i == tap_i) *tap = pre;
    pre += v[it];
  }
  if (total_out && blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) *total_out = tp + tot;
}

// out[0..L-1] = exclusive scan of in; *total_out = sum (if non-null);
// *tap = out[tap_i] (if tap).  Works in place (out == in).  ws:
// scan_ws_words(L) words.  Up to SCAN_FUSE tiles: two launches (tile sums,
// then the tile scans, each adding up its own prefix).
constexpr long SCAN_FUSE = 4096;
static int scan_exclusive(const u32 *in, long L, u32 *out, u32 *total_out,
                          u32 *ws, cudaStream_t s, u32 *tap = nullptr, long tap_i = -1) {
  if (L <= 0) return CCL_OK;
  long nb = (L + SCAN_TILE - 1) / SCAN_TILE;
  if (nb == 1) {
    launch_pdl(k_scan_tile, 1, SCAN_THREADS, 0, s, in, L, nullptr, 0, out, total_out, tap, tap_i);
    CCL_LAUNCH_CHECK("scan_tile");
    return CCL_OK;
  }
  u32 *part = ws;
  launch_pdl(k_scan_reduce, (unsigned)nb, SCAN_THREADS, 0, s, in, L, part);
  CCL_LAUNCH_CHECK("scan_reduce");
  int fused = nb <= SCAN_FUSE;
  if (!fused) {
    int rc = scan_exclusive(part, nb, part, nullptr, ws + nb, s);
    if (rc) return rc;
  }
  launch_pdl(k_scan_tile, (unsigned)nb, SCAN_THREADS, 0, s, in, L, part, fused, out, total_out, tap,
             tap_i);
  CCL_LAUNCH_CHECK("scan_tile");
  return CCL_OK;
}

// ---------------------------------------------------------------------
// Single-pass exclusive scan of the per-cell counts (the cell offsets),
// with a decoupled look-back between tiles.
//
// Tiles of LB_TILE counts are numbered in the order their blocks start (a
// ticket), so every tile's predecessors are running or done.  A tile
// publishes its own sum (flag 1) as soon as it has it, then looks back --
// the whole block reading LB_THREADS predecessors' words per round, nearest
// first -- until it meets an inclusive prefix (flag 2), and publishes its
// own inclusive prefix.  Flag and value share one 64-bit word, so no fence
// is needed between them.  (One warp reading 32 predecessors per round
// measured 7.6 us for the 255 tiles of a 2048 x 256 grid: the tiles start
// together, and the last ones walked back eight rounds before meeting an
// inclusive prefix.)  The status words and the ticket must be zero when the scan
// starts: the sort's key pass clears them together with the scatter
// cursors.
//
// Every poll is bounded: after spin_limit rounds on a window that still
// holds an unpublished word the tile records the give-up in *err (the
// sort's status word when err is null), counts the missing sums as zero and
// publishes, so that no successor waits on it.
constexpr int LB_THREADS = 256, LB_ITEMS = 8, LB_TILE = LB_THREADS * LB_ITEMS;
constexpr long SORT_SPIN_LIMIT = 1L << 20;
constexpr u32 LB_AGG = 1u, LB_INCL = 2u;

__device__ __forceinline__ unsigned long long ld_relaxed(const unsigned long long *p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_relaxed(unsigned long long *p, unsigned long long v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

static __global__ void __launch_bounds__(LB_THREADS)
    k_scan_lookback(const u32 *__restrict__ in, long L, u32 *__restrict__ out,
                    u32 *__restrict__ total_out, u32 *__restrict__ tap, long tap_i,
                    unsigned long long *status, u32 *ticket, long ntiles, long spin_limit,
                    int *err, long tile0) {
  pdl_wait();
  __shared__ u32 sh[32];
  __shared__ u32 s_tile, s_stop;
  if (threadIdx.x == 0) s_tile = atomicAdd(ticket, 1u);
  __syncthreads();
  const long t = s_tile;
  if (t >= ntiles) {  // a ticket that was not cleared: no tile of this scan
    if (threadIdx.x == 0) atomicExch(err ? err : &g_sort_error, 1);
    return;
  }
  // (tile0: the tile that in[0] starts -- 0 but for the wait probe, whose
  // one tile of data is tile 1 of its scan)
  const long base = (t - tile0) * LB_TILE + (long)threadIdx.x * LB_ITEMS;
  const bool vin = ((uintptr_t)in & 15) == 0 && base + LB_ITEMS <= L;
  u32 v[LB_ITEMS];
  if (vin) {
    const uint4 a = reinterpret_cast<const uint4 *>(in + base)[0];
    const uint4 b = reinterpret_cast<const uint4 *>(in + base)[1];
    v[0] = a.x, v[1] = a.y, v[2] = a.z, v[3] = a.w;
    v[4] = b.x, v[5] = b.y, v[6] = b.z, v[7] = b.w;
  } else {
#pragma unroll
    for (int it = 0; it < LB_ITEMS; it++) v[it] = base + it < L ? in[base + it] : 0u;
  }
  u32 sum = 0;
#pragma unroll
  for (int it = 0; it < LB_ITEMS; it++) sum += v[it];
  u32 agg;
  u32 pre = block_exclusive_scan(sum, sh, &agg);
  // publish this tile's sum, then look back block-wide: thread j reads the
  // word of tile top - j, LB_THREADS predecessors per round (the tiles of a
  // 2048 x 256 grid's offsets all in one round)
  if (threadIdx.x == 0)
    st_relaxed(status + t, ((unsigned long long)(t == 0 ? LB_INCL : LB_AGG) << 32) | agg);
  u32 before = 0;
  if (t > 0) {
    long top = t - 1, spins = 0;
    bool gave_up = false;
    while (true) {
      const long j = top - (long)threadIdx.x;
      // below tile 0: an inclusive prefix of zero
      const unsigned long long w =
          j >= 0 ? ld_relaxed(status + j) : ((unsigned long long)LB_INCL << 32);
      const u32 flag = (u32)(w >> 32);
      if (threadIdx.x == 0) s_stop = LB_THREADS;
      __syncthreads();
      if (flag == LB_INCL) atomicMin(&s_stop, (u32)threadIdx.x);  // nearest inclusive prefix
      __syncthreads();
      const u32 stop = s_stop;  // LB_THREADS: none in this window
      const bool missing = __syncthreads_or(flag == 0u && threadIdx.x <= stop);
      if (missing && !gave_up) {
        if (++spins < spin_limit) continue;
        gave_up = true;
        if (threadIdx.x == 0) atomicExch(err ? err : &g_sort_error, 1);
      }
      u32 tot;
      block_exclusive_scan((threadIdx.x <= stop && flag != 0u) ? (u32)w : 0u, sh, &tot);
      before += tot;
      if (stop < (u32)LB_THREADS) break;
      top -= LB_THREADS;
    }
  }
  if (threadIdx.x == 0 && t > 0)
    st_relaxed(status + t, ((unsigned long long)LB_INCL << 32) | (before + agg));
  pre += before;
  if (total_out && t == ntiles - 1 && threadIdx.x == 0) *total_out = before + agg;
  u32 o[LB_ITEMS];
#pragma unroll
  for (int it = 0; it < LB_ITEMS; it++) {
    o[it] = pre;
    pre += v[it];
  }
  if (tap && tap_i >= base && tap_i < base + LB_ITEMS) *tap = o[tap_i - base];
  if (((uintptr_t)out & 15) == 0 && base + LB_ITEMS <= L) {
    reinterpret_cast<uint4 *>(out + base)[0] = make_uint4(o[0], o[1], o[2], o[3]);
    reinterpret_cast<uint4 *>(out + base)[1] = make_uint4(o[4], o[5], o[6], o[7]);
  } else {
#pragma unroll
    for (int it = 0; it < LB_ITEMS; it++)
      if (base + it < L) out[base + it] = o[it];
  }
}

int scan_lookback(const u32 *in, long L, u32 *out, u32 *total_out, u32 *tap, long tap_i,
                  unsigned long long *status, u32 *ticket, cudaStream_t s) {
  if (L <= 0) return CCL_OK;
  const long nt = scan_lookback_tiles(L);
  launch_pdl(k_scan_lookback, (unsigned)nt, LB_THREADS, 0, s, in, L, out, total_out, tap, tap_i,
             status, ticket, nt, SORT_SPIN_LIMIT, (int *)nullptr, 0L);
  CCL_LAUNCH_CHECK("scan_lookback");
  return CCL_OK;
}

// ---------------------------------------------------------------------
// Counting-sort scatter.  In-window particles take their slot in their
// cell's segment through a per-cell cursor (one atomic per distinct cell per
// warp; lanes of a warp keep index order); out-of-window particles take
// cell_offset[C] + (overflow particles in earlier tiles) + (rank in this
// tile), so that segment is in index order.  A cell whose claims may have
// landed out of index order is flagged -- a claim that is not the cell's
// first, unless it directly follows the same warp's claim on the cell in
// the round before (a warp's rounds are in index order) -- and
// k_cell_fixup sorts just those cells' segments by particle number, which
// makes the result that of a stable sort: within a cell, ascending particle
// number -- the order of the reference's sort kernel run serially.  (Any
// disorder in a cell leaves at least one of its claims flagged: the first
// claim that lands after a claim of later particles is neither first nor a
// continuation.)
static __global__ void __launch_bounds__(ST_THREADS)
    k_scatter(long np, const u32 *__restrict__ keys, u32 C,
              const u32 *__restrict__ cell_offset, u32 *__restrict__ cursor,
              u32 *__restrict__ multi, const u32 *__restrict__ ovf_off, int ovf_scanned,
              u32 *__restrict__ sort_indx) {
  pdl_wait();
  __shared__ u32 sh[32];
  const int lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  const long base = (long)blockIdx.x * ST_TILE;
  // overflow items before this tile: the block adds up the per-tile counts
  // itself (ovf_scanned == 0) or reads their exclusive scan
  u32 ovf_before;
  if (!ovf_scanned) {
    u32 ps = 0;
    for (long t = threadIdx.x; t < blockIdx.x; t += blockDim.x) ps += ovf_off[t];
    block_exclusive_scan(ps, sh, &ovf_before);
  } else {
    ovf_before = ovf_off[blockIdx.x];
  }
  u32 tile_run = ovf_before + cell_offset[C];
  // overflow items of this tile (block-uniform)
  const u32 ovf_next = ovf_scanned ? (blockIdx.x + 1 < gridDim.x ? ovf_off[blockIdx.x + 1]
                                                                 : (u32)np - cell_offset[C])
                                   : ovf_before + ovf_off[blockIdx.x];
  const bool tile_has_ovf = ovf_next != ovf_before;
  if (tile_has_ovf) {
    // overflow: block-ordered rank within each round of ST_THREADS
    // consecutive items
#pragma unroll
    for (int it = 0; it < ST_ITEMS; it++) {
      const long i = base + it * ST_THREADS + threadIdx.x;
      const bool ovf = i < np && keys[i] == C;
      u32 rtot;
      const u32 r = block_exclusive_scan(ovf ? 1u : 0u, sh, &rtot);
      if (ovf) sort_indx[tile_run + r] = (u32)i;
      tile_run += rtot;
    }
  }
  // in-window: each warp takes ST_ITEMS rounds of 32 consecutive items of
  // its own 32 * ST_ITEMS (a cell split between rounds is claimed by the
  // same warp, in order); one cursor atomic per distinct cell per warp and
  // round (lanes keep index order), all of the thread's atomics issued
  // before any result is used
  const long wbase = base + (long)(threadIdx.x >> 5) * (32 * ST_ITEMS) + lane;
  u32 kk[ST_ITEMS];
#pragma unroll
  for (int it = 0; it < ST_ITEMS; it++) {
    const long i = wbase + it * 32;
    kk[it] = i < np ? keys[i] : 0xffffffffu;
  }
  unsigned peers[ST_ITEMS];
  u32 b0[ST_ITEMS];
#pragma unroll
  for (int it = 0; it < ST_ITEMS; it++) {
    const u32 k = kk[it];
    const bool win = k < C;
    peers[it] = __match_any_sync(0xffffffffu, win ? k : 0xffffffffu);
    b0[it] = 0;
    if (win && lane == __ffs(peers[it]) - 1) b0[it] = atomicAdd(&cursor[k], __popc(peers[it]));
  }

  // end of the claim made in the previous round by the group of its last
  // lane (the cell a cell-sorted round continues in the next)
  u32 kprev = 0xffffffffu, eprev = 0;
#pragma unroll
  for (int it = 0; it < ST_ITEMS; it++) {
    const long i = wbase + it * 32;
    const u32 k = kk[it];
    const bool win = k < C;
    const int leader = __ffs(peers[it]) - 1;
    // a claim that is neither the cell's first nor the direct continuation
    // of this warp's claim in the previous round: the cell's order may need
    // the fix-up
    if (win && lane == leader && b0[it] != 0 && !(k == kprev && b0[it] == eprev))
      atomicOr(&multi[k >> 5], 1u << (k & 31));
    const u32 b = __shfl_sync(0xffffffffu, b0[it], leader);
    // (cursors left from an earlier sort -- no key pass cleared them, which
    // the scan's ticket reports -- must not write past the array)
    if (win) {
      const u32 pos = cell_offset[k] + b + __popc(peers[it] & lt);
      if (pos < (u32)np) sort_indx[pos] = (u32)i;
    }
    const unsigned pl = __shfl_sync(0xffffffffu, peers[it], 31);
    kprev = __shfl_sync(0xffffffffu, k, 31);
    eprev = __shfl_sync(0xffffffffu, b, 31) + __popc(pl);
  }
}

// Fix-up of the cells the scatter flagged (claims possibly out of index
// order; the items of one claim are written in ascending order).  A warp takes
// 32 consecutive cells, one per lane: segments of up to FX_REG items are
// sorted by their lane in registers (Batcher's odd-even merge network over
// 16 or 32 inputs);
// longer ones -- a dense bunch of the plasma, or a whole layout of
// particles on cell faces -- by the whole warp, one at a time, with a
// bitonic sort in shared memory (up to FX_BUF items; a longer segment, not
// met in practice, by insertion sort in place).  Every other cell is left
// untouched without reading it.
constexpr int FX_REG = 32, FX_WARPS = 4, FX_BUF = 2048;

__device__ __forceinline__ void cswap(u32 &a, u32 &b) {
  const u32 lo = a < b ? a : b, hi = a < b ? b : a;
  a = lo;
  b = hi;
}

// ascending sort of g[0 .. n), n <= N, by one thread in registers
// (Batcher's odd-even merge network over N inputs)
template <int N>
__device__ __forceinline__ void reg_sort(u32 *__restrict__ g, u32 n) {
  u32 v[N];
#pragma unroll
  for (int i = 0; i < N; i++) v[i] = (u32)i < n ? g[i] : 0xffffffffu;
  // a segment whose claims landed in order is left as it is
  bool sorted = true;
#pragma unroll
  for (int i = 1; i < N; i++) sorted = sorted && ((u32)i >= n || v[i - 1] < v[i]);
  if (sorted) return;
#pragma unroll
  for (int p = 1; p < N; p <<= 1)
#pragma unroll
    for (int k = p; k >= 1; k >>= 1)
#pragma unroll
      for (int j = k % p; j <= N - 1 - k; j += 2 * k)
#pragma unroll
        for (int i = 0; i <= k - 1 && i + j + k <= N - 1; i++)
          if ((i + j) / (2 * p) == (i + j + k) / (2 * p)) cswap(v[i + j], v[i + j + k]);
#pragma unroll
  for (int i = 0; i < N; i++)
    if ((u32)i < n) g[i] = v[i];
}

// ascending sort of g[0 .. n) (distinct values) by the 32 lanes of a warp
// through buf (FX_BUF words of shared memory)
__device__ __forceinline__ void warp_bitonic_sort(u32 *__restrict__ g, u32 n, u32 *buf,
                                                  int lane) {
  u32 P = 32;
  while (P < n) P <<= 1;
  for (u32 i = lane; i < P; i += 32) buf[i] = i < n ? g[i] : 0xffffffffu;
  __syncwarp();
  for (u32 k = 2; k <= P; k <<= 1)
    for (u32 j = k >> 1; j > 0; j >>= 1) {
      for (u32 i = lane; i < P; i += 32) {
        const u32 l = i ^ j;
        if (l > i) {
          const u32 a = buf[i], b = buf[l];
          if ((a > b) == ((i & k) == 0)) {
            buf[i] = b;
            buf[l] = a;
          }
        }
      }
      __syncwarp();
    }
  for (u32 i = lane; i < n; i += 32) g[i] = buf[i];
  __syncwarp();
}

static __global__ void __launch_bounds__(FX_WARPS * 32)
    k_cell_fixup(u32 C, const u32 *__restrict__ cell_offset, const u32 *__restrict__ multi,
                 u32 *__restrict__ sort_indx) {
  pdl_wait();
  __shared__ u32 buf[FX_WARPS][FX_BUF];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const long stride = (long)gridDim.x * FX_WARPS * 32;
  for (long c0 = ((long)blockIdx.x * FX_WARPS + warp) * 32; c0 < (long)C; c0 += stride) {
    const long c = c0 + lane;
    const bool flagged = c < (long)C && (multi[c >> 5] & (1u << (c & 31)));
    u32 p0 = 0, n = 0;
    if (flagged) {
      p0 = cell_offset[c];
      n = cell_offset[c + 1] - p0;
    }
    if (flagged && n <= (u32)FX_REG / 2) reg_sort<FX_REG / 2>(sort_indx + p0, n);
    else if (flagged && n <= (u32)FX_REG) reg_sort<FX_REG>(sort_indx + p0, n);
    unsigned big = __ballot_sync(0xffffffffu, flagged && n > (u32)FX_REG);
    while (big) {
      const int l = __ffs(big) - 1;
      big &= big - 1;
      const u32 q0 = __shfl_sync(0xffffffffu, p0, l), qn = __shfl_sync(0xffffffffu, n, l);
      if (qn <= (u32)FX_BUF) {
        warp_bitonic_sort(sort_indx + q0, qn, buf[warp], lane);
      } else {
        if (lane == 0)
          for (u32 a = q0 + 1; a < q0 + qn; a++) {
            const u32 v = sort_indx[a];
            u32 b = a;
            while (b > q0 && sort_indx[b - 1] > v) {
              sort_indx[b] = sort_indx[b - 1];
              b--;
            }
            sort_indx[b] = v;
          }
        __syncwarp();
      }
    }
  }
}

// The sort after its first pass (keys in indx, counts in counts, the tiles'
// overflow counts in the workspace, the cleared region zero): offsets,
// scatter, fix-up.
int index_sort_keyed(long np, long C, const u32 *indx, u32 *counts, u32 *cell_offset,
                     u32 *sort_indx, u32 *np_stay, void *ws, size_t ws_bytes, cudaStream_t s) {
  CCL_REQUIRE(ws_bytes >= sort_ws_bytes(np, C), CCL_ERR_WORKSPACE,
              "index_sort: workspace %zu < %zu bytes", ws_bytes, sort_ws_bytes(np, C));
  SortWs w = carve_sort_ws(ws, np, C);
  const long ntiles = (np + ST_TILE - 1) / ST_TILE;
  // offsets, total, and np_stay = cell_offset[C] from the scan's own tap;
  // with no particles no key pass ran (nothing cleared): the two-launch scan
  if (np == 0)
    return scan_exclusive(counts, C + 1, cell_offset, cell_offset + C + 1, w.scan, s, np_stay, C);
  int rc = scan_lookback(counts, C + 1, cell_offset, cell_offset + C + 1, np_stay, C, w.status,
                         w.ticket, s);
  if (rc) return rc;
  // few tiles: each scatter block adds up the overflow counts before it
  const int ovf_scanned = ntiles > SCAN_FUSE;
  if (ovf_scanned) {
    rc = scan_exclusive(w.tile_ovf, ntiles, w.tile_ovf, nullptr, w.scan, s);
    if (rc) return rc;
  }
  launch_pdl(k_scatter, (unsigned)ntiles, ST_THREADS, 0, s, np, indx, (u32)C, cell_offset, w.cursor,
             w.multi, w.tile_ovf, ovf_scanned, sort_indx);
  CCL_LAUNCH_CHECK("scatter");
  if (C > 0)
    launch_pdl(k_cell_fixup, grid_for(C, FX_WARPS * 32), FX_WARPS * 32, 0, s, (u32)C, cell_offset,
               w.multi, sort_indx);
  CCL_LAUNCH_CHECK("cell_fixup");
  return CCL_OK;
}

long scan_lookback_tiles(long L) { return (L + LB_TILE - 1) / LB_TILE; }

int index_sort_keyed_launch(long np, long ncells, const uint32_t *indx, uint32_t *counts,
                            uint32_t *cell_offset, uint32_t *sort_indx, uint32_t *np_stay,
                            void *ws, size_t ws_bytes, cudaStream_t s) {
  return index_sort_keyed(np, ncells, indx, counts, cell_offset, sort_indx, np_stay, ws,
                          ws_bytes, s);
}

int sort_status(int reset) {
  int v = 0;
  cudaMemcpyFromSymbol(&v, g_sort_error, sizeof(int));
  if (reset) {
    int z = 0;
    cudaMemcpyToSymbol(g_sort_error, &z, sizeof(int));
  }
  return v;
}

// The look-back's bounded wait on its own: one block that holds ticket 1
// looks back at tile 0, whose status word is published (publish != 0) or
// never written; scratch: 4 words (tile 0's and 1's status words), 1 word
// (ticket), 1 word (in), 1 word (out).
static __global__ void k_scan_probe_setup(unsigned long long *status, u32 *ticket, u32 *in,
                                          int publish) {
  status[0] = publish ? (((unsigned long long)LB_INCL << 32) | 5u) : 0ull;
  status[1] = 0ull;
  *ticket = 1u;
  *in = 7u;
}

int scan_wait_probe(long spins, int publish, int *gave_up, u32 *scratch, cudaStream_t s) {
  CCL_REQUIRE(spins >= 1 && spins <= SORT_SPIN_LIMIT, CCL_ERR_ARG,
              "scan wait probe: spins=%ld outside [1, %ld]", spins, SORT_SPIN_LIMIT);
  CCL_REQUIRE(((uintptr_t)scratch & 7) == 0, CCL_ERR_ARG,
              "scan wait probe: scratch not 8-byte aligned");
  unsigned long long *status = (unsigned long long *)scratch;
  u32 *ticket = scratch + 4, *in = scratch + 5, *out = scratch + 6;
  cudaError_t e = cudaMemsetAsync(gave_up, 0, sizeof(int), s);
  CCL_REQUIRE(e == cudaSuccess, CCL_ERR_CUDA, "scan wait probe: %s", cudaGetErrorString(e));
  k_scan_probe_setup<<<1, 1, 0, s>>>(status, ticket, in, publish);
  CCL_LAUNCH_CHECK("scan_probe_setup");
  // one item (L = 1) in tile 1 of a scan whose tile 0 is status[0]
  k_scan_lookback<<<1, LB_THREADS, 0, s>>>(in, 1, out, nullptr, nullptr, -1, status, ticket, 2,
                                           spins, gave_up, 1);
  CCL_LAUNCH_CHECK("scan_wait_probe");
  return CCL_OK;
}

}  // namespace ccl
