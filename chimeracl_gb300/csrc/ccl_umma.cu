// The discrete Hankel transform as a BF16x3 split-precision GEMM on the
// 5th-generation tensor cores (tcgen05.mma, FP32 accumulation in TMEM):
//   Y = beta*Y + alpha * (A X),  A ~ A_hi + A_lo,  X ~ X_hi + X_lo  (bf16),
//   A X ~ A_hi X_hi + A_hi X_lo + A_lo X_hi,
// A real (m x k, k <= 256), X FP32 (k x ncols real columns, interleaved
// complex allowed), Y FP32.
//
// The pre-split A (hi then lo per 128-row tile, K-major, no-swizzle
// core-matrix layout, produced by k_umma_split_a) is bulk-copied into shared
// memory and stays resident while a CTA walks its N tiles; X is split into
// bf16 hi/lo on the fly.  Every mbarrier wait is bounded; a wait that gives up
// records an error code in a device flag, the CTA skips the rest of its work,
// drains what it issued (bounded) and frees its TMEM.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>
#include <stdint.h>

#include <mutex>

#include "ccl_common.cuh"
#include "ccl_launch.h"

namespace ccl {

constexpr int UM_BM = 128, UM_BK = 128;
constexpr int UM_MAXK = 256, UM_MAXBATCH = 32;
constexpr long UM_SPIN_LIMIT = 20000000L;  // ~ a second of try_wait polls

__device__ int g_umma_error = 0;

// bytes of one pre-split M tile: hi and lo, 128 rows x kp columns of bf16
__host__ __device__ constexpr long umma_tile_bytes(int kp) { return 2L * UM_BM * kp * 2; }

static inline int umma_kpad(int k) { return k <= UM_BK ? UM_BK : UM_MAXK; }

// ------------------------------------------------------------------ PTX
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n"
      " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// bounded wait: true when the phase completed, false after the spin limit
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
  for (long i = 0; i < UM_SPIN_LIMIT; i++)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

__device__ __forceinline__ void fence_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// shared-memory matrix descriptor, no swizzle: start, leading-dimension
// (K-adjacent core matrices) and stride-dimension (M/N-adjacent 8-row
// groups) byte offsets, fixed field 0b001 at bits 46-48
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((addr & 0x3FFFF) >> 4);
  d |= (uint64_t)((lbo & 0x3FFFF) >> 4) << 16;
  d |= (uint64_t)((sbo & 0x3FFFF) >> 4) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// instruction descriptor, kind::f16: D f32, A/B bf16, both K-major
__host__ __device__ constexpr uint32_t umma_idesc(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) |
         ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void umma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b,
                                          uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void umma_commit(uint64_t *bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float *v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,"
      "%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
#pragma unroll
  for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void tmem_wait_ld() {
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ uint32_t pack_bf16(__nv_bfloat16 lo_k, __nv_bfloat16 hi_k) {
  return (uint32_t)__bfloat16_as_ushort(lo_k) | ((uint32_t)__bfloat16_as_ushort(hi_k) << 16);
}

// ------------------------------------------------------------- A split
// A (m x k, row-major, lda = k) -> per 128-row tile: hi block then lo block,
// core matrix (g = row/8, j = col/8) at ((g * kp/8 + j) * 128) bytes, each
// core matrix 8 rows x 8 consecutive k values.  Zero outside m x k.
template <typename TA>
__global__ void k_umma_split_a(const TA *__restrict__ A, int m, int k, int kp, int ntile,
                               uint4 *__restrict__ out) {
  const long per_tile = (long)UM_BM * kp / 8;  // core-matrix rows (16 B) per block
  const long total = (long)ntile * 2 * per_tile;
  for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < total;
       q += (long)gridDim.x * blockDim.x) {
    long t = q / (2 * per_tile), rem = q - t * 2 * per_tile;
    int lo = rem >= per_tile;
    long w = rem - lo * per_tile;            // 16-B row index within the block
    long cm = w / 8, i = w - cm * 8;         // core matrix, row within it
    long g = cm / (kp / 8), j = cm - g * (kp / 8);
    long row = t * UM_BM + g * 8 + i;
    __nv_bfloat16 e[8];
#pragma unroll
    for (int c = 0; c < 8; c++) {
      long col = j * 8 + c;
      float v = (row < m && col < k) ? (float)A[row * k + col] : 0.f;
      __nv_bfloat16 h = __float2bfloat16_rn(v);
      e[c] = lo ? __float2bfloat16_rn(v - __bfloat162float(h)) : h;
    }
    uint4 o;
    o.x = pack_bf16(e[0], e[1]);
    o.y = pack_bf16(e[2], e[3]);
    o.z = pack_bf16(e[4], e[5]);
    o.w = pack_bf16(e[6], e[7]);
    out[q] = o;
  }
}

// ---------------------------------------------------------------- GEMM
// Persistent, warp-specialised kernel.  Work item = (batch entry e, 128-row
// M tile mt, 128-column N tile nt), ordered (e, mt, nt); CTA c takes a
// contiguous run of items, so the resident A tile is reloaded only when
// (e, mt) changes (one bulk copy into shared memory).
//   warps 0-3  epilogue: TMEM lanes 32w..32w+31 (= output rows) -> alpha,
//              optional +Y, row-contiguous stores
//   warps 4-11 converters: raw FP32 stage (32 k x 128 n) -> K-major bf16
//              hi/lo core matrices in a ring of UM_NS slots.  They issue no
//              global loads, so their proxy fence has nothing to drain.
//   warp 12    lane 0: TMA producer, one 2-D tensor copy per stage into a
//              ring of UM_NR raw slots (out-of-range rows/columns read as 0)
//   warp 13    lane 0: A bulk copies and the MMAs (3 per 16-deep k step),
//              double-buffered 128 x 128 FP32 accumulators in TMEM
// Every wait is bounded (and gives up early once another role has aborted);
// the MMA thread drains its MMAs and the producer its copies before the CTA
// releases TMEM and exits.
constexpr int UM_EPI_WARPS = 4, UM_CVT_WARPS = 8;
constexpr int UM_THREADS2 = (UM_EPI_WARPS + UM_CVT_WARPS + 2) * 32;  // 448
constexpr int UM_TN = 128;        // N tile (columns of X / Y)
constexpr int UM_KC = 32;         // K depth of one stage
constexpr int UM_NS = 2;          // bf16 slots
constexpr int UM_NR = 4;          // raw FP32 slots
constexpr uint32_t UM_SLOT = 2u * UM_KC * UM_TN * 2;  // hi + lo bf16: 16 KB
constexpr uint32_t UM_RAW = (uint32_t)UM_KC * UM_TN * 4;  // FP32: 16 KB
constexpr int UM_CVT_THREADS = UM_CVT_WARPS * 32;

struct UmmaWork {
  const void *A[UM_MAXBATCH];
  float *Y[UM_MAXBATCH];
  int ncols[UM_MAXBATCH];
  int ntn[UM_MAXBATCH];    // N tiles of the entry
  int base[UM_MAXBATCH];   // first item of the entry
  long ldy[UM_MAXBATCH];
  int batch, items, mtiles;
};

// X of every entry as a 2-D tensor map (inner dim = columns, box 128 x 32)
struct UmmaArgs {
  CUtensorMap tx[UM_MAXBATCH];
  UmmaWork w;
};

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes,
                                         uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"((uint64_t)__cvta_generic_to_global(src)), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}
// 2-D tiled tensor copy global -> shared; x (columns) must be a multiple of
// 4 floats (16 bytes), which every N tile origin is
__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, int x, int y,
                                            uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(dst)),
      "l"((uint64_t)map), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

// bounded wait that also gives up once `abort` is set by another role
__device__ __forceinline__ bool mbar_wait_ab(uint64_t *bar, uint32_t parity,
                                             volatile int *abort) {
  for (long i = 0; i < UM_SPIN_LIMIT; i++) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((i & 255) == 255 && *abort) return false;
  }
  return false;
}

__device__ __forceinline__ void um_fail(volatile int *abort, int code) {
  if (!*abort) atomicCAS(&g_umma_error, 0, code);
  *abort = 1;
}

__device__ __forceinline__ void um_decode(const UmmaWork &w, int item, int &e, int &mt,
                                          int &nt) {
  e = 0;
  while (e + 1 < w.batch && w.base[e + 1] <= item) e++;
  const int r = item - w.base[e];
  mt = r / w.ntn[e];
  nt = r - mt * w.ntn[e];
}

// converter: k rows kb*8 .. +7, columns n, n+1 of a raw stage -> one core
// matrix row (8 k values) of hi and of lo for each column; core matrix
// (gn = n/8, kb) at (gn*4 + kb)*128, row n%8; hi block, then lo block.
// Pairs of k values are rounded and packed by one cvt.rn.bf16x2 each.
__device__ __forceinline__ uint32_t bf2_bits(__nv_bfloat162 h) {
  return *reinterpret_cast<uint32_t *>(&h);
}
__device__ __forceinline__ void cvt_stage(const float *raw, int kb, int ncol_local,
                                          uint4 (&o)[4]) {
  float2 t[8];
#pragma unroll
  for (int q = 0; q < 8; q++) t[q] = *(const float2 *)(raw + (kb * 8 + q) * UM_TN + ncol_local);
  uint32_t hw[2][4], lw[2][4];
#pragma unroll
  for (int p = 0; p < 4; p++) {
    // column n (.x) and n+1 (.y), k values 2p and 2p+1 (low half = lower k)
    const __nv_bfloat162 h0 = __floats2bfloat162_rn(t[2 * p].x, t[2 * p + 1].x);
    const __nv_bfloat162 h1 = __floats2bfloat162_rn(t[2 * p].y, t[2 * p + 1].y);
    const float2 f0 = __bfloat1622float2(h0), f1 = __bfloat1622float2(h1);
    const __nv_bfloat162 l0 = __floats2bfloat162_rn(t[2 * p].x - f0.x, t[2 * p + 1].x - f0.y);
    const __nv_bfloat162 l1 = __floats2bfloat162_rn(t[2 * p].y - f1.x, t[2 * p + 1].y - f1.y);
    hw[0][p] = bf2_bits(h0);
    hw[1][p] = bf2_bits(h1);
    lw[0][p] = bf2_bits(l0);
    lw[1][p] = bf2_bits(l1);
  }
  o[0] = make_uint4(hw[0][0], hw[0][1], hw[0][2], hw[0][3]);
  o[1] = make_uint4(lw[0][0], lw[0][1], lw[0][2], lw[0][3]);
  o[2] = make_uint4(hw[1][0], hw[1][1], hw[1][2], hw[1][3]);
  o[3] = make_uint4(lw[1][0], lw[1][1], lw[1][2], lw[1][3]);
}

template <bool CPLX, bool ACC>
__global__ void __launch_bounds__(UM_THREADS2, 1)
    k_umma_gemm(const __grid_constant__ UmmaArgs args, int M, int K, int KP, int vec_y,
                float are, float aim) {
  extern __shared__ __align__(1024) unsigned char smraw[];
  const UmmaWork &w = args.w;
  unsigned char *sm = (unsigned char *)(((uintptr_t)smraw + 1023) & ~(uintptr_t)1023);
  const uint32_t a_bytes = (uint32_t)umma_tile_bytes(KP);
  unsigned char *sA = sm;
  unsigned char *sX = sA + a_bytes;       // UM_NS bf16 slots
  unsigned char *sR = sX + UM_NS * UM_SLOT;  // UM_NR raw slots
  uint64_t *full = (uint64_t *)(sR + UM_NR * UM_RAW);
  uint64_t *empty = full + UM_NS;
  uint64_t *rfull = empty + UM_NS;
  uint64_t *rempty = rfull + UM_NR;
  uint64_t *tfull = rempty + UM_NR;  // [2]
  uint64_t *tempty = tfull + 2;      // [2]
  uint64_t *abar = tempty + 2;
  uint64_t *dbar = abar + 1;
  uint32_t *tmem_slot = (uint32_t *)(dbar + 1);
  volatile int *abort = (volatile int *)(tmem_slot + 1);

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int nkc = (K + UM_KC - 1) / UM_KC;
  const int i0 = (int)((long)blockIdx.x * w.items / gridDim.x);
  const int i1 = (int)((long)(blockIdx.x + 1) * w.items / gridDim.x);
  const int S = (i1 - i0) * nkc;  // stages of this CTA

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 256;" ::"r"(
        smem_u32(tmem_slot)));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    for (int i = 0; i < UM_NS; i++) {
      mbar_init(&full[i], UM_CVT_THREADS);
      mbar_init(&empty[i], 1);
    }
    for (int i = 0; i < UM_NR; i++) {
      mbar_init(&rfull[i], 1);
      mbar_init(&rempty[i], UM_CVT_THREADS);
    }
    for (int i = 0; i < 2; i++) {
      mbar_init(&tfull[i], 1);
      mbar_init(&tempty[i], UM_EPI_WARPS * 32);
    }
    mbar_init(abar, 1);
    mbar_init(dbar, 1);
    *abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp < UM_EPI_WARPS) {
    // ------------------------------------------------------------ epilogue
    // tcgen05.ld is warp-collective: every exit decision is taken warp-wide
    for (int j = 0, item = i0; item < i1; j++, item++) {
      if (__any_sync(0xffffffffu, *abort)) break;
      int e, mt, nt;
      um_decode(w, item, e, mt, nt);
      const int b = j & 1;
      const bool got = mbar_wait_ab(&tfull[b], (j >> 1) & 1, abort);
      if (!__all_sync(0xffffffffu, got)) {
        um_fail(abort, 2);
        break;
      }
      tc_fence_after();
      const int N = w.ncols[e];
      const int n0 = nt * UM_TN;
      const uint32_t tb = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(b * UM_TN);
      const int gm = mt * UM_BM + warp * 32 + lane;
      float *__restrict__ yrow = w.Y[e] + (long)gm * w.ldy[e];
      // row-contiguous stores: lane = output row, 32 columns per chunk
#pragma unroll 1
      for (int q = 0; q < UM_TN / 32; q++) {
        float v[32];
        tmem_ld16(tb + q * 32, v);
        tmem_ld16(tb + q * 32 + 16, v + 16);
        tmem_wait_ld();
        if (gm < M) {
          const int c0 = n0 + q * 32;
          if (vec_y && c0 + 32 <= N) {
#pragma unroll
            for (int c = 0; c < 32; c += 4) {
              float4 r;
              if (CPLX) {
                r.x = are * v[c] - aim * v[c + 1];
                r.y = are * v[c + 1] + aim * v[c];
                r.z = are * v[c + 2] - aim * v[c + 3];
                r.w = are * v[c + 3] + aim * v[c + 2];
              } else {
                r.x = are * v[c];
                r.y = are * v[c + 1];
                r.z = are * v[c + 2];
                r.w = are * v[c + 3];
              }
              if (ACC) {
                const float4 o = *(const float4 *)(yrow + c0 + c);
                r.x += o.x; r.y += o.y; r.z += o.z; r.w += o.w;
              }
              *(float4 *)(yrow + c0 + c) = r;
            }
          } else {
#pragma unroll
            for (int c = 0; c < 32; c += 2) {
              const int gn = c0 + c;
              if (gn >= N) break;
              float r0, r1;
              if (CPLX) {
                r0 = are * v[c] - aim * v[c + 1];
                r1 = are * v[c + 1] + aim * v[c];
              } else {
                r0 = are * v[c];
                r1 = are * v[c + 1];
              }
              if (ACC) {
                r0 += yrow[gn];
                if (gn + 1 < N) r1 += yrow[gn + 1];
              }
              yrow[gn] = r0;
              if (gn + 1 < N) yrow[gn + 1] = r1;
            }
          }
        }
      }
      tc_fence_before();
      mbar_arrive(&tempty[b]);
    }
  } else if (warp < UM_EPI_WARPS + UM_CVT_WARPS) {
    // ---------------------------------------------------------- converters
    const int ct = tid - UM_EPI_WARPS * 32;
    const int cw = ct >> 5;
    const int kb = cw >> 1;                              // k block 0..3
    const int ncol_local = 2 * ((cw & 1) * 32 + lane);   // 0..126
    const uint32_t o0 = (uint32_t)(((ncol_local >> 3) * (UM_KC / 8) + kb) * 128 +
                                   (ncol_local & 7) * 16);
    for (int s = 0; s < S; s++) {
      if (*abort) break;
      const int r = s % UM_NR, slot = s % UM_NS;
      if (!mbar_wait_ab(&rfull[r], (s / UM_NR) & 1, abort)) {
        um_fail(abort, 7);
        break;
      }
      uint4 o[4];
      cvt_stage((const float *)(sR + r * UM_RAW), kb, ncol_local, o);
      if (s >= UM_NS && !mbar_wait_ab(&empty[slot], ((s / UM_NS) - 1) & 1, abort)) {
        um_fail(abort, 1);
        break;
      }
      unsigned char *dst = sX + slot * UM_SLOT + o0;
      *(uint4 *)(dst) = o[0];              // column n: hi
      *(uint4 *)(dst + UM_SLOT / 2) = o[1];  //           lo
      *(uint4 *)(dst + 16) = o[2];         // column n+1 (next core-matrix row)
      *(uint4 *)(dst + 16 + UM_SLOT / 2) = o[3];
      // one proxy fence orders both hand-offs against the async proxy: the
      // raw slot's generic-proxy reads before the next tensor copy into it
      // (the barrier's release alone does not order across proxies), and the
      // bf16 stores before the MMAs that read them
      fence_async_smem();
      mbar_arrive(&rempty[r]);
      mbar_arrive(&full[slot]);
    }
  } else if (warp == UM_EPI_WARPS + UM_CVT_WARPS) {
    // ------------------------------------------------- TMA producer (one lane)
    if (lane == 0) {
      int issued = 0;
      for (int s = 0; s < S; s++) {
        if (*abort) break;
        const int r = s % UM_NR;
        if (s >= UM_NR && !mbar_wait_ab(&rempty[r], ((s / UM_NR) - 1) & 1, abort)) {
          um_fail(abort, 8);
          break;
        }
        int e, mt, nt;
        um_decode(w, i0 + s / nkc, e, mt, nt);
        mbar_expect_tx(&rfull[r], UM_RAW);
        tma_load_2d(sR + r * UM_RAW, &args.tx[e], nt * UM_TN, (s % nkc) * UM_KC, &rfull[r]);
        issued = s + 1;
      }
      // every copy this lane issued has landed before the CTA may exit
      for (int s = issued - UM_NR < 0 ? 0 : issued - UM_NR; s < issued; s++)
        (void)mbar_wait(&rfull[s % UM_NR], (s / UM_NR) & 1);
    }
  } else if (lane == 0) {
    // ------------------------------------------------------ MMA (one lane)
    const uint32_t idesc = umma_idesc(UM_BM, UM_TN);
    const uint32_t sA_u = smem_u32(sA), sX_u = smem_u32(sX);
    const uint32_t a_sbo = (uint32_t)(KP / 8) * 128, a_lo = a_bytes / 2;
    const uint32_t x_sbo = (UM_KC / 8) * 128;
    int a_key = -1, a_phase = 0, d_phase = 0, s = 0;
    bool issued = false;
    for (int j = 0, item = i0; item < i1; j++, item++) {
      if (*abort) break;
      int e, mt, nt;
      um_decode(w, item, e, mt, nt);
      const int key = e * 1024 + mt;
      if (key != a_key) {
        if (issued) {  // every MMA reading the old tile has completed
          umma_commit(dbar);
          if (!mbar_wait_ab(dbar, d_phase & 1, abort)) { um_fail(abort, 3); break; }
          d_phase++;
          issued = false;
        }
        const unsigned char *src = (const unsigned char *)w.A[e] + (long)mt * a_bytes;
        mbar_expect_tx(abar, a_bytes);
        for (uint32_t off = 0; off < a_bytes; off += 32768u)
          bulk_g2s(sA + off, src + off, min(32768u, a_bytes - off), abar);
        // the copy must land before anything else happens in this CTA
        if (!mbar_wait(abar, a_phase & 1)) { um_fail(abort, 4); break; }
        a_phase++;
        a_key = key;
      }
      const int b = j & 1;
      if (j >= 2 && !mbar_wait_ab(&tempty[b], ((j - 2) >> 1) & 1, abort)) {
        um_fail(abort, 5);
        break;
      }
      tc_fence_after();
      const uint32_t d = tmem + (uint32_t)(b * UM_TN);
      bool ok = true;
      for (int kc = 0; kc < nkc; kc++, s++) {
        const int slot = s % UM_NS;
        if (!mbar_wait_ab(&full[slot], (s / UM_NS) & 1, abort)) {
          um_fail(abort, 6);
          ok = false;
          break;
        }
        tc_fence_after();
        const uint32_t xs = sX_u + slot * UM_SLOT;
#pragma unroll
        for (int ks = 0; ks < UM_KC / 16; ks++) {
          const uint32_t ja = (uint32_t)(kc * (UM_KC / 8) + 2 * ks) * 128;
          const uint64_t ahi = smem_desc(sA_u + ja, 128, a_sbo);
          const uint64_t alo = smem_desc(sA_u + a_lo + ja, 128, a_sbo);
          const uint64_t bhi = smem_desc(xs + (uint32_t)(2 * ks) * 128, 128, x_sbo);
          const uint64_t blo = smem_desc(xs + UM_SLOT / 2 + (uint32_t)(2 * ks) * 128, 128, x_sbo);
          umma_bf16(d, ahi, bhi, idesc, (kc > 0 || ks > 0) ? 1u : 0u);
          umma_bf16(d, ahi, blo, idesc, 1u);
          umma_bf16(d, alo, bhi, idesc, 1u);
        }
        umma_commit(&empty[slot]);
        issued = true;
      }
      if (!ok) break;
      umma_commit(&tfull[b]);
    }
    // drain: whatever was issued completes before TMEM is released
    umma_commit(dbar);
    (void)mbar_wait(dbar, d_phase & 1);
  }
  __syncwarp();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 256;" ::"r"(tmem));
}

static size_t umma_smem(int kp) {
  return 1024 + umma_tile_bytes(kp) + UM_NS * UM_SLOT + UM_NR * UM_RAW + 256;
}

size_t umma_split_bytes(int m, int k) {
  if (k > UM_MAXK) return 0;
  int kp = umma_kpad(k);
  long ntile = (m + UM_BM - 1) / UM_BM;
  return (size_t)(ntile * umma_tile_bytes(kp));
}

template <typename TA>
int umma_split_a(const TA *A, int m, int k, void *out, size_t bytes, cudaStream_t s) {
  CCL_REQUIRE(k > 0 && k <= UM_MAXK && m > 0, CCL_ERR_UNSUPPORTED,
              "umma split: m=%d k=%d (k <= %d)", m, k, UM_MAXK);
  CCL_REQUIRE(bytes >= umma_split_bytes(m, k), CCL_ERR_WORKSPACE,
              "umma split: %zu < %zu bytes", bytes, umma_split_bytes(m, k));
  CCL_REQUIRE(((uintptr_t)out & 15) == 0, CCL_ERR_ARG, "umma split: output not 16-B aligned");
  int kp = umma_kpad(k);
  int ntile = (m + UM_BM - 1) / UM_BM;
  long total = (long)ntile * 2 * UM_BM * kp / 8;
  k_umma_split_a<TA><<<grid_for(total, 256), 256, 0, s>>>(A, m, k, kp, ntile, (uint4 *)out);
  CCL_LAUNCH_CHECK("umma_split_a");
  return CCL_OK;
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// against the driver library); looked up once
static PFN_cuTensorMapEncodeTiled_v12000 encode_tiled() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
  });
  return fn;
}

static int device_sm_count() {
  int dev = 0, n = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return kNumSM;
  if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0)
    return kNumSM;
  return n;
}

int umma_gemm_batch(int batch, int m, int k, const int *ncols, int cplx, const void *const *Ap,
                    const void *const *X, const long *ldx, void *const *Y, const long *ldy,
                    double are, double aim, double beta, cudaStream_t s) {
  CCL_REQUIRE(batch >= 0 && batch <= UM_MAXBATCH, CCL_ERR_ARG, "umma: batch %d", batch);
  CCL_REQUIRE(m > 0 && k > 0 && k <= UM_MAXK, CCL_ERR_UNSUPPORTED,
              "umma: m=%d k=%d (k <= %d)", m, k, UM_MAXK);
  CCL_REQUIRE(beta == 0.0 || beta == 1.0, CCL_ERR_ARG, "umma: beta must be 0 or 1");
  if (batch == 0) return CCL_OK;
  static UmmaArgs args;  // host staging of the kernel parameters
  static std::mutex args_mu;
  std::lock_guard<std::mutex> lock(args_mu);
  UmmaWork &w = args.w;
  auto encode = encode_tiled();
  CCL_REQUIRE(encode, CCL_ERR_CUDA, "umma: cuTensorMapEncodeTiled unavailable");
  const int mtiles = (m + UM_BM - 1) / UM_BM;
  int vec_y = 1;
  long items = 0;
  for (int i = 0; i < batch; i++) {
    CCL_REQUIRE(Ap[i] && X[i] && Y[i], CCL_ERR_ARG, "umma: null operand %d", i);
    CCL_REQUIRE(ncols[i] > 0 && (!cplx || ncols[i] % 2 == 0), CCL_ERR_ARG,
                "umma: entry %d ncols %d", i, ncols[i]);
    CCL_REQUIRE(ldx[i] >= ncols[i] && ldy[i] >= ncols[i], CCL_ERR_ARG,
                "umma: entry %d ldx %ld / ldy %ld < ncols %d", i, ldx[i], ldy[i], ncols[i]);
    // X is read by tensor copies: 16-B aligned base and row pitch
    CCL_REQUIRE(((uintptr_t)X[i] & 15) == 0 && ldx[i] % 4 == 0, CCL_ERR_ARG,
                "umma: entry %d X not 16-B aligned (ldx %ld)", i, ldx[i]);
    {
      const cuuint64_t dims[2] = {(cuuint64_t)ncols[i], (cuuint64_t)k};
      const cuuint64_t pitch[1] = {(cuuint64_t)ldx[i] * 4};
      const cuuint32_t box[2] = {(cuuint32_t)UM_TN, (cuuint32_t)UM_KC};
      const cuuint32_t estr[2] = {1, 1};
      CUresult r = encode(&args.tx[i], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, (void *)X[i], dims,
                          pitch, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                          CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
      CCL_REQUIRE(r == CUDA_SUCCESS, CCL_ERR_CUDA, "umma: tensor map of entry %d (error %d)", i,
                  (int)r);
    }
    CCL_REQUIRE(((uintptr_t)Ap[i] & 15) == 0, CCL_ERR_ARG, "umma: entry %d A not aligned", i);
    if (((uintptr_t)Y[i] & 15) != 0 || ldy[i] % 4 != 0) vec_y = 0;
    w.A[i] = Ap[i];
    w.Y[i] = (float *)Y[i];
    w.ncols[i] = ncols[i];
    w.ntn[i] = (ncols[i] + UM_TN - 1) / UM_TN;
    w.base[i] = (int)items;
    w.ldy[i] = ldy[i];
    items += (long)mtiles * w.ntn[i];
  }
  CCL_REQUIRE(items < (1L << 30), CCL_ERR_ARG, "umma: %ld work items", items);
  w.batch = batch;
  w.items = (int)items;
  w.mtiles = mtiles;
  const int kp = umma_kpad(k);
  const size_t smem = umma_smem(kp);
  static int sms = 0;
  if (!sms) sms = device_sm_count();
  const int grid = (int)(items < sms ? items : sms);
  const float ar = (float)are, ai = (float)aim;
#define CCL_UMMA(C, A_)                                                              \
  {                                                                                  \
    auto kern = k_umma_gemm<C, A_>;                                                  \
    static size_t set_smem = 0; /* the attribute is set once per size, not per launch */ \
    if (set_smem < smem) {                                                           \
      cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem); \
      set_smem = smem;                                                               \
    }                                                                                \
    kern<<<grid, UM_THREADS2, smem, s>>>(args, m, k, kp, vec_y, ar, ai);                \
  }
  if (cplx) {
    if (beta == 1.0) CCL_UMMA(true, true) else CCL_UMMA(true, false)
  } else {
    if (beta == 1.0) CCL_UMMA(false, true) else CCL_UMMA(false, false)
  }
#undef CCL_UMMA
  CCL_LAUNCH_CHECK("umma_gemm");
  return CCL_OK;
}

int umma_status(int reset) {
  int v = 0;
  cudaMemcpyFromSymbol(&v, g_umma_error, sizeof(int));
  if (reset) {
    int z = 0;
    cudaMemcpyToSymbol(g_umma_error, &z, sizeof(int));
  }
  return v;
}

template int umma_split_a<float>(const float *, int, int, void *, size_t, cudaStream_t);
template int umma_split_a<double>(const double *, int, int, void *, size_t, cudaStream_t);

}  // namespace ccl
