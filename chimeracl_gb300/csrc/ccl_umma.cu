// The discrete Hankel transform as a BF16x3 split-precision GEMM on the
// 5th-generation tensor cores (tcgen05.mma, FP32 accumulation in TMEM):
//   Y = beta*Y + alpha * (A X),  A ~ A_hi + A_lo,  X ~ X_hi + X_lo  (bf16),
//   A X ~ A_hi X_hi + A_hi X_lo + A_lo X_hi,
// A real (m x k, m, k <= 512), X FP32 (k x ncols real columns, interleaved
// complex allowed), Y FP32.  One MMA covers at most 256 rows of A (its N):
// for m > 256 the rows are taken in two halves of 256, each a work item of
// its own over the same X tile.
//
// A is split once into bf16 hi/lo (k_umma_split_a); X is split on the fly.
// Every mbarrier wait is bounded; a wait that gives up records an error code
// in a device flag, the CTA skips the rest of its work, drains what it issued
// (bounded) and frees its TMEM.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>
#include <stdint.h>

#include <mutex>

#include "ccl_common.cuh"
#include "ccl_launch.h"

namespace ccl {

constexpr int UM_MAXK = 512, UM_MAXBATCH = 32;
constexpr long UM_SPIN_LIMIT = 20000000L;  // ~ a second of try_wait polls

__device__ int g_umma_error = 0;


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
// The matrix A (m x k, row-major, lda = k, m <= 512) is stored for the MMA's
// B operand, in row halves of NP rows (one half when m <= 256), each
// streamed per 32-deep K chunk: chunk c of half h (at (h*nchunk + c) chunk
// sizes) holds a hi block then a lo block of NP x 32 bf16 (NP = 128 or 256
// padded rows), K-major no-swizzle core matrices, core matrix (g = row/8,
// j = (col%32)/8) at (g*4 + j)*128 bytes, each 8 rows x 8 consecutive k
// values.  Zero outside m x k.
constexpr int UM_KC = 32;  // K depth of one stage
__host__ __device__ constexpr int umma_np(int m) { return m <= 128 ? 128 : 256; }
__host__ __device__ constexpr int umma_halves(int m) { return m <= 256 ? 1 : 2; }
__host__ __device__ constexpr uint32_t umma_chunk_bytes(int np) { return 2u * np * UM_KC * 2; }

template <typename TA>
__global__ void k_umma_split_a(const TA *__restrict__ A, int m, int k, int np, int nchunk,
                               int nh, uint4 *__restrict__ out) {
  const long per_block = (long)np * (UM_KC / 8);  // 16-B rows of one hi or lo block
  const long per_half = (long)nchunk * 2 * per_block;
  const long total = nh * per_half;
  for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < total;
       q += (long)gridDim.x * blockDim.x) {
    const long h = q / per_half, qh = q - h * per_half;
    const long c = qh / (2 * per_block), rem = qh - c * 2 * per_block;
    const int lo = rem >= per_block;
    const long w = rem - lo * per_block;
    const long cm = w / 8, i8 = w - cm * 8;
    const long g = cm / (UM_KC / 8), j = cm - g * (UM_KC / 8);
    const long row = h * np + g * 8 + i8;
    __nv_bfloat16 e[8];
#pragma unroll
    for (int t = 0; t < 8; t++) {
      const long col = c * UM_KC + j * 8 + t;
      const float v = (row < m && col < k) ? (float)A[row * k + col] : 0.f;
      const __nv_bfloat16 h = __float2bfloat16_rn(v);
      e[t] = lo ? __float2bfloat16_rn(v - __bfloat162float(h)) : h;
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
// Persistent, warp-specialised kernel computing the transpose on the tensor
// cores, Y^T = X^T A^T: the MMA's M = 128 columns of X (one work item = one
// 128-column tile of one batch entry and one row half of A), its N = NP rows
// of A, K = 16 per instruction.  Each X tile is therefore read and converted
// once for all output rows of a half (m <= 256: for all of them); A streams
// per K chunk from L2 (it is shared by every CTA).
//   warps 0-7  epilogue: TMEM lane = X column n, TMEM column = output row i;
//              warps w and w + 4 share lanes 32(w % 4) .. + 31 (the lanes a
//              warp may read) and take the first and the second half of the
//              rows; alpha (complex pairs are adjacent columns n, n+1: one
//              shuffle), optional +Y, stores of 32 consecutive columns of one
//              row per instruction (128 contiguous bytes)
//   warps 8-15 converters: raw FP32 stage (32 k x 128 n) -> K-major bf16
//              hi/lo core matrices in a ring of UM_NS slots
//   warp 16    lane 0: producer -- per stage one 2-D tensor copy of X into a
//              ring of UM_NR raw slots (out-of-range rows/columns read as 0)
//              and one bulk copy of A's K chunk into a ring of UM_NA slots
//   warp 17    lane 0: the MMAs (X_hi A_hi, X_lo A_hi, X_hi A_lo per 16-deep k
//              step) into double-buffered 128 x NP FP32 accumulators in TMEM
// Every wait is bounded (and gives up early once another role has aborted);
// the MMA thread drains its MMAs and the producer its copies before the CTA
// releases TMEM and exits.
constexpr int UM_EPI_WARPS = 8, UM_CVT_WARPS = 8;
constexpr int UM_THREADS2 = (UM_EPI_WARPS + UM_CVT_WARPS + 2) * 32;  // 576
constexpr int UM_TN = 128;        // X columns per work item (the MMA's M)
constexpr int UM_NS = 3;          // bf16 X slots
constexpr int UM_NR = 4;          // raw FP32 X slots
constexpr int UM_NA = 3;          // A chunk slots
constexpr uint32_t UM_SLOT = 2u * UM_KC * UM_TN * 2;  // hi + lo bf16: 16 KB
constexpr uint32_t UM_RAW = (uint32_t)UM_KC * UM_TN * 4;  // FP32: 16 KB

struct UmmaWork {
  const void *A[UM_MAXBATCH];
  float *Y[UM_MAXBATCH];
  int ncols[UM_MAXBATCH];
  int base[UM_MAXBATCH];   // first item of the entry
  long ldy[UM_MAXBATCH];
  int batch, items;
  int nh;  // row halves of A: items of an entry are (column tile, half), half fastest
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

__device__ __forceinline__ void um_decode(const UmmaWork &w, int item, int &e, int &nt,
                                          int &h) {
  e = 0;
  while (e + 1 < w.batch && w.base[e + 1] <= item) e++;
  const int local = item - w.base[e];  // nh is 1 or 2
  nt = w.nh == 2 ? local >> 1 : local;
  h = local & (w.nh - 1);
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

template <bool CPLX, bool ACC, int NP>
__global__ void __launch_bounds__(UM_THREADS2, 1)
    k_umma_gemm(const __grid_constant__ UmmaArgs args, int M, int K, float are, float aim) {
  constexpr uint32_t ACH = umma_chunk_bytes(NP);  // A chunk: hi + lo
  constexpr uint32_t TCOLS = 2 * NP;               // TMEM columns (two accumulators)
  extern __shared__ __align__(1024) unsigned char smraw[];
  const UmmaWork &w = args.w;
  unsigned char *sm = (unsigned char *)(((uintptr_t)smraw + 1023) & ~(uintptr_t)1023);
  unsigned char *sA = sm;                     // UM_NA A chunks
  unsigned char *sX = sA + UM_NA * ACH;       // UM_NS bf16 X slots
  unsigned char *sR = sX + UM_NS * UM_SLOT;   // UM_NR raw X slots
  uint64_t *full = (uint64_t *)(sR + UM_NR * UM_RAW);
  uint64_t *empty = full + UM_NS;
  uint64_t *rfull = empty + UM_NS;
  uint64_t *rempty = rfull + UM_NR;
  uint64_t *afull = rempty + UM_NR;
  uint64_t *aempty = afull + UM_NA;
  uint64_t *tfull = aempty + UM_NA;  // [2]
  uint64_t *tempty = tfull + 2;      // [2]
  uint64_t *dbar = tempty + 2;
  uint32_t *tmem_slot = (uint32_t *)(dbar + 1);
  volatile int *abort = (volatile int *)(tmem_slot + 1);

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int nkc = (K + UM_KC - 1) / UM_KC;
  const int i0 = (int)((long)blockIdx.x * w.items / gridDim.x);
  const int i1 = (int)((long)(blockIdx.x + 1) * w.items / gridDim.x);
  const int S = (i1 - i0) * nkc;  // stages of this CTA

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"(TCOLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    for (int i = 0; i < UM_NS; i++) {
      mbar_init(&full[i], UM_CVT_WARPS);  // one arrival per converter warp
      mbar_init(&empty[i], 1);
    }
    for (int i = 0; i < UM_NR; i++) {
      mbar_init(&rfull[i], 1);
      mbar_init(&rempty[i], UM_CVT_WARPS);
    }
    for (int i = 0; i < UM_NA; i++) {
      mbar_init(&afull[i], 1);
      mbar_init(&aempty[i], 1);
    }
    for (int i = 0; i < 2; i++) {
      mbar_init(&tfull[i], 1);
      mbar_init(&tempty[i], UM_EPI_WARPS * 32);
    }
    mbar_init(dbar, 1);
    *abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  // the set-up above touches only this CTA's shared and tensor memory: the
  // operands written by earlier kernels are read after this point
  pdl_wait();

  if (warp < UM_EPI_WARPS) {
    // ------------------------------------------------------------ epilogue
    // tcgen05.ld is warp-collective: every exit decision is taken warp-wide
    for (int j = 0, item = i0; item < i1; j++, item++) {
      if (__any_sync(0xffffffffu, *abort)) break;
      int e, nt, h;
      um_decode(w, item, e, nt, h);
      const int b = j & 1;
      const bool got = mbar_wait_ab(&tfull[b], (j >> 1) & 1, abort);
      if (!__all_sync(0xffffffffu, got)) {
        um_fail(abort, 2);
        break;
      }
      tc_fence_after();
      const int N = w.ncols[e];
      const int quarter = warp & 3, part = warp >> 2;  // TMEM lanes, row part
      const int n = nt * UM_TN + quarter * 32 + lane;  // this lane's column of X and Y
      const bool nin = n < N;
      const long ldy = w.ldy[e];
      float *__restrict__ ycol = w.Y[e] + n;
      if (h) ycol += (long)NP * ldy;  // first row of the half
      const uint32_t tb = tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(b * NP);
      const int mrow = M - h * NP < NP ? M - h * NP : NP;  // rows of this half
      const int r0 = part * (NP / 2);                     // this warp's rows r0 ..
      const int r1 = mrow < r0 + NP / 2 ? mrow : r0 + NP / 2;
      float *yp = ycol + (long)r0 * ldy;  // row i of this lane's column
#pragma unroll 1
      for (int i0c = r0; i0c < r1; i0c += 32) {
        float v[32];
        tmem_ld16(tb + i0c, v);  // two loads in flight per wait
        tmem_ld16(tb + i0c + 16, v + 16);
        tmem_wait_ld();
#pragma unroll
        for (int t = 0; t < 32; t++) {
          float r;
          if (CPLX) {  // (re, im) = columns (n even, n odd): partner via shuffle
            const float o = __shfl_xor_sync(0xffffffffu, v[t], 1);
            r = (lane & 1) ? are * v[t] + aim * o : are * v[t] - aim * o;
          } else {
            r = are * v[t];
          }
          if (nin && i0c + t < r1) {
            if (ACC) r += *yp;
            *yp = r;
          }
          yp += ldy;
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
    // exit decisions are taken warp-wide (the loop holds a __syncwarp)
    for (int s = 0; s < S; s++) {
      if (__any_sync(0xffffffffu, *abort)) break;
      const int r = s % UM_NR, slot = s % UM_NS;
      if (!__all_sync(0xffffffffu, mbar_wait_ab(&rfull[r], (s / UM_NR) & 1, abort))) {
        um_fail(abort, 7);
        break;
      }
      uint4 o[4];
      cvt_stage((const float *)(sR + r * UM_RAW), kb, ncol_local, o);
      if (s >= UM_NS &&
          !__all_sync(0xffffffffu, mbar_wait_ab(&empty[slot], ((s / UM_NS) - 1) & 1, abort))) {
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
      // bf16 stores before the MMAs that read them.  The warp then arrives
      // once (256 arrivals on one barrier serialise): __syncwarp orders the
      // lanes' accesses before lane 0's release.
      fence_async_smem();
      __syncwarp();
      if (lane == 0) {
        mbar_arrive(&rempty[r]);
        mbar_arrive(&full[slot]);
      }
    }
  } else if (warp == UM_EPI_WARPS + UM_CVT_WARPS) {
    // --------------------------------------------------- producer (one lane)
    if (lane == 0) {
      int issued_x = 0, issued_a = 0;
      for (int s = 0; s < S; s++) {
        if (*abort) break;
        const int r = s % UM_NR, a = s % UM_NA;
        if (s >= UM_NR && !mbar_wait_ab(&rempty[r], ((s / UM_NR) - 1) & 1, abort)) {
          um_fail(abort, 8);
          break;
        }
        int e, nt, h;
        um_decode(w, i0 + s / nkc, e, nt, h);
        const int kc = s % nkc;
        mbar_expect_tx(&rfull[r], UM_RAW);
        tma_load_2d(sR + r * UM_RAW, &args.tx[e], nt * UM_TN, kc * UM_KC, &rfull[r]);
        issued_x = s + 1;
        if (s >= UM_NA && !mbar_wait_ab(&aempty[a], ((s / UM_NA) - 1) & 1, abort)) {
          um_fail(abort, 9);
          break;
        }
        mbar_expect_tx(&afull[a], ACH);
        bulk_g2s(sA + a * ACH, (const unsigned char *)w.A[e] + ((long)h * nkc + kc) * ACH, ACH,
                 &afull[a]);
        issued_a = s + 1;
      }
      // every copy this lane issued has landed before the CTA may exit
      for (int s = issued_x - UM_NR < 0 ? 0 : issued_x - UM_NR; s < issued_x; s++)
        (void)mbar_wait(&rfull[s % UM_NR], (s / UM_NR) & 1);
      for (int s = issued_a - UM_NA < 0 ? 0 : issued_a - UM_NA; s < issued_a; s++)
        (void)mbar_wait(&afull[s % UM_NA], (s / UM_NA) & 1);
    }
  } else if (lane == 0) {
    // ------------------------------------------------------ MMA (one lane)
    const uint32_t idesc = umma_idesc(UM_TN, NP);
    const uint32_t sA_u = smem_u32(sA), sX_u = smem_u32(sX);
    const uint32_t sbo = (UM_KC / 8) * 128;  // 8-row groups, both operands
    int s = 0;
    for (int j = 0, item = i0; item < i1; j++, item++) {
      if (*abort) break;
      const int b = j & 1;
      if (j >= 2 && !mbar_wait_ab(&tempty[b], ((j - 2) >> 1) & 1, abort)) {
        um_fail(abort, 5);
        break;
      }
      tc_fence_after();
      const uint32_t d = tmem + (uint32_t)(b * NP);
      bool ok = true;
      for (int kc = 0; kc < nkc; kc++, s++) {
        const int slot = s % UM_NS, a = s % UM_NA;
        if (!mbar_wait_ab(&full[slot], (s / UM_NS) & 1, abort) ||
            !mbar_wait_ab(&afull[a], (s / UM_NA) & 1, abort)) {
          um_fail(abort, 6);
          ok = false;
          break;
        }
        tc_fence_after();
        const uint32_t xs = sX_u + slot * UM_SLOT, as = sA_u + a * ACH;
#pragma unroll
        for (int ks = 0; ks < UM_KC / 16; ks++) {
          const uint32_t o = (uint32_t)(2 * ks) * 128;
          const uint64_t xhi = smem_desc(xs + o, 128, sbo);
          const uint64_t xlo = smem_desc(xs + UM_SLOT / 2 + o, 128, sbo);
          const uint64_t ahi = smem_desc(as + o, 128, sbo);
          const uint64_t alo = smem_desc(as + ACH / 2 + o, 128, sbo);
          umma_bf16(d, xhi, ahi, idesc, (kc > 0 || ks > 0) ? 1u : 0u);
          umma_bf16(d, xlo, ahi, idesc, 1u);
          umma_bf16(d, xhi, alo, idesc, 1u);
        }
        umma_commit(&empty[slot]);
        umma_commit(&aempty[a]);
      }
      if (!ok) break;
      umma_commit(&tfull[b]);
    }
    // drain: whatever was issued completes before TMEM is released
    umma_commit(dbar);
    (void)mbar_wait(dbar, 0);
  }
  __syncwarp();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TCOLS));
}

static size_t umma_smem(int np) {
  return 1024 + UM_NA * umma_chunk_bytes(np) + UM_NS * UM_SLOT + UM_NR * UM_RAW + 256;
}

size_t umma_split_bytes(int m, int k) {
  if (k > UM_MAXK || m > UM_MAXK || m <= 0 || k <= 0) return 0;
  const int nchunk = (k + UM_KC - 1) / UM_KC;
  return (size_t)umma_halves(m) * nchunk * umma_chunk_bytes(umma_np(m));
}

template <typename TA>
int umma_split_a(const TA *A, int m, int k, void *out, size_t bytes, cudaStream_t s) {
  CCL_REQUIRE(k > 0 && k <= UM_MAXK && m > 0 && m <= UM_MAXK, CCL_ERR_UNSUPPORTED,
              "umma split: m=%d k=%d (m, k <= %d)", m, k, UM_MAXK);
  CCL_REQUIRE(bytes >= umma_split_bytes(m, k), CCL_ERR_WORKSPACE,
              "umma split: %zu < %zu bytes", bytes, umma_split_bytes(m, k));
  CCL_REQUIRE(((uintptr_t)out & 15) == 0, CCL_ERR_ARG, "umma split: output not 16-B aligned");
  const int np = umma_np(m), nchunk = (k + UM_KC - 1) / UM_KC, nh = umma_halves(m);
  const long total = (long)nh * nchunk * 2 * np * (UM_KC / 8);
  k_umma_split_a<TA><<<grid_for(total, 256), 256, 0, s>>>(A, m, k, np, nchunk, nh,
                                                          (uint4 *)out);
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

template <bool C, bool A_, int NP>
static void umma_launch(int grid, size_t smem, const UmmaArgs &args, int m, int k, float ar,
                        float ai, cudaStream_t s) {
  auto kern = k_umma_gemm<C, A_, NP>;
  static size_t set_smem = 0;  // the attribute is set once per size, not per launch
  if (set_smem < smem) {
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    set_smem = smem;
  }
  launch_pdl(kern, grid, UM_THREADS2, smem, s, args, m, k, ar, ai);
}

int umma_gemm_batch(int batch, int m, int k, const int *ncols, int cplx, const void *const *Ap,
                    const void *const *X, const long *ldx, void *const *Y, const long *ldy,
                    double are, double aim, double beta, cudaStream_t s) {
  CCL_REQUIRE(batch >= 0 && batch <= UM_MAXBATCH, CCL_ERR_ARG, "umma: batch %d", batch);
  CCL_REQUIRE(m > 0 && k > 0 && k <= UM_MAXK && m <= UM_MAXK, CCL_ERR_UNSUPPORTED,
              "umma: m=%d k=%d (m, k <= %d)", m, k, UM_MAXK);
  CCL_REQUIRE(beta == 0.0 || beta == 1.0, CCL_ERR_ARG, "umma: beta must be 0 or 1");
  if (batch == 0) return CCL_OK;
  static UmmaArgs args;  // host staging of the kernel parameters
  static std::mutex args_mu;
  std::lock_guard<std::mutex> lock(args_mu);
  UmmaWork &w = args.w;
  auto encode = encode_tiled();
  CCL_REQUIRE(encode, CCL_ERR_CUDA, "umma: cuTensorMapEncodeTiled unavailable");
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
    w.A[i] = Ap[i];
    w.Y[i] = (float *)Y[i];
    w.ncols[i] = ncols[i];
    w.base[i] = (int)items;
    w.ldy[i] = ldy[i];
    items += (long)umma_halves(m) * ((ncols[i] + UM_TN - 1) / UM_TN);
  }
  CCL_REQUIRE(items < (1L << 30), CCL_ERR_ARG, "umma: %ld work items", items);
  w.batch = batch;
  w.items = (int)items;
  w.nh = umma_halves(m);
  static int sms = 0;
  if (!sms) sms = device_sm_count();
  const int grid = (int)(items < sms ? items : sms);
  const float ar = (float)are, ai = (float)aim;
  const bool acc = beta == 1.0;
  if (umma_np(m) == 128) {
    const size_t smem = umma_smem(128);
    if (cplx) {
      if (acc) umma_launch<true, true, 128>(grid, smem, args, m, k, ar, ai, s);
      else umma_launch<true, false, 128>(grid, smem, args, m, k, ar, ai, s);
    } else {
      if (acc) umma_launch<false, true, 128>(grid, smem, args, m, k, ar, ai, s);
      else umma_launch<false, false, 128>(grid, smem, args, m, k, ar, ai, s);
    }
  } else {
    const size_t smem = umma_smem(256);
    if (cplx) {
      if (acc) umma_launch<true, true, 256>(grid, smem, args, m, k, ar, ai, s);
      else umma_launch<true, false, 256>(grid, smem, args, m, k, ar, ai, s);
    } else {
      if (acc) umma_launch<false, true, 256>(grid, smem, args, m, k, ar, ai, s);
      else umma_launch<false, false, 256>(grid, smem, args, m, k, ar, ai, s);
    }
  }
  CCL_LAUNCH_CHECK("umma_gemm");
  return CCL_OK;
}

// ------------------------------------------------------------------ wait probe
// The bounded wait of the kernels above, made to run out on purpose: one
// thread initialises an mbarrier that expects one arrival and (unless
// `arrive`) nothing arrives; it polls phase 0 at most `spins` times and
// writes 1 to *gave_up when the wait ran out, 0 when the phase completed.
// It touches only its own shared memory and *gave_up, and ends after at
// most `spins` polls.
__global__ void k_wait_probe(long spins, int arrive, int *gave_up) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x != 0) return;
  mbar_init(&bar, 1);
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  if (arrive) mbar_arrive(&bar);
  bool done = false;
  for (long i = 0; i < spins && !done; i++) done = mbar_try_wait(&bar, 0);
  *gave_up = done ? 0 : 1;
}

int umma_wait_probe(long spins, int arrive, int *gave_up, cudaStream_t s) {
  CCL_REQUIRE(spins >= 1 && spins <= UM_SPIN_LIMIT, CCL_ERR_ARG,
              "wait probe: spins=%ld outside [1, %ld]", spins, UM_SPIN_LIMIT);
  k_wait_probe<<<1, 32, 0, s>>>(spins, arrive, gave_up);
  CCL_LAUNCH_CHECK("wait_probe");
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
