// The discrete Hankel transform as a BF16x3 split-precision GEMM on the
// 5th-generation tensor cores (tcgen05.mma, FP32 accumulation in TMEM):
//   Y = beta*Y + alpha * (A X),  A ~ A_hi + A_lo,  X ~ X_hi + X_lo  (bf16),
//   A X ~ A_hi X_hi + A_hi X_lo + A_lo X_hi,
// A real (m x k, k <= 256), X FP32 (k x ncols real columns, interleaved
// complex allowed), Y FP32.
//
// CTA = 128 threads (one warpgroup), one 128-row M tile of one batch entry
// and a run of 64-column N tiles.  The pre-split A tile (hi then lo, K-major,
// no-swizzle core-matrix layout, produced by k_umma_split_a) is copied once
// into shared memory and stays resident.  X is staged per 128-deep K chunk:
// each thread loads one 8 (k) x 8 (n) block of FP32, splits it and writes
// one K-major 8x8 bf16 core matrix for X_hi and one for X_lo.  Two X
// buffers and two TMEM accumulators (128 lanes x 64 columns each) let thread
// 0 issue the next chunk's MMAs while the others stage and drain.  Every
// mbarrier wait is bounded; a wait that gives up records an error code in a
// device flag, the CTA skips the rest of its work, drains what it issued
// (bounded) and frees its TMEM.
#include <cuda_bf16.h>
#include <stdint.h>

#include "ccl_common.cuh"
#include "ccl_launch.h"

namespace ccl {

constexpr int UM_THREADS = 128, UM_BM = 128, UM_BN = 64, UM_BK = 128;
constexpr int UM_MAXK = 256, UM_MAXBATCH = 32;
constexpr int UM_MAX_TILES_PER_CTA = 4;
constexpr long UM_SPIN_LIMIT = 20000000L;  // ~ a second of try_wait polls

__device__ int g_umma_error = 0;

struct UmmaBatch {
  const void *A[UM_MAXBATCH];  // pre-split A tiles
  const float *X[UM_MAXBATCH];
  float *Y[UM_MAXBATCH];
  int ncols[UM_MAXBATCH];
  long ldx[UM_MAXBATCH], ldy[UM_MAXBATCH];
};

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
template <bool CPLX, bool ACC>
__global__ void __launch_bounds__(UM_THREADS, 1)
    k_umma_gemm(UmmaBatch b, int M, int K, int KP, int tiles_per_cta, float are, float aim) {
  extern __shared__ __align__(1024) unsigned char smraw[];
  unsigned char *sm = (unsigned char *)(((uintptr_t)smraw + 1023) & ~(uintptr_t)1023);
  unsigned char *sA = sm;                                   // umma_tile_bytes(KP)
  unsigned char *sX = sA + umma_tile_bytes(KP);             // 2 stages x 32 KB
  uint64_t *bar = (uint64_t *)(sX + 2 * 2 * UM_BK * UM_BN * 2);  // [2]
  uint32_t *tmem_slot = (uint32_t *)(bar + 2);
  int *abort_flag = (int *)(tmem_slot + 1);
  int *last_issued = abort_flag + 1;  // last stage whose MMAs were committed

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int e = blockIdx.z, mt = blockIdx.y;
  const int N = b.ncols[e];
  const int n_begin = blockIdx.x * tiles_per_cta * UM_BN;
  if (n_begin >= N) return;
  const int ntiles = min(tiles_per_cta, (N - n_begin + UM_BN - 1) / UM_BN);
  const int nkc = KP / UM_BK;
  const float *__restrict__ X = b.X[e];
  float *__restrict__ Y = b.Y[e];
  const long ldx = b.ldx[e], ldy = b.ldy[e];

  // TMEM: 2 accumulators of 64 columns
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 128;" ::"r"(
        smem_u32(tmem_slot)));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    *abort_flag = 0;
    *last_issued = -1;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  // resident A tile
  {
    const uint4 *src = (const uint4 *)((const unsigned char *)b.A[e] + mt * umma_tile_bytes(KP));
    uint4 *dst = (uint4 *)sA;
    const int n16 = (int)(umma_tile_bytes(KP) / 16);
    for (int i = tid; i < n16; i += UM_THREADS) dst[i] = src[i];
  }
  fence_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  const uint32_t idesc = umma_idesc(UM_BM, UM_BN);
  const uint32_t sA_u = smem_u32(sA), sX_u = smem_u32(sX);
  const uint32_t a_lo_off = (uint32_t)(umma_tile_bytes(KP) / 2);
  const uint32_t a_sbo = (uint32_t)(KP / 8) * 128;
  const uint32_t x_stage = 2 * UM_BK * UM_BN * 2, x_lo_off = UM_BK * UM_BN * 2;
  const uint32_t x_sbo = (UM_BK / 8) * 128;
  bool ok = true;

  // thread's 8x8 staging block within a 128 (k) x 64 (n) chunk
  const int nb = tid & 7, kb = tid >> 3;

  auto epilogue = [&](int t) {
    const int st_last = t * nkc + nkc - 1;
    bool got = mbar_wait(&bar[st_last & 1], (st_last >> 1) & 1);
    if (!got) {
      atomicExch(&g_umma_error, 2);
      *abort_flag = 1;
    }
    tc_fence_after();
    const int gm = mt * UM_BM + warp * 32 + lane;
    const int n0 = n_begin + t * UM_BN;
    const uint32_t tbase = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)((t & 1) * UM_BN);
#pragma unroll
    for (int q = 0; q < UM_BN / 16; q++) {
      float v[16];
      tmem_ld16(tbase + q * 16, v);
      tmem_wait_ld();
      if (got && gm < M) {
        float *yrow = Y + (long)gm * ldy;
#pragma unroll
        for (int c = 0; c < 16; c += 2) {
          const int gn = n0 + q * 16 + c;
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
    tc_fence_before();
  };

  const int S = ntiles * nkc;
  for (int st = 0; st < S; st++) {
    const int buf = st & 1, t = st / nkc, kc = st - t * nkc;
    if (st >= 2 && tid == 0) {
      if (!mbar_wait(&bar[buf], ((st - 2) >> 1) & 1)) {
        atomicExch(&g_umma_error, 1);
        *abort_flag = 1;
      }
    }
    __syncthreads();
    if (*abort_flag) { ok = false; break; }
    // stage X chunk: rows kc*128 + kb*8 + r, columns n_begin + t*64 + nb*8 + c
    {
      float v[8][8];
      const int n = n_begin + t * UM_BN + nb * 8;
#pragma unroll
      for (int r = 0; r < 8; r++) {
        const int kk = kc * UM_BK + kb * 8 + r;
        const float *row = X + (long)kk * ldx + n;
        if (kk < K && n + 8 <= N) {
          float4 p = *(const float4 *)row, q = *(const float4 *)(row + 4);
          v[r][0] = p.x; v[r][1] = p.y; v[r][2] = p.z; v[r][3] = p.w;
          v[r][4] = q.x; v[r][5] = q.y; v[r][6] = q.z; v[r][7] = q.w;
        } else {
#pragma unroll
          for (int c = 0; c < 8; c++) v[r][c] = (kk < K && n + c < N) ? row[c] : 0.f;
        }
      }
      unsigned char *dst_hi = sX + buf * x_stage + (nb * (UM_BK / 8) + kb) * 128;
      unsigned char *dst_lo = dst_hi + x_lo_off;
#pragma unroll
      for (int c = 0; c < 8; c++) {  // core-matrix row = column n of the block
        __nv_bfloat16 h[8], l[8];
#pragma unroll
        for (int r = 0; r < 8; r++) {
          h[r] = __float2bfloat16_rn(v[r][c]);
          l[r] = __float2bfloat16_rn(v[r][c] - __bfloat162float(h[r]));
        }
        uint4 ph = {pack_bf16(h[0], h[1]), pack_bf16(h[2], h[3]), pack_bf16(h[4], h[5]),
                    pack_bf16(h[6], h[7])};
        uint4 pl = {pack_bf16(l[0], l[1]), pack_bf16(l[2], l[3]), pack_bf16(l[4], l[5]),
                    pack_bf16(l[6], l[7])};
        *(uint4 *)(dst_hi + c * 16) = ph;
        *(uint4 *)(dst_lo + c * 16) = pl;
      }
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    if (tid == 0) {
      tc_fence_after();
      const uint32_t d = tmem + (uint32_t)((t & 1) * UM_BN);
      const uint32_t xs = sX_u + buf * x_stage;
#pragma unroll
      for (int ks = 0; ks < UM_BK / 16; ks++) {
        const uint32_t ja = (uint32_t)(kc * (UM_BK / 8) + 2 * ks) * 128;
        const uint64_t ahi = smem_desc(sA_u + ja, 128, a_sbo);
        const uint64_t alo = smem_desc(sA_u + a_lo_off + ja, 128, a_sbo);
        const uint64_t bhi = smem_desc(xs + (uint32_t)(2 * ks) * 128, 128, x_sbo);
        const uint64_t blo = smem_desc(xs + x_lo_off + (uint32_t)(2 * ks) * 128, 128, x_sbo);
        umma_bf16(d, ahi, bhi, idesc, (kc > 0 || ks > 0) ? 1u : 0u);
        umma_bf16(d, ahi, blo, idesc, 1u);
        umma_bf16(d, alo, bhi, idesc, 1u);
      }
      umma_commit(&bar[buf]);
      *last_issued = st;
    }
    if (kc == 0 && t >= 1) {
      epilogue(t - 1);
      __syncthreads();
    }
  }
  if (ok) {
    epilogue(ntiles - 1);
  } else if (tid == 0) {
    // drain: the MMAs of the last committed stage (bounded) before TMEM is
    // released; the stages before it completed in issue order
    const int li = *last_issued;
    if (li >= 0) (void)mbar_wait(&bar[li & 1], (li >> 1) & 1);
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 128;" ::"r"(tmem));
}

static size_t umma_smem(int kp) {
  return 1024 + umma_tile_bytes(kp) + 2 * 2 * UM_BK * UM_BN * 2 + 64;
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

int umma_gemm_batch(int batch, int m, int k, const int *ncols, int cplx, const void *const *Ap,
                    const void *const *X, const long *ldx, void *const *Y, const long *ldy,
                    double are, double aim, double beta, cudaStream_t s) {
  CCL_REQUIRE(batch >= 0 && batch <= UM_MAXBATCH, CCL_ERR_ARG, "umma: batch %d", batch);
  CCL_REQUIRE(m > 0 && k > 0 && k <= UM_MAXK, CCL_ERR_UNSUPPORTED,
              "umma: m=%d k=%d (k <= %d)", m, k, UM_MAXK);
  CCL_REQUIRE(beta == 0.0 || beta == 1.0, CCL_ERR_ARG, "umma: beta must be 0 or 1");
  if (batch == 0) return CCL_OK;
  UmmaBatch b;
  int nmax = 0;
  for (int i = 0; i < batch; i++) {
    CCL_REQUIRE(Ap[i] && X[i] && Y[i], CCL_ERR_ARG, "umma: null operand %d", i);
    CCL_REQUIRE(ncols[i] > 0 && (!cplx || ncols[i] % 2 == 0), CCL_ERR_ARG,
                "umma: entry %d ncols %d", i, ncols[i]);
    CCL_REQUIRE(ldx[i] >= ncols[i] && ldy[i] >= ncols[i], CCL_ERR_ARG,
                "umma: entry %d ldx %ld / ldy %ld < ncols %d", i, ldx[i], ldy[i], ncols[i]);
    // the staging loads read 8 floats at a time: rows must be 16-B aligned
    CCL_REQUIRE(((uintptr_t)X[i] & 15) == 0 && ldx[i] % 4 == 0, CCL_ERR_ARG,
                "umma: entry %d X not 16-B aligned (ldx %ld)", i, ldx[i]);
    CCL_REQUIRE(((uintptr_t)Ap[i] & 15) == 0, CCL_ERR_ARG, "umma: entry %d A not aligned", i);
    b.A[i] = Ap[i];
    b.X[i] = (const float *)X[i];
    b.Y[i] = (float *)Y[i];
    b.ncols[i] = ncols[i];
    b.ldx[i] = ldx[i];
    b.ldy[i] = ldy[i];
    if (ncols[i] > nmax) nmax = ncols[i];
  }
  const int kp = umma_kpad(k);
  const size_t smem = umma_smem(kp);
  // N tiles per CTA: amortise the resident A tile over up to 4 tiles, but
  // keep at least ~3 CTAs per SM of work in the launch (one CTA is resident
  // per SM at this shared-memory size)
  const int mtiles = (m + UM_BM - 1) / UM_BM;
  long tiles = 0;
  for (int i = 0; i < batch; i++) tiles += (ncols[i] + UM_BN - 1) / UM_BN;
  tiles *= mtiles;
  int tpc = (int)(tiles / (3L * kNumSM));
  tpc = tpc < 1 ? 1 : (tpc > UM_MAX_TILES_PER_CTA ? UM_MAX_TILES_PER_CTA : tpc);
  dim3 grid((nmax + tpc * UM_BN - 1) / (tpc * UM_BN), mtiles, batch);
  const float ar = (float)are, ai = (float)aim;
#define CCL_UMMA(C, A_)                                                              \
  {                                                                                  \
    auto kern = k_umma_gemm<C, A_>;                                                  \
    static size_t set_smem = 0; /* the attribute is set once per size, not per launch */ \
    if (set_smem < smem) {                                                           \
      cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem); \
      set_smem = smem;                                                               \
    }                                                                                \
    kern<<<grid, UM_THREADS, smem, s>>>(b, m, k, kp, tpc, ar, ai);                   \
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
