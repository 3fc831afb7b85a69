/*
 * cgfd_sg_gemm.cu -- BF16 matrix products on the 5th-generation tensor cores
 * (tcgen05, sm_103a) for the learned seismogram surrogate (cgfd_sg.cu).
 *
 *   C[M, N] = alpha * A[M, K] . B[N, K]^T   (+ bias[N], optional GELU)
 *
 * A and B are bf16, row-major with K contiguous ("K-major" for both
 * operands); the product accumulates in FP32 in tensor memory (TMEM).
 * Products with at least two 32768-output tiles (128 x 256 or 256 x 128)
 * per SM (and no split along K) run in the persistent form k_gemm_tn_p
 * further down; the others
 * in k_gemm_tn, where one CTA computes one 128 x 128 tile of C (or, split
 * along K, its share of one), with four warps:
 *
 *   warp 0, lane 0   producer: bulk tensor copies (cp.async.bulk.tensor,
 *                    128-byte swizzle) of the A and B tiles of each 64-wide
 *                    K block into a 3-stage shared-memory ring (97 KiB, so
 *                    two CTAs share an SM and one's epilogue overlaps the
 *                    other's main loop);
 *   warp 1, lane 0   MMA issuer: four tcgen05.mma (M 128, N 128, K 16) per K
 *                    block, then tcgen05.commit to the stage's `empty`
 *                    barrier, which frees the stage when those MMAs are done;
 *   warps 0-3        epilogue: each warp reads its 32 TMEM lanes (rows) with
 *                    tcgen05.ld, applies alpha, bias and GELU, and stores
 *                    bf16, fp32, or adds fp32 atomically (split-K partial
 *                    products of weight gradients).
 *
 * Warp 0 allocates the 128 TMEM columns of the accumulator and frees them
 * at the end.  Every mbarrier wait is bounded: on timeout the thread sets
 * the error word (a device int the caller reads), the pipeline stops
 * issuing, and the kernel still drains what it issued, frees TMEM and
 * returns.  Rows of A or B beyond M, N or K read as zeros (the tensor
 * maps' out-of-bounds fill); stores are guarded.
 */
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstring>

#include "../../include/cgfd3d_gpu.h"

__attribute__((visibility("hidden"))) int cgfd_set_error_msg(int code, const char *msg);

namespace sgg {

constexpr int BM = 128, BN = 128, BK = 64;   /* BK: one 128-byte swizzle row of bf16 */
constexpr int STAGES = 3;
constexpr int TILE_A = BM * BK * 2;          /* 16 KiB */
constexpr int TILE_B = BN * BK * 2;          /* 16 KiB */
constexpr int SMEM_BYTES = STAGES * (TILE_A + TILE_B) + 1024;   /* + alignment slack */
constexpr int NTHREADS = 128;
constexpr uint32_t TMEM_COLS = 128;
constexpr int WAIT_LIMIT = 1 << 24;

struct Epi {
  void *C;
  long long ldc;
  __nv_bfloat16 *Z;      /* pre-activation copy (bf16), or null */
  const float *bias;     /* per column, or null */
  float alpha;
  int act;               /* CGFD_SG_ACT_* */
  int mode;              /* CGFD_SG_OUT_* */
  int M, N;
  int *err;
};

__device__ __forceinline__ uint32_t smem_u32(const void *p)
{
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *b, uint32_t n)
{
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(n) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *b, uint32_t bytes)
{
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(b)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try(uint64_t *b, uint32_t parity)
{
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(b)), "r"(parity)
      : "memory");
  return ok != 0;
}

/* bounded wait: false after `limit` polls (the caller records the error) */
__device__ __forceinline__ bool mbar_wait(uint64_t *b, uint32_t parity, int limit)
{
  for (int n = 0; n < limit; n++) {
    if (mbar_try(b, parity)) return true;
    if (n > 64) __nanosleep(64);
  }
  return false;
}

__device__ __forceinline__ void tma_2d(void *dst, const CUtensorMap *map, int c0, int c1,
                                       uint64_t *bar)
{
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(smem_u32(bar))
      : "memory");
}

/* bulk tensor store of one box from shared memory (bulk-group completion;
 * rows and columns outside the tensor are not written) */
__device__ __forceinline__ void tma_store_2d(const CUtensorMap *map, const void *src, int c0,
                                             int c1)
{
  asm volatile(
      "cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%1, %2}], [%3];" ::"l"(
          reinterpret_cast<uint64_t>(map)),
      "r"(c0), "r"(c1), "r"(smem_u32(src))
      : "memory");
}

/* shared-memory matrix descriptor of a K-major tile with 128-byte swizzle:
 * start address (>> 4), leading byte offset 16 B (unused by swizzled
 * K-major layouts), stride byte offset 1024 B (eight 128-byte rows),
 * descriptor version 1, layout "128-byte swizzle" (2) */
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr)
{
  uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)(16 >> 4) << 16;
  d |= (uint64_t)(1024 >> 4) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)2 << 61;
  return d;
}

/* instruction descriptor of kind::f16: D fp32 (bits 4-5 = 1), A and B bf16
 * (bits 7-9 and 10-12 = 1), both K-major (bits 15, 16 = 0), N >> 3 at bit
 * 17, M >> 4 at bit 24 */
constexpr uint32_t idesc_mn(int m, int n)
{
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) |
         ((uint32_t)(m >> 4) << 24);
}
constexpr uint32_t IDESC = idesc_mn(BM, BN);           /* M 128, N 128 */
constexpr uint32_t IDESC_N256 = idesc_mn(BM, 2 * BN);  /* M 128, N 256 */

__device__ __forceinline__ void umma(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t acc,
                                     uint32_t idesc = IDESC)
{
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(a), "l"(b), "r"(idesc), "r"(acc)
      : "memory");
}

__device__ __forceinline__ void umma_commit(uint64_t *bar)
{
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

/* 32 consecutive fp32 columns of this warp's 32 TMEM lanes */
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t *r)
{
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, "
      "%11, %12, %13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, "
      "%28, %29, %30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
        "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]),
        "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]),
        "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

/* 64 consecutive fp32 columns of this warp's 32 TMEM lanes (one wait) */
__device__ __forceinline__ void tmem_ld64(uint32_t taddr, uint32_t *r)
{
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x64.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, "
      "%11, %12, %13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, "
      "%28, %29, %30, %31, %32, %33, %34, %35, %36, %37, %38, %39, %40, %41, %42, %43, %44, "
      "%45, %46, %47, %48, %49, %50, %51, %52, %53, %54, %55, %56, %57, %58, %59, %60, %61, "
      "%62, %63}, [%64];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
        "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]),
        "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]),
        "=r"(r[31]), "=r"(r[32]), "=r"(r[33]), "=r"(r[34]), "=r"(r[35]), "=r"(r[36]),
        "=r"(r[37]), "=r"(r[38]), "=r"(r[39]), "=r"(r[40]), "=r"(r[41]), "=r"(r[42]),
        "=r"(r[43]), "=r"(r[44]), "=r"(r[45]), "=r"(r[46]), "=r"(r[47]), "=r"(r[48]),
        "=r"(r[49]), "=r"(r[50]), "=r"(r[51]), "=r"(r[52]), "=r"(r[53]), "=r"(r[54]),
        "=r"(r[55]), "=r"(r[56]), "=r"(r[57]), "=r"(r[58]), "=r"(r[59]), "=r"(r[60]),
        "=r"(r[61]), "=r"(r[62]), "=r"(r[63])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ float gelu(float x)
{
  const float u = 0.7978845608028654f * (x + 0.044715f * x * x * x);
  return 0.5f * x * (1.0f + tanhf(u));
}

/* two floats as a bf16 pair in one register (a at the lower address) */
__device__ __forceinline__ uint32_t pack_bf16(float a, float b)
{
  __nv_bfloat162 t = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<uint32_t *>(&t);
}

/* 32 consecutive outputs of one row as bf16: C = act(v), Z = v (Z may be
 * null); `n` of them lie inside the product (32: one full, aligned run) */
__device__ __forceinline__ void store_bf16_32(__nv_bfloat16 *C, __nv_bfloat16 *Z,
                                              const float *v, int act, int n)
{
  if (n >= 32) {
    uint32_t hp[16], zp[16];
#pragma unroll
    for (int u = 0; u < 16; u++) {
      zp[u] = pack_bf16(v[2 * u], v[2 * u + 1]);
      hp[u] = act == CGFD_SG_ACT_GELU ? pack_bf16(gelu(v[2 * u]), gelu(v[2 * u + 1])) : zp[u];
    }
#pragma unroll
    for (int u = 0; u < 4; u++) {
      reinterpret_cast<uint4 *>(C)[u] = make_uint4(hp[4 * u], hp[4 * u + 1], hp[4 * u + 2],
                                                   hp[4 * u + 3]);
      if (Z)
        reinterpret_cast<uint4 *>(Z)[u] = make_uint4(zp[4 * u], zp[4 * u + 1], zp[4 * u + 2],
                                                     zp[4 * u + 3]);
    }
  } else {
#pragma unroll
    for (int u = 0; u < 32; u++) {
      if (u >= n) continue;
      C[u] = __float2bfloat16_rn(act == CGFD_SG_ACT_GELU ? gelu(v[u]) : v[u]);
      if (Z) Z[u] = __float2bfloat16_rn(v[u]);
    }
  }
}

__global__ void __launch_bounds__(NTHREADS, 2)
    k_gemm_tn(const __grid_constant__ CUtensorMap ta, const __grid_constant__ CUtensorMap tb,
              Epi e, int K, int kper)
{
  extern __shared__ uint8_t smem_raw[];
  __shared__ __align__(8) uint64_t full[STAGES], empty[STAGES], accum;
  __shared__ uint32_t tmem_sh;
  __shared__ int abort_sh;
  /* 128-byte swizzled tiles sit on 1024-byte boundaries */
  uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint8_t *sA = smem, *sB = smem + STAGES * TILE_A;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
  const int kb0 = blockIdx.z * kper;
  const int kend = min(K, kb0 + kper);
  const int nkb = kend > kb0 ? (kend - kb0 + BK - 1) / BK : 0;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; s++) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(&accum, 1);
    abort_sh = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&tmem_sh)),
                 "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_sh;

  if (warp == 0 && lane == 0) {
    /* producer */
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&ta)) : "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tb)) : "memory");
    for (int kb = 0; kb < nkb; kb++) {
      const int s = kb % STAGES;
      if (kb >= STAGES) {
        if (!mbar_wait(&empty[s], ((kb / STAGES) - 1) & 1,
                       *(volatile int *)&abort_sh ? 64 : WAIT_LIMIT)) {
          atomicOr(e.err, 1);
          abort_sh = 1;
          break;
        }
      }
      if (*(volatile int *)&abort_sh) break;
      mbar_expect_tx(&full[s], TILE_A + TILE_B);
      tma_2d(sA + s * TILE_A, &ta, kb0 + kb * BK, m0, &full[s]);
      tma_2d(sB + s * TILE_B, &tb, kb0 + kb * BK, n0, &full[s]);
    }
  } else if (warp == 1 && lane == 0) {
    /* MMA issuer: every issued copy is waited for, also after an error */
    bool ok = true;
    for (int kb = 0; kb < nkb; kb++) {
      const int s = kb % STAGES;
      if (!mbar_wait(&full[s], (kb / STAGES) & 1, ok ? WAIT_LIMIT : 64)) {
        if (ok) atomicOr(e.err, 2);
        ok = false;
        abort_sh = 1;
        continue;
      }
      tc_fence_after();
      if (ok) {
        const uint32_t a0 = smem_u32(sA + s * TILE_A), b0 = smem_u32(sB + s * TILE_B);
#pragma unroll
        for (int kk = 0; kk < BK / 16; kk++)
          umma(tmem, sdesc(a0 + kk * 32), sdesc(b0 + kk * 32), (kb | kk) != 0);
      }
      umma_commit(&empty[s]);
    }
    umma_commit(&accum);
  }
  __syncwarp();

  /* epilogue */
  bool have = nkb > 0;
  if (have && !mbar_wait(&accum, 0, WAIT_LIMIT)) {
    atomicOr(e.err, 4);
    have = false;
  }
  tc_fence_after();
  __syncwarp();
  const int row = m0 + warp * 32 + lane;
  const uint32_t tl = tmem + ((uint32_t)(warp * 32) << 16);
#pragma unroll 1
  for (int c0 = 0; c0 < BN; c0 += 32) {
    const int col0 = n0 + c0;
    if (col0 >= e.N) break;                /* warp-uniform */
    uint32_t r[32];
    tmem_ld32(tl + c0, r);
    /* bias: one coalesced load per warp, lane t's value broadcast */
    const float bv = e.bias && col0 + lane < e.N ? e.bias[col0 + lane] : 0.0f;
    float v[32];
#pragma unroll
    for (int t = 0; t < 32; t++)
      v[t] = __uint_as_float(r[t]) * e.alpha + __shfl_sync(0xffffffffu, bv, t);
    if (!have || row >= e.M) continue;
    const bool full_row = col0 + 32 <= e.N;
    if (e.mode == CGFD_SG_OUT_BF16) {
      store_bf16_32((__nv_bfloat16 *)e.C + (long long)row * e.ldc + col0,
                    e.Z ? e.Z + (long long)row * e.ldc + col0 : nullptr, v, e.act, e.N - col0);
    } else if (e.mode == CGFD_SG_OUT_F32) {
      float *C = (float *)e.C + (long long)row * e.ldc + col0;
      if (full_row) {
#pragma unroll
        for (int t = 0; t < 8; t++)
          reinterpret_cast<float4 *>(C)[t] = make_float4(v[4 * t], v[4 * t + 1], v[4 * t + 2],
                                                         v[4 * t + 3]);
      } else {
#pragma unroll
        for (int t = 0; t < 32; t++)
          if (col0 + t < e.N) C[t] = v[t];
      }
    } else {
      float *C = (float *)e.C + (long long)row * e.ldc + col0;
#pragma unroll
      for (int t = 0; t < 32; t++)
        if (col0 + t < e.N) atomicAdd(C + t, v[t]);
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(TMEM_COLS)
                 : "memory");
  }
}

/* ---- persistent form for large products ---------------------------------
 * One CTA per SM walks the output tiles (t = blockIdx.x, + gridDim.x, ...;
 * the N tiles of a row of A are neighbours, so A is re-read from L2).  Ten
 * warps: warp 0 lane 0 the producer, warp 1 lane 0 the MMA issuer, warps 2-9
 * the epilogue.  Two tile forms, each 32768 outputs and 48 KiB of operands
 * per K block:
 *   WIDE (N > 128)   128 x 256: one M 128 x N 256 MMA per K step (the
 *                    tensor pipe does twice the work per cycle at N 256
 *                    than at N 128); a last tile of at most 128 columns
 *                    loads one B box and issues N 128;
 *   narrow (N <= 128) 256 x 128: two M-128 MMAs per K step share the B tile.
 * Epilogue warp w reads TMEM lane quarter w & 3 of the 128-column (WIDE) or
 * 128-row (narrow) half (w - 2) >> 2 of the tile.  Two accumulators of 256
 * TMEM columns alternate between
 * tiles: the MMAs of tile i+1 run while the epilogue reads tile i
 * (tfull[a]: the MMAs of a tile are done; tempty[a]: its accumulator has
 * been read).  The smem ring runs on across tiles.  Outputs: bf16 blocks of
 * 32 x 32 leave through shared memory by bulk tensor stores (tc, tz; rows
 * past M clipped), ragged bf16 blocks and fp32 outputs by the threads' own
 * stores; no split along K. */
constexpr int PSTAGES = 4;
constexpr int P_STAGE = 2 * TILE_A + TILE_B; /* 48 KiB (TILE_A == TILE_B) */
/* epilogue staging, per epilogue warp: 32 rows x 64 B of C and of Z */
constexpr int P_EPI_BUF = 32 * 64;
constexpr int P_THREADS = 320;
constexpr int P_EPI_WARPS = 8;
constexpr int P_SMEM_BYTES = PSTAGES * P_STAGE + 1024 + P_EPI_WARPS * 2 * P_EPI_BUF;
static_assert(P_SMEM_BYTES <= 232448, "more shared memory than one CTA gets");
constexpr uint32_t P_TMEM_COLS = 512;   /* 2 accumulators x 2 halves x 128 */

template <bool WIDE>
__global__ void __launch_bounds__(P_THREADS, 1)
    k_gemm_tn_p(const __grid_constant__ CUtensorMap ta, const __grid_constant__ CUtensorMap tb,
                const __grid_constant__ CUtensorMap tc, const __grid_constant__ CUtensorMap tz,
                Epi e, int K, int ntn, int ntiles)
{
  constexpr int TM = WIDE ? BM : 2 * BM, TN = WIDE ? 2 * BN : BN;
  extern __shared__ uint8_t smem_raw[];
  __shared__ __align__(8) uint64_t full[PSTAGES], empty[PSTAGES], tfull[2], tempty[2], done;
  __shared__ uint32_t tmem_sh;
  __shared__ int abort_sh;
  uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  /* stage s, each a 128 x 64 tile: narrow A rows 0-127, A rows 128-255, B;
   * WIDE A, B rows 0-127, B rows 128-255 (one 256-row K-major operand) */
  auto stA = [&](int s, int h) { return smem + s * P_STAGE + h * TILE_A; };
  auto stB = [&](int s) { return smem + s * P_STAGE + (WIDE ? TILE_A : 2 * TILE_A); };
  /* B boxes of the tile at column n0: a WIDE tile's second box only where
   * columns beyond n0 + 128 exist */
  auto nbox = [&](int n0) { return WIDE && e.N - n0 > BN ? 2 : 1; };
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nkb = (K + BK - 1) / BK;

  if (threadIdx.x == 0) {
    for (int s = 0; s < PSTAGES; s++) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int a = 0; a < 2; a++) {
      mbar_init(&tfull[a], 1);
      mbar_init(&tempty[a], P_EPI_WARPS);
    }
    mbar_init(&done, 1);
    abort_sh = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&tmem_sh)),
                 "r"(P_TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_sh;
  auto live = [&]() { return *(volatile int *)&abort_sh == 0; };

  if (warp == 0 && lane == 0) {
    /* producer; last[s]: the latest ring position issued into stage s */
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&ta)) : "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tb)) : "memory");
    int last[PSTAGES];
#pragma unroll
    for (int s = 0; s < PSTAGES; s++) last[s] = -1;
    int g = 0;
    for (int t = blockIdx.x; t < ntiles && live(); t += gridDim.x) {
      const int m0 = (t / ntn) * TM, n0 = (t % ntn) * TN;
      const int nb = nbox(n0);
      for (int kb = 0; kb < nkb; kb++, g++) {
        const int s = g % PSTAGES;
        if (g >= PSTAGES && !mbar_wait(&empty[s], ((g / PSTAGES) - 1) & 1, WAIT_LIMIT)) {
          atomicOr(e.err, 1);
          abort_sh = 1;
        }
        if (!live()) break;
        if (WIDE) {
          mbar_expect_tx(&full[s], TILE_A + nb * TILE_B);
          tma_2d(stA(s, 0), &ta, kb * BK, m0, &full[s]);
          tma_2d(stB(s), &tb, kb * BK, n0, &full[s]);
          if (nb == 2) tma_2d(stB(s) + TILE_B, &tb, kb * BK, n0 + BN, &full[s]);
        } else {
          mbar_expect_tx(&full[s], P_STAGE);
          tma_2d(stA(s, 0), &ta, kb * BK, m0, &full[s]);
          tma_2d(stA(s, 1), &ta, kb * BK, m0 + BM, &full[s]);
          tma_2d(stB(s), &tb, kb * BK, n0, &full[s]);
        }
        last[s] = g;
      }
    }
    if (!live()) {
      /* the CTA leaves only after its copies have landed */
#pragma unroll
      for (int s = 0; s < PSTAGES; s++)
        if (last[s] >= 0) mbar_wait(&full[s], (last[s] / PSTAGES) & 1, WAIT_LIMIT);
    }
  } else if (warp == 1 && lane == 0) {
    /* MMA issuer */
    int g = 0, i = 0;
    for (int t = blockIdx.x; t < ntiles && live(); t += gridDim.x, i++) {
      const int acc = i & 1;
      if (i >= 2 && !mbar_wait(&tempty[acc], ((i / 2) - 1) & 1, WAIT_LIMIT)) {
        atomicOr(e.err, 2);
        abort_sh = 1;
        break;
      }
      tc_fence_after();
      const uint32_t d = tmem + (uint32_t)(acc * 2 * BN);
      const uint32_t idesc = nbox((t % ntn) * TN) == 2 ? IDESC_N256 : IDESC;
      bool ok = true;
      for (int kb = 0; kb < nkb; kb++, g++) {
        const int s = g % PSTAGES;
        if (!mbar_wait(&full[s], (g / PSTAGES) & 1, WAIT_LIMIT)) {
          atomicOr(e.err, 2);
          abort_sh = 1;
          ok = false;
          break;
        }
        tc_fence_after();
        const uint32_t a0 = smem_u32(stA(s, 0)), a1 = smem_u32(stA(s, 1));
        const uint32_t b0 = smem_u32(stB(s));
#pragma unroll
        for (int kk = 0; kk < BK / 16; kk++) {
          if (WIDE) {
            umma(d, sdesc(a0 + kk * 32), sdesc(b0 + kk * 32), (kb | kk) != 0, idesc);
          } else {
            umma(d, sdesc(a0 + kk * 32), sdesc(b0 + kk * 32), (kb | kk) != 0);
            umma(d + BN, sdesc(a1 + kk * 32), sdesc(b0 + kk * 32), (kb | kk) != 0);
          }
        }
        umma_commit(&empty[s]);
      }
      if (!ok) break;
      umma_commit(&tfull[acc]);
    }
    /* every MMA issued has finished before TMEM is freed */
    umma_commit(&done);
    mbar_wait(&done, 0, WAIT_LIMIT);
  } else if (warp >= 2) {
    /* epilogue: warp w reads TMEM lanes 32 (w % 4) .. + 31 of the
     * accumulator half h = (w - 2) / 4: rows 32 (w % 4) .. of columns
     * h 128 .. (WIDE), rows h 128 + 32 (w % 4) .. (narrow) */
    const int q = warp & 3, half = (warp - 2) >> 2;
    uint8_t *ebuf = smem + PSTAGES * P_STAGE + (warp - 2) * 2 * P_EPI_BUF;
    int i = 0;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x, i++) {
      const int acc = i & 1;
      bool have = live() && mbar_wait(&tfull[acc], (i / 2) & 1, WAIT_LIMIT);
      have = __all_sync(0xffffffffu, have);
      if (!have) {
        if (lane == 0) {
          atomicOr(e.err, 4);
          abort_sh = 1;
        }
        break;
      }
      tc_fence_after();
      const int m0 = (t / ntn) * TM + (WIDE ? 0 : half * BM);
      const int n0 = (t % ntn) * TN + (WIDE ? half * BN : 0);
      const int row = m0 + q * 32 + lane;
      const uint32_t tl = tmem + (uint32_t)(acc * 2 * BN + half * BN) + ((uint32_t)(q * 32) << 16);
      /* 64 columns per TMEM load, then two 32-column blocks from registers */
#pragma unroll 1
      for (int c64 = 0; c64 < BN; c64 += 64) {
        if (n0 + c64 >= e.N) break;        /* warp-uniform: nothing left of this half */
        uint32_t r64[64];
        tmem_ld64(tl + c64, r64);
#pragma unroll
        for (int sub = 0; sub < 2; sub++) {
          const int c0 = c64 + 32 * sub;
          const int col0 = n0 + c0;
          if (col0 >= e.N) break;
          const uint32_t *r = r64 + 32 * sub;
          /* bias: one coalesced load per warp, lane u's value broadcast */
          const float bv = e.bias && col0 + lane < e.N ? e.bias[col0 + lane] : 0.0f;
          float v[32];
  #pragma unroll
          for (int u = 0; u < 32; u++)
            v[u] = __uint_as_float(r[u]) * e.alpha + __shfl_sync(0xffffffffu, bv, u);
          if (e.mode == CGFD_SG_OUT_BF16 && col0 + 32 <= e.N) {
            /* the warp's 32 x 32 block goes out through shared memory as one
             * bulk tensor store per output: lane = row writes its 64 bytes,
             * 16-byte chunk c of row r at c ^ ((r >> 1) & 3), the layout of
             * the stores' 64-byte swizzle (bank-conflict free as well); rows
             * beyond M are clipped by the store */
            uint32_t hp[16], zp[16];
  #pragma unroll
            for (int u = 0; u < 16; u++) {
              zp[u] = pack_bf16(v[2 * u], v[2 * u + 1]);
              hp[u] = e.act == CGFD_SG_ACT_GELU ? pack_bf16(gelu(v[2 * u]), gelu(v[2 * u + 1]))
                                                : zp[u];
            }
            /* the previous block's stores have read the buffer */
            if (lane == 0) asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
            __syncwarp();
            const int sw = (lane >> 1) & 3;
  #pragma unroll
            for (int c = 0; c < 4; c++) {
              *reinterpret_cast<uint4 *>(ebuf + lane * 64 + ((c ^ sw) << 4)) =
                  make_uint4(hp[4 * c], hp[4 * c + 1], hp[4 * c + 2], hp[4 * c + 3]);
              if (e.Z)
                *reinterpret_cast<uint4 *>(ebuf + P_EPI_BUF + lane * 64 + ((c ^ sw) << 4)) =
                    make_uint4(zp[4 * c], zp[4 * c + 1], zp[4 * c + 2], zp[4 * c + 3]);
            }
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            __syncwarp();
            if (lane == 0) {
              tma_store_2d(&tc, ebuf, col0, m0 + q * 32);
              if (e.Z) tma_store_2d(&tz, ebuf + P_EPI_BUF, col0, m0 + q * 32);
              asm volatile("cp.async.bulk.commit_group;" ::: "memory");
            }
            continue;
          }
          if (row >= e.M) continue;
          if (e.mode == CGFD_SG_OUT_BF16) {
            store_bf16_32((__nv_bfloat16 *)e.C + (long long)row * e.ldc + col0,
                          e.Z ? e.Z + (long long)row * e.ldc + col0 : nullptr, v, e.act,
                          e.N - col0);
          } else {
            float *C = (float *)e.C + (long long)row * e.ldc + col0;
            if (col0 + 32 <= e.N) {
  #pragma unroll
              for (int u = 0; u < 8; u++)
                reinterpret_cast<float4 *>(C)[u] =
                    make_float4(v[4 * u], v[4 * u + 1], v[4 * u + 2], v[4 * u + 3]);
            } else {
  #pragma unroll
              for (int u = 0; u < 32; u++)
                if (col0 + u < e.N) C[u] = v[u];
            }
          }
        }
      }
      /* this warp's lanes of the accumulator are read: hand it back */
      tc_fence_before();
      __syncwarp();
      if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(
                                      smem_u32(&tempty[acc]))
                                  : "memory");
    }
    /* the warp's bulk stores are complete before the CTA leaves */
    if (lane == 0) asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
    __syncwarp();
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(P_TMEM_COLS)
                 : "memory");
  }
}

typedef CUresult (*encode_fn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                              const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                              const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                              CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static encode_fn encoder(void)
{
  static encode_fn fn = nullptr;
  if (!fn) {
    cudaDriverEntryPointQueryResult q;
    void *p = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (encode_fn)p;
  }
  return fn;
}

/* a [rows, K] bf16 operand with row stride ld elements, 64 x 128 boxes */
static bool operand_map(CUtensorMap *m, const void *p, int rows, int K, long long ld)
{
  encode_fn fn = encoder();
  if (!fn) return false;
  cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)ld * 2};
  cuuint32_t box[2] = {BK, 128};
  cuuint32_t es[2] = {1, 1};
  return fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(p), dims, strides, box,
            es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
            CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

/* a bf16 [rows, N] output with row stride ld elements, 32 x 32 boxes in the
 * 64-byte swizzle the persistent epilogue stages its blocks in */
static bool output_map(CUtensorMap *m, void *p, int rows, int N, long long ld)
{
  encode_fn fn = encoder();
  if (!fn) return false;
  cuuint64_t dims[2] = {(cuuint64_t)N, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)ld * 2};
  cuuint32_t box[2] = {32, 32};
  cuuint32_t es[2] = {1, 1};
  return fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, p, dims, strides, box, es,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B,
            CU_TENSOR_MAP_L2_PROMOTION_NONE, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

static int gemm_err(int code, const char *fmt, ...)
{
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  return cgfd_set_error_msg(code, buf);
}

}  // namespace sgg

using namespace sgg;

extern "C" int cgfd_sg_gemm(const void *A, long long lda, const void *B, long long ldb, void *C,
                            long long ldc, int M, int N, int K, float alpha, const float *bias,
                            int act, int mode, void *Z, int splits, int *d_err, void *stream)
{
  if (!A || !B || !C || !d_err || M < 1 || N < 1 || K < 1)
    return gemm_err(CGFD_EINVAL, "sg_gemm: missing operand or empty product (%d x %d x %d)",
                    M, N, K);
  if (K % 8 || lda % 8 || ldb % 8 || lda < K || ldb < K || ldc < N ||
      ((uintptr_t)A & 15) || ((uintptr_t)B & 15))
    return gemm_err(CGFD_EINVAL, "sg_gemm: K, lda, ldb must be multiples of 8 (16-byte rows) "
                    "and the operands 16-byte aligned (K %d, lda %lld, ldb %lld)", K, lda, ldb);
  if (mode != CGFD_SG_OUT_BF16 && mode != CGFD_SG_OUT_F32 && mode != CGFD_SG_OUT_F32_ADD)
    return gemm_err(CGFD_EINVAL, "sg_gemm: output mode %d", mode);
  if ((mode == CGFD_SG_OUT_BF16 && (ldc % 8 || ((uintptr_t)C & 15) ||
                                    (Z && ((uintptr_t)Z & 15)))) ||
      (mode == CGFD_SG_OUT_F32 && (ldc % 4 || ((uintptr_t)C & 15))))
    return gemm_err(CGFD_EINVAL, "sg_gemm: output rows must be 16-byte aligned");
  if (splits < 1) splits = 1;
  if (splits > 1 && mode != CGFD_SG_OUT_F32_ADD)
    return gemm_err(CGFD_EINVAL, "sg_gemm: a split product must add into fp32");
  CUtensorMap ta, tb;
  if (!operand_map(&ta, A, M, K, lda) || !operand_map(&tb, B, N, K, ldb))
    return gemm_err(CGFD_ECUDA, "sg_gemm: tensor map encoding failed");
  const int nkb = (K + BK - 1) / BK;
  const int kper = ((nkb + splits - 1) / splits) * BK;
  const int nz = (K + kper - 1) / kper;
  static bool attr = false;
  static int nsm = 0;
  if (!attr) {
    int dev = 0;
    if (cudaFuncSetAttribute(k_gemm_tn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             SMEM_BYTES) != cudaSuccess ||
        cudaFuncSetAttribute(k_gemm_tn_p<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             P_SMEM_BYTES) != cudaSuccess ||
        cudaFuncSetAttribute(k_gemm_tn_p<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             P_SMEM_BYTES) != cudaSuccess ||
        cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
      return gemm_err(CGFD_ECUDA, "sg_gemm: kernel attributes");
    attr = true;
  }
  Epi e;
  e.C = C;
  e.ldc = ldc;
  e.Z = (__nv_bfloat16 *)Z;
  e.bias = bias;
  e.alpha = alpha;
  e.act = act;
  e.mode = mode;
  e.M = M;
  e.N = N;
  e.err = d_err;
  const int ntn = (N + BN - 1) / BN, ntm = (M + BM - 1) / BM;
  const bool wide = N > BN;
  const int ptn = wide ? (N + 2 * BN - 1) / (2 * BN) : ntn;
  const long long ptiles = (long long)ptn * (wide ? ntm : (M + 2 * BM - 1) / (2 * BM));
  if (nz == 1 && mode != CGFD_SG_OUT_F32_ADD && ptiles >= 2LL * nsm && ptiles < (1LL << 31)) {
    /* large products: one persistent CTA per SM, 32768-output tiles,
     * epilogue overlapped; bf16 outputs leave by bulk tensor stores */
    CUtensorMap tc, tz;
    memset(&tc, 0, sizeof(tc));
    memset(&tz, 0, sizeof(tz));
    if (mode == CGFD_SG_OUT_BF16 &&
        (!output_map(&tc, C, M, N, ldc) || (Z && !output_map(&tz, Z, M, N, ldc))))
      return gemm_err(CGFD_ECUDA, "sg_gemm: output tensor map encoding failed");
    if (wide)
      k_gemm_tn_p<true><<<nsm, P_THREADS, P_SMEM_BYTES, (cudaStream_t)stream>>>(
          ta, tb, tc, tz, e, K, ptn, (int)ptiles);
    else
      k_gemm_tn_p<false><<<nsm, P_THREADS, P_SMEM_BYTES, (cudaStream_t)stream>>>(
          ta, tb, tc, tz, e, K, ptn, (int)ptiles);
  } else {
    dim3 grid(ntn, ntm, nz);
    k_gemm_tn<<<grid, NTHREADS, SMEM_BYTES, (cudaStream_t)stream>>>(ta, tb, e, K, kper);
  }
  const cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) return gemm_err(CGFD_ECUDA, "sg_gemm launch: %s", cudaGetErrorString(err));
  return 0;
}
