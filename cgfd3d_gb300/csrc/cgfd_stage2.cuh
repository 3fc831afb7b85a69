/*
 * Shared-memory building blocks of the TMA-fed stage kernel
 * (cgfd_stage3.cuh): mbarrier and bulk-tensor-copy wrappers (inline PTX),
 * the plane-tile layout, and the MacCormack operators evaluated on plane
 * tiles held in shared memory.
 *
 * Plane tile: the nine wavefield components of one k plane over the CTA's
 * 32 x TY columns plus a halo of 4 columns in x (one/three are used,
 * depending on the operator bias; 4 keeps the box origin 16-byte aligned)
 * and 2+2 rows in y, stored [component][row][column] exactly as one 5-D
 * bulk tensor copy lands it.
 */
#ifndef CGFD_STAGE2_CUH
#define CGFD_STAGE2_CUH

#include <cuda.h>

#include "cgfd_common.h"
#include "cgfd_stage.cuh"

namespace s2 {

constexpr int TX = 32;
/* tile rows (one consumer warp each); set per translation unit: more rows
 * give more warps per SM to hide latency where the shared memory allows */
#ifndef CGFD_TILE_ROWS
#define CGFD_TILE_ROWS 8
#endif
constexpr int TY = CGFD_TILE_ROWS;
constexpr int BW = 40;               /* box width (x), multiple of 4 */
constexpr int BH = TY + 4;           /* box height (y) */
constexpr int XL = 4;                /* smem column of the tile's first i */
constexpr int PLANE_DATA = 9 * BH * BW;  /* floats one plane copy lands */
/* plane buffer stride: every bulk tensor copy must land on a 128-byte
 * aligned shared-memory address, so the ring stride is rounded up */
constexpr int PLANE = (PLANE_DATA + 31) / 32 * 32;
static_assert(PLANE % 32 == 0, "plane buffers must stay 128-byte aligned");

__device__ __forceinline__ uint32_t smem_u32(const void *p)
{
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(count)
               : "memory");
}

/* the barrier's memory may be initialised again (after every use has ended) */
__device__ __forceinline__ void mbar_inval(uint64_t *bar)
{
  asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes)
{
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(
                   smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity)
{
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n"
      " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

/* bounded wait; returns false (and flags the error) after `limit` polls */
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity,
                                          int *err, int limit = 1 << 22)
{
  for (int n = 0; n < limit; n++) {
    if (mbar_try_wait(bar, parity)) return true;
    if (n > 16) __nanosleep(128);
  }
  atomicOr(err, 1);
  return false;
}

__device__ __forceinline__ void tma_load_4d(float *dst, const CUtensorMap *map,
                                            int c0, int c1, int c2, int c3,
                                            uint64_t *bar)
{
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_"
      "tx::bytes [%0], [%1, {%2, %3, %4, %5}], [%6];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3),
      "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar)
{
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void tma_load_5d(float *dst, const CUtensorMap *map,
                                            int c0, int c1, int c2, int c3,
                                            int c4, uint64_t *bar)
{
  asm volatile(
      "cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_"
      "tx::bytes [%0], [%1, {%2, %3, %4, %5, %6}], [%7];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3),
      "r"(c4), "r"(smem_u32(bar))
      : "memory");
}

/* L2 prefetch of one tensor tile (no shared memory, no completion) */
__device__ __forceinline__ void tma_prefetch_4d(const CUtensorMap *map, int c0,
                                                int c1, int c2, int c3)
{
  asm volatile(
      "cp.async.bulk.prefetch.tensor.4d.L2.global.tile [%0, {%1, %2, %3, %4}];" ::"l"(
          reinterpret_cast<uint64_t>(map)),
      "r"(c0), "r"(c1), "r"(c2), "r"(c3)
      : "memory");
}

__device__ __forceinline__ void tma_prefetch_5d(const CUtensorMap *map, int c0,
                                                int c1, int c2, int c3, int c4)
{
  asm volatile(
      "cp.async.bulk.prefetch.tensor.5d.L2.global.tile [%0, {%1, %2, %3, %4, "
      "%5}];" ::"l"(reinterpret_cast<uint64_t>(map)),
      "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(c4)
      : "memory");
}

template <int B>
__device__ __forceinline__ float sdop(const float *p, int s)
{
  if (B == 0)
    return -0.30874f * p[-s] + -0.6326f * p[0] + 1.233f * p[s] +
           -0.3334f * p[2 * s] + 0.04168f * p[3 * s];
  else
    return -0.04168f * p[-3 * s] + 0.3334f * p[-2 * s] + -1.233f * p[-s] +
           0.6326f * p[0] + 0.30874f * p[s];
}

/* the five z-tap planes of the current window, lowest first */
struct Win {
  const float *p0, *p1, *p2, *p3, *p4;
  __device__ __forceinline__ const float *at(int n) const
  {
    return n == 0 ? p0 : n == 1 ? p1 : n == 2 ? p2 : n == 3 ? p3 : p4;
  }
};

template <int BZ>
__device__ __forceinline__ float zdop(const Win &w, int o)
{
  if (BZ == 0)
    return -0.30874f * w.p0[o] + -0.6326f * w.p1[o] + 1.233f * w.p2[o] +
           -0.3334f * w.p3[o] + 0.04168f * w.p4[o];
  else
    return -0.04168f * w.p0[o] + 0.3334f * w.p1[o] + -1.233f * w.p2[o] +
           0.6326f * w.p3[o] + 0.30874f * w.p4[o];
}

/* offset of component c inside a plane buffer at smem row/col */
__device__ __forceinline__ int soff(int c, int row, int col)
{
  return (c * BH + row) * BW + col;
}

template <int BX, int BY, int BZ>
__device__ __forceinline__ void sderiv9(const float *cen, const Win &w,
                                        int row, int col, int dim, Deriv9 &d)
{
  float v[9];
#pragma unroll
  for (int c = 0; c < 9; c++) {
    int o = soff(c, row, col);
    if (dim == 0) v[c] = sdop<BX>(cen + o, 1);
    else if (dim == 1) v[c] = sdop<BY>(cen + o, BW);
    else v[c] = zdop<BZ>(w, o);
  }
  d.Vx = v[C_VX]; d.Vy = v[C_VY]; d.Vz = v[C_VZ];
  d.Txx = v[C_TXX]; d.Tyy = v[C_TYY]; d.Tzz = v[C_TZZ];
  d.Txz = v[C_TXZ]; d.Tyz = v[C_TYZ]; d.Txy = v[C_TXY];
}

/* conservative traction flux J (m . T) with T read from a plane buffer */
__device__ __forceinline__ float scons(const StageArgs &a, const float *P,
                                       int ca, int cb, int cc, int row,
                                       int col, long long q, const float *m1,
                                       const float *m2, const float *m3)
{
  return LDG(a.jac + q) * (LDG(m1 + q) * P[soff(ca, row, col)] +
                           LDG(m2 + q) * P[soff(cb, row, col)] +
                           LDG(m3 + q) * P[soff(cc, row, col)]);
}

/* traction image, smem operands (same formula as timg_row) */
template <int BX, int BY, int BZ>
__device__ float stimg_row(const StageArgs &a, const Win &w,
                           const float *cen, int row, int col, long long q,
                           int k, int r, float ts)
{
  const long long px = a.g.px, sl = a.g.sl;
  int ca, cb, cc;
  if (r == 0) { ca = C_TXX; cb = C_TXY; cc = C_TXZ; }
  else if (r == 1) { ca = C_TXY; cb = C_TYY; cc = C_TYZ; }
  else { ca = C_TXZ; cb = C_TYZ; cc = C_TZZ; }
  float Dx = 0.f, Dy = 0.f, Dz = 0.f;
#pragma unroll
  for (int n = 0; n < 5; n++) {
    int sx = tap_shift<BX>(n), sy = tap_shift<BY>(n);
    Dx += tap_coef<BX>(n) *
          scons(a, cen, ca, cb, cc, row, col + sx, q + sx, a.xix, a.xiy, a.xiz);
    Dy += tap_coef<BY>(n) * scons(a, cen, ca, cb, cc, row + sy, col,
                                  q + (long long)sy * px, a.etx, a.ety, a.etz);
  }
  const int nk2 = a.g.nk2;
  const int klow = k + tap_shift<BZ>(0);
#pragma unroll
  for (int n = 0; n < 5; n++) {
    int kk = k + tap_shift<BZ>(n);
    float v;
    if (kk < nk2) {
      v = scons(a, w.at(n), ca, cb, cc, row, col, q + (long long)(kk - k) * sl,
                a.ztx, a.zty, a.ztz);
    } else if (kk == nk2) {
      v = ts;                     /* surface traction (TxSrc/TySrc/TzSrc) */
    } else {
      int km = 2 * nk2 - kk;
      /* mirror 2 ts - flux(km); the image point km lies inside the 5-plane
       * window whenever km >= klow (else the reference reads zeros) */
      v = 2.0f * ts -
          ((km >= klow) ? scons(a, w.at(km - klow), ca, cb, cc, row, col,
                                q + (long long)(km - k) * sl, a.ztx, a.zty, a.ztz)
                        : 0.f);
    }
    Dz += tap_coef<BZ>(n) * v;
  }
  float slwjac = LDG(a.slw + q) / LDG(a.jac + q);
  return (Dx + Dy + Dz) * slwjac;
}

}  // namespace s2

#endif
