/*
 * Stage kernel, 2.5-D form: z-marching thread blocks fed by TMA.
 *
 * A CTA owns a 32 x 8 column tile of the (i, j) plane and a run of k planes.
 * For every k plane it needs the nine wavefield components of five planes
 * (the z operator's taps) and, on the current plane, a halo of one/three
 * points in x and y (the MacCormack operators are one-sided).  Those plane
 * tiles stream through a ring of NB shared-memory buffers: one elected
 * thread issues a single 5-D bulk tensor copy per plane (40 x 12 points x 9
 * components = 17 KiB, cp.async.bulk.tensor with an mbarrier carrying the
 * byte count), one plane ahead of use.  Each wavefield value therefore
 * leaves HBM once per stage; the halo re-reads are served by L2.  The
 * per-point streams (metrics, media, pre/end levels, PML auxiliaries) are
 * plain coalesced loads from the same pitched layout.
 *
 * The arithmetic per point is that of cgfd_stage.cuh (reference:
 * forward/sv_curv_col_el_iso.c:208-1146, forward/sv_curv_col_el.c:30-479,
 * forward/drv_rk_curv_col.c:292-446); only where the operands come from
 * differs.  Directional derivatives the CFS-PML and the free-surface code
 * need are recomputed from shared memory where they are used, which keeps
 * the register footprint of the common path small.
 *
 * Every mbarrier wait is bounded: after ~2^22 polls the thread records
 * CGFD device error 1 in a.err and continues, so the kernel always ends and
 * the host reports the failure.
 */
#ifndef CGFD_STAGE2_CUH
#define CGFD_STAGE2_CUH

#include <cuda.h>

#include "cgfd_common.h"
#include "cgfd_stage.cuh"

namespace s2 {

constexpr int TX = 32;
constexpr int TY = 8;
constexpr int BW = 40;               /* box width (x), multiple of 4 */
constexpr int BH = TY + 4;           /* box height (y) */
constexpr int XL = 4;                /* smem column of the tile's first i */
constexpr int NB = 6;                /* ring: 5 window planes + 1 in flight */
constexpr int PLANE = 9 * BH * BW;   /* floats per buffer */
constexpr int SMEM_BYTES = NB * PLANE * 4;

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

/* bounded wait; returns false (and flags the error) on timeout */
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity,
                                          int *err)
{
  for (int n = 0; n < (1 << 22); n++) {
    if (mbar_try_wait(bar, parity)) return true;
    if (n > 16) __nanosleep(128);
  }
  atomicOr(err, 1);
  return false;
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

template <int BZ>
__device__ __forceinline__ float zdop(const float *const *w, int o)
{
  if (BZ == 0)
    return -0.30874f * w[0][o] + -0.6326f * w[1][o] + 1.233f * w[2][o] +
           -0.3334f * w[3][o] + 0.04168f * w[4][o];
  else
    return -0.04168f * w[0][o] + 0.3334f * w[1][o] + -1.233f * w[2][o] +
           0.6326f * w[3][o] + 0.30874f * w[4][o];
}

/* offset of component c inside a plane buffer at smem row/col */
__device__ __forceinline__ int soff(int c, int row, int col)
{
  return (c * BH + row) * BW + col;
}

template <int BX, int BY, int BZ>
__device__ __forceinline__ void sderiv9(const float *cen, const float *const *w,
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
__device__ float stimg_row(const StageArgs &a, const float *const *w,
                           const float *cen, int row, int col, long long q,
                           int k, int r)
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
      v = scons(a, w[n], ca, cb, cc, row, col, q + (long long)(kk - k) * sl,
                a.ztx, a.zty, a.ztz);
    } else if (kk == nk2) {
      v = 0.f;
    } else {
      int km = 2 * nk2 - kk;
      /* image point km lies inside the 5-plane window whenever km >= klow */
      v = (km >= klow)
              ? -scons(a, w[km - klow], ca, cb, cc, row, col,
                       q + (long long)(km - k) * sl, a.ztx, a.zty, a.ztz)
              : 0.f;
    }
    Dz += tap_coef<BZ>(n) * v;
  }
  float slwjac = LDG(a.slw + q) / LDG(a.jac + q);
  return (Dx + Dy + Dz) * slwjac;
}

template <int BX, int BY, int BZ, int KIND>
__global__ void __launch_bounds__(TX *TY, 2)
    k_stage2(const __grid_constant__ StageArgs a,
             const __grid_constant__ CUtensorMap tmap)
{
  extern __shared__ __align__(128) float sm[];
  __shared__ __align__(8) uint64_t bars[NB];

  const int tx = threadIdx.x, ty = threadIdx.y;
  const int tid = ty * TX + tx;
  const DevGrid &g = a.g;
  const int i0 = g.ni1 + blockIdx.x * TX;
  const int j0 = g.nj1 + blockIdx.y * TY;
  const int i = i0 + tx, j = j0 + ty;
  const bool valid = (i <= g.ni2) && (j <= g.nj2);
  const int kbeg = g.nk1 + blockIdx.z * a.kchunk;
  const int kend = min(kbeg + a.kchunk - 1, g.nk2);

  constexpr int ZS0 = BZ == 0 ? -1 : -3;  /* lowest z tap */
  constexpr int YL = BY == 0 ? 1 : 3;     /* smem row of j0 */
  constexpr int ZC = BZ == 0 ? 1 : 3;     /* window index of plane k */
  const int pbase = kbeg + ZS0;
  const int nplanes = kend - kbeg + 5;
  const int bx0 = i0 + g.xoff - XL;       /* box origin, multiple of 4 */
  const int by0 = j0 - YL;

  if (tid == 0) {
    for (int b = 0; b < NB; b++) mbar_init(&bars[b], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  __syncthreads();
  if (tid == 0) {
    for (int r = 0; r < NB && r < nplanes; r++) {
      mbar_expect_tx(&bars[r], PLANE * 4);
      tma_load_5d(sm + r * PLANE, &tmap, bx0, by0, pbase + r, 0, a.cur_level,
                  &bars[r]);
    }
  }

  const int row = ty + YL, col = tx + XL;
  const long long px = g.px, sl = g.sl, vol = g.vol;

  for (int k = kbeg; k <= kend; k++) {
    const int rtop = k - kbeg + 4;  /* newest plane of the window (rel) */
    const float *w[5];
#pragma unroll
    for (int n = 0; n < 5; n++) {
      int rel = rtop - 4 + n;
      w[n] = sm + (rel % NB) * PLANE;
      mbar_wait(&bars[rel % NB], (rel / NB) & 1, a.err);
    }
    const float *cen = w[ZC];

    if (valid) {
      const long long q = (long long)(i + g.xoff) + (long long)j * px +
                          (long long)k * sl;
      float xix = LDG(a.xix + q), xiy = LDG(a.xiy + q), xiz = LDG(a.xiz + q);
      float etx = LDG(a.etx + q), ety = LDG(a.ety + q), etz = LDG(a.etz + q);
      float ztx = LDG(a.ztx + q), zty = LDG(a.zty + q), ztz = LDG(a.ztz + q);
      float lam = LDG(a.lam + q), mu = LDG(a.mu + q), slw = LDG(a.slw + q);
      float l2m = lam + 2.0f * mu;
      float r[9];
      {
        /* momentum: stress derivatives */
        const float *cT;
#define DX(c) sdop<BX>(cen + soff(c, row, col), 1)
#define DY(c) sdop<BY>(cen + soff(c, row, col), BW)
#define DZ(c) zdop<BZ>(w, soff(c, row, col))
        float DxTxx = DX(C_TXX), DyTxx = DY(C_TXX), DzTxx = DZ(C_TXX);
        float DxTxy = DX(C_TXY), DyTxy = DY(C_TXY), DzTxy = DZ(C_TXY);
        float DxTxz = DX(C_TXZ), DyTxz = DY(C_TXZ), DzTxz = DZ(C_TXZ);
        r[C_VX] = slw * (xix * DxTxx + xiy * DxTxy + xiz * DxTxz +
                         etx * DyTxx + ety * DyTxy + etz * DyTxz +
                         ztx * DzTxx + zty * DzTxy + ztz * DzTxz);
        float DxTyy = DX(C_TYY), DyTyy = DY(C_TYY), DzTyy = DZ(C_TYY);
        float DxTyz = DX(C_TYZ), DyTyz = DY(C_TYZ), DzTyz = DZ(C_TYZ);
        r[C_VY] = slw * (xix * DxTxy + xiy * DxTyy + xiz * DxTyz +
                         etx * DyTxy + ety * DyTyy + etz * DyTyz +
                         ztx * DzTxy + zty * DzTyy + ztz * DzTyz);
        float DxTzz = DX(C_TZZ), DyTzz = DY(C_TZZ), DzTzz = DZ(C_TZZ);
        r[C_VZ] = slw * (xix * DxTxz + xiy * DxTyz + xiz * DxTzz +
                         etx * DyTxz + ety * DyTyz + etz * DyTzz +
                         ztx * DzTxz + zty * DzTyz + ztz * DzTzz);
        (void)cT;
      }
      {
        /* Hooke: velocity derivatives (vlow near the free surface) */
        float DxVx = DX(C_VX), DyVx = DY(C_VX);
        float DxVy = DX(C_VY), DyVy = DY(C_VY);
        float DxVz = DX(C_VZ), DyVz = DY(C_VZ);
        float DzVx, DzVy, DzVz;
        const int nk2 = g.nk2;
        if (a.free_top && k >= nk2 - 2) {
          if (k == nk2) {
            long long ij = ((long long)i + (long long)j * g.nx) * 9;
            const float *A = a.mVx + ij, *Bm = a.mVy + ij;
            DzVx = LDG(A + 0) * DxVx + LDG(A + 1) * DxVy + LDG(A + 2) * DxVz +
                   LDG(Bm + 0) * DyVx + LDG(Bm + 1) * DyVy + LDG(Bm + 2) * DyVz;
            DzVy = LDG(A + 3) * DxVx + LDG(A + 4) * DxVy + LDG(A + 5) * DxVz +
                   LDG(Bm + 3) * DyVx + LDG(Bm + 4) * DyVy + LDG(Bm + 5) * DyVz;
            DzVz = LDG(A + 6) * DxVx + LDG(A + 7) * DxVy + LDG(A + 8) * DxVz +
                   LDG(Bm + 6) * DyVx + LDG(Bm + 7) * DyVy + LDG(Bm + 8) * DyVz;
          } else if (k == nk2 - 1) {
            /* second order: taps {0,1} (bias 0) or {-1,0} (bias 1) */
            const float *lo = BZ == 0 ? w[ZC] : w[ZC - 1];
            const float *hi = BZ == 0 ? w[ZC + 1] : w[ZC];
            int ox = soff(C_VX, row, col), oy = soff(C_VY, row, col),
                oz = soff(C_VZ, row, col);
            DzVx = -lo[ox] + hi[ox];
            DzVy = -lo[oy] + hi[oy];
            DzVz = -lo[oz] + hi[oz];
          } else {
            /* fourth order: {0,1,2} or {-2,-1,0} */
            const float c0 = BZ == 0 ? (float)(-7.0 / 6.0) : (float)(1.0 / 6.0);
            const float c1 = BZ == 0 ? (float)(8.0 / 6.0) : (float)(-8.0 / 6.0);
            const float c2 = BZ == 0 ? (float)(-1.0 / 6.0) : (float)(7.0 / 6.0);
            const float *p0 = BZ == 0 ? w[ZC] : w[ZC - 2];
            const float *p1 = BZ == 0 ? w[ZC + 1] : w[ZC - 1];
            const float *p2 = BZ == 0 ? w[ZC + 2] : w[ZC];
            int ox = soff(C_VX, row, col), oy = soff(C_VY, row, col),
                oz = soff(C_VZ, row, col);
            DzVx = c0 * p0[ox] + c1 * p1[ox] + c2 * p2[ox];
            DzVy = c0 * p0[oy] + c1 * p1[oy] + c2 * p2[oy];
            DzVz = c0 * p0[oz] + c1 * p1[oz] + c2 * p2[oz];
          }
        } else {
          DzVx = DZ(C_VX);
          DzVy = DZ(C_VY);
          DzVz = DZ(C_VZ);
        }
        hooke_iso(lam, mu, l2m, xix, xiy, xiz, etx, ety, etz, ztx, zty, ztz,
                  DxVx, DxVy, DxVz, DyVx, DyVy, DyVz, DzVx, DzVy, DzVz, r);
#undef DX
#undef DY
#undef DZ
      }
      if (a.free_top && k >= g.nk2 - (BZ == 0 ? 3 : 1)) {
        r[C_VX] = stimg_row<BX, BY, BZ>(a, w, cen, row, col, q, k, 0);
        r[C_VY] = stimg_row<BX, BY, BZ>(a, w, cen, row, col, q, k, 1);
        r[C_VZ] = stimg_row<BX, BY, BZ>(a, w, cen, row, col, q, k, 2);
      }

      /* CFS-PML, faces in reference order */
#pragma unroll 1
      for (int f = 0; f < CGFD_NFACE; f++) {
        const DevFace &F = a.face[f];
        if (!F.on || i < F.i1 || i > F.i2 || j < F.j1 || j > F.j2 ||
            k < F.k1 || k > F.k2)
          continue;
        Deriv9 d;
        sderiv9<BX, BY, BZ>(cen, w, row, col, F.dim, d);
        if (F.dim == 0)
          pml_face<KIND>(a, f, i, j, k, q, d, xix, xiy, xiz, lam, mu, l2m, slw, r);
        else if (F.dim == 1)
          pml_face<KIND>(a, f, i, j, k, q, d, etx, ety, etz, lam, mu, l2m, slw, r);
        else
          pml_face<KIND>(a, f, i, j, k, q, d, ztx, zty, ztz, lam, mu, l2m, slw, r);
      }

      /* sources */
      if (a.src_n > 0) {
        long long colidx = (long long)(i - g.ni1) + (long long)(j - g.nj1) * g.ni;
        int e0 = LDG(a.src_col + colidx), e1 = LDG(a.src_col + colidx + 1);
        if (e0 < e1) {
          int it = *a.d_it;
          for (int e = e0; e < e1; e++) {
            SrcEntry s = a.src_ent[e];
            if (s.k != k) continue;
            if (it < a.src_it_begin[s.is] || it > a.src_it_end[s.is]) continue;
            long long t = ((long long)s.is * a.src_max_nt +
                           (it - a.src_it_begin[s.is])) * a.src_max_stage + a.istage;
            if (a.src_force && s.force_on) {
              r[C_VX] += a.Fx[t] * s.vf;
              r[C_VY] += a.Fy[t] * s.vf;
              r[C_VZ] += a.Fz[t] * s.vf;
            }
            if (a.src_moment) {
              r[C_TXX] -= a.Mxx[t] * s.rjac;
              r[C_TYY] -= a.Myy[t] * s.rjac;
              r[C_TZZ] -= a.Mzz[t] * s.rjac;
              r[C_TXZ] -= a.Mxz[t] * s.rjac;
              r[C_TYZ] -= a.Myz[t] * s.rjac;
              r[C_TXY] -= a.Mxy[t] * s.rjac;
            }
          }
        }
      }

      /* RK combine */
#pragma unroll
      for (int c = 0; c < 9; c++) {
        long long x = c * vol + q;
        if (KIND == 0) {
          float p = cen[soff(c, row, col)]; /* cur is pre at stage 0 */
          a.tmp_out[x] = p + a.ca * r[c];
          a.end[x] = p + a.cb * r[c];
        } else if (KIND == 1) {
          a.tmp_out[x] = LDG(a.pre + x) + a.ca * r[c];
          a.end[x] = a.end[x] + a.cb * r[c];
        } else {
          a.end[x] = a.end[x] + a.cb * r[c];
        }
      }
    }

    /* the oldest window plane is free: refill its buffer two planes ahead */
    __syncthreads();
    if (tid == 0 && rtop + 2 < nplanes) {
      int rel = rtop + 2;
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      mbar_expect_tx(&bars[rel % NB], PLANE * 4);
      tma_load_5d(sm + (rel % NB) * PLANE, &tmap, bx0, by0, pbase + rel, 0,
                  a.cur_level, &bars[rel % NB]);
    }
  }
}

}  // namespace s2

#endif
