/*
 * Per-point update of one RK stage for isotropic elastic media, sm_103a.
 *
 * One call computes, for one physical grid point, what the reference spreads
 * over five passes and three full-volume sweeps per stage
 * (forward/sv_curv_col_el_iso.c:22-202 then forward/drv_rk_curv_col.c:292-446):
 *
 *   r  = interior RHS                      (sv_curv_col_el_iso.c:304-440)
 *   r.V <- traction image at the top layers (sv_curv_col_el.c:84-304)
 *   r.T <- velocity-gradient "vlow" at the top three layers
 *                                          (sv_curv_col_el_iso.c:501-633)
 *   r += CFS-PML correction of each face containing the point, faces in the
 *        reference order x1,x2,y1,y2,z1,z2 (sv_curv_col_el_iso.c:708-1143),
 *        and the face's auxiliary variables are advanced in the same pass
 *   r += sources at this point, in source order (sv_curv_col_el.c:350-476)
 *   tmp = pre + a*dt*r ;  end = pre + b*dt*r  or  end += b*dt*r
 *
 * so the stage never stores r.  Template parameters fix the bias of the
 * x/y/z MacCormack operators (forward/fd_t.c:182-236): bias 0 uses the taps
 * -1..3, bias 1 the taps -3..1.  KIND: 0 first stage, 1 middle, 2 last.
 *
 * The traction image reads, at k = nk2 with z bias 0, the conservative flux
 * at mirror points k-2 and k-3 that the reference never computes (it reads
 * before the start of its local array); those terms are taken as 0, which is
 * what the reference computes when that memory holds (near) zero.
 */
#ifndef CGFD_STAGE_CUH
#define CGFD_STAGE_CUH

#include "cgfd_common.h"

#define LDG(p) __ldg(p)

template <int B>
__device__ __forceinline__ float dop(const float *__restrict__ p, long long s)
{
  if (B == 0)
    return -0.30874f * LDG(p - s) + -0.6326f * LDG(p) + 1.233f * LDG(p + s) +
           -0.3334f * LDG(p + 2 * s) + 0.04168f * LDG(p + 3 * s);
  else
    return -0.04168f * LDG(p - 3 * s) + 0.3334f * LDG(p - 2 * s) +
           -1.233f * LDG(p - s) + 0.6326f * LDG(p) + 0.30874f * LDG(p + s);
}

template <int B>
__device__ __forceinline__ int tap_shift(int n)
{
  return B == 0 ? n - 1 : n - 3;
}

template <int B>
__device__ __forceinline__ float tap_coef(int n)
{
  if (B == 0) {
    return n == 0 ? -0.30874f : n == 1 ? -0.6326f : n == 2 ? 1.233f
         : n == 3 ? -0.3334f : 0.04168f;
  } else {
    return n == 0 ? -0.04168f : n == 1 ? 0.3334f : n == 2 ? -1.233f
         : n == 3 ? 0.6326f : 0.30874f;
  }
}

struct Deriv9 {
  float Vx, Vy, Vz, Txx, Tyy, Tzz, Txz, Tyz, Txy;
};

template <int B>
__device__ __forceinline__ void deriv9(const float *__restrict__ w,
                                       long long q, long long vol,
                                       long long s, Deriv9 &d)
{
  d.Vx = dop<B>(w + C_VX * vol + q, s);
  d.Vy = dop<B>(w + C_VY * vol + q, s);
  d.Vz = dop<B>(w + C_VZ * vol + q, s);
  d.Txx = dop<B>(w + C_TXX * vol + q, s);
  d.Tyy = dop<B>(w + C_TYY * vol + q, s);
  d.Tzz = dop<B>(w + C_TZZ * vol + q, s);
  d.Txz = dop<B>(w + C_TXZ * vol + q, s);
  d.Tyz = dop<B>(w + C_TYZ * vol + q, s);
  d.Txy = dop<B>(w + C_TXY * vol + q, s);
}

/* J * (m1*Ta + m2*Tb + m3*Tc) at point q (conservative traction flux) */
__device__ __forceinline__ float cons_flux(const float *__restrict__ jac,
                                           const float *__restrict__ m1,
                                           const float *__restrict__ m2,
                                           const float *__restrict__ m3,
                                           const float *__restrict__ Ta,
                                           const float *__restrict__ Tb,
                                           const float *__restrict__ Tc,
                                           long long q)
{
  return LDG(jac + q) *
         (LDG(m1 + q) * LDG(Ta + q) + LDG(m2 + q) * LDG(Tb + q) +
          LDG(m3 + q) * LDG(Tc + q));
}

/* traction-image hV (row r: 0 x, 1 y, 2 z) at (i,j,k) */
template <int BX, int BY, int BZ>
__device__ float timg_row(const StageArgs &a, long long q, int k, int r)
{
  const long long vol = a.g.vol, nx = a.g.px, sl = a.g.sl;
  const float *w = a.cur;
  const float *Ta, *Tb, *Tc;
  if (r == 0) { Ta = w + C_TXX * vol; Tb = w + C_TXY * vol; Tc = w + C_TXZ * vol; }
  else if (r == 1) { Ta = w + C_TXY * vol; Tb = w + C_TYY * vol; Tc = w + C_TYZ * vol; }
  else { Ta = w + C_TXZ * vol; Tb = w + C_TYZ * vol; Tc = w + C_TZZ * vol; }
  float Dx = 0.f, Dy = 0.f, Dz = 0.f;
#pragma unroll
  for (int n = 0; n < 5; n++) {
    float vx = cons_flux(a.jac, a.xix, a.xiy, a.xiz, Ta, Tb, Tc, q + tap_shift<BX>(n));
    float vy = cons_flux(a.jac, a.etx, a.ety, a.etz, Ta, Tb, Tc,
                         q + (long long)tap_shift<BY>(n) * nx);
    Dx += tap_coef<BX>(n) * vx;
    Dy += tap_coef<BY>(n) * vy;
  }
  const int nk2 = a.g.nk2;
  const int klow = k + tap_shift<BZ>(0); /* lowest computed tap */
#pragma unroll
  for (int n = 0; n < 5; n++) {
    int kk = k + tap_shift<BZ>(n);
    float v;
    if (kk < nk2) {
      v = cons_flux(a.jac, a.ztx, a.zty, a.ztz, Ta, Tb, Tc, q + (long long)(kk - k) * sl);
    } else if (kk == nk2) {
      v = 0.f; /* surface traction (no surface force) */
    } else {
      int km = 2 * nk2 - kk; /* image point */
      v = (km >= klow)
              ? -cons_flux(a.jac, a.ztx, a.zty, a.ztz, Ta, Tb, Tc, q + (long long)(km - k) * sl)
              : 0.f;
    }
    Dz += tap_coef<BZ>(n) * v;
  }
  float slwjac = LDG(a.slw + q) / LDG(a.jac + q);
  return (Dx + Dy + Dz) * slwjac;
}

/* Hooke's law for the isotropic medium from the 9 velocity gradients */
__device__ __forceinline__ void hooke_iso(float lam, float mu, float l2m,
                                          float xix, float xiy, float xiz,
                                          float etx, float ety, float etz,
                                          float ztx, float zty, float ztz,
                                          float DxVx, float DxVy, float DxVz,
                                          float DyVx, float DyVy, float DyVz,
                                          float DzVx, float DzVy, float DzVz,
                                          float *r)
{
  r[C_TXX] = l2m * (xix * DxVx + etx * DyVx + ztx * DzVx) +
             lam * (xiy * DxVy + ety * DyVy + zty * DzVy + xiz * DxVz +
                    etz * DyVz + ztz * DzVz);
  r[C_TYY] = l2m * (xiy * DxVy + ety * DyVy + zty * DzVy) +
             lam * (xix * DxVx + etx * DyVx + ztx * DzVx + xiz * DxVz +
                    etz * DyVz + ztz * DzVz);
  r[C_TZZ] = l2m * (xiz * DxVz + etz * DyVz + ztz * DzVz) +
             lam * (xix * DxVx + etx * DyVx + ztx * DzVx + xiy * DxVy +
                    ety * DyVy + zty * DzVy);
  r[C_TXY] = mu * (xiy * DxVx + xix * DxVy + ety * DyVx + etx * DyVy +
                   zty * DzVx + ztx * DzVy);
  r[C_TXZ] = mu * (xiz * DxVx + xix * DxVz + etz * DyVx + etx * DyVz +
                   ztz * DzVx + ztx * DzVz);
  r[C_TYZ] = mu * (xiz * DxVy + xiy * DxVz + etz * DyVy + ety * DyVz +
                   ztz * DzVy + zty * DzVz);
}

/* CFS-PML correction of one face at one point; advances the face's aux */
template <int KIND>
__device__ __forceinline__ void pml_face(const StageArgs &a, int f, int i,
                                         int j, int k, long long q,
                                         const Deriv9 &d, float e1, float e2,
                                         float e3, float lam, float mu,
                                         float l2m, float slw, float *r)
{
  const DevFace &F = a.face[f];
  int n = F.dim == 0 ? i - F.i1 : (F.dim == 1 ? j - F.j1 : k - F.k1);
  long long ai = (long long)(i - F.i1) + (long long)(j - F.j1) * F.bx +
                 (long long)(k - F.k1) * F.bx * F.by;
  float cD = LDG(F.D + n), cA = LDG(F.A + n), cB = LDG(F.B + n);
  float cB1 = cB - 1.0f;
  float s[9];
  s[C_VX] = slw * (e1 * d.Txx + e2 * d.Txy + e3 * d.Txz);
  s[C_VY] = slw * (e1 * d.Txy + e2 * d.Tyy + e3 * d.Tyz);
  s[C_VZ] = slw * (e1 * d.Txz + e2 * d.Tyz + e3 * d.Tzz);
  s[C_TXX] = l2m * e1 * d.Vx + lam * e2 * d.Vy + lam * e3 * d.Vz;
  s[C_TYY] = lam * e1 * d.Vx + l2m * e2 * d.Vy + lam * e3 * d.Vz;
  s[C_TZZ] = lam * e1 * d.Vx + lam * e2 * d.Vy + l2m * e3 * d.Vz;
  s[C_TXY] = mu * (e2 * d.Vx + e1 * d.Vy);
  s[C_TXZ] = mu * (e3 * d.Vx + e1 * d.Vz);
  s[C_TYZ] = mu * (e3 * d.Vy + e2 * d.Vz);
  const long long av = F.avol;
  const float *acur = a.acur[f];
  float arhs[9];
#pragma unroll
  for (int c = 0; c < 9; c++) {
    float ac = LDG(acur + c * av + ai);
    r[c] += cB1 * s[c] - cB * ac;
    arhs[c] = cD * s[c] - cA * ac;
  }
  if (F.dim < 2 && a.free_top && k == a.g.nk2) {
    long long ij = ((long long)i + (long long)j * a.g.nx) * 9;
    const float *M = (F.dim == 0 ? a.mVx : a.mVy) + ij;
    float DzVx = LDG(M + 0) * d.Vx + LDG(M + 1) * d.Vy + LDG(M + 2) * d.Vz;
    float DzVy = LDG(M + 3) * d.Vx + LDG(M + 4) * d.Vy + LDG(M + 5) * d.Vz;
    float DzVz = LDG(M + 6) * d.Vx + LDG(M + 7) * d.Vy + LDG(M + 8) * d.Vz;
    float ztx = LDG(a.ztx + q), zty = LDG(a.zty + q), ztz = LDG(a.ztz + q);
    float t[9];
    t[C_TXX] = l2m * (ztx * DzVx) + lam * (zty * DzVy + ztz * DzVz);
    t[C_TYY] = l2m * (zty * DzVy) + lam * (ztx * DzVx + ztz * DzVz);
    t[C_TZZ] = l2m * (ztz * DzVz) + lam * (ztx * DzVx + zty * DzVy);
    t[C_TXY] = mu * (zty * DzVx + ztx * DzVy);
    t[C_TXZ] = mu * (ztz * DzVx + ztx * DzVz);
    t[C_TYZ] = mu * (ztz * DzVy + zty * DzVz);
#pragma unroll
    for (int c = C_TXX; c <= C_TXY; c++) {
      r[c] += cB1 * t[c];
      arhs[c] += cD * t[c];
    }
  }
  /* RK combine of the auxiliary variables */
  const float *apre = a.apre[f];
  float *aend = a.aend[f];
#pragma unroll
  for (int c = 0; c < 9; c++) {
    long long x = c * av + ai;
    if (KIND == 0) {
      float p = LDG(apre + x);
      a.atmp_out[f][x] = p + a.ca * arhs[c];
      aend[x] = p + a.cb * arhs[c];
    } else if (KIND == 1) {
      a.atmp_out[f][x] = LDG(apre + x) + a.ca * arhs[c];
      aend[x] = aend[x] + a.cb * arhs[c];
    } else {
      aend[x] = aend[x] + a.cb * arhs[c];
    }
  }
}

template <int BX, int BY, int BZ, int KIND>
__device__ __forceinline__ void stage_point(const StageArgs &a, int i, int j,
                                            int k)
{
  const DevGrid &g = a.g;
  const long long vol = g.vol, nx = g.px, sl = g.sl;
  const long long q = (long long)(i + g.xoff) + (long long)j * nx + (long long)k * sl;
  const float *w = a.cur;

  Deriv9 dx, dy, dz;
  deriv9<BX>(w, q, vol, 1, dx);
  deriv9<BY>(w, q, vol, nx, dy);
  deriv9<BZ>(w, q, vol, sl, dz);

  float xix = LDG(a.xix + q), xiy = LDG(a.xiy + q), xiz = LDG(a.xiz + q);
  float etx = LDG(a.etx + q), ety = LDG(a.ety + q), etz = LDG(a.etz + q);
  float ztx = LDG(a.ztx + q), zty = LDG(a.zty + q), ztz = LDG(a.ztz + q);
  float lam = LDG(a.lam + q), mu = LDG(a.mu + q), slw = LDG(a.slw + q);
  float l2m = lam + 2.0f * mu;

  float r[9];
  r[C_VX] = slw * (xix * dx.Txx + xiy * dx.Txy + xiz * dx.Txz +
                   etx * dy.Txx + ety * dy.Txy + etz * dy.Txz +
                   ztx * dz.Txx + zty * dz.Txy + ztz * dz.Txz);
  r[C_VY] = slw * (xix * dx.Txy + xiy * dx.Tyy + xiz * dx.Tyz +
                   etx * dy.Txy + ety * dy.Tyy + etz * dy.Tyz +
                   ztx * dz.Txy + zty * dz.Tyy + ztz * dz.Tyz);
  r[C_VZ] = slw * (xix * dx.Txz + xiy * dx.Tyz + xiz * dx.Tzz +
                   etx * dy.Txz + ety * dy.Tyz + etz * dy.Tzz +
                   ztx * dz.Txz + zty * dz.Tyz + ztz * dz.Tzz);

  const int nk2 = g.nk2;
  if (a.free_top && k >= nk2 - 2) {
    /* vlow: z-derivatives of V replaced near the surface */
    float DzVx, DzVy, DzVz;
    if (k == nk2) {
      long long ij = ((long long)i + (long long)j * g.nx) * 9;
      const float *A = a.mVx + ij, *Bm = a.mVy + ij;
      DzVx = LDG(A + 0) * dx.Vx + LDG(A + 1) * dx.Vy + LDG(A + 2) * dx.Vz +
             LDG(Bm + 0) * dy.Vx + LDG(Bm + 1) * dy.Vy + LDG(Bm + 2) * dy.Vz;
      DzVy = LDG(A + 3) * dx.Vx + LDG(A + 4) * dx.Vy + LDG(A + 5) * dx.Vz +
             LDG(Bm + 3) * dy.Vx + LDG(Bm + 4) * dy.Vy + LDG(Bm + 5) * dy.Vz;
      DzVz = LDG(A + 6) * dx.Vx + LDG(A + 7) * dx.Vy + LDG(A + 8) * dx.Vz +
             LDG(Bm + 6) * dy.Vx + LDG(Bm + 7) * dy.Vy + LDG(Bm + 8) * dy.Vz;
    } else {
      const float *Vx = w + C_VX * vol + q, *Vy = w + C_VY * vol + q,
                  *Vz = w + C_VZ * vol + q;
      if (k == nk2 - 1) {
        /* second order: {0,1} or {-1,0}, coefficients -1, 1 */
        long long s0 = BZ == 0 ? 0 : -sl, s1 = BZ == 0 ? sl : 0;
        DzVx = -LDG(Vx + s0) + LDG(Vx + s1);
        DzVy = -LDG(Vy + s0) + LDG(Vy + s1);
        DzVz = -LDG(Vz + s0) + LDG(Vz + s1);
      } else {
        /* fourth order: {0,1,2} or {-2,-1,0} */
        const float c0 = BZ == 0 ? (float)(-7.0 / 6.0) : (float)(1.0 / 6.0);
        const float c1 = BZ == 0 ? (float)(8.0 / 6.0) : (float)(-8.0 / 6.0);
        const float c2 = BZ == 0 ? (float)(-1.0 / 6.0) : (float)(7.0 / 6.0);
        long long s0 = BZ == 0 ? 0 : -2 * sl, s1 = BZ == 0 ? sl : -sl,
                  s2 = BZ == 0 ? 2 * sl : 0;
        DzVx = c0 * LDG(Vx + s0) + c1 * LDG(Vx + s1) + c2 * LDG(Vx + s2);
        DzVy = c0 * LDG(Vy + s0) + c1 * LDG(Vy + s1) + c2 * LDG(Vy + s2);
        DzVz = c0 * LDG(Vz + s0) + c1 * LDG(Vz + s1) + c2 * LDG(Vz + s2);
      }
    }
    hooke_iso(lam, mu, l2m, xix, xiy, xiz, etx, ety, etz, ztx, zty, ztz,
              dx.Vx, dx.Vy, dx.Vz, dy.Vx, dy.Vy, dy.Vz, DzVx, DzVy, DzVz, r);
  } else {
    hooke_iso(lam, mu, l2m, xix, xiy, xiz, etx, ety, etz, ztx, zty, ztz,
              dx.Vx, dx.Vy, dx.Vz, dy.Vx, dy.Vy, dy.Vz, dz.Vx, dz.Vy, dz.Vz, r);
  }
  if (a.free_top && k >= nk2 - (BZ == 0 ? 3 : 1)) {
    r[C_VX] = timg_row<BX, BY, BZ>(a, q, k, 0);
    r[C_VY] = timg_row<BX, BY, BZ>(a, q, k, 1);
    r[C_VZ] = timg_row<BX, BY, BZ>(a, q, k, 2);
  }

  /* CFS-PML, faces in reference order */
#pragma unroll 1
  for (int f = 0; f < CGFD_NFACE; f++) {
    const DevFace &F = a.face[f];
    if (!F.on || i < F.i1 || i > F.i2 || j < F.j1 || j > F.j2 || k < F.k1 ||
        k > F.k2)
      continue;
    if (F.dim == 0)
      pml_face<KIND>(a, f, i, j, k, q, dx, xix, xiy, xiz, lam, mu, l2m, slw, r);
    else if (F.dim == 1)
      pml_face<KIND>(a, f, i, j, k, q, dy, etx, ety, etz, lam, mu, l2m, slw, r);
    else
      pml_face<KIND>(a, f, i, j, k, q, dz, ztx, zty, ztz, lam, mu, l2m, slw, r);
  }

  /* sources */
  if (a.src_n > 0) {
    long long col = (long long)(i - g.ni1) + (long long)(j - g.nj1) * g.ni;
    int e0 = LDG(a.src_col + col), e1 = LDG(a.src_col + col + 1);
    if (e0 < e1) {
      int it = *a.d_it;
      for (int e = e0; e < e1; e++) {
        SrcEntry s = a.src_ent[e];
        if (s.k != k) continue;
        if (it < a.src_it_begin[s.is] || it > a.src_it_end[s.is]) continue;
        long long t = ((long long)s.is * a.src_max_nt + (it - a.src_it_begin[s.is])) *
                          a.src_max_stage + a.istage;
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
      float p = LDG(a.pre + x);
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

#endif
