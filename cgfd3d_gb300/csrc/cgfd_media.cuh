/*
 * Medium policies of the stage and CFS-PML kernels (sm_103a).
 *
 * MED_ISO  isotropic elastic        (forward/sv_curv_col_el_iso.c)
 * MED_VTI  VTI elastic, 5 constants (forward/sv_curv_col_el_vti.c)
 * MED_VIS  GMB visco-elastic isotropic: the isotropic elastic operators
 *          plus 6 memory variables per Maxwell body
 *          (forward/sv_curv_col_vis_iso.c)
 * MED_ANI  fully anisotropic elastic, 21 constants
 *          (forward/sv_curv_col_el_aniso.c)
 *
 * Device media block (one padded volume per component, stride g.vol):
 *   iso  slw, lambda, mu
 *   vti  slw, c11, c13, c33, c55, c66
 *   vis  slw, lambda, mu, Ylam[0..nmw-1], Ymu[0..nmw-1]
 *   ani  slw, c11, c12, .., c16, c22, .., c26, c33, .., c66 (21)
 * slw is 1/rho, as the reference holds it (forward/md_t.c:601-623).
 */
#ifndef CGFD_MEDIA_CUH
#define CGFD_MEDIA_CUH

#include "cgfd_common.h"

enum { MED_ISO = 0, MED_VTI = 1, MED_VIS = 2, MED_ANI = 3 };

/* media components of the device block for a medium */
__host__ __device__ constexpr int med_ncomp(int med, int nmw)
{
  return med == MED_VTI ? 6 : med == MED_VIS ? 3 + 2 * nmw : med == MED_ANI ? 22 : 3;
}

/* elastic constants of one point */
struct MedPt {
  float slw;
  float lam, mu, l2m;                    /* iso, vis */
  float c11, c12, c13, c33, c55, c66;    /* vti */
  float c[21];                           /* ani: c11 c12 .. c16 c22 .. c66 */
};

/* C_IJ (Voigt indices 1..6, compile-time) of the packed anisotropic set */
template <int I, int J>
__device__ __forceinline__ float cij(const MedPt &m)
{
  constexpr int a = I < J ? I : J, b = I < J ? J : I;
  constexpr int off = a == 1 ? 0 : a == 2 ? 6 : a == 3 ? 11 : a == 4 ? 15 : a == 5 ? 18 : 20;
  return m.c[off + b - a];
}

/* anisotropic stress rates from the six strain-rate sums: exx, eyy, ezz
 * and the engineering shears gyz, gxz, gxy (rows Txx Tyy Tzz Tyz Txz Txy =
 * Voigt 1..6); algebraically the reference's expanded expression,
 * forward/sv_curv_col_el_aniso.c:453-470 */
__device__ __forceinline__ void ani_hooke(const MedPt &m, float exx, float eyy,
                                          float ezz, float gyz, float gxz,
                                          float gxy, float *r)
{
#define ANI_ROW(R)                                                              \
  (cij<R, 1>(m) * exx + cij<R, 2>(m) * eyy + cij<R, 3>(m) * ezz +              \
   cij<R, 4>(m) * gyz + cij<R, 5>(m) * gxz + cij<R, 6>(m) * gxy)
  r[C_TXX] = ANI_ROW(1);
  r[C_TYY] = ANI_ROW(2);
  r[C_TZZ] = ANI_ROW(3);
  r[C_TYZ] = ANI_ROW(4);
  r[C_TXZ] = ANI_ROW(5);
  r[C_TXY] = ANI_ROW(6);
#undef ANI_ROW
}

/* constants at p (component stride s); c12 = c11 - 2 c66
 * (forward/sv_curv_col_el_vti.c:351) */
template <int MED, bool GLOBAL>
__device__ __forceinline__ MedPt med_from(const float *p, long long s)
{
  MedPt m;
  auto ld = [&](long long o) { return GLOBAL ? __ldg(p + o) : p[o]; };
  m.slw = ld(0);
  if (MED == MED_ANI) {
#pragma unroll
    for (int n = 0; n < 21; n++) m.c[n] = ld((n + 1) * s);
    m.lam = m.mu = m.l2m = 0.f;
    m.c11 = m.c12 = m.c13 = m.c33 = m.c55 = m.c66 = 0.f;
  } else if (MED == MED_VTI) {
    m.c11 = ld(s); m.c13 = ld(2 * s); m.c33 = ld(3 * s);
    m.c55 = ld(4 * s); m.c66 = ld(5 * s);
    m.c12 = m.c11 - 2.0f * m.c66;
    m.lam = m.mu = m.l2m = 0.f;
  } else {
    m.lam = ld(s); m.mu = ld(2 * s);
    m.l2m = m.lam + 2.0f * m.mu;
    m.c11 = m.c12 = m.c13 = m.c33 = m.c55 = m.c66 = 0.f;
  }
  return m;
}

/* Hooke's law from the nine velocity gradients (interior and vlow):
 * forward/sv_curv_col_el_iso.c:409-435, forward/sv_curv_col_el_vti.c:366-389 */
template <int MED>
__device__ __forceinline__ void hooke9(const MedPt &m, float xix, float xiy,
                                       float xiz, float etx, float ety,
                                       float etz, float ztx, float zty,
                                       float ztz, float DxVx, float DxVy,
                                       float DxVz, float DyVx, float DyVy,
                                       float DyVz, float DzVx, float DzVy,
                                       float DzVz, float *r)
{
  if (MED == MED_ANI) {
    const float exx = xix * DxVx + etx * DyVx + ztx * DzVx;
    const float eyy = xiy * DxVy + ety * DyVy + zty * DzVy;
    const float ezz = xiz * DxVz + etz * DyVz + ztz * DzVz;
    const float gyz = xiz * DxVy + xiy * DxVz + etz * DyVy + ety * DyVz +
                      ztz * DzVy + zty * DzVz;
    const float gxz = xiz * DxVx + xix * DxVz + etz * DyVx + etx * DyVz +
                      ztz * DzVx + ztx * DzVz;
    const float gxy = xiy * DxVx + xix * DxVy + ety * DyVx + etx * DyVy +
                      zty * DzVx + ztx * DzVy;
    ani_hooke(m, exx, eyy, ezz, gyz, gxz, gxy, r);
  } else if (MED != MED_VTI) {
    const float lam = m.lam, mu = m.mu, l2m = m.l2m;
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
  } else {
    /* strain-rate sums first: each constant multiplies a metric-weighted
     * gradient sum (algebraically the reference's expression) */
    const float ex = xix * DxVx + etx * DyVx + ztx * DzVx;   /* d vx / dx */
    const float ey = xiy * DxVy + ety * DyVy + zty * DzVy;   /* d vy / dy */
    const float ez = xiz * DxVz + etz * DyVz + ztz * DzVz;   /* d vz / dz */
    r[C_TXX] = m.c11 * ex + m.c12 * ey + m.c13 * ez;
    r[C_TYY] = m.c12 * ex + m.c11 * ey + m.c13 * ez;
    r[C_TZZ] = m.c13 * ex + m.c13 * ey + m.c33 * ez;
    r[C_TYZ] = m.c55 * (xiz * DxVy + xiy * DxVz + etz * DyVy + ety * DyVz +
                        ztz * DzVy + zty * DzVz);
    r[C_TXZ] = m.c55 * (xiz * DxVx + xix * DxVz + etz * DyVx + etx * DyVz +
                        ztz * DzVx + ztx * DzVz);
    r[C_TXY] = m.c66 * (xiy * DxVx + xix * DxVy + ety * DyVx + etx * DyVy +
                        zty * DzVx + ztx * DzVy);
  }
}

/* Hooke's law with the gradients along one direction (metric e1..e3):
 * CFS-PML terms, forward/sv_curv_col_el_iso.c:806-811,
 * forward/sv_curv_col_el_vti.c:760-765; also the free-surface part of the
 * x/y faces at k = nk2 with the zeta metric (iso :863-877, vti :817-822) */
template <int MED>
__device__ __forceinline__ void hooke1(const MedPt &m, float e1, float e2,
                                       float e3, float DVx, float DVy,
                                       float DVz, float *s)
{
  if (MED == MED_ANI) {
    ani_hooke(m, e1 * DVx, e2 * DVy, e3 * DVz, e3 * DVy + e2 * DVz,
              e3 * DVx + e1 * DVz, e2 * DVx + e1 * DVy, s);
  } else if (MED != MED_VTI) {
    const float lam = m.lam, mu = m.mu, l2m = m.l2m;
    s[C_TXX] = l2m * e1 * DVx + lam * e2 * DVy + lam * e3 * DVz;
    s[C_TYY] = lam * e1 * DVx + l2m * e2 * DVy + lam * e3 * DVz;
    s[C_TZZ] = lam * e1 * DVx + lam * e2 * DVy + l2m * e3 * DVz;
    s[C_TXY] = mu * (e2 * DVx + e1 * DVy);
    s[C_TXZ] = mu * (e3 * DVx + e1 * DVz);
    s[C_TYZ] = mu * (e3 * DVy + e2 * DVz);
  } else {
    const float ex = e1 * DVx, ey = e2 * DVy, ez = e3 * DVz;
    s[C_TXX] = m.c11 * ex + m.c12 * ey + m.c13 * ez;
    s[C_TYY] = m.c12 * ex + m.c11 * ey + m.c13 * ez;
    s[C_TZZ] = m.c13 * ex + m.c13 * ey + m.c33 * ez;
    s[C_TYZ] = m.c55 * (e3 * DVy + e2 * DVz);
    s[C_TXZ] = m.c55 * (e3 * DVx + e1 * DVz);
    s[C_TXY] = m.c66 * (e2 * DVx + e1 * DVy);
  }
}

/* Strain rates implied by a stress rate h (6 components, C_TXX..C_TXY
 * order) for the GMB memory variables, forward/sv_curv_col_vis_iso.c:
 * 285-297: deviatoric part over 2 mu plus the mean part over 3 lam + 2 mu.
 * Output order xx, yy, zz, yz, xz, xy (the memory-variable order of
 * forward/wav_t.c:140-170). */
__device__ __forceinline__ void vis_strain_rate(float lam, float mu,
                                                const float *h, float *ev)
{
  const float hxx = h[C_TXX], hyy = h[C_TYY], hzz = h[C_TZZ];
  const float sum = (hxx + hyy + hzz) / (3.0f * lam + 2.0f * mu);
  const float i2mu = 1.0f / (2.0f * mu);
  ev[0] = ((2.0f * hxx - hyy - hzz) * i2mu + sum) * (1.0f / 3.0f);
  ev[1] = ((2.0f * hyy - hxx - hzz) * i2mu + sum) * (1.0f / 3.0f);
  ev[2] = ((2.0f * hzz - hxx - hyy) * i2mu + sum) * (1.0f / 3.0f);
  ev[3] = h[C_TYZ] * i2mu;
  ev[4] = h[C_TXZ] * i2mu;
  ev[5] = h[C_TXY] * i2mu;
}

/* memory-variable component c (xx,yy,zz,yz,xz,xy) -> stress component */
__host__ __device__ constexpr int vis_tcomp(int c)
{
  return c == 0 ? C_TXX : c == 1 ? C_TYY : c == 2 ? C_TZZ
       : c == 3 ? C_TYZ : c == 4 ? C_TXZ : C_TXY;
}

#endif
