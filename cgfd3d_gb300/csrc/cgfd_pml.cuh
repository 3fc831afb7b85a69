/*
 * CFS-PML face kernel (ADE, unsplit), one launch per enabled face per stage.
 *
 * The interior stage kernel (cgfd_stage3.cuh) writes tmp = pre + a*dt*r and
 * end (+)= b*dt*r with r the RHS without PML terms.  The PML terms of the
 * reference (forward/sv_curv_col_el_iso.c:708-1143) are linear additions to
 * r, so this kernel adds them afterwards:
 *
 *   corr = (B-1) * r_d - B * aux_cur        (+ the free-surface term of
 *                                             x/y faces at k = nk2)
 *   aux_rhs = D * r_d - A * aux_cur
 *   tmp += a*dt*corr ;  end += b*dt*corr ;  aux levels advanced by RK4
 *
 * where r_d is the part of the RHS made of derivatives along the face normal.
 * Faces are launched in the reference order x1, x2, y1, y2, z1, z2, so a
 * corner point receives its corrections in the same order.  Rounding differs
 * from the reference only by the association (pre + a r) + a corr versus
 * pre + a (r + corr).
 *
 * One thread per point of the face box, linear index with i fastest, plain
 * coalesced loads (the face boxes are thin; their operands are read once).
 *
 * MED selects Hooke's law (cgfd_media.cuh; VTI: forward/sv_curv_col_el_vti.c:
 * 592-1075).  For the GMB visco-elastic medium the reference's attenuation
 * pass reads hT after the PML corrections (forward/sv_curv_col_vis_iso.c:
 * 200-232); its memory-variable rates are linear in hT, so this kernel also
 * adds wl_n EV(corr) to the memory variables' tmp/end.
 */
#ifndef CGFD_PML_CUH
#define CGFD_PML_CUH

#include "cgfd_common.h"
#include "cgfd_media.cuh"
#include "cgfd_stage.cuh"

template <int DIM, int B, int KIND, int MED>
__global__ void __launch_bounds__(256)
    k_pml_face(const __grid_constant__ StageArgs a, int f)
{
  const DevFace &F = a.face[f];
  const long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (n >= F.avol) return;
  const int bxy = F.bx * F.by;
  const int ii = (int)(n % F.bx);
  const int jj = (int)((n / F.bx) % F.by);
  const int kk = (int)(n / bxy);
  const int i = F.i1 + ii, j = F.j1 + jj, k = F.k1 + kk;
  const DevGrid &g = a.g;
  const long long vol = g.vol;
  const long long q = (long long)(i + g.xoff) + (long long)j * g.px + (long long)k * g.sl;
  const long long s = DIM == 0 ? 1 : (DIM == 1 ? (long long)g.px : g.sl);

  const float *e1p = DIM == 0 ? a.xix : (DIM == 1 ? a.etx : a.ztx);
  const float *e2p = DIM == 0 ? a.xiy : (DIM == 1 ? a.ety : a.zty);
  const float *e3p = DIM == 0 ? a.xiz : (DIM == 1 ? a.etz : a.ztz);
  float e1 = LDG(e1p + q), e2 = LDG(e2p + q), e3 = LDG(e3p + q);
  const MedPt m = med_from<MED, true>(a.med + q, vol);
  const float slw = m.slw;

  Deriv9 d;
  deriv9<B>(a.cur, q, vol, s, d);

  const int nidx = DIM == 0 ? ii : (DIM == 1 ? jj : kk);
  float cD = LDG(F.D + nidx), cA = LDG(F.A + nidx), cB = LDG(F.B + nidx);
  float cB1 = cB - 1.0f;
  float sv[9];
  sv[C_VX] = slw * (e1 * d.Txx + e2 * d.Txy + e3 * d.Txz);
  sv[C_VY] = slw * (e1 * d.Txy + e2 * d.Tyy + e3 * d.Tyz);
  sv[C_VZ] = slw * (e1 * d.Txz + e2 * d.Tyz + e3 * d.Tzz);
  hooke1<MED>(m, e1, e2, e3, d.Vx, d.Vy, d.Vz, sv);

  const long long av = F.avol;
  const float *acur = a.acur[f];
  float corr[9], arhs[9];
#pragma unroll
  for (int c = 0; c < 9; c++) {
    float ac = LDG(acur + c * av + n);
    corr[c] = cB1 * sv[c] - cB * ac;
    arhs[c] = cD * sv[c] - cA * ac;
  }
  if (DIM < 2 && a.free_top && k == g.nk2) {
    long long ij = ((long long)i + (long long)j * g.nx) * 9;
    const float *M = (DIM == 0 ? a.mVx : a.mVy) + ij;
    float DzVx = LDG(M + 0) * d.Vx + LDG(M + 1) * d.Vy + LDG(M + 2) * d.Vz;
    float DzVy = LDG(M + 3) * d.Vx + LDG(M + 4) * d.Vy + LDG(M + 5) * d.Vz;
    float DzVz = LDG(M + 6) * d.Vx + LDG(M + 7) * d.Vy + LDG(M + 8) * d.Vz;
    float ztx = LDG(a.ztx + q), zty = LDG(a.zty + q), ztz = LDG(a.ztz + q);
    float t[9];
    hooke1<MED>(m, ztx, zty, ztz, DzVx, DzVy, DzVz, t);
#pragma unroll
    for (int c = C_TXX; c <= C_TXY; c++) {
      corr[c] += cB1 * t[c];
      arhs[c] += cD * t[c];
    }
  }

  /* auxiliary RK combine and the corrections of tmp / end */
  const float *apre = a.apre[f];
  float *aend = a.aend[f];
#pragma unroll
  for (int c = 0; c < 9; c++) {
    long long xa = c * av + n;
    long long x = c * vol + q;
    if (KIND == 0) {
      float p = LDG(apre + xa);
      a.atmp_out[f][xa] = p + a.ca * arhs[c];
      aend[xa] = p + a.cb * arhs[c];
      a.tmp_out[x] += a.ca * corr[c];
      a.end[x] += a.cb * corr[c];
    } else if (KIND == 1) {
      a.atmp_out[f][xa] = LDG(apre + xa) + a.ca * arhs[c];
      aend[xa] = aend[xa] + a.cb * arhs[c];
      a.tmp_out[x] += a.ca * corr[c];
      a.end[x] += a.cb * corr[c];
    } else {
      aend[xa] = aend[xa] + a.cb * arhs[c];
      a.end[x] += a.cb * corr[c];
    }
  }
  if (MED == MED_VIS) {
    /* memory-variable rates of the correction: wl_n EV(corr) */
    float ev[6];
    vis_strain_rate(m.lam, m.mu, corr, ev);
#pragma unroll
    for (int n = 0; n < CGFD_VIS_NMW_MAX; n++) {
      if (n >= a.nmw) break;
#pragma unroll
      for (int c = 0; c < 6; c++) {
        long long x = (long long)(9 + 6 * n + c) * vol + q;
        float h = a.wl[n] * ev[c];
        if (KIND <= 1) a.tmp_out[x] += a.ca * h;
        a.end[x] += a.cb * h;
      }
    }
  }
}

#endif
