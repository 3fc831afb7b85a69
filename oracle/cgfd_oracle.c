/*
 * cgfd_oracle.c -- CPU restatement of the CGFD3D time-stepping hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker the GPU library is
 * compared against: tests/, __graft_entry__.smoke() and the cpu_baseline leg
 * of bench.py may load it; the product path never does.
 *
 * It restates, for the flat problem description of include/cgfd3d_gpu.h,
 * what the reference's drv_rk_curv_col_allstep does for isotropic elastic,
 * VTI elastic, fully anisotropic elastic and GMB visco-elastic isotropic media (the float arithmetic
 * is ordered as in the reference so that the results are bit-identical to
 * the reference's own CPU build, which is checked against the golden
 * fixtures under tests/golden/):
 *
 *   time loop, pair/stage schedule, RK4 combine
 *                        forward/drv_rk_curv_col.c:167-544, fd_t.c:36-49,182-289
 *   operator tables      forward/fd_t.c:75-122 (MacCormack DRP + surface ops)
 *   interior RHS         forward/sv_curv_col_el_iso.c:208-441
 *   traction image       forward/sv_curv_col_el.c:30-305
 *   velocity "vlow"      forward/sv_curv_col_el_iso.c:451-634
 *   ADE CFS-PML          forward/sv_curv_col_el_iso.c:644-1146
 *   source injection     forward/sv_curv_col_el.c:311-479, src_t.c:2111-2151
 *   distributed sources  forward/sv_curv_col_el.c:487-590
 *   surface force layers forward/src_t.c:153-314 (traction and velocity-rate
 *                        layers of the forces whose spread reaches the
 *                        surface, used by the traction image and vlow)
 *   receivers / lines    forward/io_funcs.c:1584-1645
 *   free-surface matrices forward/sv_curv_col_el_iso.c:1258-1375,
 *                        lib/fdlib_math.c:8-48
 *   grid metrics         forward/gd_t.c:190-402 (set-up, restated for the
 *                        device metric calculation's parity)
 *   VTI media            forward/sv_curv_col_el_vti.c:200-397 (interior),
 *                        :407-590 (vlow), :592-1075 (CFS-PML),
 *                        :1085-1206 (free-surface matrices)
 *   anisotropic media    forward/sv_curv_col_el_aniso.c:234-503 (interior),
 *                        :507-716 (vlow), :718-1265 (CFS-PML),
 *                        :1267-1423 (free-surface matrices)
 *   GMB visco-elastic    forward/sv_curv_col_vis_iso.c:22-245 (stage order),
 *                        :250-347 (attenuation), :353-507 (free-surface
 *                        matrices), :509-623 (surface stress rotation, after
 *                        the last stage: forward/drv_rk_curv_col.c:440-445)
 *
 * Multi-threaded with pthreads (one slab of k-planes per thread) so that it
 * can serve as the host-core baseline.
 */
#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "cgfd3d_gpu.h"

/* ------------------------------------------------------------------------ */
/* operator tables                                                          */
/* ------------------------------------------------------------------------ */

/* bias 0: taps at -1..3; bias 1: taps at -3..1 (fd_t.c:75-122, layer 3) */
static const int OP_SHIFT[2][5] = {{-1, 0, 1, 2, 3}, {-3, -2, -1, 0, 1}};
static const float OP_COEF[2][5] = {
  {-0.30874f, -0.6326f, 1.233f, -0.3334f, 0.04168f},
  {-0.04168f, 0.3334f, -1.233f, 0.6326f, 0.30874f}};
/* z operators of the two layers below the surface (fd_t.c:81-99):
 * layer 1 (k = nk2-1) second order, layer 2 (k = nk2-2) fourth order */
static const int OPZ1_SHIFT[2][2] = {{0, 1}, {-1, 0}};
static const float OPZ1_COEF[2][2] = {{-1.0f, 1.0f}, {-1.0f, 1.0f}};
static const int OPZ2_SHIFT[2][3] = {{0, 1, 2}, {-2, -1, 0}};
static const float OPZ2_COEF[2][3] = {
  {(float)(-7.0 / 6.0), (float)(8.0 / 6.0), (float)(-1.0 / 6.0)},
  {(float)(1.0 / 6.0), (float)(-8.0 / 6.0), (float)(7.0 / 6.0)}};
/* forward/backward flags of the 8 pairs (fd_t.c:185-195) */
static const int PAIR_FLAGS[8][3] = {{0, 0, 0}, {1, 1, 0}, {1, 1, 1}, {0, 0, 1},
                                     {0, 1, 0}, {1, 0, 0}, {1, 0, 1}, {0, 1, 1}};
static const float RK_A[3] = {0.5f, 0.5f, 1.0f};
static const float RK_B[4] = {(float)(1.0 / 6.0), (float)(1.0 / 3.0),
                              (float)(1.0 / 3.0), (float)(1.0 / 6.0)};

/* 5-tap derivative, evaluated left to right as in M_FD_SHIFT_PTR_MACDRP */
static inline float d5(const float *p, const float *c, long s0, long s1,
                       long s2, long s3, long s4)
{
  return c[0] * p[s0] + c[1] * p[s1] + c[2] * p[s2] + c[3] * p[s3] +
         c[4] * p[s4];
}

typedef struct {
  const float *c;
  long s[5];
} op5_t;

static op5_t make_op(int bias, long stride)
{
  op5_t o;
  o.c = OP_COEF[bias];
  for (int n = 0; n < 5; n++) o.s[n] = OP_SHIFT[bias][n] * stride;
  return o;
}

static inline float D5(const op5_t *o, const float *p)
{
  return d5(p, o->c, o->s[0], o->s[1], o->s[2], o->s[3], o->s[4]);
}

/* ------------------------------------------------------------------------ */
/* state                                                                    */
/* ------------------------------------------------------------------------ */

enum { VX, VY, VZ, TXX, TYY, TZZ, TYZ, TXZ, TXY };

typedef struct {
  const cgfd_problem_t *p;
  size_t vol, sl, ln;        /* volume, slice, line strides */
  float *lev[4];             /* pre, tmp, rhs, end (rotating pre/end) */
  float *aux[3][2][4];
  size_t aux_vol[3][2];
  float *mVx, *mVy, *mF;     /* free-surface matrices, 9 per (i,j) */
  float *mD;                 /* visco: surface rotation matrix, 9 per (i,j) */
  int med;                   /* medium_type */
  float **ext;               /* per source Gaussian weights (or NULL) */
  float *TS, *VS;            /* surface force layers: Tx,Ty,Tz / Vx,Vy,Vz Src,
                                3 x nx*ny each (NULL without surface forces) */
  int nthreads;
  int timg_mode;
  float *pg, *dis;           /* peak-motion maps (NULL: not computed) */
  pthread_barrier_t bar;
} orc_t;

typedef struct {
  orc_t *o;
  int tid;
} thr_t;

static inline float lam2mu_of(float lam, float mu)
{
  return (float)((double)lam + 2.0 * (double)mu);
}

/* ------------------------------------------------------------------------ */
/* media                                                                    */
/* ------------------------------------------------------------------------ */

/* elastic constants of one point: isotropic (lam, mu, l2m) or VTI (c11,
 * c12 = c11 - 2 c66 evaluated in double as the reference's `2.0 *` does,
 * c13, c33, c55, c66; forward/sv_curv_col_el_vti.c:345-351) */
typedef struct {
  int vti, aniso;
  float lam, mu, l2m;
  float c11, c12, c13, c33, c55, c66;
  float c[21];      /* anisotropic: c11 c12 .. c16 c22 .. c26 c33 .. c66 */
} med_t;

/* C_IJ (Voigt indices 1..6) of the packed anisotropic constants */
static inline float cij(const med_t *m, int I, int J)
{
  static const int off[7] = {0, 0, 6, 11, 15, 18, 20};
  if (I > J) { int t = I; I = J; J = t; }
  return m->c[off[I] + J - I];
}

/* Voigt index of the strain component (a, b), a, b in x, y, z = 0, 1, 2 */
static inline int voigt(int a, int b)
{
  static const int v[3][3] = {{1, 6, 5}, {6, 2, 4}, {5, 4, 3}};
  return v[a][b];
}

/* the reference's factor of output row R and velocity component v for a
 * metric direction (m0, m1, m2): C(R,V(v,x))*m0 + C(R,V(v,y))*m1 +
 * C(R,V(v,z))*m2 (forward/sv_curv_col_el_aniso.c:453-470) */
static inline float ani_f(const med_t *m, int R, int v, float m0, float m1, float m2)
{
  return cij(m, R, voigt(v, 0)) * m0 + cij(m, R, voigt(v, 1)) * m1 +
         cij(m, R, voigt(v, 2)) * m2;
}

/* output rows in the reference's order hTxx hTyy hTzz hTyz hTxz hTxy */
static const int ANI_ROW_COMP[6] = {TXX, TYY, TZZ, TYZ, TXZ, TXY};

static inline void med_at(const cgfd_problem_t *p, size_t q, med_t *m)
{
  memset(m, 0, sizeof(*m));
  if (p->medium_type == CGFD_MEDIUM_ELASTIC_ANISO) {
    const float *c[21] = {p->c11, p->c12, p->c13, p->c14, p->c15, p->c16, p->c22,
                          p->c23, p->c24, p->c25, p->c26, p->c33, p->c34, p->c35,
                          p->c36, p->c44, p->c45, p->c46, p->c55, p->c56, p->c66};
    m->aniso = 1;
    for (int n = 0; n < 21; n++) m->c[n] = c[n][q];
    return;
  }
  if (p->medium_type == CGFD_MEDIUM_ELASTIC_VTI) {
    m->vti = 1;
    m->c11 = p->c11[q]; m->c13 = p->c13[q]; m->c33 = p->c33[q];
    m->c55 = p->c55[q]; m->c66 = p->c66[q];
    m->c12 = (float)((double)m->c11 - 2.0 * (double)m->c66);
  } else {
    m->vti = 0;
    m->lam = p->lambda[q];
    m->mu = p->mu[q];
    m->l2m = (float)((double)m->lam + 2.0 * (double)m->mu);
  }
}

/* Hooke's law with all nine velocity gradients (interior and vlow):
 * isotropic forward/sv_curv_col_el_iso.c:409-435, VTI
 * forward/sv_curv_col_el_vti.c:366-389 (same expression order) */
static inline void hooke9(const med_t *m, float xix, float xiy, float xiz,
                          float etx, float ety, float etz, float ztx,
                          float zty, float ztz, float DxVx, float DxVy,
                          float DxVz, float DyVx, float DyVy, float DyVz,
                          float DzVx, float DzVy, float DzVz, float *h,
                          size_t V, size_t q)
{
  if (m->aniso) {
    /* forward/sv_curv_col_el_aniso.c:453-470: nine terms, xi / eta / zeta
     * gradients in turn, x y z velocity in each */
    const float mt[3][3] = {{xix, xiy, xiz}, {etx, ety, etz}, {ztx, zty, ztz}};
    const float D[3][3] = {{DxVx, DxVy, DxVz}, {DyVx, DyVy, DyVz}, {DzVx, DzVy, DzVz}};
    for (int r = 0; r < 6; r++) {
      float acc = ani_f(m, r + 1, 0, mt[0][0], mt[0][1], mt[0][2]) * D[0][0];
      for (int t = 1; t < 9; t++) {
        int d = t / 3, v = t % 3;
        acc = acc + ani_f(m, r + 1, v, mt[d][0], mt[d][1], mt[d][2]) * D[d][v];
      }
      h[ANI_ROW_COMP[r] * V + q] = acc;
    }
    return;
  }
  if (!m->vti) {
    float lam = m->lam, mu = m->mu, l2m = m->l2m;
    h[TXX * V + q] = l2m * (xix * DxVx + etx * DyVx + ztx * DzVx) +
                     lam * (xiy * DxVy + ety * DyVy + zty * DzVy +
                            xiz * DxVz + etz * DyVz + ztz * DzVz);
    h[TYY * V + q] = l2m * (xiy * DxVy + ety * DyVy + zty * DzVy) +
                     lam * (xix * DxVx + etx * DyVx + ztx * DzVx +
                            xiz * DxVz + etz * DyVz + ztz * DzVz);
    h[TZZ * V + q] = l2m * (xiz * DxVz + etz * DyVz + ztz * DzVz) +
                     lam * (xix * DxVx + etx * DyVx + ztx * DzVx +
                            xiy * DxVy + ety * DyVy + zty * DzVy);
    h[TXY * V + q] = mu * (xiy * DxVx + xix * DxVy + ety * DyVx +
                           etx * DyVy + zty * DzVx + ztx * DzVy);
    h[TXZ * V + q] = mu * (xiz * DxVx + xix * DxVz + etz * DyVx +
                           etx * DyVz + ztz * DzVx + ztx * DzVz);
    h[TYZ * V + q] = mu * (xiz * DxVy + xiy * DxVz + etz * DyVy +
                           ety * DyVz + ztz * DzVy + zty * DzVz);
    return;
  }
  float c11 = m->c11, c12 = m->c12, c13 = m->c13, c33 = m->c33,
        c55 = m->c55, c66 = m->c66;
  h[TXX * V + q] = (c11 * xix) * DxVx + (c12 * xiy) * DxVy + (c13 * xiz) * DxVz +
                   (c11 * etx) * DyVx + (c12 * ety) * DyVy + (c13 * etz) * DyVz +
                   (c11 * ztx) * DzVx + (c12 * zty) * DzVy + (c13 * ztz) * DzVz;
  h[TYY * V + q] = (c12 * xix) * DxVx + (c11 * xiy) * DxVy + (c13 * xiz) * DxVz +
                   (c12 * etx) * DyVx + (c11 * ety) * DyVy + (c13 * etz) * DyVz +
                   (c12 * ztx) * DzVx + (c11 * zty) * DzVy + (c13 * ztz) * DzVz;
  h[TZZ * V + q] = (c13 * xix) * DxVx + (c13 * xiy) * DxVy + (c33 * xiz) * DxVz +
                   (c13 * etx) * DyVx + (c13 * ety) * DyVy + (c33 * etz) * DyVz +
                   (c13 * ztx) * DzVx + (c13 * zty) * DzVy + (c33 * ztz) * DzVz;
  h[TYZ * V + q] = (c55 * xiz) * DxVy + (c55 * xiy) * DxVz +
                   (c55 * etz) * DyVy + (c55 * ety) * DyVz +
                   (c55 * ztz) * DzVy + (c55 * zty) * DzVz;
  h[TXZ * V + q] = (c55 * xiz) * DxVx + (c55 * xix) * DxVz +
                   (c55 * etz) * DyVx + (c55 * etx) * DyVz +
                   (c55 * ztz) * DzVx + (c55 * ztx) * DzVz;
  h[TXY * V + q] = (c66 * xiy) * DxVx + (c66 * xix) * DxVy +
                   (c66 * ety) * DyVx + (c66 * etx) * DyVy +
                   (c66 * zty) * DzVx + (c66 * ztx) * DzVy;
}

/* Hooke's law with the gradients along one direction only (CFS-PML terms;
 * e1..e3 the metric of that direction): isotropic
 * forward/sv_curv_col_el_iso.c:806-811, VTI forward/sv_curv_col_el_vti.c:
 * 760-765 */
static inline void hooke1(const med_t *m, float e1, float e2, float e3,
                          float DVx, float DVy, float DVz, float *r)
{
  if (m->aniso) {
    /* forward/sv_curv_col_el_aniso.c:824-829 */
    for (int w = 0; w < 6; w++)
      r[ANI_ROW_COMP[w]] = ani_f(m, w + 1, 0, e1, e2, e3) * DVx +
                           ani_f(m, w + 1, 1, e1, e2, e3) * DVy +
                           ani_f(m, w + 1, 2, e1, e2, e3) * DVz;
    return;
  }
  if (!m->vti) {
    float lam = m->lam, mu = m->mu, l2m = m->l2m;
    r[TXX] = l2m * e1 * DVx + lam * e2 * DVy + lam * e3 * DVz;
    r[TYY] = lam * e1 * DVx + l2m * e2 * DVy + lam * e3 * DVz;
    r[TZZ] = lam * e1 * DVx + lam * e2 * DVy + l2m * e3 * DVz;
    r[TXY] = mu * (e2 * DVx + e1 * DVy);
    r[TXZ] = mu * (e3 * DVx + e1 * DVz);
    r[TYZ] = mu * (e3 * DVy + e2 * DVz);
    return;
  }
  float c11 = m->c11, c12 = m->c12, c13 = m->c13, c33 = m->c33,
        c55 = m->c55, c66 = m->c66;
  r[TXX] = (c11 * e1) * DVx + (c12 * e2) * DVy + (c13 * e3) * DVz;
  r[TYY] = (c12 * e1) * DVx + (c11 * e2) * DVy + (c13 * e3) * DVz;
  r[TZZ] = (c13 * e1) * DVx + (c13 * e2) * DVy + (c33 * e3) * DVz;
  r[TYZ] = (c55 * e3) * DVy + (c55 * e2) * DVz;
  r[TXZ] = (c55 * e3) * DVx + (c55 * e1) * DVz;
  r[TXY] = (c66 * e2) * DVx + (c66 * e1) * DVy;
}

/* free-surface part of the x/y-face PML terms at k = nk2: zeta-metric
 * Hooke's law applied to the converted z gradients (isotropic
 * forward/sv_curv_col_el_iso.c:863-877, VTI forward/sv_curv_col_el_vti.c:
 * 817-822) */
static inline void hooke_surf(const med_t *m, float ztx, float zty, float ztz,
                              float DzVx, float DzVy, float DzVz, float *s)
{
  if (m->aniso) {   /* forward/sv_curv_col_el_aniso.c:875-880 */
    hooke1(m, ztx, zty, ztz, DzVx, DzVy, DzVz, s);
    return;
  }
  if (!m->vti) {
    float lam = m->lam, mu = m->mu, l2m = m->l2m;
    s[TXX] = l2m * (ztx * DzVx) + lam * (zty * DzVy + ztz * DzVz);
    s[TYY] = l2m * (zty * DzVy) + lam * (ztx * DzVx + ztz * DzVz);
    s[TZZ] = l2m * (ztz * DzVz) + lam * (ztx * DzVx + zty * DzVy);
    s[TXY] = mu * (zty * DzVx + ztx * DzVy);
    s[TXZ] = mu * (ztz * DzVx + ztx * DzVz);
    s[TYZ] = mu * (ztz * DzVy + zty * DzVz);
    return;
  }
  hooke1(m, ztx, zty, ztz, DzVx, DzVy, DzVz, s);
}

/* ------------------------------------------------------------------------ */
/* free-surface conversion matrices                                          */
/* ------------------------------------------------------------------------ */

static void inv3(float m[3][3])
{
  float v[3][3];
  v[0][0] = m[1][1] * m[2][2] - m[2][1] * m[1][2];
  v[0][1] = m[2][1] * m[0][2] - m[0][1] * m[2][2];
  v[0][2] = m[0][1] * m[1][2] - m[0][2] * m[1][1];
  v[1][0] = m[1][2] * m[2][0] - m[1][0] * m[2][2];
  v[1][1] = m[0][0] * m[2][2] - m[2][0] * m[0][2];
  v[1][2] = m[1][0] * m[0][2] - m[0][0] * m[1][2];
  v[2][0] = m[1][0] * m[2][1] - m[1][1] * m[2][0];
  v[2][1] = m[2][0] * m[0][1] - m[0][0] * m[2][1];
  v[2][2] = m[0][0] * m[1][1] - m[0][1] * m[1][0];
  float det = v[0][0] * m[0][0] + v[0][1] * m[1][0] + v[0][2] * m[2][0];
  det = 1.0f / det;
  for (int a = 0; a < 3; a++)
    for (int b = 0; b < 3; b++) m[a][b] = v[a][b] * det;
}

static void mul3(float A[3][3], float B[3][3], float C[3][3])
{
  for (int a = 0; a < 3; a++)
    for (int b = 0; b < 3; b++) {
      C[a][b] = 0.0f;
      for (int k = 0; k < 3; k++) C[a][b] += A[a][k] * B[k][b];
    }
}

/* matVx2Vz = A^-1 B, matVy2Vz = A^-1 C, matF2Vz = A^-1 at k = nk2 */
int oracle_dvh2dvz_iso(const cgfd_problem_t *p, float *mVx, float *mVy,
                       float *mF)
{
  size_t ln = p->nx, sl = (size_t)p->nx * p->ny;
  int k = p->nk2;
  for (int j = p->nj1; j <= p->nj2; j++)
    for (int i = p->ni1; i <= p->ni2; i++) {
      size_t q = i + j * ln + k * sl;
      float e11 = p->xi_x[q], e12 = p->xi_y[q], e13 = p->xi_z[q];
      float e21 = p->eta_x[q], e22 = p->eta_y[q], e23 = p->eta_z[q];
      float e31 = p->zeta_x[q], e32 = p->zeta_y[q], e33 = p->zeta_z[q];
      float lam = p->lambda[q], mu = p->mu[q];
      float l2m = lam + 2.0f * mu;
      float A[3][3], B[3][3], C[3][3], AB[3][3], AC[3][3];
      A[0][0] = l2m * e31 * e31 + mu * (e32 * e32 + e33 * e33);
      A[0][1] = lam * e31 * e32 + mu * e32 * e31;
      A[0][2] = lam * e31 * e33 + mu * e33 * e31;
      A[1][0] = lam * e32 * e31 + mu * e31 * e32;
      A[1][1] = l2m * e32 * e32 + mu * (e31 * e31 + e33 * e33);
      A[1][2] = lam * e32 * e33 + mu * e33 * e32;
      A[2][0] = lam * e33 * e31 + mu * e31 * e33;
      A[2][1] = lam * e33 * e32 + mu * e32 * e33;
      A[2][2] = l2m * e33 * e33 + mu * (e31 * e31 + e32 * e32);
      inv3(A);
      B[0][0] = -l2m * e31 * e11 - mu * (e32 * e12 + e33 * e13);
      B[0][1] = -lam * e31 * e12 - mu * e32 * e11;
      B[0][2] = -lam * e31 * e13 - mu * e33 * e11;
      B[1][0] = -lam * e32 * e11 - mu * e31 * e12;
      B[1][1] = -l2m * e32 * e12 - mu * (e31 * e11 + e33 * e13);
      B[1][2] = -lam * e32 * e13 - mu * e33 * e12;
      B[2][0] = -lam * e33 * e11 - mu * e31 * e13;
      B[2][1] = -lam * e33 * e12 - mu * e32 * e13;
      B[2][2] = -l2m * e33 * e13 - mu * (e31 * e11 + e32 * e12);
      C[0][0] = -l2m * e31 * e21 - mu * (e32 * e22 + e33 * e23);
      C[0][1] = -lam * e31 * e22 - mu * e32 * e21;
      C[0][2] = -lam * e31 * e23 - mu * e33 * e21;
      C[1][0] = -lam * e32 * e21 - mu * e31 * e22;
      C[1][1] = -l2m * e32 * e22 - mu * (e31 * e21 + e33 * e23);
      C[1][2] = -lam * e32 * e23 - mu * e33 * e22;
      C[2][0] = -lam * e33 * e21 - mu * e31 * e23;
      C[2][1] = -lam * e33 * e22 - mu * e32 * e23;
      C[2][2] = -l2m * e33 * e23 - mu * (e31 * e21 + e32 * e22);
      mul3(A, B, AB);
      mul3(A, C, AC);
      size_t ij = (j * ln + i) * 9;
      for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) {
          mVx[ij + r * 3 + c] = AB[r][c];
          mVy[ij + r * 3 + c] = AC[r][c];
          mF[ij + r * 3 + c] = A[r][c];
        }
    }
  return 0;
}

/* VTI: matVx2Vz = -A^-1 B, matVy2Vz = -A^-1 C at k = nk2
 * (forward/sv_curv_col_el_vti.c:1085-1206); matF2Vz is left untouched */
int oracle_dvh2dvz_vti(const cgfd_problem_t *p, float *mVx, float *mVy)
{
  size_t ln = p->nx, sl = (size_t)p->nx * p->ny;
  int k = p->nk2;
  for (int j = p->nj1; j <= p->nj2; j++)
    for (int i = p->ni1; i <= p->ni2; i++) {
      size_t q = i + j * ln + k * sl;
      float xix = p->xi_x[q], xiy = p->xi_y[q], xiz = p->xi_z[q];
      float etx = p->eta_x[q], ety = p->eta_y[q], etz = p->eta_z[q];
      float ztx = p->zeta_x[q], zty = p->zeta_y[q], ztz = p->zeta_z[q];
      med_t m;
      med_at(p, q, &m);
      float c11 = m.c11, c12 = m.c12, c13 = m.c13, c33 = m.c33, c55 = m.c55,
            c66 = m.c66;
      float A[3][3], B[3][3], C[3][3], AB[3][3], AC[3][3];
      A[0][0] = (c11 * ztx) * ztx + (c66 * zty) * zty + (c55 * ztz) * ztz;
      A[0][1] = (c12 * zty) * ztx + (c66 * ztx) * zty;
      A[0][2] = (c13 * ztz) * ztx + (c55 * ztx) * ztz;
      A[1][0] = (c66 * zty) * ztx + (c12 * ztx) * zty;
      A[1][1] = (c66 * ztx) * ztx + (c11 * zty) * zty + (c55 * ztz) * ztz;
      A[1][2] = (c13 * ztz) * zty + (c55 * zty) * ztz;
      A[2][0] = (c55 * ztz) * ztx + (c13 * ztx) * ztz;
      A[2][1] = (c55 * ztz) * zty + (c13 * zty) * ztz;
      A[2][2] = (c55 * ztx) * ztx + (c55 * zty) * zty + (c33 * ztz) * ztz;
      inv3(A);
      B[0][0] = (c11 * xix) * ztx + (c66 * xiy) * zty + (c55 * xiz) * ztz;
      B[0][1] = (c12 * xiy) * ztx + (c66 * xix) * zty;
      B[0][2] = (c13 * xiz) * ztx + (c55 * xix) * ztz;
      B[1][0] = (c66 * xiy) * ztx + (c12 * xix) * zty;
      B[1][1] = (c66 * xix) * ztx + (c11 * xiy) * zty + (c55 * xiz) * ztz;
      B[1][2] = (c13 * xiz) * zty + (c55 * xiy) * ztz;
      B[2][0] = (c55 * xiz) * ztx + (c13 * xix) * ztz;
      B[2][1] = (c55 * xiz) * zty + (c13 * xiy) * ztz;
      B[2][2] = (c55 * xix) * ztx + (c55 * xiy) * zty + (c33 * xiz) * ztz;
      C[0][0] = (c11 * etx) * ztx + (c66 * ety) * zty + (c55 * etz) * ztz;
      C[0][1] = (c12 * ety) * ztx + (c66 * etx) * zty;
      C[0][2] = (c13 * etz) * ztx + (c55 * etx) * ztz;
      C[1][0] = (c66 * ety) * ztx + (c12 * etx) * zty;
      C[1][1] = (c66 * etx) * ztx + (c11 * ety) * zty + (c55 * etz) * ztz;
      C[1][2] = (c13 * etz) * zty + (c55 * ety) * ztz;
      C[2][0] = (c55 * etz) * ztx + (c13 * etx) * ztz;
      C[2][1] = (c55 * etz) * zty + (c13 * ety) * ztz;
      C[2][2] = (c55 * etx) * ztx + (c55 * ety) * zty + (c33 * etz) * ztz;
      mul3(A, B, AB);
      mul3(A, C, AC);
      size_t ij = (j * ln + i) * 9;
      for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) {
          mVx[ij + r * 3 + c] = -1.0f * AB[r][c];
          mVy[ij + r * 3 + c] = -1.0f * AC[r][c];
        }
    }
  return 0;
}

/* anisotropic: matVx2Vz = -A^-1 B, matVy2Vz = -A^-1 C at k = nk2
 * (forward/sv_curv_col_el_aniso.c:1267-1423), with
 * M[a][b] = sum over n of (sum over m of C(V(a,n),V(b,m)) g_m) zeta_n for the
 * metric g = zeta (A), xi (B), eta (C); matF2Vz is left untouched */
int oracle_dvh2dvz_aniso(const cgfd_problem_t *p, float *mVx, float *mVy)
{
  size_t ln = p->nx, sl = (size_t)p->nx * p->ny;
  int k = p->nk2;
  for (int j = p->nj1; j <= p->nj2; j++)
    for (int i = p->ni1; i <= p->ni2; i++) {
      size_t q = i + j * ln + k * sl;
      const float g[3][3] = {{p->xi_x[q], p->xi_y[q], p->xi_z[q]},
                             {p->eta_x[q], p->eta_y[q], p->eta_z[q]},
                             {p->zeta_x[q], p->zeta_y[q], p->zeta_z[q]}};
      const float *zt = g[2];
      med_t m;
      med_at(p, q, &m);
      float M[3][3][3];     /* [A, B, C] */
      const int gsel[3] = {2, 0, 1};
      for (int w = 0; w < 3; w++) {
        const float *gm = g[gsel[w]];
        for (int a = 0; a < 3; a++)
          for (int b = 0; b < 3; b++) {
            float t[3];
            for (int n = 0; n < 3; n++)
              t[n] = cij(&m, voigt(a, n), voigt(b, 0)) * gm[0] +
                     cij(&m, voigt(a, n), voigt(b, 1)) * gm[1] +
                     cij(&m, voigt(a, n), voigt(b, 2)) * gm[2];
            M[w][a][b] = t[0] * zt[0] + t[1] * zt[1] + t[2] * zt[2];
          }
      }
      float AB[3][3], AC[3][3];
      inv3(M[0]);
      mul3(M[0], M[1], AB);
      mul3(M[0], M[2], AC);
      size_t ij = (j * ln + i) * 9;
      for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) {
          mVx[ij + r * 3 + c] = -1.0f * AB[r][c];
          mVy[ij + r * 3 + c] = -1.0f * AC[r][c];
        }
    }
  return 0;
}

/* centred 7-point operator of the metric calculation (fd_t.c:152-176,
 * layer 3), used along j on the grid coordinates */
static const float FDC_COEF[7] = {-0.02084f, 0.1667f, -0.7709f, 0.0f,
                                  0.7709f, -0.1667f, 0.02084f};

/* visco-elastic (GMB): matVx2Vz = A^-1 B, matVy2Vz = A^-1 C and the
 * rotation matrix matD of the local surface frame at k = nk2
 * (forward/sv_curv_col_vis_iso.c:353-507); matF2Vz is left untouched */
int oracle_dvh2dvz_vis(const cgfd_problem_t *p, float *mVx, float *mVy,
                       float *mD)
{
  size_t ln = p->nx, sl = (size_t)p->nx * p->ny;
  int k = p->nk2;
  for (int j = p->nj1; j <= p->nj2; j++)
    for (int i = p->ni1; i <= p->ni2; i++) {
      size_t q = i + j * ln + k * sl;
      float xix = p->xi_x[q], xiy = p->xi_y[q], xiz = p->xi_z[q];
      float etx = p->eta_x[q], ety = p->eta_y[q], etz = p->eta_z[q];
      float ztx = p->zeta_x[q], zty = p->zeta_y[q], ztz = p->zeta_z[q];
      float xet, yet, zet;
      xet = FDC_COEF[0] * p->x3d[q - 3 * ln];
      yet = FDC_COEF[0] * p->y3d[q - 3 * ln];
      zet = FDC_COEF[0] * p->z3d[q - 3 * ln];
      for (int n = 1; n < 7; n++) {
        long s = (long)(n - 3) * (long)ln;
        xet += FDC_COEF[n] * p->x3d[q + s];
      }
      for (int n = 1; n < 7; n++) {
        long s = (long)(n - 3) * (long)ln;
        yet += FDC_COEF[n] * p->y3d[q + s];
      }
      for (int n = 1; n < 7; n++) {
        long s = (long)(n - 3) * (long)ln;
        zet += FDC_COEF[n] * p->z3d[q + s];
      }
      float e_n = (float)(1.0 / sqrt((double)(xet * xet + yet * yet + zet * zet)));
      float e_m = (float)(1.0 / sqrt((double)(ztx * ztx + zty * zty + ztz * ztz)));
      float e_nm = e_n * e_m;
      float lam = p->lambda[q], mu = p->mu[q];
      float l2m = lam + 2.0f * mu;
      float A[3][3], B[3][3], C[3][3], D[3][3], AB[3][3], AC[3][3];
      A[0][0] = l2m * ztx * ztx + mu * (zty * zty + ztz * ztz);
      A[0][1] = lam * ztx * zty + mu * zty * ztx;
      A[0][2] = lam * ztx * ztz + mu * ztz * ztx;
      A[1][0] = lam * zty * ztx + mu * ztx * zty;
      A[1][1] = l2m * zty * zty + mu * (ztx * ztx + ztz * ztz);
      A[1][2] = lam * zty * ztz + mu * ztz * zty;
      A[2][0] = lam * ztz * ztx + mu * ztx * ztz;
      A[2][1] = lam * ztz * zty + mu * zty * ztz;
      A[2][2] = l2m * ztz * ztz + mu * (ztx * ztx + zty * zty);
      inv3(A);
      B[0][0] = -l2m * ztx * xix - mu * (zty * xiy + ztz * xiz);
      B[0][1] = -lam * ztx * xiy - mu * zty * xix;
      B[0][2] = -lam * ztx * xiz - mu * ztz * xix;
      B[1][0] = -lam * zty * xix - mu * ztx * xiy;
      B[1][1] = -l2m * zty * xiy - mu * (ztx * xix + ztz * xiz);
      B[1][2] = -lam * zty * xiz - mu * ztz * xiy;
      B[2][0] = -lam * ztz * xix - mu * ztx * xiz;
      B[2][1] = -lam * ztz * xiy - mu * zty * xiz;
      B[2][2] = -l2m * ztz * xiz - mu * (ztx * xix + zty * xiy);
      C[0][0] = -l2m * ztx * etx - mu * (zty * ety + ztz * etz);
      C[0][1] = -lam * ztx * ety - mu * zty * etx;
      C[0][2] = -lam * ztx * etz - mu * ztz * etx;
      C[1][0] = -lam * zty * etx - mu * ztx * ety;
      C[1][1] = -l2m * zty * ety - mu * (ztx * etx + ztz * etz);
      C[1][2] = -lam * zty * etz - mu * ztz * ety;
      C[2][0] = -lam * ztz * etx - mu * ztx * etz;
      C[2][1] = -lam * ztz * ety - mu * zty * etz;
      C[2][2] = -l2m * ztz * etz - mu * (ztx * etx + zty * ety);
      mul3(A, B, AB);
      mul3(A, C, AC);
      D[0][0] = (yet * ztz - zet * zty) * e_nm;
      D[0][1] = (zet * ztx - xet * ztz) * e_nm;
      D[0][2] = (xet * zty - yet * ztx) * e_nm;
      D[1][0] = xet * e_n;
      D[1][1] = yet * e_n;
      D[1][2] = zet * e_n;
      D[2][0] = ztx * e_m;
      D[2][1] = zty * e_m;
      D[2][2] = ztz * e_m;
      size_t ij = (j * ln + i) * 9;
      for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) {
          mVx[ij + r * 3 + c] = AB[r][c];
          mVy[ij + r * 3 + c] = AC[r][c];
          mD[ij + r * 3 + c] = D[r][c];
        }
    }
  return 0;
}

/* ------------------------------------------------------------------------ */
/* RHS passes                                                               */
/* ------------------------------------------------------------------------ */

/* interior RHS of one k-plane (sv_curv_col_el_iso.c:304-440) */
static void rhs_inner_plane(orc_t *o, const float *w, float *h, int k,
                            const op5_t *ox, const op5_t *oy, const op5_t *oz)
{
  const cgfd_problem_t *p = o->p;
  size_t V = o->vol;
  const float *Vx = w + VX * V, *Vy = w + VY * V, *Vz = w + VZ * V;
  const float *Txx = w + TXX * V, *Tyy = w + TYY * V, *Tzz = w + TZZ * V;
  const float *Tyz = w + TYZ * V, *Txz = w + TXZ * V, *Txy = w + TXY * V;
  for (int j = p->nj1; j <= p->nj2; j++) {
    size_t q = p->ni1 + j * o->ln + (size_t)k * o->sl;
    for (int i = p->ni1; i <= p->ni2; i++, q++) {
      float DxVx = D5(ox, Vx + q), DyVx = D5(oy, Vx + q), DzVx = D5(oz, Vx + q);
      float DxVy = D5(ox, Vy + q), DyVy = D5(oy, Vy + q), DzVy = D5(oz, Vy + q);
      float DxVz = D5(ox, Vz + q), DyVz = D5(oy, Vz + q), DzVz = D5(oz, Vz + q);
      float DxTxx = D5(ox, Txx + q), DyTxx = D5(oy, Txx + q), DzTxx = D5(oz, Txx + q);
      float DxTyy = D5(ox, Tyy + q), DyTyy = D5(oy, Tyy + q), DzTyy = D5(oz, Tyy + q);
      float DxTzz = D5(ox, Tzz + q), DyTzz = D5(oy, Tzz + q), DzTzz = D5(oz, Tzz + q);
      float DxTxz = D5(ox, Txz + q), DyTxz = D5(oy, Txz + q), DzTxz = D5(oz, Txz + q);
      float DxTyz = D5(ox, Tyz + q), DyTyz = D5(oy, Tyz + q), DzTyz = D5(oz, Tyz + q);
      float DxTxy = D5(ox, Txy + q), DyTxy = D5(oy, Txy + q), DzTxy = D5(oz, Txy + q);
      float xix = p->xi_x[q], xiy = p->xi_y[q], xiz = p->xi_z[q];
      float etx = p->eta_x[q], ety = p->eta_y[q], etz = p->eta_z[q];
      float ztx = p->zeta_x[q], zty = p->zeta_y[q], ztz = p->zeta_z[q];
      float slw = p->slw[q];
      med_t m;
      med_at(p, q, &m);
      h[VX * V + q] = slw * (xix * DxTxx + xiy * DxTxy + xiz * DxTxz +
                             etx * DyTxx + ety * DyTxy + etz * DyTxz +
                             ztx * DzTxx + zty * DzTxy + ztz * DzTxz);
      h[VY * V + q] = slw * (xix * DxTxy + xiy * DxTyy + xiz * DxTyz +
                             etx * DyTxy + ety * DyTyy + etz * DyTyz +
                             ztx * DzTxy + zty * DzTyy + ztz * DzTyz);
      h[VZ * V + q] = slw * (xix * DxTxz + xiy * DxTyz + xiz * DxTzz +
                             etx * DyTxz + ety * DyTyz + etz * DyTzz +
                             ztx * DzTxz + zty * DzTyz + ztz * DzTzz);
      hooke9(&m, xix, xiy, xiz, etx, ety, etz, ztx, zty, ztz, DxVx, DxVy, DxVz,
             DyVx, DyVy, DyVz, DzVx, DzVy, DzVz, h, V, q);
    }
  }
}

/* conservative traction term J * (m . T) at one point, for one momentum row */
static inline float cons(const float *jac, const float *mx, const float *my,
                         const float *mz, const float *Ta, const float *Tb,
                         const float *Tc, size_t q)
{
  return jac[q] * (mx[q] * Ta[q] + my[q] * Tb[q] + mz[q] * Tc[q]);
}

/*
 * Traction image for the top layers of row j (sv_curv_col_el.c:84-304).
 * Above the surface the conservative z-flux is mirrored:
 * vec[n] = 2 T_surf - vec[2 n_free - n].  At k = nk2 with the taps at -1..3
 * the mirror needs n = -1, -2, i.e. values of the points k-2, k-3 that the
 * reference never computes: it reads past the start of its local array.
 * timg_mode chooses what stands there: 0 = zero (the value that array slot
 * holds in the reference build this oracle is pinned against), 1 = the
 * conservative value at k-2/k-3 (the mirror the formula intends).
 */
static void rhs_timg_row(orc_t *o, const float *w, float *h, int j, int zbias,
                         const op5_t *ox, const op5_t *oy)
{
  const cgfd_problem_t *p = o->p;
  size_t V = o->vol, ln = o->ln, sl = o->sl;
  const float *T[9];
  for (int c = 0; c < 9; c++) T[c] = w + c * V;
  const int *zs = OP_SHIFT[zbias];
  const float *zc = OP_COEF[zbias];
  int k_min = p->nk2 - zs[4];
  /* momentum rows: (x-flux metric set) x (stress triplet) */
  const int rowT[3][3] = {{TXX, TXY, TXZ}, {TXY, TYY, TYZ}, {TXZ, TYZ, TZZ}};
  for (int k = k_min; k <= p->nk2; k++) {
    int n_free = p->nk2 - k - zs[0];
    size_t q = p->ni1 + j * ln + (size_t)k * sl;
    for (int i = p->ni1; i <= p->ni2; i++, q++) {
      float slwjac = p->slw[q] / p->jac[q];
      for (int r = 0; r < 3; r++) {
        const float *Ta = T[rowT[r][0]], *Tb = T[rowT[r][1]], *Tc = T[rowT[r][2]];
        float vx[5], vy[5], vzb[7];
        float *vz = vzb + 2; /* vz[-2], vz[-1] addressable */
        for (int n = 0; n < 5; n++) {
          vx[n] = cons(p->jac, p->xi_x, p->xi_y, p->xi_z, Ta, Tb, Tc, q + ox->s[n]);
          vy[n] = cons(p->jac, p->eta_x, p->eta_y, p->eta_z, Ta, Tb, Tc, q + oy->s[n]);
        }
        for (int n = 0; n < n_free; n++)
          vz[n] = cons(p->jac, p->zeta_x, p->zeta_y, p->zeta_z, Ta, Tb, Tc,
                       q + zs[n] * (long)sl);
        if (o->timg_mode == 1) {
          for (int n = -2; n < 0; n++)
            vz[n] = cons(p->jac, p->zeta_x, p->zeta_y, p->zeta_z, Ta, Tb, Tc,
                         q + (zs[0] + n) * (long)sl);
        } else {
          vz[-2] = 0.0f;
          vz[-1] = 0.0f;
        }
        float tsurf = o->TS ? o->TS[r * sl + i + j * ln] : 0.0f; /* TxSrc.. */
        vz[n_free] = tsurf;
        for (int n = n_free + 1; n < 5; n++)
          vz[n] = (float)(2.0 * (double)tsurf - (double)vz[2 * n_free - n]);
        float Dx = ox->c[0] * vx[0];
        for (int n = 1; n < 5; n++) Dx += ox->c[n] * vx[n];
        float Dy = oy->c[0] * vy[0];
        for (int n = 1; n < 5; n++) Dy += oy->c[n] * vy[n];
        float Dz = zc[0] * vz[0];
        for (int n = 1; n < 5; n++) Dz += zc[n] * vz[n];
        h[(VX + r) * V + q] = (Dx + Dy + Dz) * slwjac;
      }
    }
  }
}

/* velocity-gradient conversion on the top three layers of row j
 * (sv_curv_col_el_iso.c:501-633) */
static void rhs_vlow_row(orc_t *o, const float *w, float *h, int j, int zbias,
                         const op5_t *ox, const op5_t *oy)
{
  const cgfd_problem_t *p = o->p;
  size_t V = o->vol, ln = o->ln, sl = o->sl;
  const float *Vx = w + VX * V, *Vy = w + VY * V, *Vz = w + VZ * V;
  for (int n = 0; n < 3; n++) {
    int k = p->nk2 - n;
    size_t q = p->ni1 + j * ln + (size_t)k * sl;
    for (int i = p->ni1; i <= p->ni2; i++, q++) {
      float xix = p->xi_x[q], xiy = p->xi_y[q], xiz = p->xi_z[q];
      float etx = p->eta_x[q], ety = p->eta_y[q], etz = p->eta_z[q];
      float ztx = p->zeta_x[q], zty = p->zeta_y[q], ztz = p->zeta_z[q];
      med_t m;
      med_at(p, q, &m);
      float DxVx = D5(ox, Vx + q), DyVx = D5(oy, Vx + q);
      float DxVy = D5(ox, Vy + q), DyVy = D5(oy, Vy + q);
      float DxVz = D5(ox, Vz + q), DyVz = D5(oy, Vz + q);
      float DzVx, DzVy, DzVz;
      if (n == 0) {
        size_t ij = (i + j * ln) * 9;
        const float *a = o->mVx + ij, *b = o->mVy + ij;
        DzVx = a[0] * DxVx + a[1] * DxVy + a[2] * DxVz + b[0] * DyVx +
               b[1] * DyVy + b[2] * DyVz;
        DzVy = a[3] * DxVx + a[4] * DxVy + a[5] * DxVz + b[3] * DyVx +
               b[4] * DyVy + b[5] * DyVz;
        DzVz = a[6] * DxVx + a[7] * DxVy + a[8] * DxVz + b[6] * DyVx +
               b[7] * DyVy + b[8] * DyVz;
        /* + matF2Vz * (VxSrc,VySrc,VzSrc): zero without surface forces;
           the VTI routine has no such term (sv_curv_col_el_vti.c:525-547) */
        if (!m.vti && !m.aniso) {
          const float *f = o->mF + ij;
          size_t i2 = i + j * ln;
          float vx = 0.0f, vy = 0.0f, vz = 0.0f;
          if (o->VS) { vx = o->VS[i2]; vy = o->VS[sl + i2]; vz = o->VS[2 * sl + i2]; }
          DzVx += f[0] * vx + f[1] * vy + f[2] * vz;
          DzVy += f[3] * vx + f[4] * vy + f[5] * vz;
          DzVz += f[6] * vx + f[7] * vy + f[8] * vz;
        }
      } else if (n == 1) {
        long s0 = OPZ1_SHIFT[zbias][0] * (long)sl, s1 = OPZ1_SHIFT[zbias][1] * (long)sl;
        const float *c = OPZ1_COEF[zbias];
        DzVx = c[0] * Vx[q + s0]; DzVx += c[1] * Vx[q + s1];
        DzVy = c[0] * Vy[q + s0]; DzVy += c[1] * Vy[q + s1];
        DzVz = c[0] * Vz[q + s0]; DzVz += c[1] * Vz[q + s1];
      } else {
        long s0 = OPZ2_SHIFT[zbias][0] * (long)sl, s1 = OPZ2_SHIFT[zbias][1] * (long)sl,
             s2 = OPZ2_SHIFT[zbias][2] * (long)sl;
        const float *c = OPZ2_COEF[zbias];
        DzVx = c[0] * Vx[q + s0]; DzVx += c[1] * Vx[q + s1]; DzVx += c[2] * Vx[q + s2];
        DzVy = c[0] * Vy[q + s0]; DzVy += c[1] * Vy[q + s1]; DzVy += c[2] * Vy[q + s2];
        DzVz = c[0] * Vz[q + s0]; DzVz += c[1] * Vz[q + s1]; DzVz += c[2] * Vz[q + s2];
      }
      hooke9(&m, xix, xiy, xiz, etx, ety, etz, ztx, zty, ztz, DxVx, DxVy, DxVz,
             DyVx, DyVy, DyVz, DzVx, DzVy, DzVz, h, V, q);
    }
  }
}

/* CFS-PML corrections of one face for the points of plane k
 * (sv_curv_col_el_iso.c:708-1143) */
static void rhs_pml_face_plane(orc_t *o, const float *w, float *h, int idim,
                               int iside, int k, const op5_t *op,
                               const float *acur, float *arhs)
{
  const cgfd_problem_t *p = o->p;
  const cgfd_pml_face_t *f = &p->pml[idim][iside];
  size_t V = o->vol, ln = o->ln, sl = o->sl;
  int nbx = f->ni2 - f->ni1 + 1, nby = f->nj2 - f->nj1 + 1;
  size_t AV = o->aux_vol[idim][iside];
  const float *m1, *m2, *m3;
  if (idim == 0) { m1 = p->xi_x; m2 = p->xi_y; m3 = p->xi_z; }
  else if (idim == 1) { m1 = p->eta_x; m2 = p->eta_y; m3 = p->eta_z; }
  else { m1 = p->zeta_x; m2 = p->zeta_y; m3 = p->zeta_z; }
  const float *W[9];
  for (int c = 0; c < 9; c++) W[c] = w + c * V;
  for (int j = f->nj1; j <= f->nj2; j++) {
    for (int i = f->ni1; i <= f->ni2; i++) {
      size_t q = i + j * ln + (size_t)k * sl;
      size_t a = (size_t)(i - f->ni1) + (size_t)(j - f->nj1) * nbx +
                 (size_t)(k - f->nk1) * nbx * nby;
      int n = idim == 0 ? i - f->ni1 : (idim == 1 ? j - f->nj1 : k - f->nk1);
      float cD = f->D[n], cA = f->A[n], cB = f->B[n];
      float cB1 = (float)((double)cB - 1.0);
      float e1 = m1[q], e2 = m2[q], e3 = m3[q];
      float slw = p->slw[q];
      med_t m;
      med_at(p, q, &m);
      float DVx = D5(op, W[VX] + q), DVy = D5(op, W[VY] + q), DVz = D5(op, W[VZ] + q);
      float DTxx = D5(op, W[TXX] + q), DTyy = D5(op, W[TYY] + q),
            DTzz = D5(op, W[TZZ] + q), DTxz = D5(op, W[TXZ] + q),
            DTyz = D5(op, W[TYZ] + q), DTxy = D5(op, W[TXY] + q);
      float r[9];
      r[VX] = slw * (e1 * DTxx + e2 * DTxy + e3 * DTxz);
      r[VY] = slw * (e1 * DTxy + e2 * DTyy + e3 * DTyz);
      r[VZ] = slw * (e1 * DTxz + e2 * DTyz + e3 * DTzz);
      hooke1(&m, e1, e2, e3, DVx, DVy, DVz, r);
      /* same component order of updates as the reference */
      static const int ord[9] = {VX, VY, VZ, TXX, TYY, TZZ, TXZ, TYZ, TXY};
      for (int m = 0; m < 9; m++) {
        int c = ord[m];
        h[c * V + q] += cB1 * r[c] - cB * acur[c * AV + a];
      }
      for (int m = 0; m < 9; m++) {
        int c = ord[m];
        arhs[c * AV + a] = cD * r[c] - cA * acur[c * AV + a];
      }
      if (idim < 2 && p->free_top && k == p->nk2) {
        size_t ij = (i + j * ln) * 9;
        const float *M = (idim == 0 ? o->mVx : o->mVy) + ij;
        float DzVx = M[0] * DVx + M[1] * DVy + M[2] * DVz;
        float DzVy = M[3] * DVx + M[4] * DVy + M[5] * DVz;
        float DzVz = M[6] * DVx + M[7] * DVy + M[8] * DVz;
        float ztx = p->zeta_x[q], zty = p->zeta_y[q], ztz = p->zeta_z[q];
        float s[9];
        hooke_surf(&m, ztx, zty, ztz, DzVx, DzVy, DzVz, s);
        static const int ordT[6] = {TXX, TYY, TZZ, TXZ, TYZ, TXY};
        for (int m = 0; m < 6; m++) {
          int c = ordT[m];
          h[c * V + q] = (float)((double)h[c * V + q] +
                                 ((double)cB - 1.0) * (double)s[c]);
        }
        for (int m = 0; m < 6; m++) {
          int c = ordT[m];
          arhs[c * AV + a] += cD * s[c];
        }
      }
    }
  }
}

/* GMB attenuation of one k plane (forward/sv_curv_col_vis_iso.c:250-347):
 * memory-variable rates from the strain rates implied by hT, and the
 * memory-stress correction of hT.  Runs after the PML pass and before the
 * sources, as in sv_curv_col_vis_iso_onestage (:165-232). */
static void rhs_atten_plane(orc_t *o, const float *w, float *h, int k)
{
  const cgfd_problem_t *p = o->p;
  size_t V = o->vol;
  int nm = p->nmaxwell;
  for (int j = p->nj1; j <= p->nj2; j++) {
    size_t q = p->ni1 + j * o->ln + (size_t)k * o->sl;
    for (int i = p->ni1; i <= p->ni2; i++, q++) {
      float lam = p->lambda[q], mu = p->mu[q];
      float hxx = h[TXX * V + q], hyy = h[TYY * V + q], hzz = h[TZZ * V + q];
      float hxy = h[TXY * V + q], hxz = h[TXZ * V + q], hyz = h[TYZ * V + q];
      float sum_hxyz = (hxx + hyy + hzz) / (3 * lam + 2 * mu);
      double mu2 = (double)(2 * mu);
      float EVxx = (float)(((2.0 * hxx - hyy - hzz) / mu2 + sum_hxyz) / 3);
      float EVyy = (float)(((2.0 * hyy - hxx - hzz) / mu2 + sum_hxyz) / 3);
      float EVzz = (float)(((2.0 * hzz - hxx - hyy) / mu2 + sum_hxyz) / 3);
      float EVxy = (float)(hxy / mu * 0.5);
      float EVxz = (float)(hxz / mu * 0.5);
      float EVyz = (float)(hyz / mu * 0.5);
      for (int n = 0; n < nm; n++) {
        size_t b = (size_t)(9 + 6 * n) * V + q;
        float wl = p->wl[n];
        h[b + 0 * V] = wl * (EVxx - w[b + 0 * V]);
        h[b + 1 * V] = wl * (EVyy - w[b + 1 * V]);
        h[b + 2 * V] = wl * (EVzz - w[b + 2 * V]);
        h[b + 5 * V] = wl * (EVxy - w[b + 5 * V]);
        h[b + 4 * V] = wl * (EVxz - w[b + 4 * V]);
        h[b + 3 * V] = wl * (EVyz - w[b + 3 * V]);
      }
      float sxyz = 0.0f, sxx = 0.0f, syy = 0.0f, szz = 0.0f, sxy = 0.0f,
            sxz = 0.0f, syz = 0.0f;
      for (int n = 0; n < nm; n++) {
        size_t b = (size_t)(9 + 6 * n) * V + q;
        float yl = p->Ylam[n][q], ym = p->Ymu[n][q];
        float Jxx = w[b], Jyy = w[b + V], Jzz = w[b + 2 * V];
        float Jyz = w[b + 3 * V], Jxz = w[b + 4 * V], Jxy = w[b + 5 * V];
        sxyz += yl * (Jxx + Jyy + Jzz);
        sxx += ym * Jxx;
        syy += ym * Jyy;
        szz += ym * Jzz;
        sxy += ym * Jxy;
        sxz += ym * Jxz;
        syz += ym * Jyz;
      }
      double mu2d = 2.0 * (double)mu;
      float mxx = (float)((double)(lam * sxyz) + mu2d * (double)sxx);
      float myy = (float)((double)(lam * sxyz) + mu2d * (double)syy);
      float mzz = (float)((double)(lam * sxyz) + mu2d * (double)szz);
      float mxy = (float)(mu2d * (double)sxy);
      float mxz = (float)(mu2d * (double)sxz);
      float myz = (float)(mu2d * (double)syz);
      h[TXX * V + q] = hxx - mxx;
      h[TYY * V + q] = hyy - myy;
      h[TZZ * V + q] = hzz - mzz;
      h[TXY * V + q] = hxy - mxy;
      h[TXZ * V + q] = hxz - mxz;
      h[TYZ * V + q] = hyz - myz;
    }
  }
}

/* distributed sources at grid points after the other sources
 * (forward/sv_curv_col_el.c:487-590): force rates times slw/jac, moment
 * rates times 1/jac (evaluated in double as the reference's 1.0 / jac) */
static void rhs_srcdd(orc_t *o, float *h, int it, int is)
{
  const cgfd_problem_t *p = o->p;
  const size_t V = o->vol;
  if (p->dd_vi) {
    const float *vi = p->dd_vi + ((size_t)it * 4 + is) * p->dd_n * 3;
    for (int n = 0; n < p->dd_n; n++, vi += 3) {
      size_t q = p->dd_si[n] + p->dd_sj[n] * o->ln + (size_t)p->dd_sk[n] * o->sl;
      float v = p->slw[q] / p->jac[q];
      h[VX * V + q] += vi[0] * v;
      h[VY * V + q] += vi[1] * v;
      h[VZ * V + q] += vi[2] * v;
    }
  }
  if (p->dd_mij) {
    const float *m = p->dd_mij + ((size_t)it * 4 + is) * p->dd_n * 6;
    for (int n = 0; n < p->dd_n; n++, m += 6) {
      size_t q = p->dd_si[n] + p->dd_sj[n] * o->ln + (size_t)p->dd_sk[n] * o->sl;
      float rjac = 1.0 / p->jac[q];
      h[TXX * V + q] -= m[0] * rjac;
      h[TYY * V + q] -= m[1] * rjac;
      h[TZZ * V + q] -= m[2] * rjac;
      h[TYZ * V + q] -= m[3] * rjac;
      h[TXZ * V + q] -= m[4] * rjac;
      h[TXY * V + q] -= m[5] * rjac;
    }
  }
}

/* Graves Q attenuation after the last stage's combine, physical points of
 * one k-slab (forward/sv_curv_col_el.c:638-666) */
static void graves_qs_slab(orc_t *o, float *w, long k0, long k1)
{
  const cgfd_problem_t *p = o->p;
  float coef = -3.14159265358979323846 * p->qs_freq * p->dt;
  for (int c = 0; c < p->ncmp; c++)
    for (long k = k0; k < k1; k++)
      for (int j = p->nj1; j <= p->nj2; j++)
        for (int i = p->ni1; i <= p->ni2; i++) {
          size_t q = (size_t)i + j * o->ln + (size_t)k * o->sl;
          float qatt = expf(coef / p->Qs[q]);
          w[c * o->vol + q] *= qatt;
        }
}

/* exponential sponge after each step (forward/bdry_t.c:841-890): the
 * points of the enabled blocks times min(Ex[i], Ey[j], Ez[k]) */
static void ablexp_apply(orc_t *o, float *w)
{
  const cgfd_problem_t *p = o->p;
  for (int c = 0; c < p->ncmp; c++)
    for (int n = 0; n < 6; n++) {
      const int *b = p->ablexp_blk[n];
      if (b[0] != 1) continue;
      for (int k = b[5]; k <= b[6]; k++)
        for (int j = b[3]; j <= b[4]; j++)
          for (int i = b[1]; i <= b[2]; i++) {
            float mask = (p->ablexp_Ex[i] < p->ablexp_Ey[j]) ? p->ablexp_Ex[i] : p->ablexp_Ey[j];
            if (mask > p->ablexp_Ez[k]) mask = p->ablexp_Ez[k];
            w[c * o->vol + (size_t)i + j * o->ln + (size_t)k * o->sl] *= mask;
          }
    }
}

/* visco-elastic free surface after the last stage: rotate the surface
 * stress into the local frame, drop the traction components, rotate back
 * (forward/sv_curv_col_vis_iso.c:509-623) */
static void vis_free_row(orc_t *o, float *w, int j)
{
  const cgfd_problem_t *p = o->p;
  size_t V = o->vol, ln = o->ln;
  size_t q = p->ni1 + j * ln + (size_t)p->nk2 * o->sl;
  for (int i = p->ni1; i <= p->ni2; i++, q++) {
    const float *M = o->mD + (i + j * ln) * 9;
    float D[3][3], DT[3][3], Tl[3][3], DTl[3][3], Tg[3][3];
    for (int r = 0; r < 3; r++)
      for (int c = 0; c < 3; c++) {
        D[r][c] = M[r * 3 + c];
        DT[c][r] = M[r * 3 + c];
      }
    float d11 = D[0][0], d12 = D[0][1], d13 = D[0][2];
    float d21 = D[1][0], d22 = D[1][1], d23 = D[1][2];
    float Txx = w[TXX * V + q], Tyy = w[TYY * V + q], Tzz = w[TZZ * V + q];
    float Txy = w[TXY * V + q], Txz = w[TXZ * V + q], Tyz = w[TYZ * V + q];
    Tl[0][0] = d11 * d11 * Txx + d12 * d12 * Tyy + d13 * d13 * Tzz +
               2 * (d11 * d12 * Txy + d11 * d13 * Txz + d12 * d13 * Tyz);
    Tl[0][1] = d11 * d21 * Txx + d12 * d22 * Tyy + d13 * d23 * Tzz +
               (d11 * d22 + d12 * d21) * Txy + (d11 * d23 + d21 * d13) * Txz +
               (d12 * d23 + d22 * d13) * Tyz;
    Tl[1][1] = d21 * d21 * Txx + d22 * d22 * Tyy + d23 * d23 * Tzz +
               2 * (d21 * d22 * Txy + d21 * d23 * Txz + d22 * d23 * Tyz);
    Tl[1][0] = Tl[0][1];
    Tl[0][2] = 0.0f; Tl[1][2] = 0.0f; Tl[2][0] = 0.0f; Tl[2][1] = 0.0f;
    Tl[2][2] = 0.0f;
    mul3(DT, Tl, DTl);
    mul3(DTl, D, Tg);
    w[TXX * V + q] = Tg[0][0];
    w[TYY * V + q] = Tg[1][1];
    w[TZZ * V + q] = Tg[2][2];
    w[TXY * V + q] = Tg[0][1];
    w[TXZ * V + q] = Tg[0][2];
    w[TYZ * V + q] = Tg[1][2];
  }
}

/* Gaussian weights normalised over the points at or below the surface
 * (src_t.c:2111-2151; fun_gauss src_t.c:2179) */
static float gauss1(float t, float a)
{
  float tt = t - 0.0f;
  float e = (-tt) * tt / (a * a);
  float den = sqrtf((float)3.14159265358979323846) * a;
  return (float)(exp((double)e) / (double)den);
}

static void src_weights(float *delt, float x0, float y0, float z0, float r,
                        int half, int half_z2)
{
  int idx = 0;
  for (int k = -half; k <= half; k++)
    for (int j = -half; j <= half; j++)
      for (int i = -half; i <= half; i++) {
        float D1 = gauss1(i - x0, r), D2 = gauss1(j - y0, r), D3 = gauss1(k - z0, r);
        delt[idx++] = D1 * D2 * D3;
      }
  float sum = 0.0f;
  idx = 0;
  for (int k = -half; k <= half_z2; k++)
    for (int j = -half; j <= half; j++)
      for (int i = -half; i <= half; i++) sum += delt[idx++];
  int n1 = 2 * half + 1;
  for (int m = 0; m < n1 * n1 * n1; m++) delt[m] /= sum;
}

/* surface traction (TxSrc..) and velocity-rate (VxSrc..) layers of the
 * surface forces at (it, istage) (forward/src_t.c:153-314): a point force
 * adds its value at its column, a spread one the surface layer of its
 * Gaussian weights (the same weights as its volume injection). */
static void surf_layer(orc_t *o, int it, int istage)
{
  const cgfd_problem_t *p = o->p;
  size_t s2 = o->sl, ln = o->ln;
  memset(o->TS, 0, 3 * s2 * sizeof(float));
  memset(o->VS, 0, 3 * s2 * sizeof(float));
  for (int n = 0; n < p->src_n_surface_force; n++) {
    int is = p->src_force_rate_indx[n];
    if (it < p->src_it_begin[is] || it > p->src_it_end[is]) continue;
    int si = p->src_si[is], sj = p->src_sj[is], sk = p->src_sk[is];
    size_t t = (size_t)is * p->src_max_nt * p->src_max_stage +
               (size_t)(it - p->src_it_begin[is]) * p->src_max_stage + istage;
    size_t tr = (size_t)n * p->src_max_nt * p->src_max_stage +
                (size_t)(it - p->src_it_begin[is]) * p->src_max_stage + istage;
    float fx = p->Fx[t], fy = p->Fy[t], fz = p->Fz[t];
    float rx = p->Fx_rate[tr], ry = p->Fy_rate[tr], rz = p->Fz_rate[tr];
    if (p->src_spatial == CGFD_SRC_POINT) {
      size_t q = si + sj * ln + (size_t)sk * s2, i2 = si + sj * ln;
      o->TS[i2] += fx; o->TS[s2 + i2] += fy; o->TS[2 * s2 + i2] += fz;
      o->VS[i2] += rx / p->jac[q];
      o->VS[s2 + i2] += ry / p->jac[q];
      o->VS[2 * s2 + i2] += rz / p->jac[q];
    } else {
      int half = p->src_ext_half, len = 2 * half + 1;
      int kx = p->nk2 - sk;                     /* k_ext of the surface */
      const float *wgt = o->ext[is] + (size_t)(kx + half) * len * len;
      int k = sk + kx;
      for (int jj = -half; jj <= half; jj++)
        for (int ii = -half; ii <= half; ii++) {
          float c = *wgt++;
          int i = si + ii, j = sj + jj;
          if (i < 0 || i >= p->nx || j < 0 || j >= p->ny) continue;
          size_t q = i + j * ln + (size_t)k * s2, i2 = i + j * ln;
          o->TS[i2] += fx * c; o->TS[s2 + i2] += fy * c; o->TS[2 * s2 + i2] += fz * c;
          o->VS[i2] += rx * c / p->jac[q];
          o->VS[s2 + i2] += ry * c / p->jac[q];
          o->VS[2 * s2 + i2] += rz * c / p->jac[q];
        }
    }
  }
}

/* source injection (sv_curv_col_el.c:350-476) */
static void rhs_src(orc_t *o, float *h, int it, int istage)
{
  const cgfd_problem_t *p = o->p;
  size_t V = o->vol, ln = o->ln, sl = o->sl;
  for (int is = 0; is < p->src_n; is++) {
    if (it < p->src_it_begin[is] || it > p->src_it_end[is]) continue;
    size_t t = (size_t)is * p->src_max_nt * p->src_max_stage +
               (size_t)(it - p->src_it_begin[is]) * p->src_max_stage + istage;
    float fx = 0, fy = 0, fz = 0, Mxx = 0, Myy = 0, Mzz = 0, Mxz = 0, Myz = 0, Mxy = 0;
    if (p->src_force) { fx = p->Fx[t]; fy = p->Fy[t]; fz = p->Fz[t]; }
    if (p->src_moment) {
      Mxx = p->Mxx[t]; Myy = p->Myy[t]; Mzz = p->Mzz[t];
      Mxz = p->Mxz[t]; Myz = p->Myz[t]; Mxy = p->Mxy[t];
    }
    int si = p->src_si[is], sj = p->src_sj[is], sk = p->src_sk[is];
    if (p->src_spatial == CGFD_SRC_POINT) {
      /* a point source outside the physical region is not located
         (src_t.c:481-495 keeps only sources inside the domain) */
      if (si < p->ni1 || si > p->ni2 || sj < p->nj1 || sj > p->nj2 ||
          sk < p->nk1 || sk > p->nk2)
        continue;
      size_t q = si + sj * ln + (size_t)sk * sl;
      if (p->src_force && (p->src_surface_strict == 0 || sk < p->nk2)) {
        float Vf = p->slw[q] / p->jac[q];
        h[VX * V + q] += fx * Vf;
        h[VY * V + q] += fy * Vf;
        h[VZ * V + q] += fz * Vf;
      }
      if (p->src_moment) {
        float rjac = (float)(1.0 / (double)p->jac[q]);
        h[TXX * V + q] -= Mxx * rjac;
        h[TYY * V + q] -= Myy * rjac;
        h[TZZ * V + q] -= Mzz * rjac;
        h[TXZ * V + q] -= Mxz * rjac;
        h[TYZ * V + q] -= Myz * rjac;
        h[TXY * V + q] -= Mxy * rjac;
      }
    } else {
      int half = p->src_ext_half;
      int kz2 = (sk + half < p->nk2) ? half : p->nk2 - sk;
      const float *wgt = o->ext[is];
      int idx = 0;
      for (int kk = -half; kk <= kz2; kk++)
        for (int jj = -half; jj <= half; jj++)
          for (int ii = -half; ii <= half; ii++, idx++) {
            int i = si + ii, j = sj + jj, k = sk + kk;
            if (i < p->ni1 || i > p->ni2 || j < p->nj1 || j > p->nj2 ||
                k < p->nk1 || k > p->nk2)
              continue;
            size_t q = i + j * ln + (size_t)k * sl;
            float c = wgt[idx];
            if (p->src_force && (p->src_surface_strict == 0 || k < p->nk2)) {
              float Vf = c * p->slw[q] / p->jac[q];
              h[VX * V + q] += fx * Vf;
              h[VY * V + q] += fy * Vf;
              h[VZ * V + q] += fz * Vf;
            }
            if (p->src_moment) {
              float rjac = c / p->jac[q];
              h[TXX * V + q] -= Mxx * rjac;
              h[TYY * V + q] -= Myy * rjac;
              h[TZZ * V + q] -= Mzz * rjac;
              h[TXZ * V + q] -= Mxz * rjac;
              h[TYZ * V + q] -= Myz * rjac;
              h[TXY * V + q] -= Mxy * rjac;
            }
          }
    }
  }
}

/* receivers (io_funcs.c:1584-1645), including the reference's use of
 * corner 5 twice and corner 4 never */
static void keep_recv(orc_t *o, const float *w, int it)
{
  const cgfd_problem_t *p = o->p;
  for (int n = 0; n < p->recv_n; n++) {
    const int *x = p->recv_indx1d + 8 * n;
    float Lx2 = p->recv_dijk[3 * n], Ly2 = p->recv_dijk[3 * n + 1],
          Lz2 = p->recv_dijk[3 * n + 2];
    float Lx1 = (float)(1.0 - (double)Lx2), Ly1 = (float)(1.0 - (double)Ly2),
          Lz1 = (float)(1.0 - (double)Lz2);
    for (int c = 0; c < p->recv_ncmp; c++) {
      const float *v = w + c * o->vol;
      p->recv_seismo[((size_t)n * p->recv_ncmp + c) * p->recv_max_nt + it] =
          v[x[0]] * Lx1 * Ly1 * Lz1 + v[x[1]] * Lx2 * Ly1 * Lz1 +
          v[x[2]] * Lx1 * Ly2 * Lz1 + v[x[3]] * Lx2 * Ly2 * Lz1 +
          v[x[5]] * Lx1 * Ly1 * Lz2 + v[x[5]] * Lx2 * Ly1 * Lz2 +
          v[x[6]] * Lx1 * Ly2 * Lz2 + v[x[7]] * Lx2 * Ly2 * Lz2;
    }
  }
  for (int n = 0; n < p->line_n; n++)
    for (int c = 0; c < p->ncmp; c++)
      p->line_seismo[((size_t)n * p->ncmp + c) * p->line_max_nt + it] =
          w[c * o->vol + p->line_iptr[n]];
}

/* surface peak ground motion after a step (forward/wav_t.c:379-455) */
static void pg_calcu(orc_t *o, const float *w1, const float *w0, float *PG,
                     float *Dis)
{
  const cgfd_problem_t *p = o->p;
  size_t s2 = o->sl, V = o->vol;
  float dt = p->dt;
  for (int j = p->nj1; j <= p->nj2; j++)
    for (int i = p->ni1; i <= p->ni2; i++) {
      size_t q = i + j * o->ln + (size_t)p->nk2 * s2, q1 = i + j * o->ln;
      float vx1 = w1[q], vy1 = w1[V + q], vz1 = w1[2 * V + q];
      float vx0 = w0[q], vy0 = w0[V + q], vz0 = w0[2 * V + q];
      float Ax = fabsf((vx1 - vx0) / dt), Ay = fabsf((vy1 - vy0) / dt),
            Az = fabsf((vz1 - vz0) / dt);
      float *Dx = Dis + q1, *Dy = Dis + s2 + q1, *Dz = Dis + 2 * s2 + q1;
      *Dx = (float)(*Dx + 0.5 * (vx1 + vx0) * dt);
      *Dy = (float)(*Dy + 0.5 * (vy1 + vy0) * dt);
      *Dz = (float)(*Dz + 0.5 * (vz1 + vz0) * dt);
      float v[15];
      v[0] = (float)sqrt(vx1 * vx1 + vy1 * vy1 + vz1 * vz1);
      v[1] = (float)sqrt(vx1 * vx1 + vy1 * vy1);
      v[2] = fabsf(vx1); v[3] = fabsf(vy1); v[4] = fabsf(vz1);
      v[5] = (float)sqrt(Ax * Ax + Ay * Ay + Az * Az);
      v[6] = (float)sqrt(Ax * Ax + Ay * Ay);
      v[7] = Ax; v[8] = Ay; v[9] = Az;
      v[10] = (float)sqrt(*Dx * *Dx + *Dy * *Dy + *Dz * *Dz);
      v[11] = (float)sqrt(*Dx * *Dx + *Dy * *Dy);
      v[12] = fabsf(*Dx); v[13] = fabsf(*Dy); v[14] = fabsf(*Dz);
      for (int m = 0; m < 15; m++)
        if (PG[m * s2 + q1] < v[m]) PG[m * s2 + q1] = v[m];
    }
}

/* ------------------------------------------------------------------------ */
/* time loop                                                                */
/* ------------------------------------------------------------------------ */

static void slab(const orc_t *o, int tid, long n0, long n1, long *a, long *b)
{
  long n = n1 - n0, T = o->nthreads;
  *a = n0 + n * tid / T;
  *b = n0 + n * (tid + 1) / T;
}

static void *worker(void *arg)
{
  thr_t *th = (thr_t *)arg;
  orc_t *o = th->o;
  const cgfd_problem_t *p = o->p;
  int tid = th->tid;
  size_t V = o->vol;
  size_t L = V * p->ncmp;
  float *pre = o->lev[0], *tmp = o->lev[1], *rhs = o->lev[2], *end = o->lev[3];
  float *apre[3][2], *atmp[3][2], *arhs[3][2], *aend[3][2];
  for (int d = 0; d < 3; d++)
    for (int s = 0; s < 2; s++) {
      apre[d][s] = o->aux[d][s][0]; atmp[d][s] = o->aux[d][s][1];
      arhs[d][s] = o->aux[d][s][2]; aend[d][s] = o->aux[d][s][3];
    }
  long k0, k1, e0, e1;
  slab(o, tid, p->nk1, p->nk2 + 1, &k0, &k1);
  slab(o, tid, 0, (long)L, &e0, &e1);

  for (int it = 0; it < p->nt_total; it++) {
    int ipair = it % 8;
    for (int is = 0; is < 4; is++) {
      const float *cur = (is == 0) ? pre : tmp;
      int bx = (PAIR_FLAGS[ipair][0] + is) % 2;
      int by = (PAIR_FLAGS[ipair][1] + is) % 2;
      int bz = (PAIR_FLAGS[ipair][2] + is) % 2;
      op5_t ox = make_op(bx, 1), oy = make_op(by, (long)o->ln),
            oz = make_op(bz, (long)o->sl);
      /* 0. surface force layers of this stage (drv_rk_curv_col.c:230) */
      if (o->TS) {
        if (tid == 0) surf_layer(o, it, is);
        pthread_barrier_wait(&o->bar);
      }
      /* 1. interior RHS on all physical points */
      for (long k = k0; k < k1; k++) rhs_inner_plane(o, cur, rhs, (int)k, &ox, &oy, &oz);
      pthread_barrier_wait(&o->bar);
      /* 2./3. free surface overwrites (rows split over threads) */
      if (p->free_top) {
        for (int j = p->nj1 + tid; j <= p->nj2; j += o->nthreads) {
          rhs_timg_row(o, cur, rhs, j, bz, &ox, &oy);
          rhs_vlow_row(o, cur, rhs, j, bz, &ox, &oy);
        }
      }
      pthread_barrier_wait(&o->bar);
      /* 4. PML corrections, faces in reference order, per point */
      for (int d = 0; d < 3; d++)
        for (int s = 0; s < 2; s++) {
          const cgfd_pml_face_t *f = &p->pml[d][s];
          if (!f->enabled) continue;
          const op5_t *op = d == 0 ? &ox : (d == 1 ? &oy : &oz);
          const float *acur = (is == 0) ? apre[d][s] : atmp[d][s];
          for (long k = k0; k < k1; k++) {
            if (k < f->nk1 || k > f->nk2) continue;
            rhs_pml_face_plane(o, cur, rhs, d, s, (int)k, op, acur, arhs[d][s]);
          }
        }
      pthread_barrier_wait(&o->bar);
      /* 4b. GMB attenuation (visco-elastic media) */
      if (p->medium_type == CGFD_MEDIUM_VISCOELASTIC_ISO) {
        for (long k = k0; k < k1; k++) rhs_atten_plane(o, cur, rhs, (int)k);
        pthread_barrier_wait(&o->bar);
      }
      /* 5. sources */
      if (tid == 0 && p->src_n > 0) rhs_src(o, rhs, it, is);
      if (tid == 0 && p->dd_n > 0 && it < p->dd_max_nt) rhs_srcdd(o, rhs, it, is);
      pthread_barrier_wait(&o->bar);
      /* RK combine over the whole padded volume (drv_rk_curv_col.c:292-446) */
      if (is < 3) {
        float ca = RK_A[is] * p->dt;
        float cb = RK_B[is] * p->dt;
        for (long e = e0; e < e1; e++) tmp[e] = pre[e] + ca * rhs[e];
        for (int d = 0; d < 3; d++)
          for (int s = 0; s < 2; s++) {
            if (!p->pml[d][s].enabled) continue;
            long a0, a1;
            slab(o, tid, 0, (long)(o->aux_vol[d][s] * p->ncmp), &a0, &a1);
            for (long e = a0; e < a1; e++)
              atmp[d][s][e] = apre[d][s][e] + ca * arhs[d][s][e];
          }
        if (is == 0)
          for (long e = e0; e < e1; e++) end[e] = pre[e] + cb * rhs[e];
        else
          for (long e = e0; e < e1; e++) end[e] += cb * rhs[e];
        for (int d = 0; d < 3; d++)
          for (int s = 0; s < 2; s++) {
            if (!p->pml[d][s].enabled) continue;
            long a0, a1;
            slab(o, tid, 0, (long)(o->aux_vol[d][s] * p->ncmp), &a0, &a1);
            if (is == 0)
              for (long e = a0; e < a1; e++)
                aend[d][s][e] = apre[d][s][e] + cb * arhs[d][s][e];
            else
              for (long e = a0; e < a1; e++) aend[d][s][e] += cb * arhs[d][s][e];
          }
      } else {
        float cb = RK_B[is] * p->dt;
        for (long e = e0; e < e1; e++) end[e] += cb * rhs[e];
        if (p->graves_qs) {      /* drv_rk_curv_col.c:414-416 */
          pthread_barrier_wait(&o->bar);
          graves_qs_slab(o, end, k0, k1);
        }
        for (int d = 0; d < 3; d++)
          for (int s = 0; s < 2; s++) {
            if (!p->pml[d][s].enabled) continue;
            long a0, a1;
            slab(o, tid, 0, (long)(o->aux_vol[d][s] * p->ncmp), &a0, &a1);
            for (long e = a0; e < a1; e++) aend[d][s][e] += cb * arhs[d][s][e];
          }
        /* visco-elastic free surface (drv_rk_curv_col.c:440-445) */
        if (p->medium_type == CGFD_MEDIUM_VISCOELASTIC_ISO && p->free_top) {
          pthread_barrier_wait(&o->bar);
          for (int j = p->nj1 + tid; j <= p->nj2; j += o->nthreads)
            vis_free_row(o, end, j);
        }
      }
      pthread_barrier_wait(&o->bar);
    }
    if (tid == 0) {
      if (p->ablexp) ablexp_apply(o, end);      /* drv_rk_curv_col.c:484-486 */
      if (o->pg) pg_calcu(o, end, pre, o->pg, o->dis);
      keep_recv(o, end, it);
    }
    /* swap pre and end (drv_rk_curv_col.c:530-542) */
    float *t = pre; pre = end; end = t;
    for (int d = 0; d < 3; d++)
      for (int s = 0; s < 2; s++) {
        float *u = apre[d][s]; apre[d][s] = aend[d][s]; aend[d][s] = u;
      }
    pthread_barrier_wait(&o->bar);
  }
  (void)V;
  return NULL;
}

/*
 * Runs the whole time loop on the host arrays of `p` (wav and PML aux are
 * updated in place, level semantics as in the reference; seismograms
 * written).  mVx/mVy/mF receive the free-surface matrices (nx*ny*9 each,
 * may be NULL when there is no free surface).
 */
int oracle_allstep_pg(const cgfd_problem_t *p, int timg_mode, int nthreads,
                      float *mVx, float *mVy, float *mF, float *pg);

int oracle_allstep(const cgfd_problem_t *p, int timg_mode, int nthreads,
                   float *mVx, float *mVy, float *mF)
{
  return oracle_allstep_pg(p, timg_mode, nthreads, mVx, mVy, mF, NULL);
}

/* as oracle_allstep; pg (15 x nx*ny, zero on entry) receives the surface
 * peak-motion maps when non-NULL and the top is free */
int oracle_allstep_pg(const cgfd_problem_t *p, int timg_mode, int nthreads,
                      float *mVx, float *mVy, float *mF, float *pg)
{
  int med = p->medium_type;
  if (med != CGFD_MEDIUM_ELASTIC_ISO && med != CGFD_MEDIUM_ELASTIC_VTI &&
      med != CGFD_MEDIUM_ELASTIC_ANISO && med != CGFD_MEDIUM_VISCOELASTIC_ISO)
    return CGFD_EINVAL;
  if (p->src_n_surface_force > 0 &&
      (!p->src_force || !p->src_force_rate_indx || !p->Fx_rate || !p->Fy_rate ||
       !p->Fz_rate || !p->free_top))
    return CGFD_EINVAL;
  int ncmp_want = 9;
  if (med == CGFD_MEDIUM_VISCOELASTIC_ISO) {
    if (p->nmaxwell < 1 || p->nmaxwell > CGFD_MAX_MAXWELL || !p->wl) return CGFD_EINVAL;
    if (p->free_top && (!p->x3d || !p->y3d || !p->z3d)) return CGFD_EINVAL;
    ncmp_want += 6 * p->nmaxwell;
  }
  if (p->nlevel != 4 || p->ncmp != ncmp_want) return CGFD_EINVAL;
  orc_t o;
  memset(&o, 0, sizeof(o));
  o.p = p;
  o.ln = p->nx;
  o.sl = (size_t)p->nx * p->ny;
  o.vol = o.sl * p->nz;
  o.timg_mode = timg_mode;
  o.nthreads = nthreads < 1 ? 1 : nthreads;
  for (int l = 0; l < 4; l++) o.lev[l] = p->wav + (size_t)l * o.vol * p->ncmp;
  for (int d = 0; d < 3; d++)
    for (int s = 0; s < 2; s++) {
      const cgfd_pml_face_t *f = &p->pml[d][s];
      if (!f->enabled) continue;
      size_t av = (size_t)(f->ni2 - f->ni1 + 1) * (f->nj2 - f->nj1 + 1) *
                  (f->nk2 - f->nk1 + 1);
      o.aux_vol[d][s] = av;
      for (int l = 0; l < 4; l++) o.aux[d][s][l] = f->aux + (size_t)l * av * p->ncmp;
    }
  size_t n2 = o.sl * 9;
  int own_m = 0;
  if (p->free_top) {
    if (!mVx) {
      mVx = calloc(n2, sizeof(float));
      mVy = calloc(n2, sizeof(float));
      mF = calloc(n2, sizeof(float));
      own_m = 1;
    } else {
      memset(mVx, 0, n2 * 4); memset(mVy, 0, n2 * 4); memset(mF, 0, n2 * 4);
    }
    if (med == CGFD_MEDIUM_ELASTIC_VTI) {
      oracle_dvh2dvz_vti(p, mVx, mVy);
    } else if (med == CGFD_MEDIUM_ELASTIC_ANISO) {
      oracle_dvh2dvz_aniso(p, mVx, mVy);
    } else if (med == CGFD_MEDIUM_VISCOELASTIC_ISO) {
      o.mD = calloc(n2, sizeof(float));
      oracle_dvh2dvz_vis(p, mVx, mVy, o.mD);
    } else {
      oracle_dvh2dvz_iso(p, mVx, mVy, mF);
    }
  }
  o.mVx = mVx; o.mVy = mVy; o.mF = mF;
  o.med = med;
  if (p->src_n > 0 && p->src_spatial != CGFD_SRC_POINT) {
    int n1 = 2 * p->src_ext_half + 1;
    o.ext = calloc(p->src_n, sizeof(float *));
    for (int is = 0; is < p->src_n; is++) {
      o.ext[is] = calloc((size_t)n1 * n1 * n1, sizeof(float));
      int sk = p->src_sk[is], half = p->src_ext_half;
      int kz2 = (sk + half < p->nk2) ? half : p->nk2 - sk;
      src_weights(o.ext[is], p->src_si_inc[is], p->src_sj_inc[is],
                  p->src_sk_inc[is], p->src_ext_coef, half, kz2);
    }
  }
  if (p->src_n > 0 && p->src_n_surface_force > 0) {
    o.TS = calloc(3 * o.sl, sizeof(float));
    o.VS = calloc(3 * o.sl, sizeof(float));
  }
  if (pg && p->free_top) {
    o.pg = pg;
    o.dis = calloc(3 * o.sl, sizeof(float));
  }
  pthread_barrier_init(&o.bar, NULL, o.nthreads);
  pthread_t *ths = calloc(o.nthreads, sizeof(pthread_t));
  thr_t *ta = calloc(o.nthreads, sizeof(thr_t));
  for (int t = 0; t < o.nthreads; t++) {
    ta[t].o = &o;
    ta[t].tid = t;
    if (t > 0) pthread_create(&ths[t], NULL, worker, &ta[t]);
  }
  worker(&ta[0]);
  for (int t = 1; t < o.nthreads; t++) pthread_join(ths[t], NULL);
  pthread_barrier_destroy(&o.bar);
  free(ths);
  free(ta);
  if (o.ext) {
    for (int is = 0; is < p->src_n; is++) free(o.ext[is]);
    free(o.ext);
  }
  if (own_m) { free(mVx); free(mVy); free(mF); }
  free(o.mD);
  free(o.TS);
  free(o.VS);
  free(o.dis);
  return 0;
}

/* ------------------------------------------------------------------------ */
/* grid metrics (forward/gd_t.c:190-402)                                    */
/* ------------------------------------------------------------------------ */

/* Restatement of gd_curv_metric_cal: centred 7-point derivatives of the
 * node coordinates along i, j, k (all seven taps, the zero centre
 * included, left to right), the Jacobian as (x_xi x x_et) . x_zt and the
 * contravariant metrics as cross products over it, then the ghost layers
 * mirrored x, y, z in turn.  out: 10 x nx*ny*nz (jac, xi_x..zeta_z). */
int oracle_metric_calc(int nx, int ny, int nz, int ni1, int ni2, int nj1,
                       int nj2, int nk1, int nk2, const float *x3d,
                       const float *y3d, const float *z3d, float *out)
{
  size_t ln = nx, sl = (size_t)nx * ny, V = sl * nz;
  float *m[10];
  for (int c = 0; c < 10; c++) m[c] = out + c * V;
  long sx[7], sy[7], sz[7];
  for (int n = 0; n < 7; n++) {
    sx[n] = n - 3;
    sy[n] = (long)(n - 3) * (long)ln;
    sz[n] = (long)(n - 3) * (long)sl;
  }
  for (int k = nk1; k <= nk2; k++)
    for (int j = nj1; j <= nj2; j++)
      for (int i = ni1; i <= ni2; i++) {
        size_t q = i + j * ln + (size_t)k * sl;
        const float *cx[3] = {x3d, y3d, z3d};
        float d[3][3];                 /* d[axis][coord] */
        const long *sh[3] = {sx, sy, sz};
        for (int ax = 0; ax < 3; ax++)
          for (int c = 0; c < 3; c++) {
            float v = FDC_COEF[0] * cx[c][q + sh[ax][0]];
            for (int n = 1; n < 7; n++) v += FDC_COEF[n] * cx[c][q + sh[ax][n]];
            d[ax][c] = v;
          }
        const float *v1 = d[0], *v2 = d[1], *v3 = d[2];
        float g[3];
        g[0] = v1[1] * v2[2] - v1[2] * v2[1];
        g[1] = v1[2] * v2[0] - v1[0] * v2[2];
        g[2] = v1[0] * v2[1] - v1[1] * v2[0];
        float jac = 0.0f;
        for (int c = 0; c < 3; c++) jac += g[c] * v3[c];
        m[0][q] = jac;
        const float *pa[3] = {v2, v3, v1}, *pb[3] = {v3, v1, v2};
        for (int r = 0; r < 3; r++) {
          const float *A = pa[r], *B = pb[r];
          g[0] = A[1] * B[2] - A[2] * B[1];
          g[1] = A[2] * B[0] - A[0] * B[2];
          g[2] = A[0] * B[1] - A[1] * B[0];
          for (int c = 0; c < 3; c++) m[1 + 3 * r + c][q] = g[c] / jac;
        }
      }
  /* ghosts: mirrored about the physical boundary, x then y then z */
  for (int c = 0; c < 10; c++) {
    float *a = m[c];
    for (int k = 0; k < nz; k++)
      for (int j = 0; j < ny; j++) {
        size_t r = j * ln + (size_t)k * sl;
        for (int i = 0; i < ni1; i++) a[r + i] = a[r + 2 * ni1 - 1 - i];
        for (int i = ni2 + 1; i < nx; i++) a[r + i] = a[r + 2 * ni2 + 1 - i];
      }
    for (int k = 0; k < nz; k++)
      for (int j = 0; j < ny; j++) {
        size_t r = j * ln + (size_t)k * sl;
        if (j < nj1) memcpy(a + r, a + (2 * nj1 - 1 - j) * ln + (size_t)k * sl, ln * 4);
        if (j > nj2) memcpy(a + r, a + (2 * nj2 + 1 - j) * ln + (size_t)k * sl, ln * 4);
      }
    for (int k = 0; k < nz; k++) {
      if (k < nk1) memcpy(a + (size_t)k * sl, a + (size_t)(2 * nk1 - 1 - k) * sl, sl * 4);
      if (k > nk2) memcpy(a + (size_t)k * sl, a + (size_t)(2 * nk2 + 1 - k) * sl, sl * 4);
    }
  }
  return 0;
}

/* ------------------------------------------------------------------------ */
/* point location on a curvilinear grid: stations and sources given by      */
/* coordinates (set-up beside the time loop)                                 */
/* ------------------------------------------------------------------------ */

/* Restates, for a grid with 3 ghost layers on one rank:
 *   gd_curv_set_minmax            forward/gd_t.c:1708-1880 (global bounds,
 *                                 cell and 4x4x4 tile boxes)
 *   gd_curv_depth_to_axis         forward/gd_t.c:2179-2297
 *   gd_curv_coord_to_local_indx   forward/gd_t.c:1998-2171
 *   gd_curv_coord2shift_sample    forward/gd_t.c:2304-2370
 *   isPointInHexahedron           media/media_geometry3d.cpp:150-265
 *   fdlib_math_isPoint2InTri, _Point2InWhichTri, _computeZfromTri
 *                                 lib/fdlib_math.c:246-338
 * in float arithmetic ordered as there (-ffp-contract=off). */

#define LOC_TILES 4
#define LOC_SAMPLES 100

typedef struct { float x, y, z; } v3_t;

static v3_t v3_sub(v3_t a, v3_t b)
{
  v3_t r = {a.x - b.x, a.y - b.y, a.z - b.z};
  return r;
}
static float v3_dot(v3_t a, v3_t b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static v3_t v3_cross(v3_t a, v3_t b)
{
  v3_t r = {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
  return r;
}
static float v3_len(v3_t a) { return sqrtf(v3_dot(a, a)); }
static float tri_area2(v3_t a, v3_t b, v3_t c)
{
  return v3_len(v3_cross(v3_sub(b, a), v3_sub(c, a)));
}

/* a point on a triangle: the three sub-areas add up to its area */
static int on_tri(v3_t p, v3_t a, v3_t b, v3_t c)
{
  float s = tri_area2(p, a, b) + tri_area2(p, b, c) + tri_area2(p, c, a) -
            tri_area2(a, b, c);
  return fabs(s) < 1e-6;
}

/* the ten tetrahedra (two cuts into five) of a hexahedron with corners
 * numbered i + 2 j + 4 k, each as four faces */
static const unsigned char TETRA_FACES[10][4][3] = {
    {{0, 4, 2}, {2, 4, 1}, {1, 4, 0}, {0, 2, 1}},
    {{4, 6, 2}, {2, 6, 7}, {7, 6, 4}, {4, 2, 7}},
    {{2, 7, 3}, {3, 7, 1}, {1, 2, 3}, {1, 7, 2}},
    {{7, 4, 5}, {1, 7, 5}, {5, 4, 1}, {1, 4, 7}},
    {{2, 4, 7}, {7, 4, 1}, {2, 7, 1}, {4, 2, 1}},
    {{4, 5, 6}, {4, 6, 0}, {4, 0, 5}, {6, 5, 0}},
    {{6, 2, 0}, {6, 3, 2}, {0, 2, 3}, {3, 6, 0}},
    {{6, 5, 7}, {3, 6, 7}, {7, 5, 3}, {5, 6, 3}},
    {{5, 0, 1}, {3, 5, 1}, {0, 3, 1}, {0, 5, 3}},
    {{5, 6, 0}, {5, 0, 3}, {0, 6, 3}, {3, 6, 5}}};

static int in_hexahedron(v3_t p, const v3_t *v)
{
  for (int t = 0; t < 10; t++) {
    int inside = 1;
    for (int f = 0; f < 4 && inside; f++) {
      v3_t a = v[TETRA_FACES[t][f][0]], b = v[TETRA_FACES[t][f][1]];
      v3_t c = v[TETRA_FACES[t][f][2]];
      if (on_tri(p, a, b, c)) break;          /* on a face: inside */
      v3_t p2f = v3_sub(a, p);
      v3_t n = v3_cross(v3_sub(b, a), v3_sub(c, a));
      float d = v3_len(n);
      n.x = n.x / d; n.y = n.y / d; n.z = n.z / d;
      float sign = v3_dot(p2f, n);
      sign /= v3_len(p2f);
      if (sign <= -1.0e-6f) inside = 0;
    }
    if (inside) return 1;
  }
  return 0;
}

/* shift of p inside a cell: the closest of 101^3 trilinear samples, the
 * first in (k, j, i) order on ties */
static void cell_shift(v3_t p, const v3_t *v, float *si, float *sj, float *sk)
{
  float min_dist = sqrtf((p.x - v[0].x) * (p.x - v[0].x) + (p.y - v[0].y) * (p.y - v[0].y) +
                         (p.z - v[0].z) * (p.z - v[0].z));
  int bi = 0, bj = 0, bk = 0;
  for (int n3 = 0; n3 <= LOC_SAMPLES; n3++) {
    float lz[2];
    lz[1] = (float)n3 / (float)LOC_SAMPLES;
    lz[0] = 1.0 - lz[1];
    for (int n2 = 0; n2 <= LOC_SAMPLES; n2++) {
      float ly[2];
      ly[1] = (float)n2 / (float)LOC_SAMPLES;
      ly[0] = 1.0 - ly[1];
      for (int n1 = 0; n1 <= LOC_SAMPLES; n1++) {
        float lx[2];
        lx[1] = (float)n1 / (float)LOC_SAMPLES;
        lx[0] = 1.0 - lx[1];
        float x = 0, y = 0, z = 0;
        for (int c = 0; c < 8; c++) {
          float w = lx[c & 1] * ly[(c >> 1) & 1] * lz[c >> 2];
          x += w * v[c].x;
          y += w * v[c].y;
          z += w * v[c].z;
        }
        float d = sqrtf((p.x - x) * (p.x - x) + (p.y - y) * (p.y - y) + (p.z - z) * (p.z - z));
        if (min_dist > d) {
          min_dist = d;
          bi = n1; bj = n2; bk = n3;
        }
      }
    }
  }
  *si = (float)bi / (float)LOC_SAMPLES;
  *sj = (float)bj / (float)LOC_SAMPLES;
  *sk = (float)bk / (float)LOC_SAMPLES;
}

static int in_tri2(float px, float py, const float *vx, const float *vy)
{
  for (int i = 0; i < 3; i++) {
    float ex = i == 2 ? vx[0] - vx[2] : vx[i + 1] - vx[i];
    float ey = i == 2 ? vy[0] - vy[2] : vy[i + 1] - vy[i];
    float tx = px - vx[i], ty = py - vy[i];
    float sign = ex * ty - ey * tx;
    sign /= sqrt(ex * ex + ey * ey);
    if (sign < 0) return 0;
  }
  return 1;
}

static float z_on_tri(float x, float y, v3_t p1, v3_t p2, v3_t p3)
{
  float v1x = p2.x - p1.x, v1y = p2.y - p1.y, v1z = p2.z - p1.z;
  float v2x = p3.x - p1.x, v2y = p3.y - p1.y, v2z = p3.z - p1.z;
  float a = v1y * v2z - v1z * v2y;
  float b = v1z * v2x - v1x * v2z;
  float c = v1x * v2y - v1y * v2x;
  float d = -(a * p1.x + b * p1.y + c * p1.z);
  return -(a * x + b * y + d) / c;
}

typedef struct {
  int nx, ny, nz;
  size_t sl;
  const float *x, *y, *z;
  float xmin, xmax, ymin, ymax, zmin, zmax;
  int ts[3][LOC_TILES], te[3][LOC_TILES];
  float tb[LOC_TILES][LOC_TILES][LOC_TILES][6];   /* [kt][jt][it]: x0 x1 y0 y1 z0 z1 */
} loc_grid_t;

static v3_t grid_pt(const loc_grid_t *g, int i, int j, int k)
{
  size_t q = (size_t)i + (size_t)j * g->nx + (size_t)k * g->sl;
  v3_t r = {g->x[q], g->y[q], g->z[q]};
  return r;
}

static void cell_box(const loc_grid_t *g, int i, int j, int k, float *b)
{
  v3_t p = grid_pt(g, i, j, k);
  b[0] = b[1] = p.x; b[2] = b[3] = p.y; b[4] = b[5] = p.z;
  for (int c = 1; c < 8; c++) {
    v3_t q = grid_pt(g, i + (c & 1), j + ((c >> 1) & 1), k + (c >> 2));
    b[0] = b[0] < q.x ? b[0] : q.x; b[1] = b[1] > q.x ? b[1] : q.x;
    b[2] = b[2] < q.y ? b[2] : q.y; b[3] = b[3] > q.y ? b[3] : q.y;
    b[4] = b[4] < q.z ? b[4] : q.z; b[5] = b[5] > q.z ? b[5] : q.z;
  }
}

static void loc_grid_init(loc_grid_t *g, int nx, int ny, int nz, const float *x,
                          const float *y, const float *z)
{
  g->nx = nx; g->ny = ny; g->nz = nz;
  g->sl = (size_t)nx * ny;
  g->x = x; g->y = y; g->z = z;
  size_t vol = g->sl * nz;
  g->xmin = g->xmax = x[0]; g->ymin = g->ymax = y[0]; g->zmin = g->zmax = z[0];
  for (size_t q = 0; q < vol; q++) {
    g->xmin = g->xmin < x[q] ? g->xmin : x[q]; g->xmax = g->xmax > x[q] ? g->xmax : x[q];
    g->ymin = g->ymin < y[q] ? g->ymin : y[q]; g->ymax = g->ymax > y[q] ? g->ymax : y[q];
    g->zmin = g->zmin < z[q] ? g->zmin : z[q]; g->zmax = g->zmax > z[q] ? g->zmax : z[q];
  }
  const int n[3] = {nx - 6, ny - 6, nz - 6};
  for (int d = 0; d < 3; d++) {
    int avg = n[d] / LOC_TILES, left = n[d] % LOC_TILES;
    for (int t = 0; t < LOC_TILES; t++) {
      g->ts[d][t] = t == 0 ? 3 : g->te[d][t - 1] + 1;
      g->te[d][t] = g->ts[d][t] + avg - 1 + (t < left ? 1 : 0);
    }
  }
  for (int kt = 0; kt < LOC_TILES; kt++)
    for (int jt = 0; jt < LOC_TILES; jt++)
      for (int it = 0; it < LOC_TILES; it++) {
        float *tb = g->tb[kt][jt][it];
        tb[0] = tb[2] = tb[4] = 1.0e26f;
        tb[1] = tb[3] = tb[5] = -1.0e26f;
        for (int k = g->ts[2][kt]; k <= g->te[2][kt]; k++)
          for (int j = g->ts[1][jt]; j <= g->te[1][jt]; j++)
            for (int i = g->ts[0][it]; i <= g->te[0][it]; i++) {
              float b[6];
              cell_box(g, i, j, k, b);
              for (int e = 0; e < 6; e += 2) {
                tb[e] = tb[e] < b[e] ? tb[e] : b[e];
                tb[e + 1] = tb[e + 1] > b[e + 1] ? tb[e + 1] : b[e + 1];
              }
            }
      }
}

static void depth_to_axis(const loc_grid_t *g, float sx, float sy, float *sz)
{
  if (sx < g->xmin || sx > g->xmax || sy < g->ymin || sy > g->ymax) return;
  const int kt = LOC_TILES - 1, k = g->te[2][kt];
  for (int jt = 0; jt < LOC_TILES; jt++)
    for (int it = 0; it < LOC_TILES; it++) {
      const float *tb = g->tb[kt][jt][it];
      if (sx < tb[0] || sx > tb[1] || sy < tb[2] || sy > tb[3]) continue;
      for (int j = g->ts[1][jt]; j <= g->te[1][jt]; j++)
        for (int i = g->ts[0][it]; i <= g->te[0][it]; i++) {
          float b[6];
          cell_box(g, i, j, k, b);
          if (sx < b[0] || sx > b[1] || sy < b[2] || sy > b[3]) continue;
          v3_t p[4];
          float vx[5], vy[5];
          for (int c = 0; c < 4; c++) p[c] = grid_pt(g, i + (c & 1), j + (c >> 1), k);
          /* corners 0, 1, 3, 2 around the quadrilateral */
          vx[0] = p[0].x; vx[1] = p[1].x; vx[2] = p[3].x; vx[3] = p[2].x; vx[4] = p[0].x;
          vy[0] = p[0].y; vy[1] = p[1].y; vy[2] = p[3].y; vy[3] = p[2].y; vy[4] = p[0].y;
          if (in_tri2(sx, sy, vx + 2, vy + 2)) {
            *sz = z_on_tri(sx, sy, p[3], p[2], p[0]) - *sz;
            return;
          }
          if (in_tri2(sx, sy, vx, vy)) {
            *sz = z_on_tri(sx, sy, p[0], p[1], p[3]) - *sz;
            return;
          }
        }
    }
}

static int locate_one(const loc_grid_t *g, float sx, float sy, float sz, int *gi,
                      float *shift)
{
  gi[0] = gi[1] = gi[2] = -1000;
  shift[0] = shift[1] = shift[2] = 0.0f;
  if (sx < g->xmin || sx > g->xmax || sy < g->ymin || sy > g->ymax || sz < g->zmin ||
      sz > g->zmax)
    return 0;
  const v3_t p = {sx, sy, sz};
  for (int kt = 0; kt < LOC_TILES; kt++)
    for (int jt = 0; jt < LOC_TILES; jt++)
      for (int it = 0; it < LOC_TILES; it++) {
        const float *tb = g->tb[kt][jt][it];
        if (sx < tb[0] || sx > tb[1] || sy < tb[2] || sy > tb[3] || sz < tb[4] ||
            sz > tb[5])
          continue;
        for (int k = g->ts[2][kt]; k <= g->te[2][kt]; k++)
          for (int j = g->ts[1][jt]; j <= g->te[1][jt]; j++)
            for (int i = g->ts[0][it]; i <= g->te[0][it]; i++) {
              float b[6];
              cell_box(g, i, j, k, b);
              if (sx < b[0] || sx > b[1] || sy < b[2] || sy > b[3] || sz < b[4] ||
                  sz > b[5])
                continue;
              v3_t v[8];
              for (int c = 0; c < 8; c++)
                v[c] = grid_pt(g, i + (c & 1), j + ((c >> 1) & 1), k + (c >> 2));
              if (!in_hexahedron(p, v)) continue;
              int li[3] = {i, j, k};
              cell_shift(p, v, &shift[0], &shift[1], &shift[2]);
              for (int d = 0; d < 3; d++) {
                if (shift[d] > 0.5) {
                  li[d] += 1;
                  shift[d] -= 1.0;
                }
                gi[d] = li[d] - 3;      /* local with ghosts -> global physical */
              }
              return 1;
            }
      }
  return 0;
}

/* Locates n points (is_depth[q]: pz[q] is a depth below the surface, first
 * converted to z).  Per point: found, global physical indices (-1000 when
 * not found), shifts in the cell, and the z that was located. */
int oracle_locate(int nx, int ny, int nz, const float *x3d, const float *y3d,
                  const float *z3d, int n, const float *px, const float *py,
                  const float *pz, const int *is_depth, int *found, int *idx,
                  float *shift, float *zout)
{
  loc_grid_t g;
  loc_grid_init(&g, nx, ny, nz, x3d, y3d, z3d);
  for (int q = 0; q < n; q++) {
    float sz = pz[q];
    if (is_depth && is_depth[q]) depth_to_axis(&g, px[q], py[q], &sz);
    found[q] = locate_one(&g, px[q], py[q], sz, idx + 3 * q, shift + 3 * q);
    zout[q] = sz;
  }
  return 0;
}

/* ------------------------------------------------------------------------ */
/* layered media: elastic isotropic model discretised with the "loc" method  */
/* ------------------------------------------------------------------------ */

/* Restates media_layer2model_el_iso with "loc" (media/media_layer2model.cpp:
 * 140-190, 422-560, 1334-1384) and its helpers (media/media_utility.cpp:
 * 53-55, 88-140, 173-209).  rec: [NI][NY][NX][10] = elevation, rho,
 * rho_grad, rho_pow, vp, vp_grad, vp_pow, vs, vs_grad, vs_pow.  Returns 1
 * when a point lies outside the interface mesh or vp <= sqrt(2) vs (where
 * the reference exits), else 0. */

#define LAY_MAXI 64

static float lay_bilinear(const float *xv, int NX, const float *yv, int NY,
                          const float *v, int stride, float xq, float yq)
{
  int ix = (xq - xv[0]) / (xv[1] - xv[0]);
  int iy = (yq - yv[0]) / (yv[1] - yv[0]);
  if (ix < 0 || iy < 0) return FLT_MAX;
  int indx = iy * NX + ix;
  if (ix == NX - 1 || iy == NY - 1) return v[indx * stride];
  float area = (xv[ix + 1] - xv[ix]) * (yv[iy + 1] - yv[iy]);
  float vq = v[indx * stride] * (xv[ix + 1] - xq) * (yv[iy + 1] - yq) +
             v[(indx + 1) * stride] * (xq - xv[ix]) * (yv[iy + 1] - yq) +
             v[(indx + NX) * stride] * (xv[ix + 1] - xq) * (yq - yv[iy]) +
             v[(indx + 1 + NX) * stride] * (xq - xv[ix]) * (yq - yv[iy]);
  vq /= area;
  return vq;
}

static int lay_last_ge(float value, const float *x, int n)
{
  if (value > x[0]) return -1;
  float dist = FLT_MAX;
  int indx = -1;
  for (int i = 0; i < n; i++) {
    if (x[i] == -FLT_MAX) continue;
    float d = x[i] - value;
    if (d < 0) break;
    if (d >= 0 && d <= dist) { dist = d; indx = i; }
  }
  return indx;
}

static int lay_first_ge(float value, const float *x, int n)
{
  float dist = FLT_MAX;
  int idx = -1;
  for (int i = 0; i < n; i++) {
    if (x[i] == -FLT_MAX) continue;
    float d = x[i] - value;
    if (d >= 0 && d <= dist) {
      if (d <= 1e-6) return i;
      dist = d;
      idx = i;
    }
  }
  return idx;
}

/* media kinds of a layered model, with the reference's numbers
 * (media/media_utility.hpp:38-43): one component (Qp, Qs, ...), elastic
 * isotropic (rho vp vs) and the
 * three VTI parametrisations (rho vph vpv vsh vsv eta / rho vp0 vs0 epsilon
 * delta gamma / rho c11 c33 c55 c66 c13) */
#define LAY_ONE 0
#define LAY_ISO 21
#define LAY_VTI_PREM 22
#define LAY_VTI_THOMSEN 23
#define LAY_VTI_CIJ 24

typedef struct {
  int kind, np, nc;          /* properties per point; record width 1 + 3 np */
  int NI, NX, NY;
  const float *xv, *yv, *rec;
  size_t slice;
  float minx, maxx, miny, maxy;
  float *elev;
} lay_model_t;

/* value + pow(dz, power) * grad of property p of layer mi at (x, y) */
static float lay_value(const lay_model_t *m, int mi, int p, float dz, float x, float y)
{
  const float *r = m->rec + mi * m->slice * m->nc + 1 + 3 * p;
  float v = lay_bilinear(m->xv, m->NX, m->yv, m->NY, r, m->nc, x, y);
  float g = lay_bilinear(m->xv, m->NX, m->yv, m->NY, r + 1, m->nc, x, y);
  float pw = lay_bilinear(m->xv, m->NX, m->yv, m->NY, r + 2, m->nc, x, y);
  return v + pow(dz, pw) * g;
}

/* the properties of one point: AssignLayerMediaPara2Point with
 * CalPointValue_layer (media/media_layer2model.cpp:422-830).  Returns 1
 * where the reference exits (outside the mesh; for elastic isotropic media
 * also vp <= sqrt(2) vs), else 0. */
static int lay_point(const lay_model_t *m, float x, float y, float z, float *var)
{
  const int NI = m->NI;
  float *elev = m->elev;
  if (x < m->minx || x > m->maxx || y < m->miny || y > m->maxy) return 1;
  for (int n = 0; n < NI; n++)
    elev[n] = lay_bilinear(m->xv, m->NX, m->yv, m->NY, m->rec + n * m->slice * m->nc, m->nc,
                           x, y);
  int mi = lay_last_ge(z, elev, NI);
  if (mi == -1) {
    mi = lay_last_ge(elev[0], elev, NI);
    for (int p = 0; p < m->np; p++)
      var[p] = lay_bilinear(m->xv, m->NX, m->yv, m->NY, m->rec + mi * m->slice * m->nc + 1 + 3 * p,
                            m->nc, x, y);
    return 0;
  }
  float dz = elev[mi] - z;
  for (int p = 0; p < m->np; p++) var[p] = lay_value(m, mi, p, dz, x, y);
  if (m->kind == LAY_ISO && var[1] <= var[2] * sqrt(2)) return 1;
  if (fabsf(dz - 0.0f) < FLT_EPSILON) {
    int m2 = lay_first_ge(z, elev, NI) - 1;
    if (m2 >= 0) {
      /* the layer above is taken at its own interface's depth, except for
       * elastic_vti_cij models: that branch of the reference keeps the
       * point's dz (media/media_layer2model.cpp:742-774; the others
       * recompute it, :617, :690) */
      float dz2 = m->kind == LAY_VTI_CIJ ? dz : elev[m2] - z;
      for (int p = 0; p < m->np; p++) {
        float top = lay_value(m, m2, p, dz2, x, y);
        var[p] = (var[p] + top) / 2.0;
      }
    }
  }
  return 0;
}

/* VTI stiffness from the point's parameters (para2vti,
 * media/media_utility.cpp:827-882): c = c11 c33 c55 c66 c13 rho */
static void lay_para2vti(int kind, const float *var, float *c)
{
  if (kind == LAY_VTI_PREM) {
    float vph = var[1], vpv = var[2], vsh = var[3], vsv = var[4], rho = var[0], eta = var[5];
    c[0] = vph * vph * rho;
    c[1] = vpv * vpv * rho;
    c[3] = vsh * vsh * rho;
    c[2] = vsv * vsv * rho;
    c[5] = rho;
    c[4] = eta * (c[0] - 2.0 * c[2]);
  } else if (kind == LAY_VTI_THOMSEN) {
    float rho = var[0], vp0 = var[1], vs0 = var[2], epsil = var[3], delta = var[4];
    float gamma = var[5];
    float c33 = vp0 * vp0 * rho, c55 = vs0 * vs0 * rho;
    c[5] = rho;
    c[1] = c33;
    c[2] = c55;
    c[3] = 2.0 * gamma * c55 + c55;
    c[0] = 2.0 * epsil * c33 + c33;
    c[4] = sqrt(2.0 * delta * c33 * (c33 - c55) + (c33 - c55) * (c33 - c55)) - c55;
  } else {
    c[0] = var[1];
    c[1] = var[2];
    c[2] = var[3];
    c[3] = var[4];
    c[4] = var[5];
    c[5] = var[0];
  }
}

/* the half grid of a curvilinear grid: each point but the last along an
 * axis moved to the centre of the cell above it (media/media_utility.cpp:
 * 656-760, GRID_CURV) */
static void lay_half_grid(int nx, int ny, int nz, const float *G, float *H)
{
  const size_t line = nx, sl = (size_t)nx * ny, vol = sl * nz;
  memcpy(H, G, vol * sizeof(float));
  for (int k = 0; k < nz - 1; k++)
    for (int j = 0; j < ny - 1; j++)
      for (int i = 0; i < nx - 1; i++) {
        size_t q = i + j * line + k * sl;
        H[q] = (G[q] + G[q + 1] + G[q + line + 1] + G[q + line] + G[q + sl] + G[q + sl + 1] +
                G[q + sl + line + 1] + G[q + line + sl]) / 8.0;
      }
}

/* the layer number of each half-grid point (MarkInterfaceNumber,
 * media/media_layer2model.cpp:1515-1598, GRID_CURV) */
static void lay_mark(const lay_model_t *m, size_t vol, const float *Hx, const float *Hy,
                     const float *Hz, int *mat)
{
  for (size_t q = 0; q < vol; q++) {
    for (int n = 0; n < m->NI; n++)
      m->elev[n] = lay_bilinear(m->xv, m->NX, m->yv, m->NY, m->rec + n * m->slice * m->nc,
                                m->nc, Hx[q], Hy[q]);
    int mi = lay_last_ge(Hz[q], m->elev, m->NI);
    if (mi == -1) mi = lay_last_ge(m->elev[0], m->elev, m->NI);
    mat[q] = mi;
  }
}

/* distinct values among 8 layer numbers, 0 when one is -1
 * (NumOfValues, media/media_utility.cpp:610-624) */
static int lay_num_values(const int *v)
{
  int tab[LAY_MAXI] = {0}, num = 0;
  for (int i = 0; i < 8; i++) {
    if (v[i] == -1) return 0;
    if (tab[v[i]] == 0) num++;
    tab[v[i]]++;
  }
  return num;
}

#define LAY_NG 8

/* sample (i, j, k) of the (NG+1)^3 points spanning a cell of 8 vertices
 * (MeshSubdivide, media/media_utility.cpp:627-654) */
static void lay_subpoint(const float (*v)[3], int i, int j, int k, float *p)
{
  const float ng = LAY_NG;
  for (int d = 0; d < 3; d++) {
    float ly00 = v[0][d] + (v[1][d] - v[0][d]) / ng * j;
    float ly10 = v[3][d] + (v[2][d] - v[3][d]) / ng * j;
    float ly01 = v[4][d] + (v[5][d] - v[4][d]) / ng * j;
    float ly11 = v[7][d] + (v[6][d] - v[7][d]) / ng * j;
    float lxy0 = ly00 + (ly10 - ly00) / ng * i;
    float lxy1 = ly01 + (ly11 - ly01) / ng * i;
    p[d] = lxy0 + (lxy1 - lxy0) / ng * k;
  }
}

/* The output of one point from its properties: lambda, mu, rho (elastic
 * isotropic; media/media_layer2model.cpp:1375-1380) or c11 c33 c55 c66 c13
 * rho (VTI). */
static void lay_store(int kind, const float *var, float **out, size_t q)
{
  if (kind == LAY_ONE) {
    out[0][q] = var[0];
  } else if (kind == LAY_ISO) {
    float vp = var[1], vs = var[2], r = var[0];
    out[1][q] = vs * vs * r;
    out[0][q] = vp * vp * r - 2.0 * out[1][q];
    out[2][q] = r;
  } else {
    float c[6];
    lay_para2vti(kind, var, c);
    for (int n = 0; n < 6; n++) out[n][q] = c[n];
  }
}

/* kind: LAY_ONE, LAY_ISO or LAY_VTI_*; method 0: loc; 1: har; 2: ari.  har and ari
 * start from loc and recompute the points whose cell (between the half-grid
 * points around them) touches more than one layer from its 9^3 samples:
 * elastic isotropic har: harmonic kappa and mu, arithmetic rho
 * (media/media_layer2model.cpp:1984-2095); ari: arithmetic lambda, mu, rho
 * (:2098-2190); VTI har: harmonic c11 c13 c33 c55 c66, arithmetic rho
 * (:2197-2314); ari: all arithmetic (:2317-2436); one component: the value
 * harmonically or arithmetically (:1603-1782).  out: 1 (one component), 3
 * (isotropic: lambda, mu, rho) or 6 (VTI: c11 c33 c55 c66 c13 rho) arrays. */
int oracle_layer(int kind, int method, int NI, int NX, int NY, float MINX, float MINY,
                 float DX, float DY, const float *rec, int nx, int ny, int nz,
                 const float *x3d, const float *y3d, const float *z3d, float **out)
{
  if (NI < 1 || NI > LAY_MAXI) return 1;
  if (kind != LAY_ONE && kind != LAY_ISO && kind != LAY_VTI_PREM && kind != LAY_VTI_THOMSEN &&
      kind != LAY_VTI_CIJ)
    return 1;
  const int np = kind == LAY_ONE ? 1 : kind == LAY_ISO ? 3 : 6;
  float *xv = malloc(NX * sizeof(float)), *yv = malloc(NY * sizeof(float));
  float *elev = malloc(NI * sizeof(float));
  for (int i = 0; i < NX; i++) xv[i] = MINX + DX * i;
  for (int j = 0; j < NY; j++) yv[j] = MINY + DY * j;
  lay_model_t m = {kind, np, 1 + 3 * np, NI, NX, NY, xv, yv, rec, (size_t)NX * NY, MINX,
                   MINX + (NX - 1) * DX, MINY, MINY + (NY - 1) * DY, elev};
  int bad = 0;
  const size_t line = nx, sl = (size_t)nx * ny, vol = sl * nz;
  for (size_t q = 0; q < vol && !bad; q++) {
    float var[6];
    if (lay_point(&m, x3d[q], y3d[q], z3d[q], var)) { bad = 1; break; }
    lay_store(kind, var, out, q);
  }
  if (method != 0 && !bad) {
    float *Hx = malloc(vol * sizeof(float)), *Hy = malloc(vol * sizeof(float));
    float *Hz = malloc(vol * sizeof(float));
    int *mat = malloc(vol * sizeof(int));
    lay_half_grid(nx, ny, nz, x3d, Hx);
    lay_half_grid(nx, ny, nz, y3d, Hy);
    lay_half_grid(nx, ny, nz, z3d, Hz);
    lay_mark(&m, vol, Hx, Hy, Hz, mat);
    const int nsg = (LAY_NG + 1) * (LAY_NG + 1) * (LAY_NG + 1);
    for (int j = 1; j < ny - 1 && !bad; j++)
      for (int k = 1; k < nz - 1 && !bad; k++)
        for (int i = 1; i < nx - 1 && !bad; i++) {
          size_t q = i + j * line + k * sl;
          /* the cell's vertices, in the reference's order */
          const size_t c[8] = {q - 1 - line - sl, q - 1 - sl, q - sl, q - line - sl,
                               q - 1 - line, q - 1, q, q - line};
          int v[8];
          for (int n = 0; n < 8; n++) v[n] = mat[c[n]];
          if (lay_num_values(v) <= 1) continue;
          float vert[8][3];
          for (int n = 0; n < 8; n++) {
            vert[n][0] = Hx[c[n]];
            vert[n][1] = Hy[c[n]];
            vert[n][2] = Hz[c[n]];
          }
          /* isotropic: s[0] rho, s[1] kappa or lambda, s[2] mu;
           * VTI: s[0..4] c11 c33 c55 c66 c13, s[5] rho */
          float s[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
          for (int kk = 0; kk <= LAY_NG && !bad; kk++)
            for (int jj = 0; jj <= LAY_NG && !bad; jj++)
              for (int ii = 0; ii <= LAY_NG; ii++) {
                float p[3], var[6];
                lay_subpoint((const float (*)[3])vert, ii, jj, kk, p);
                if (lay_point(&m, p[0], p[1], p[2], var)) { bad = 1; break; }
                if (kind == LAY_ONE) {
                  if (method == 1)
                    s[0] += (1.0 / var[0]);
                  else
                    s[0] += var[0];
                } else if (kind == LAY_ISO) {
                  float vp = var[1], vs = var[2], r = var[0];
                  float mu_ = vs * vs * r;
                  float lambda = vp * vp * r - 2.0 * mu_;
                  s[0] += r;
                  if (method == 1) {
                    s[1] += (1.0 / (lambda + 2.0 / 3.0 * mu_));
                    s[2] += (1.0 / mu_);
                  } else {
                    s[1] += lambda;
                    s[2] += mu_;
                  }
                } else {
                  float cp[6];
                  lay_para2vti(kind, var, cp);
                  for (int n = 0; n < 5; n++) {
                    if (method == 1)
                      s[n] += (1.0 / cp[n]);
                    else
                      s[n] += cp[n];
                  }
                  s[5] += cp[5];
                }
              }
          if (bad) break;
          if (kind == LAY_ONE) {
            /* media/media_layer2model.cpp:1603-1782 (nsg is a size_t there) */
            out[0][q] = method == 1 ? (float)(nsg * 1.0 / s[0]) : (float)(s[0] / (nsg * 1.0));
          } else if (kind == LAY_ISO && method == 1) {
            s[2] = nsg * 1.0 / s[2];
            s[1] = nsg * 1.0 / s[1];
            s[0] = s[0] / (nsg * 1.0);
            out[0][q] = s[1] - 2.0 / 3.0 * s[2];
            out[1][q] = s[2];
            out[2][q] = s[0];
          } else if (kind == LAY_ISO) {
            out[0][q] = s[1] / (nsg * 1.0);
            out[1][q] = s[2] / (nsg * 1.0);
            out[2][q] = s[0] / (nsg * 1.0);
          } else {
            for (int n = 0; n < 5; n++)
              out[n][q] = method == 1 ? (float)(1.0 * nsg / s[n]) : s[n] / nsg;
            out[5][q] = s[5] / nsg;
          }
        }
    free(Hx); free(Hy); free(Hz); free(mat);
  }
  free(xv); free(yv); free(elev);
  return bad;
}

int oracle_layer_el_iso(int method, int NI, int NX, int NY, float MINX, float MINY, float DX,
                        float DY, const float *rec, int nx, int ny, int nz, const float *x3d,
                        const float *y3d, const float *z3d, float *lam, float *mu, float *rho)
{
  float *out[3] = {lam, mu, rho};
  return oracle_layer(LAY_ISO, method, NI, NX, NY, MINX, MINY, DX, DY, rec, nx, ny, nz, x3d,
                      y3d, z3d, out);
}

int oracle_layer_el_iso_loc(int NI, int NX, int NY, float MINX, float MINY, float DX,
                            float DY, const float *rec, int nx, int ny, int nz,
                            const float *x3d, const float *y3d, const float *z3d,
                            float *lam, float *mu, float *rho)
{
  return oracle_layer_el_iso(0, NI, NX, NY, MINX, MINY, DX, DY, rec, nx, ny, nz, x3d, y3d,
                             z3d, lam, mu, rho);
}

/* ------------------------------------------------------------------------ */
/* models given as binary volumes (media/media_bin2model.cpp:27-432)          */
/* ------------------------------------------------------------------------ */

/* The crop of the volumes to the grid's x/y range and the coordinate
 * vectors (media_bin2model_el_iso, media/media_bin2model.cpp:44-158).
 * Returns 1 where the reference exits (bad bin_order, no overlap), and 1
 * where the crop keeps fewer than two samples along an axis (the
 * reference's interpolation would read past its vectors). */
typedef struct {
  int dim[3];            /* file dimension holding x, y, z */
  int start[2];          /* first kept x, y sample */
  int n[3];              /* kept samples along x, y, z */
  size_t st[3];          /* file strides of x, y, z */
  float *xv, *yv, *zv;
} bin_crop_t;

static int bin_setup(const int *order, const int *size, const float *spacing,
                     const float *origin, const float *ext, size_t vol, const float *z3d,
                     bin_crop_t *b)
{
  int dimx = -1, dimy = -1, dimz = -1;
  for (int i = 0; i < 3; i++) {
    if (order[i] == 0) dimx = i;
    else if (order[i] == 1) dimy = i;
    else if (order[i] == 2) dimz = i;
    else return 1;
  }
  if (dimx == -1 || dimy == -1 || dimz == -1) return 1;
  const float xmin = ext[0], xmax = ext[1], ymin = ext[2], ymax = ext[3];
  const float bx0 = origin[dimx], by0 = origin[dimy], bz0 = origin[dimz];
  const float bdx = spacing[dimx], bdy = spacing[dimy], bdz = spacing[dimz];
  int ix_start = (xmin < bx0 ? 0 : (xmin - bx0) / bdx);
  if (ix_start >= size[dimx] || xmax < bx0) return 1;
  int ix_end = ceil((xmax - bx0) / bdx);
  if (ix_end >= size[dimx]) ix_end = size[dimx] - 1;
  int iy_start = (ymin < by0 ? 0 : (ymin - by0) / bdy);
  if (iy_start >= size[dimy] || ymax < by0) return 1;
  int iy_end = ceil((ymax - by0) / bdy);
  if (iy_end >= size[dimy]) iy_end = size[dimy] - 1;
  float zmin = FLT_MAX, zmax = -FLT_MAX;
  for (size_t i = 0; i < vol; i++) {
    zmin = fminf(zmin, z3d[i]);
    zmax = fmaxf(zmax, z3d[i]);
  }
  float bzn = bz0 + bdz * (size[dimz] - 1);
  if (zmin >= fmaxf(bzn, bz0) || zmax <= fminf(bz0, bzn)) return 1;
  b->dim[0] = dimx; b->dim[1] = dimy; b->dim[2] = dimz;
  b->start[0] = ix_start; b->start[1] = iy_start;
  b->n[0] = ix_end - ix_start + 1;
  b->n[1] = iy_end - iy_start + 1;
  b->n[2] = size[dimz];
  if (b->n[0] < 2 || b->n[1] < 2 || b->n[2] < 2) return 1;
  const size_t fst[3] = {1, (size_t)size[0], (size_t)size[0] * size[1]};
  for (int d = 0; d < 3; d++) b->st[d] = fst[b->dim[d]];
  b->xv = malloc(b->n[0] * sizeof(float));
  b->yv = malloc(b->n[1] * sizeof(float));
  b->zv = malloc(b->n[2] * sizeof(float));
  for (size_t i = 0; i < (size_t)b->n[0]; i++) b->xv[i] = bx0 + (ix_start + i) * bdx;
  for (size_t i = 0; i < (size_t)b->n[1]; i++) b->yv[i] = by0 + (iy_start + i) * bdy;
  for (size_t i = 0; i < (size_t)b->n[2]; i++) b->zv[i] = bz0 + i * bdz;
  return 0;
}

/* one volume (file order) at (xq, yq, zq): TrilinearInterpolation
 * (media/media_utility.cpp:299-391) on the cropped vectors */
static float bin_trilinear(const bin_crop_t *b, const float *v, float xq, float yq, float zq)
{
  const float *x = b->xv, *y = b->yv, *z = b->zv;
  const int nx = b->n[0], ny = b->n[1], nz = b->n[2];
  float dx = x[1] - x[0], dy = y[1] - y[0], dz = z[1] - z[0];
  int ix0 = floor((xq - x[0]) / dx), iy0 = floor((yq - y[0]) / dy);
  int ix2 = ceil((xq - x[0]) / dx), iy2 = ceil((yq - y[0]) / dy);
  ix0 = ix0 < 0 ? 0 : ix0;
  ix2 = ix2 < 0 ? 0 : ix2;
  ix0 = ix0 > nx - 1 ? nx - 1 : ix0;
  ix2 = ix2 > nx - 1 ? nx - 1 : ix2;
  iy0 = iy0 < 0 ? 0 : iy0;
  iy2 = iy2 < 0 ? 0 : iy2;
  iy0 = iy0 > ny - 1 ? ny - 1 : iy0;
  iy2 = iy2 > ny - 1 ? ny - 1 : iy2;
  int iz0 = floor((zq - z[0]) / dz), iz2 = ceil((zq - z[0]) / dz);
  iz0 = iz0 < 0 ? 0 : iz0;
  iz0 = iz0 > nz - 1 ? nz - 1 : iz0;
  iz2 = iz2 > nz - 1 ? nz - 1 : iz2;
  iz2 = iz2 < 0 ? 0 : iz2;
#define BINV(i, j, k) \
  v[(size_t)((i) + b->start[0]) * b->st[0] + (size_t)((j) + b->start[1]) * b->st[1] + \
    (size_t)(k) * b->st[2]]
  if (ix0 == ix2 && iy0 == iy2 && iz0 == iz2) return BINV(ix0, iy0, iz0);
  float v000 = BINV(ix0, iy0, iz0), v002 = BINV(ix0, iy0, iz2);
  float v200 = BINV(ix2, iy0, iz0), v202 = BINV(ix2, iy0, iz2);
  float v020 = BINV(ix0, iy2, iz0), v022 = BINV(ix0, iy2, iz2);
  float v220 = BINV(ix2, iy2, iz0), v222 = BINV(ix2, iy2, iz2);
#undef BINV
  float v100, v102, v122, v120;
  if (ix0 == ix2) {
    v100 = v000; v102 = v002; v122 = v022; v120 = v020;
  } else {
    float w = (xq - x[ix0]) / (x[ix2] - x[ix0]);
    v100 = v000 + w * (v200 - v000);
    v102 = v002 + w * (v202 - v002);
    v122 = v022 + w * (v222 - v022);
    v120 = v020 + w * (v220 - v020);
  }
  float v110, v112;
  if (iy0 == iy2) {
    v110 = v100; v112 = v102;
  } else {
    float w = (yq - y[iy0]) / (y[iy2] - y[iy0]);
    v110 = v100 + w * (v120 - v100);
    v112 = v102 + w * (v122 - v102);
  }
  if (iz0 == iz2) return v110;
  return v110 + (zq - z[iz0]) / (z[iz2] - z[iz0]) * (v112 - v110);
}

/* The box of the files the crop covers: first sample and count per file
 * dimension (the reference reads exactly these samples,
 * media/media_bin2model.cpp:91-175).  Returns 1 where the reference exits. */
int oracle_bin_crop(const int *order, const int *size, const float *spacing,
                    const float *origin, const float *ext, size_t vol, const float *z3d,
                    int *first, int *count)
{
  bin_crop_t b;
  if (bin_setup(order, size, spacing, origin, ext, vol, z3d, &b)) return 1;
  for (int d = 0; d < 3; d++) {
    first[b.dim[d]] = d < 2 ? b.start[d] : 0;
    count[b.dim[d]] = b.n[d];
  }
  free(b.xv); free(b.yv); free(b.zv);
  return 0;
}

/* vis 0: rho, lambda, mu from volumes rho, vp, vs
 * (parameterization_bin_el_iso_loc, media/media_bin2model.cpp:185-234);
 * vis 1: Qp, Qs from volumes Qp, Qs (:387-432).  ext: xmin xmax ymin ymax
 * of the grid.  Returns 1 where the reference exits. */
int oracle_bin(int vis, const int *order, const int *size, const float *spacing,
               const float *origin, const float *ext, const float *const *vols, int nx, int ny,
               int nz, const float *x3d, const float *y3d, const float *z3d, float **out)
{
  const size_t vol = (size_t)nx * ny * nz;
  bin_crop_t b;
  if (bin_setup(order, size, spacing, origin, ext, vol, z3d, &b)) return 1;
  for (size_t q = 0; q < vol; q++) {
    if (vis) {
      out[0][q] = bin_trilinear(&b, vols[0], x3d[q], y3d[q], z3d[q]);
      out[1][q] = bin_trilinear(&b, vols[1], x3d[q], y3d[q], z3d[q]);
    } else {
      float rho = bin_trilinear(&b, vols[0], x3d[q], y3d[q], z3d[q]);
      float vp = bin_trilinear(&b, vols[1], x3d[q], y3d[q], z3d[q]);
      float vs = bin_trilinear(&b, vols[2], x3d[q], y3d[q], z3d[q]);
      out[2][q] = vs * vs * rho;
      out[1][q] = vp * vp * rho - 2.0 * out[2][q];
      out[0][q] = rho;
    }
  }
  free(b.xv); free(b.yv); free(b.zv);
  return 0;
}

/* ------------------------------------------------------------------------ */
/* 3-D grid models (.md3grd), elastic isotropic (media/media_grid2model.cpp)  */
/* ------------------------------------------------------------------------ */

/* NI grid levels in NL layers of ngz[l] levels each; rec [NI][NY][NX][4] =
 * elevation, rho, vp, vs as the reference's reader leaves them (after its
 * crop to the grid's extent, media/media_read_file.cpp read_grid_file). */
typedef struct {
  int kind, np, nc;           /* LAY_ISO (rho vp vs) or LAY_VTI_*; nc = 1 + np */
  int NI, NX, NY, NL;
  int start[LAY_MAXI];        /* first level of each layer */
  const float *xv, *yv, *rec;
  size_t slice;
  float minx, maxx, miny, maxy;
  float *elev, *elev_nl;
} grd_model_t;

/* whether level mi starts a layer other than the first (the reference's
 * layer_indx set, media/media_grid2model.cpp:447-452) */
static int grd_is_start(const grd_model_t *m, int mi)
{
  for (int l = 1; l < m->NL; l++)
    if (m->start[l] == mi) return 1;
  return 0;
}

static float grd_val(const grd_model_t *m, int level, int c, float x, float y)
{
  return lay_bilinear(m->xv, m->NX, m->yv, m->NY, m->rec + level * m->slice * m->nc + c, m->nc,
                      x, y);
}

/* the parameters at a point (rho vp vs, or the six of a VTI type):
 * AssignGridMediaPara2Point with CalPointValue_grid
 * (media/media_grid2model.cpp:424-700), linear between the two levels
 * around the point.  *on: the point lies on a layer's top level
 * (isPointOnInter).  Returns 1 where the reference exits (outside the mesh;
 * isotropic: vp <= sqrt(2) vs). */
static int grd_point(const grd_model_t *m, float x, float y, float z, float *var, int *on)
{
  const int NI = m->NI;
  float *elev = m->elev;
  if (x < m->minx || x > m->maxx || y < m->miny || y > m->maxy) return 1;
  for (int n = 0; n < NI; n++) elev[n] = grd_val(m, n, 0, x, y);
  int mi = lay_last_ge(z, elev, NI);
  *on = mi >= 0 && grd_is_start(m, mi) && fabsf(z - elev[mi]) < FLT_EPSILON;
  /* the reference computes this before the branches, also where mi is -1
   * or NI-1 (it reads past its vector there; the value is not used) */
  float dis_r = 1.0 / 2.0;
  if (mi >= 0 && mi + 1 < NI && fabs(elev[mi + 1] - elev[mi]) > 1e-6)
    dis_r = (z - elev[mi]) / (elev[mi + 1] - elev[mi]);
  if (mi == -1 || mi == NI - 1) {
    if (mi == -1) mi = lay_last_ge(elev[0], elev, NI);
    for (int p = 0; p < m->np; p++) var[p] = grd_val(m, mi, 1 + p, x, y);
    return 0;
  }
  if (mi > 0 && fabsf(elev[mi] - z) < FLT_EPSILON && grd_is_start(m, mi)) {
    mi--;
    dis_r = 1.0 / 2.0;
  }
  for (int p = 0; p < m->np; p++) {
    float v0 = grd_val(m, mi, 1 + p, x, y), v1 = grd_val(m, mi + 1, 1 + p, x, y);
    var[p] = v0 + (v1 - v0) * dis_r;
  }
  if (m->kind == LAY_ISO && var[1] <= sqrt(2) * var[2]) return 1;
  return 0;
}

/* the layer of a half-grid point (LayerNumberAtPoint,
 * media/media_grid2model.cpp:1269-1310) */
static int grd_layer(const grd_model_t *m, float x, float y, float z)
{
  for (int l = 0; l < m->NL; l++) m->elev_nl[l] = grd_val(m, m->start[l], 0, x, y);
  int mi = lay_last_ge(z, m->elev_nl, m->NL);
  if (mi == -1) mi = lay_last_ge(m->elev_nl[0], m->elev_nl, m->NL);
  return mi;
}

/* method 0 loc, 1 har, 2 ari (parametrization_grid_el_iso_loc / _har /
 * _ari, media/media_grid2model.cpp:1067-1126, 1819-2079): out = rho, lambda,
 * mu (the reference's argument order).  har and ari recompute the interior
 * points whose cell touches two layers from the 9^3 samples not lying on a
 * layer's top level.  Returns 1 where the reference exits. */
static int oracle_grid_vti_loc(int kind, int NI, int NL, const int *ngz, int NX, int NY,
                               float MINX, float MINY, float DX, float DY, const float *rec,
                               int nx, int ny, int nz, const float *x3d, const float *y3d,
                               const float *z3d, float **out);

int oracle_grid_el_iso(int method, int NI, int NL, const int *ngz, int NX, int NY, float MINX,
                       float MINY, float DX, float DY, const float *rec, int nx, int ny, int nz,
                       const float *x3d, const float *y3d, const float *z3d, float **out)
{
  if (NI < 1 || NI > LAY_MAXI || NL < 1 || NL > NI) return 1;
  grd_model_t m;
  m.kind = LAY_ISO; m.np = 3; m.nc = 4;
  m.NI = NI; m.NX = NX; m.NY = NY; m.NL = NL;
  int acc = 0;
  for (int l = 0; l < NL; l++) {
    m.start[l] = acc;
    acc += ngz[l];
  }
  if (acc != NI) return 1;
  float *xv = malloc(NX * sizeof(float)), *yv = malloc(NY * sizeof(float));
  for (int i = 0; i < NX; i++) xv[i] = MINX + DX * i;
  for (int j = 0; j < NY; j++) yv[j] = MINY + DY * j;
  m.xv = xv; m.yv = yv; m.rec = rec; m.slice = (size_t)NX * NY;
  m.minx = MINX; m.maxx = MINX + (NX - 1) * DX;
  m.miny = MINY; m.maxy = MINY + (NY - 1) * DY;
  m.elev = malloc(NI * sizeof(float));
  m.elev_nl = malloc(NL * sizeof(float));
  int bad = 0;
  const size_t line = nx, sl = (size_t)nx * ny, vol = sl * nz;
  for (size_t q = 0; q < vol && !bad; q++) {
    float var[3];
    int on;
    if (grd_point(&m, x3d[q], y3d[q], z3d[q], var, &on)) { bad = 1; break; }
    float vp = var[1], vs = var[2], r = var[0];
    out[2][q] = vs * vs * r;
    out[1][q] = vp * vp * r - 2.0 * out[2][q];
    out[0][q] = r;
  }
  if (method != 0 && !bad) {
    float *Hx = malloc(vol * sizeof(float)), *Hy = malloc(vol * sizeof(float));
    float *Hz = malloc(vol * sizeof(float));
    int *mat = malloc(vol * sizeof(int));
    lay_half_grid(nx, ny, nz, x3d, Hx);
    lay_half_grid(nx, ny, nz, y3d, Hy);
    lay_half_grid(nx, ny, nz, z3d, Hz);
    for (size_t q = 0; q < vol; q++) mat[q] = grd_layer(&m, Hx[q], Hy[q], Hz[q]);
    for (int j = 1; j < ny - 1 && !bad; j++)
      for (int k = 1; k < nz - 1 && !bad; k++)
        for (int i = 1; i < nx - 1 && !bad; i++) {
          size_t q = i + j * line + k * sl;
          const size_t c[8] = {q - 1 - line - sl, q - 1 - sl, q - sl, q - line - sl,
                               q - 1 - line, q - 1, q, q - line};
          int v[8];
          for (int n = 0; n < 8; n++) v[n] = mat[c[n]];
          if (lay_num_values(v) <= 1) continue;
          float vert[8][3];
          for (int n = 0; n < 8; n++) {
            vert[n][0] = Hx[c[n]];
            vert[n][1] = Hy[c[n]];
            vert[n][2] = Hz[c[n]];
          }
          float s_rho = 0.0, s_a = 0.0, s_b = 0.0;   /* rho; kappa or lambda; mu */
          int num_dis = (LAY_NG + 1) * (LAY_NG + 1) * (LAY_NG + 1);
          for (int kk = 0; kk <= LAY_NG && !bad; kk++)
            for (int jj = 0; jj <= LAY_NG && !bad; jj++)
              for (int ii = 0; ii <= LAY_NG; ii++) {
                float p[3], var[3];
                int on;
                lay_subpoint((const float (*)[3])vert, ii, jj, kk, p);
                if (grd_point(&m, p[0], p[1], p[2], var, &on)) { bad = 1; break; }
                if (on) {
                  num_dis--;
                  continue;
                }
                float rho = var[0], vp = var[1], vs = var[2];
                float mu_ = vs * vs * rho;
                float lambda = vp * vp * rho - 2.0 * mu_;
                s_rho += rho;
                if (method == 1) {
                  s_a += (1.0 / (lambda + 2.0 / 3.0 * mu_));
                  s_b += (1.0 / mu_);
                } else {
                  s_a += lambda;
                  s_b += mu_;
                }
              }
          if (bad) break;
          if (method == 1) {
            s_b = num_dis * 1.0 / s_b;
            s_a = num_dis * 1.0 / s_a;
            s_rho = s_rho / num_dis;
            out[1][q] = s_a - 2.0 / 3.0 * s_b;
            out[2][q] = s_b;
            out[0][q] = s_rho;
          } else {
            out[1][q] = s_a / (num_dis * 1.0);
            out[2][q] = s_b / (num_dis * 1.0);
            out[0][q] = s_rho / (num_dis * 1.0);
          }
        }
    free(Hx); free(Hy); free(Hz); free(mat);
  }
  free(xv); free(yv); free(m.elev); free(m.elev_nl);
  return bad;
}

/* An elastic VTI grid model (kind LAY_VTI_*) with "loc": the six parameters
 * at each point, then para2vti (parametrization_grid_el_vti_loc,
 * media/media_grid2model.cpp:1127-1184); rec [NI][NY][NX][7]; out = c11 c33
 * c55 c66 c13 rho.  Returns 1 where the reference exits. */
static int oracle_grid_vti_loc(int kind, int NI, int NL, const int *ngz, int NX, int NY,
                               float MINX, float MINY, float DX, float DY, const float *rec,
                               int nx, int ny, int nz, const float *x3d, const float *y3d,
                               const float *z3d, float **out)
{
  if (NI < 1 || NI > LAY_MAXI || NL < 1 || NL > NI) return 1;
  grd_model_t m;
  m.kind = kind; m.np = 6; m.nc = 7;
  m.NI = NI; m.NX = NX; m.NY = NY; m.NL = NL;
  int acc = 0;
  for (int l = 0; l < NL; l++) {
    m.start[l] = acc;
    acc += ngz[l];
  }
  if (acc != NI) return 1;
  float *xv = malloc(NX * sizeof(float)), *yv = malloc(NY * sizeof(float));
  for (int i = 0; i < NX; i++) xv[i] = MINX + DX * i;
  for (int j = 0; j < NY; j++) yv[j] = MINY + DY * j;
  m.xv = xv; m.yv = yv; m.rec = rec; m.slice = (size_t)NX * NY;
  m.minx = MINX; m.maxx = MINX + (NX - 1) * DX;
  m.miny = MINY; m.maxy = MINY + (NY - 1) * DY;
  m.elev = malloc(NI * sizeof(float));
  m.elev_nl = malloc(NL * sizeof(float));
  int bad = 0;
  const size_t vol = (size_t)nx * ny * nz;
  for (size_t q = 0; q < vol && !bad; q++) {
    float var[6], c[6];
    int on;
    if (grd_point(&m, x3d[q], y3d[q], z3d[q], var, &on)) { bad = 1; break; }
    lay_para2vti(kind, var, c);
    for (int n = 0; n < 6; n++) out[n][q] = c[n];
  }
  free(xv); free(yv); free(m.elev); free(m.elev_nl);
  return bad;
}

int oracle_grid_el_vti_loc(int kind, int NI, int NL, const int *ngz, int NX, int NY, float MINX,
                           float MINY, float DX, float DY, const float *rec, int nx, int ny,
                           int nz, const float *x3d, const float *y3d, const float *z3d,
                           float **out)
{
  if (kind != LAY_VTI_PREM && kind != LAY_VTI_THOMSEN && kind != LAY_VTI_CIJ) return 1;
  return oracle_grid_vti_loc(kind, NI, NL, ngz, NX, NY, MINX, MINY, DX, DY, rec, nx, ny, nz,
                             x3d, y3d, z3d, out);
}
