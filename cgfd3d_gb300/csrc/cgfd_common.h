/*
 * Shared host/device definitions of the GB300 time-stepping library.
 *
 * Device layout in HBM (per solver):
 *   wavefield  4 levels x ncmp components x padded volume, the
 *              reference's layout (forward/wav_t.c:40-136) with the level
 *              roles  pre | tmpA | tmpB | end.  The reference keeps a
 *              separate rhs level; here the RHS lives only in registers and
 *              the former rhs level is the second tmp buffer, so that the
 *              stage that reads tmp with a +-3 stencil never writes the
 *              buffer it reads.
 *   metrics    10 x volume: jac, xi_x..zeta_z (forward/gd_t.c:142-180)
 *   media      slw (=1/rho) and the medium's constants, one volume each
 *              (cgfd_media.cuh)
 *   PML aux    per enabled face: 4 levels x 9 x face-box volume
 *   surface    3 x (nx*ny*9) conversion matrices (k = nk2)
 */
#ifndef CGFD_COMMON_H
#define CGFD_COMMON_H

#include <stddef.h>
#include <stdint.h>

#define CGFD_NCMP 9
#define CGFD_NFACE 6

/* component order of the reference (forward/wav_t.c:93-136) */
enum { C_VX = 0, C_VY, C_VZ, C_TXX, C_TYY, C_TZZ, C_TYZ, C_TXZ, C_TXY };

/* Device volumes are pitched: row pitch px >= nx + xoff (multiple of 32
 * floats) and x offset xoff chosen so that the first physical column
 * (i = 3) starts a 128-byte line; element (i,j,k) sits at
 * (i + xoff) + j*px + k*px*ny.  This keeps every warp-wide row access and
 * every TMA box aligned. */
struct DevGrid {
  int ni, nj, nk, nx, ny, nz;
  int ni1, ni2, nj1, nj2, nk1, nk2;
  int px, xoff;
  long long sl;   /* px*ny */
  long long vol;  /* px*ny*nz */
};

struct DevFace {
  int on;
  int dim;                       /* 0 x, 1 y, 2 z */
  int i1, i2, j1, j2, k1, k2;    /* box, inclusive */
  int bx, by;                    /* box extents in i and j */
  long long avol;                /* box volume */
  const float *A, *B, *D;
};

/* one surface force source (forward/src_t.c:202-311) */
struct SurfForce {
  int is;          /* source index (time window, force table) */
  int n;           /* surface-force index (rate table) */
  int si, sj, sk;  /* grid indices */
  int half;        /* Gaussian half width, 0 for a point force */
  int w0;          /* offset of its (2 half + 1)^2 surface weights */
  int pad;
};

/* one source contribution at one grid point (precomputed on the host) */
struct SrcEntry {
  int k;          /* plane */
  int is;         /* source index */
  float vf;       /* coef * slw / jac  (force weight) */
  float rjac;     /* coef / jac        (moment weight) */
  int force_on;   /* force applied at this point (strict surface rule) */
  float coef;     /* spatial weight (1 for a point source) */
  long long q;    /* device index of the point (weights filled on the device) */
};

/* Maxwell bodies the fused visco-elastic path holds in shared memory */
#define CGFD_VIS_NMW_MAX 3

struct StageArgs {
  DevGrid g;
  /* metrics and media */
  const float *jac, *xix, *xiy, *xiz, *etx, *ety, *etz, *ztx, *zty, *ztz;
  const float *slw, *lam, *mu;
  const float *med;   /* media block (cgfd_media.cuh), component stride g.vol */
  int ncmp;           /* wavefield components per level (9 + 6 nmw) */
  int nmw;            /* Maxwell bodies (visco-elastic), else 0 */
  float wl[CGFD_VIS_NMW_MAX];   /* relaxation angular frequencies */
  /* wavefield levels for this stage */
  const float *cur;   /* stencil input */
  const float *pre;   /* level "pre" */
  float *tmp_out;     /* next tmp (stages 0-2) */
  float *end;         /* accumulator */
  float ca, cb;       /* rk_a*dt, rk_b*dt */
  /* PML */
  DevFace face[CGFD_NFACE];
  const float *acur[CGFD_NFACE];
  const float *apre[CGFD_NFACE];
  float *atmp_out[CGFD_NFACE];
  float *aend[CGFD_NFACE];
  /* free surface */
  int free_top;
  const float *mVx, *mVy, *mF, *mD;
  /* surface force layers of the stage (TxSrc,TySrc,TzSrc / VxSrc,VySrc,
   * VzSrc, 3 x nx*ny each, forward/src_t.c:153-314), or null */
  const float *TS, *VS;
  /* sources */
  int src_n, src_max_nt, src_max_stage, src_force, src_moment;
  const int *src_col;          /* (ni*nj + 1) offsets into src_ent */
  const SrcEntry *src_ent;
  const int *src_it_begin, *src_it_end;
  const float *Fx, *Fy, *Fz, *Mxx, *Myy, *Mzz, *Mxz, *Myz, *Mxy;
  const int *d_it;             /* current step on the device */
  int istage;
  int *err;                    /* device error word (bounded waits) */
  int pml_fused;               /* CFS-PML inside the stage kernel (else face kernels) */
  int l2_ahead;                /* planes of L2 prefetch beyond the smem rings */
  int cur_level;               /* level index of `cur` (TMA coordinate) */
  int pre_level, end_level;    /* level indices of `pre` and `end` */
  int kchunk;                  /* planes per CTA along k */
  /* Graves Q attenuation factors expf(-PI f dt / Qs) per point (pitched
   * volume), applied to `end` by the last stage; null when off */
  const float *qatt;
  /* distributed sources: per-column entries (is = dd point), tables
   * [step][stage][point][3 | 6] */
  int dd_n, dd_max_nt;
  const int *dd_col;
  const SrcEntry *dd_ent;
  const float *dd_vi, *dd_mij;
  /* polls of an mbarrier wait before it gives up (records error 1 and the
   * CTA stops); and, for tests of that path only, a wavefield plane (ring
   * position of the k march, -1: none) whose copy the first CTA of the grid
   * does not issue, so that a wait on it runs out */
  int wait_limit;
  int test_skip_plane;
};

/* StageArgs is copied word by word into shared memory by the batched stage
 * kernel */
static_assert(sizeof(StageArgs) % 4 == 0, "StageArgs size");

#endif
