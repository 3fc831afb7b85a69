/*
 * Golden-vector capture around the reference solver entry point.
 *
 * TEST INFRASTRUCTURE ONLY.  Linked into the reference build with
 * `-Wl,--wrap=drv_rk_curv_col_allstep`, so the reference sources stay
 * unmodified: `main` (forward/main_curv_col_el_3d.c:849) calls this wrapper,
 * which
 *   1. optionally (CGFD_DUMP_SEED set) perturbs the media, and seeds the
 *      wavefield and the PML auxiliary variables with deterministic noise so
 *      that every stencil tap and every boundary branch is exercised from the
 *      first step;
 *   2. writes every input array the time loop reads;
 *   3. calls the real drv_rk_curv_col_allstep (forward/drv_rk_curv_col.c:28);
 *   4. writes every output the time loop produces: all wavefield levels, all
 *      PML auxiliary levels, receiver and line seismograms and the
 *      free-surface conversion matrices computed inside the entry point.
 *
 * File format (CGFD_DUMP_FILE): a sequence of records
 *   char name[48]; char kind ('f' float32, 'i' int32, 'd' float64);
 *   char pad[7]; int64 count; payload (count * item size bytes).
 * tests/golden/make_golden.py turns it into compressed .npz fixtures.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <stdint.h>

#include "fd_t.h"
#include "gd_t.h"
#include "md_t.h"
#include "src_t.h"
#include "bdry_t.h"
#include "wav_t.h"
#include "mympi_t.h"
#include "io_funcs.h"
#include "drv_rk_curv_col.h"

void __real_drv_rk_curv_col_allstep(
  fd_t *fd, gd_t *gd, gdcurv_metric_t *metric, md_t *md, src_t *src,
  bdry_t *bdry, wav_t *wav, mympi_t *mympi, iorecv_t *iorecv,
  ioline_t *ioline, ioslice_t *ioslice, iosnap_t *iosnap, float dt,
  int nt_total, float t0, char *output_fname_part, char *output_dir,
  int qc_check_nan_num_of_step, const int output_all, const int verbose);

static FILE *g_fp = NULL;

static void put(const char *name, char kind, const void *data, int64_t count)
{
  char hdr[56];
  memset(hdr, 0, sizeof(hdr));
  strncpy(hdr, name, 47);
  hdr[48] = kind;
  fwrite(hdr, 1, 56, g_fp);
  fwrite(&count, sizeof(int64_t), 1, g_fp);
  size_t isz = (kind == 'd') ? 8 : 4;
  if (count > 0 && data != NULL) fwrite(data, isz, (size_t)count, g_fp);
}
static void put_i(const char *name, int v) { put(name, 'i', &v, 1); }
static void put_f(const char *name, float v) { put(name, 'f', &v, 1); }

/* xorshift32 -> uniform in [-1, 1) */
static uint32_t g_rng = 1u;
static float urand(void)
{
  uint32_t x = g_rng;
  x ^= x << 13; x ^= x >> 17; x ^= x << 5;
  g_rng = x;
  return (float)((double)(x >> 8) / 8388608.0 - 1.0);
}

static int is_phys(gd_t *gd, int i, int j, int k)
{
  return i >= gd->ni1 && i <= gd->ni2 && j >= gd->nj1 && j <= gd->nj2 &&
         k >= gd->nk1 && k <= gd->nk2;
}

/* the 21 constants of an anisotropic medium, c11 c12 .. c16 c22 .. c66 */
static float **aniso_fields(md_t *md)
{
  static float *c[21];
  float *v[21] = {md->c11, md->c12, md->c13, md->c14, md->c15, md->c16, md->c22,
                  md->c23, md->c24, md->c25, md->c26, md->c33, md->c34, md->c35,
                  md->c36, md->c44, md->c45, md->c46, md->c55, md->c56, md->c66};
  memcpy(c, v, sizeof v);
  return c;
}

/* The reference's anisotropic test medium (forward/md_t.c:539-590) leaves
 * c12, c22, c44 and the off-diagonal terms zero, which is not a stable
 * medium.  With CGFD_DUMP_SEED set, an anisotropic model gets instead a
 * transversely isotropic stiffness (c11 = c22 = 25.2 GPa, c33 = 18,
 * c13 = c23 = 10.962, c44 = c55 = 5.12, c66 = 7.168, c12 = c11 - 2 c66)
 * plus every one of the 21 constants offset by up to +-0.4 GPa (seeded),
 * before the pointwise +-10 % of perturb(). */
static void aniso_base(gd_t *gd, md_t *md)
{
  const float base[21] = {25.2e9f, 10.864e9f, 10.962e9f, 0, 0, 0, 25.2e9f, 10.962e9f,
                          0, 0, 0, 18.0e9f, 0, 0, 0, 5.12e9f, 0, 0, 5.12e9f, 0, 7.168e9f};
  float off[21];
  for (int n = 0; n < 21; n++) off[n] = 0.4e9f * urand();
  float **c = aniso_fields(md);
  for (size_t p = 0; p < gd->siz_icmp; p++)
    for (int n = 0; n < 21; n++) c[n][p] = base[n] + off[n];
}

static void perturb(gd_t *gd, md_t *md, bdry_t *bdry, wav_t *wav, float amp_v)
{
  size_t n = gd->siz_icmp;
  /* media: +-10 % around the given values, physical and ghost points */
  float *fields[32];
  int nf = 0;
  fields[nf++] = md->rho; /* already slowness */
  if (md->medium_type == CONST_MEDIUM_ELASTIC_ISO ||
      md->medium_type == CONST_MEDIUM_VISCOELASTIC_ISO) {
    fields[nf++] = md->lambda;
    fields[nf++] = md->mu;
  } else if (md->medium_type == CONST_MEDIUM_ELASTIC_VTI) {
    fields[nf++] = md->c11; fields[nf++] = md->c13; fields[nf++] = md->c33;
    fields[nf++] = md->c55; fields[nf++] = md->c66;
  } else if (md->medium_type == CONST_MEDIUM_ELASTIC_ANISO) {
    float **c = aniso_fields(md);
    for (int n = 0; n < 21; n++) fields[nf++] = c[n];
  }
  if (md->visco_type == CONST_VISCO_GRAVES_QS) fields[nf++] = md->Qs;
  for (int f = 0; f < nf; f++)
    for (size_t p = 0; p < n; p++) fields[f][p] *= 1.0f + 0.1f * urand();

  /* wavefield level 0: noise in the physical region only (ghosts stay 0) */
  float *w = wav->v5d;
  float rho_ref = 2700.0f, vp_ref = 6000.0f;
  for (int c = 0; c < wav->ncmp; c++) {
    float amp = (c < 3) ? amp_v : amp_v * rho_ref * vp_ref;
    if (c >= 9) amp *= 1e-3f; /* memory variables */
    for (int k = 0; k < gd->nz; k++)
      for (int j = 0; j < gd->ny; j++)
        for (int i = 0; i < gd->nx; i++) {
          size_t p = i + j * gd->siz_iy + k * gd->siz_iz;
          w[c * n + p] = is_phys(gd, i, j, k) ? amp * urand() : 0.0f;
        }
  }
  /* PML auxiliary level 0 */
  for (int d = 0; d < 3; d++)
    for (int s = 0; s < 2; s++) {
      if (bdry->is_sides_pml[d][s] != 1) continue;
      bdrypml_auxvar_t *a = &bdry->auxvar[d][s];
      for (int c = 0; c < a->ncmp; c++) {
        float amp = (c < 3) ? amp_v : amp_v * rho_ref * vp_ref;
        amp *= 0.1f;
        for (size_t p = 0; p < a->siz_icmp; p++)
          a->var[c * a->siz_icmp + p] = amp * urand();
      }
    }
}

static void dump_fd(fd_t *fd)
{
  put_i("fd.num_rk_stages", fd->num_rk_stages);
  put("fd.rk_a", 'f', fd->rk_a, fd->num_rk_stages - 1);
  put("fd.rk_b", 'f', fd->rk_b, fd->num_rk_stages);
  put("fd.rk_rhs_time", 'f', fd->rk_rhs_time, fd->num_rk_stages);
  put_i("fd.num_of_pairs", fd->num_of_pairs);
  put_i("fd.num_of_fdz_op", fd->num_of_fdz_op);
  /* operator tables: [pair][stage] -> x, y inner op; z ops per layer */
  for (int p = 0; p < fd->num_of_pairs; p++)
    for (int s = 0; s < fd->num_rk_stages; s++) {
      char nm[48];
      fd_op_t *ox = fd->pair_fdx_op[p][s] + fd->num_of_fdx_op - 1;
      fd_op_t *oy = fd->pair_fdy_op[p][s] + fd->num_of_fdy_op - 1;
      snprintf(nm, 48, "fd.x.%d.%d.indx", p, s); put(nm, 'i', ox->indx, ox->total_len);
      snprintf(nm, 48, "fd.x.%d.%d.coef", p, s); put(nm, 'f', ox->coef, ox->total_len);
      snprintf(nm, 48, "fd.y.%d.%d.indx", p, s); put(nm, 'i', oy->indx, oy->total_len);
      snprintf(nm, 48, "fd.y.%d.%d.coef", p, s); put(nm, 'f', oy->coef, oy->total_len);
      for (int l = 0; l < fd->num_of_fdz_op; l++) {
        fd_op_t *oz = fd->pair_fdz_op[p][s] + l;
        snprintf(nm, 48, "fd.z.%d.%d.%d.indx", p, s, l); put(nm, 'i', oz->indx, oz->total_len);
        snprintf(nm, 48, "fd.z.%d.%d.%d.coef", p, s, l); put(nm, 'f', oz->coef, oz->total_len);
      }
    }
}

static void dump_inputs(fd_t *fd, gd_t *gd, gdcurv_metric_t *metric, md_t *md,
                        src_t *src, bdry_t *bdry, wav_t *wav,
                        iorecv_t *iorecv, ioline_t *ioline,
                        float dt, int nt_total, float t0)
{
  dump_fd(fd);
  put_f("dt", dt);
  put_i("nt_total", nt_total);
  put_f("t0", t0);
  int g[12] = {gd->ni, gd->nj, gd->nk, gd->nx, gd->ny, gd->nz,
               gd->ni1, gd->ni2, gd->nj1, gd->nj2, gd->nk1, gd->nk2};
  put("gd.dims", 'i', g, 12);
  size_t n = gd->siz_icmp;
  put("metric.jac", 'f', metric->jac, n);
  put("metric.xi_x", 'f', metric->xi_x, n);
  put("metric.xi_y", 'f', metric->xi_y, n);
  put("metric.xi_z", 'f', metric->xi_z, n);
  put("metric.eta_x", 'f', metric->eta_x, n);
  put("metric.eta_y", 'f', metric->eta_y, n);
  put("metric.eta_z", 'f', metric->eta_z, n);
  put("metric.zeta_x", 'f', metric->zeta_x, n);
  put("metric.zeta_y", 'f', metric->zeta_y, n);
  put("metric.zeta_z", 'f', metric->zeta_z, n);
  /* grid coordinates: read by the visco-elastic free surface, and the
   * input of the metric calculation (checked on its own) */
  if (gd->x3d) {
    put("gd.x3d", 'f', gd->x3d, n);
    put("gd.y3d", 'f', gd->y3d, n);
    put("gd.z3d", 'f', gd->z3d, n);
  }

  put_i("md.medium_type", md->medium_type);
  put_i("md.visco_type", md->visco_type);
  put("md.slw", 'f', md->rho, n);
  if (md->medium_type == CONST_MEDIUM_ELASTIC_ISO ||
      md->medium_type == CONST_MEDIUM_VISCOELASTIC_ISO) {
    put("md.lambda", 'f', md->lambda, n);
    put("md.mu", 'f', md->mu, n);
  }
  if (md->medium_type == CONST_MEDIUM_ELASTIC_VTI) {
    put("md.c11", 'f', md->c11, n);
    put("md.c13", 'f', md->c13, n);
    put("md.c33", 'f', md->c33, n);
    put("md.c55", 'f', md->c55, n);
    put("md.c66", 'f', md->c66, n);
  }
  if (md->medium_type == CONST_MEDIUM_VISCOELASTIC_ISO) {
    put_i("md.nmaxwell", md->nmaxwell);
    put("md.wl", 'f', md->wl, md->nmaxwell);
    for (int m = 0; m < md->nmaxwell; m++) {
      char nm[48];
      snprintf(nm, 48, "md.Ylam.%d", m); put(nm, 'f', md->Ylam[m], n);
      snprintf(nm, 48, "md.Ymu.%d", m); put(nm, 'f', md->Ymu[m], n);
    }
  }

  if (md->medium_type == CONST_MEDIUM_ELASTIC_ANISO) {
    static const char *nm[21] = {"c11", "c12", "c13", "c14", "c15", "c16", "c22",
                                 "c23", "c24", "c25", "c26", "c33", "c34", "c35",
                                 "c36", "c44", "c45", "c46", "c55", "c56", "c66"};
    float **c = aniso_fields(md);
    for (int m = 0; m < 21; m++) {
      char key[48];
      snprintf(key, 48, "md.%s", nm[m]);
      put(key, 'f', c[m], n);
    }
  }
  if (md->visco_type == CONST_VISCO_GRAVES_QS) {
    put("md.Qs", 'f', md->Qs, n);
    put_f("md.visco_Qs_freq", md->visco_Qs_freq);
  }

  /* boundaries */
  put("bdry.is_sides_pml", 'i', bdry->is_sides_pml, 6);
  put("bdry.is_sides_free", 'i', bdry->is_sides_free, 6);
  put_i("bdry.is_enable_pml", bdry->is_enable_pml);
  put_i("bdry.is_enable_free", bdry->is_enable_free);
  put_i("bdry.is_enable_ablexp", bdry->is_enable_ablexp);
  if (bdry->is_enable_ablexp == 1) {
    int blk[6][7];
    for (int b = 0; b < 6; b++) {
      bdry_block_t *D = &bdry->bdry_blk[b];
      int v[7] = {D->enable, D->ni1, D->ni2, D->nj1, D->nj2, D->nk1, D->nk2};
      memcpy(blk[b], v, sizeof v);
    }
    put("bdry.ablexp_blk", 'i', blk, 42);
    put("bdry.ablexp_Ex", 'f', bdry->ablexp_Ex, gd->nx);
    put("bdry.ablexp_Ey", 'f', bdry->ablexp_Ey, gd->ny);
    put("bdry.ablexp_Ez", 'f', bdry->ablexp_Ez, gd->nz);
  }
  for (int d = 0; d < 3; d++)
    for (int s = 0; s < 2; s++) {
      if (bdry->is_sides_pml[d][s] != 1) continue;
      char nm[48];
      int box[6] = {bdry->ni1[d][s], bdry->ni2[d][s], bdry->nj1[d][s],
                    bdry->nj2[d][s], bdry->nk1[d][s], bdry->nk2[d][s]};
      int np = bdry->num_of_layers[d][s] + 1;
      snprintf(nm, 48, "pml.%d.%d.box", d, s); put(nm, 'i', box, 6);
      snprintf(nm, 48, "pml.%d.%d.A", d, s); put(nm, 'f', bdry->A[d][s], np);
      snprintf(nm, 48, "pml.%d.%d.B", d, s); put(nm, 'f', bdry->B[d][s], np);
      snprintf(nm, 48, "pml.%d.%d.D", d, s); put(nm, 'f', bdry->D[d][s], np);
      bdrypml_auxvar_t *a = &bdry->auxvar[d][s];
      snprintf(nm, 48, "pml.%d.%d.aux0", d, s);
      put(nm, 'f', a->var, a->siz_ilevel);
    }

  /* source */
  put_i("src.total_number", src->total_number);
  put_i("src.max_nt", src->max_nt);
  put_i("src.max_stage", src->max_stage);
  put_i("src.force_actived", src->force_actived);
  put_i("src.moment_actived", src->moment_actived);
  put_i("src.itype_spatial_ext", src->itype_spatial_ext);
  put_i("src.ext_half_npoint", src->ext_half_npoint);
  put_f("src.ext_func_coef", src->ext_func_coef);
  put_i("src.is_surface_force_strict", src->is_surface_force_strict);
  put_i("src.total_number_surface_force", src->total_number_surface_force);
  put_i("src.dd_is_valid", src->dd_is_valid);
  if (src->dd_is_valid == 1) {
    /* distributed sources: indices and the whole per-step tables, read from
     * the files the set-up wrote (position restored for the time loop) */
    int nd = src->dd_total_number;
    put_i("src.dd_total_number", nd);
    put_i("src.dd_max_nt", src->dd_max_nt);
    put_i("src.dd_is_add_at_point", src->dd_is_add_at_point);
    put("src.dd_si", 'i', src->dd_si, nd);
    put("src.dd_sj", 'i', src->dd_sj, nd);
    put("src.dd_sk", 'i', src->dd_sk, nd);
    FILE *fps[2] = {src->dd_vi_actived == 1 ? src->fp_vi : NULL,
                    src->dd_mij_actived == 1 ? src->fp_mij : NULL};
    const char *names[2] = {"src.dd_vi", "src.dd_mij"};
    const int ncmp[2] = {3, 6};
    for (int t = 0; t < 2; t++) {
      if (!fps[t]) continue;
      size_t n = (size_t)src->dd_max_nt * src->max_stage * nd * ncmp[t];
      float *buf = malloc(n * sizeof(float));
      long pos = ftell(fps[t]);
      fseek(fps[t], 0, SEEK_SET);
      if (fread(buf, sizeof(float), n, fps[t]) != n) exit(3);
      fseek(fps[t], pos, SEEK_SET);
      put(names[t], 'f', buf, n);
      free(buf);
    }
  }
  int ns = src->total_number;
  if (ns > 0) {
    size_t nstf = (size_t)ns * src->max_nt * src->max_stage;
    put("src.si", 'i', src->si, ns);
    put("src.sj", 'i', src->sj, ns);
    put("src.sk", 'i', src->sk, ns);
    put("src.si_inc", 'f', src->si_inc, ns);
    put("src.sj_inc", 'f', src->sj_inc, ns);
    put("src.sk_inc", 'f', src->sk_inc, ns);
    put("src.it_begin", 'i', src->it_begin, ns);
    put("src.it_end", 'i', src->it_end, ns);
    if (src->force_actived == 1) {
      put("src.Fx", 'f', src->Fx, nstf);
      put("src.Fy", 'f', src->Fy, nstf);
      put("src.Fz", 'f', src->Fz, nstf);
    }
    if (src->total_number_surface_force > 0) {
      int nsf = src->total_number_surface_force;
      size_t nr = (size_t)nsf * src->max_nt * src->max_stage;
      put("src.force_rate_indx", 'i', src->force_rate_indx, nsf);
      put("src.Fx_rate", 'f', src->Fx_rate, nr);
      put("src.Fy_rate", 'f', src->Fy_rate, nr);
      put("src.Fz_rate", 'f', src->Fz_rate, nr);
    }
    if (src->moment_actived == 1) {
      put("src.Mxx", 'f', src->Mxx, nstf);
      put("src.Myy", 'f', src->Myy, nstf);
      put("src.Mzz", 'f', src->Mzz, nstf);
      put("src.Mxz", 'f', src->Mxz, nstf);
      put("src.Myz", 'f', src->Myz, nstf);
      put("src.Mxy", 'f', src->Mxy, nstf);
    }
  }

  /* wavefield layout and initial state */
  put_i("wav.ncmp", wav->ncmp);
  put_i("wav.nlevel", wav->nlevel);
  put("wav.level0", 'f', wav->v5d, wav->siz_ilevel);

  /* receivers */
  put_i("recv.total_number", iorecv->total_number);
  put_i("recv.max_nt", iorecv->max_nt);
  put_i("recv.ncmp", iorecv->ncmp);
  for (int r = 0; r < iorecv->total_number; r++) {
    iorecv_one_t *o = iorecv->recvone + r;
    char nm[48];
    float d3[3] = {o->di, o->dj, o->dk};
    int i3[3] = {o->i, o->j, o->k};
    snprintf(nm, 48, "recv.%d.dijk", r); put(nm, 'f', d3, 3);
    snprintf(nm, 48, "recv.%d.ijk", r); put(nm, 'i', i3, 3);
    snprintf(nm, 48, "recv.%d.indx1d", r); put(nm, 'i', o->indx1d, 8);
  }
  put_i("line.num_of_lines", ioline->num_of_lines);
  put_i("line.max_nt", ioline->max_nt);
  put_i("line.ncmp", ioline->ncmp);
  for (int l = 0; l < ioline->num_of_lines; l++) {
    char nm[48];
    snprintf(nm, 48, "line.%d.iptr", l);
    put(nm, 'i', ioline->recv_iptr[l], ioline->line_nr[l]);
  }
}

static void dump_outputs(gd_t *gd, bdry_t *bdry, wav_t *wav,
                         iorecv_t *iorecv, ioline_t *ioline)
{
  for (int lev = 0; lev < wav->nlevel; lev++) {
    char nm[48];
    snprintf(nm, 48, "out.wav.level%d", lev);
    put(nm, 'f', wav->v5d + (size_t)lev * wav->siz_ilevel, wav->siz_ilevel);
  }
  for (int d = 0; d < 3; d++)
    for (int s = 0; s < 2; s++) {
      if (bdry->is_sides_pml[d][s] != 1) continue;
      bdrypml_auxvar_t *a = &bdry->auxvar[d][s];
      char nm[48];
      snprintf(nm, 48, "out.pml.%d.%d.aux", d, s);
      put(nm, 'f', a->var, a->siz_ilevel * a->nlevel);
    }
  if (bdry->is_sides_free[2][1] == 1) {
    size_t n2 = gd->siz_iz * 9;
    put("out.matVx2Vz2", 'f', bdry->matVx2Vz2, n2);
    put("out.matVy2Vz2", 'f', bdry->matVy2Vz2, n2);
    put("out.matF2Vz2", 'f', bdry->matF2Vz2, n2);
    if (bdry->matD) put("out.matD", 'f', bdry->matD, n2);
  }
  for (int r = 0; r < iorecv->total_number; r++) {
    char nm[48];
    snprintf(nm, 48, "out.recv.%d.seismo", r);
    put(nm, 'f', iorecv->recvone[r].seismo, (int64_t)iorecv->max_nt * iorecv->ncmp);
  }
  for (int l = 0; l < ioline->num_of_lines; l++) {
    char nm[48];
    snprintf(nm, 48, "out.line.%d.seismo", l);
    put(nm, 'f', ioline->recv_seismo[l],
        (int64_t)ioline->line_nr[l] * ioline->max_nt * ioline->ncmp);
  }
}

void __wrap_drv_rk_curv_col_allstep(
  fd_t *fd, gd_t *gd, gdcurv_metric_t *metric, md_t *md, src_t *src,
  bdry_t *bdry, wav_t *wav, mympi_t *mympi, iorecv_t *iorecv,
  ioline_t *ioline, ioslice_t *ioslice, iosnap_t *iosnap, float dt,
  int nt_total, float t0, char *output_fname_part, char *output_dir,
  int qc_check_nan_num_of_step, const int output_all, const int verbose)
{
  const char *path = getenv("CGFD_DUMP_FILE");
  const char *seed = getenv("CGFD_DUMP_SEED");
  const char *amp = getenv("CGFD_DUMP_AMP");
  const char *media = getenv("CGFD_DUMP_MEDIA");
  if (media && md->medium_type == CONST_MEDIUM_ELASTIC_ISO) {
    /* uniform Vp,Vs,rho (the "code" medium of the reference is fixed) */
    float vp = 0, vs = 0, rho = 0;
    if (sscanf(media, "%f,%f,%f", &vp, &vs, &rho) != 3) exit(2);
    float mu = vs * vs * rho;
    float lam = vp * vp * rho - 2.0f * mu;
    for (size_t p = 0; p < gd->siz_icmp; p++) {
      md->lambda[p] = lam;
      md->mu[p] = mu;
      md->rho[p] = 1.0f / rho;
    }
  }
  if (path) {
    g_fp = fopen(path, "wb");
    if (!g_fp) { fprintf(stderr, "cannot open %s\n", path); exit(2); }
    if (seed) {
      g_rng = (uint32_t)strtoul(seed, NULL, 10);
      if (g_rng == 0) g_rng = 1;
      if (md->medium_type == CONST_MEDIUM_ELASTIC_ANISO) aniso_base(gd, md);
      perturb(gd, md, bdry, wav, amp ? (float)atof(amp) : 1e-2f);
    }
    dump_inputs(fd, gd, metric, md, src, bdry, wav, iorecv, ioline, dt,
                nt_total, t0);
  }
  __real_drv_rk_curv_col_allstep(fd, gd, metric, md, src, bdry, wav, mympi,
                                 iorecv, ioline, ioslice, iosnap, dt, nt_total,
                                 t0, output_fname_part, output_dir,
                                 qc_check_nan_num_of_step, output_all, verbose);
  if (g_fp) {
    dump_outputs(gd, bdry, wav, iorecv, ioline);
    fclose(g_fp);
    g_fp = NULL;
  }
}
