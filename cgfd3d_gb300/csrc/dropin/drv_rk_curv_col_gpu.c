/*
 * drv_rk_curv_col_gpu.c -- drop-in replacement of CGFD3D's time loop.
 *
 * Exports drv_rk_curv_col_allstep() with the reference prototype
 * (forward/drv_rk_curv_col.h:17-37), reading the reference's structs
 * unchanged, and runs the whole loop through the flat C ABI of
 * include/cgfd3d_gpu.h on the GPU.  Link it instead of
 * forward/drv_rk_curv_col.o, together with libcgfd3d_gpu.so and the CUDA
 * runtime (-lcudart).
 *
 * What the reference's loop leaves behind is left behind here too:
 *   wav->v5d         final state in level 0 (nt_total even) or 3 (odd)
 *   bdry->auxvar[][].var   final PML auxiliaries, same level rule
 *   bdry->matVx2Vz2/matVy2Vz2/matF2Vz2   free-surface matrices
 *   bdry->matD       visco-elastic surface rotation matrices
 *   iorecv->recvone[r].seismo, ioline->recv_seismo[l]   seismograms
 *   PGV/PGA/PGD surface maps (forward/wav_t.c:379-455), computed on the
 *   device every step and, inside the reference binary, written by its
 *   PG_slice_output() (forward/drv_rk_curv_col.c:547-550)
 * Slices and snapshots (NetCDF, forward/io_funcs.c:780-1268) are written by
 * the reference's own writers when this file is built inside the reference
 * tree (CGFD_DROPIN_REFERENCE_HEADERS).  The loop then runs up to each step
 * that writes and copies to the host only the points those writers read: the
 * slice planes and the due snapshot boxes, packed on the device
 * (cgfd_solver_fetch_boxes); output_all (a NetCDF volume of the whole state
 * every step, forward/drv_rk_curv_col.c:511-526) copies the whole state.
 * Built without the reference (tests, other hosts) there are no NetCDF
 * writers and requested slices/snapshots are reported and skipped.
 *
 * Errors print the library's message and call MPI_Abort when MPI is linked
 * (exit(1) otherwise), as the reference does.  Unsupported configurations
 * (dd sources spread over several points)
 * are reported the same way instead of being ignored.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../../../include/cgfd3d_dropin.h"
#include "../../../include/cgfd3d_gpu.h"

#ifdef CGFD_DROPIN_REFERENCE_HEADERS
#include "drv_rk_curv_col.h"
#define CGFD_REF_VISCO_GMB CONST_VISCO_GMB
#define CGFD_REF_VISCO_GRAVES_QS CONST_VISCO_GRAVES_QS
#else
#include "../../../include/cgfd3d_ref_abi.h"
#endif

#ifdef CGFD_DROPIN_REFERENCE_HEADERS
#define CGFD_ABORT() MPI_Abort(MPI_COMM_WORLD, 1)
#else
#define CGFD_ABORT() exit(1)
#endif

/* CGFD_* code of the failure that ended the time loop (0: none so far);
 * read by cgfd_gpu_last_error(), e.g. from an atexit handler, since the
 * failure itself ends the process as the reference's errors do */
static int g_gpu_code = 0;

int cgfd_gpu_last_error(void) { return g_gpu_code; }

static void fail(const char *what)
{
  fprintf(stderr, "drv_rk_curv_col_allstep (GPU): %s: %s\n", what,
          cgfd_last_error());
  fflush(stderr);
  CGFD_ABORT();
}

/* a library call's status: non-zero is recorded and ends the run */
static void check(int rc, const char *what)
{
  if (rc == 0) return;
  g_gpu_code = rc;
  fail(what);
}

/* Boxes of the slices io_slice_nc_put writes (forward/io_funcs.c:992-1111):
 * components 0..ncmp-1 (0..8 for GMB media), x slices over (k, j), y slices
 * over (k, i), z slices over (j, i) of the physical points. */
static int slice_boxes(const gd_t *gd, const ioslice_t *sl, const wav_t *wav,
                       cgfd_box_t *box)
{
  const int c2 = wav->visco_type == CGFD_REF_VISCO_GMB ? 8 : wav->ncmp - 1;
  int n = 0;
  for (int m = 0; m < sl->num_of_slice_x; m++, n++) {
    cgfd_box_t b = {0, c2, sl->slice_x_indx[m], 1, 1, gd->nj1, gd->nj, 1,
                    gd->nk1, gd->nk, 1};
    box[n] = b;
  }
  for (int m = 0; m < sl->num_of_slice_y; m++, n++) {
    cgfd_box_t b = {0, c2, gd->ni1, gd->ni, 1, sl->slice_y_indx[m], 1, 1,
                    gd->nk1, gd->nk, 1};
    box[n] = b;
  }
  for (int m = 0; m < sl->num_of_slice_z; m++, n++) {
    cgfd_box_t b = {0, c2, gd->ni1, gd->ni, 1, gd->nj1, gd->nj, 1,
                    sl->slice_z_indx[m], 1, 1};
    box[n] = b;
  }
  return n;
}

/* The rule of io_snap_nc_put (forward/io_funcs.c:1147-1153) for snapshot m
 * at step it. */
static int snapshot_due(const iosnap_t *sn, int m, int nt_total, int it)
{
  const int it1 = sn->it1[m], dit = sn->dit[m];
  return it >= it1 && (it - it1) / dit <= (nt_total - it1) / dit &&
         (it - it1) % dit == 0;
}

/* First step >= from at which a snapshot is due; nt_total when none is. */
static int next_snapshot(const iosnap_t *sn, int nt_total, int from)
{
  int best = nt_total;
  for (int m = 0; m < sn->num_of_snap; m++) {
    const int it1 = sn->it1[m], dit = sn->dit[m];
    int it = from <= it1 ? it1 : it1 + (from - it1 + dit - 1) / dit * dit;
    if (it < best && snapshot_due(sn, m, nt_total, it)) best = it;
  }
  return best;
}

/* Box of snapshot m: velocity (components 0..2) and/or stress (3..8, also
 * read for strain).  Returns the boxes added (0 or 1). */
static int snapshot_box(const iosnap_t *sn, int m, cgfd_box_t *b)
{
  const int v = sn->out_vel[m] == 1;
  const int t = sn->out_stress[m] == 1 || sn->out_strain[m] == 1;
  if (!v && !t) return 0;
  cgfd_box_t q = {v ? 0 : 3, t ? 8 : 2, sn->i1[m], sn->ni[m], sn->di[m],
                  sn->j1[m], sn->nj[m], sn->dj[m], sn->k1[m], sn->nk[m], sn->dk[m]};
  *b = q;
  return 1;
}

#ifdef CGFD_DROPIN_REFERENCE_HEADERS
/* What the reference's writers need at an output step. */
typedef struct {
  ioslice_t *ioslice;
  ioslice_nc_t *slice_nc;
  iosnap_t *iosnap;
  iosnap_nc_t *snap_nc;
  gd_t *gd;
  md_t *md;
  wav_t *wav;
  float *w_host, *w_buff;
  int nt_total, output_every;
  float dt, t0;
  char *output_dir;
  int *topoid;
} out_ctx_t;

/* The reference's writers for step it, handed the host state w_host, in the
 * order of forward/drv_rk_curv_col.c:501-526. */
static void write_step(const out_ctx_t *o, int it)
{
  const float t_end = it * o->dt + o->t0 + o->dt;
  io_slice_nc_put(o->ioslice, o->slice_nc, o->gd, o->w_host, o->w_buff, it, t_end, 0,
                  o->wav->ncmp - 1, o->wav->visco_type);
  io_snap_nc_put(o->iosnap, o->snap_nc, o->gd, o->md, o->wav, o->w_host, o->w_buff,
                 o->nt_total, it, t_end, 1, 1, 1);
  if (o->output_every) {
    char ou_file[CONST_MAX_STRLEN];
    io_build_fname_time(o->output_dir, "w3d", ".nc", o->topoid, it, ou_file);
    io_var3d_export_nc(ou_file, o->w_host, o->wav->cmp_pos, o->wav->cmp_name,
                       o->wav->ncmp, o->gd->index_name, o->gd->nx, o->gd->ny, o->gd->nz);
  }
}
#endif

static void fatal(const char *what)
{
  g_gpu_code = CGFD_EINVAL;
  fprintf(stderr, "drv_rk_curv_col_allstep (GPU): %s\n", what);
  fflush(stderr);
  CGFD_ABORT();
}

static void unsupported(const char *what)
{
  g_gpu_code = CGFD_EINVAL;
  fprintf(stderr, "drv_rk_curv_col_allstep (GPU): %s is not supported\n", what);
  fflush(stderr);
  CGFD_ABORT();
}

void drv_rk_curv_col_allstep(
    fd_t *fd, gd_t *gd, gdcurv_metric_t *metric, md_t *md, src_t *src,
    bdry_t *bdry, wav_t *wav, mympi_t *mympi, iorecv_t *iorecv,
    ioline_t *ioline, ioslice_t *ioslice, iosnap_t *iosnap, float dt,
    int nt_total, float t0, char *output_fname_part, char *output_dir,
    int qc_check_nan_num_of_step, const int output_all, const int verbose)
{
  (void)mympi; (void)output_fname_part; (void)output_dir;
  g_gpu_code = 0;

  if (fd->num_rk_stages != 4 || fd->num_of_pairs != 8)
    unsupported("an operator set other than MacCormack DRP with RK4");
  if (md->medium_type != CGFD_MEDIUM_ELASTIC_ISO &&
      md->medium_type != CGFD_MEDIUM_ELASTIC_VTI &&
      md->medium_type != CGFD_MEDIUM_ELASTIC_ANISO &&
      md->medium_type != CGFD_MEDIUM_VISCOELASTIC_ISO)
    unsupported("this medium type");
  if (md->medium_type == CGFD_MEDIUM_VISCOELASTIC_ISO &&
      md->visco_type != CGFD_REF_VISCO_GMB)
    unsupported("a visco-elastic model other than GMB");
  if (src->dd_is_valid == 1 && src->dd_is_add_at_point != 1)
    unsupported("a distributed (dd) source spread over several points");

  cgfd_problem_t p;
  memset(&p, 0, sizeof(p));
  p.ni = gd->ni; p.nj = gd->nj; p.nk = gd->nk;
  p.nx = gd->nx; p.ny = gd->ny; p.nz = gd->nz;
  p.ni1 = gd->ni1; p.ni2 = gd->ni2; p.nj1 = gd->nj1;
  p.nj2 = gd->nj2; p.nk1 = gd->nk1; p.nk2 = gd->nk2;
  p.jac = metric->jac;
  p.xi_x = metric->xi_x; p.xi_y = metric->xi_y; p.xi_z = metric->xi_z;
  p.eta_x = metric->eta_x; p.eta_y = metric->eta_y; p.eta_z = metric->eta_z;
  p.zeta_x = metric->zeta_x; p.zeta_y = metric->zeta_y; p.zeta_z = metric->zeta_z;
  p.medium_type = md->medium_type;
  p.slw = md->rho; /* md_rho_to_slow ran before the call */
  p.lambda = md->lambda;
  p.mu = md->mu;
  p.c11 = md->c11; p.c13 = md->c13; p.c33 = md->c33;
  p.c55 = md->c55; p.c66 = md->c66;
  if (md->medium_type == CGFD_MEDIUM_ELASTIC_ANISO) {
    p.c12 = md->c12; p.c14 = md->c14; p.c15 = md->c15; p.c16 = md->c16;
    p.c22 = md->c22; p.c23 = md->c23; p.c24 = md->c24; p.c25 = md->c25;
    p.c26 = md->c26; p.c34 = md->c34; p.c35 = md->c35; p.c36 = md->c36;
    p.c44 = md->c44; p.c45 = md->c45; p.c46 = md->c46; p.c56 = md->c56;
  }
  if (md->medium_type == CGFD_MEDIUM_VISCOELASTIC_ISO) {
    if (md->nmaxwell > CGFD_MAX_MAXWELL) unsupported("more than 8 Maxwell bodies");
    p.nmaxwell = md->nmaxwell;
    p.wl = md->wl;
    for (int n = 0; n < md->nmaxwell; n++) {
      p.Ylam[n] = md->Ylam[n];
      p.Ymu[n] = md->Ymu[n];
    }
    p.x3d = gd->x3d; p.y3d = gd->y3d; p.z3d = gd->z3d;
  }
  if (md->visco_type == CGFD_REF_VISCO_GRAVES_QS) {
    /* Graves Q (forward/drv_rk_curv_col.c:414-416) */
    p.graves_qs = 1;
    p.qs_freq = md->visco_Qs_freq;
    p.Qs = md->Qs;
  }
  if (bdry->is_enable_ablexp == 1) {
    /* exponential sponge (forward/drv_rk_curv_col.c:484-486) */
    p.ablexp = 1;
    p.ablexp_Ex = bdry->ablexp_Ex;
    p.ablexp_Ey = bdry->ablexp_Ey;
    p.ablexp_Ez = bdry->ablexp_Ez;
    for (int n = 0; n < 6; n++) {
      const bdry_block_t *D = &bdry->bdry_blk[n];
      int v[7] = {D->enable, D->ni1, D->ni2, D->nj1, D->nj2, D->nk1, D->nk2};
      memcpy(p.ablexp_blk[n], v, sizeof v);
    }
  }
  /* distributed sources: the reference streams their per-step values from
   * the files its set-up wrote (forward/src_t.c:1929-2000); here the whole
   * files are read once and handed to the device */
  float *dd_vi = NULL, *dd_mij = NULL;
  if (src->dd_is_valid == 1 && src->dd_total_number > 0) {
    size_t nt = (size_t)src->dd_max_nt * src->max_stage * src->dd_total_number;
    if (src->max_stage != 4) unsupported("dd sources with other than 4 stages");
    if (src->dd_vi_actived == 1) {
      dd_vi = (float *)malloc(3 * nt * sizeof(float));
      if (!dd_vi || fseek(src->fp_vi, 0, SEEK_SET) != 0 ||
          fread(dd_vi, sizeof(float), 3 * nt, src->fp_vi) != 3 * nt)
        fatal("cannot read the dd force-rate file");
    }
    if (src->dd_mij_actived == 1) {
      dd_mij = (float *)malloc(6 * nt * sizeof(float));
      if (!dd_mij || fseek(src->fp_mij, 0, SEEK_SET) != 0 ||
          fread(dd_mij, sizeof(float), 6 * nt, src->fp_mij) != 6 * nt)
        fatal("cannot read the dd moment-rate file");
    }
    p.dd_n = src->dd_total_number;
    p.dd_max_nt = src->dd_max_nt;
    p.dd_si = src->dd_si; p.dd_sj = src->dd_sj; p.dd_sk = src->dd_sk;
    p.dd_vi = dd_vi;
    p.dd_mij = dd_mij;
  }
  p.free_top = bdry->is_sides_free[2][1] == 1;
  for (int d = 0; d < 3; d++)
    for (int s = 0; s < 2; s++) {
      cgfd_pml_face_t *f = &p.pml[d][s];
      f->enabled = bdry->is_enable_pml == 1 && bdry->is_sides_pml[d][s] == 1;
      if (!f->enabled) continue;
      f->ni1 = bdry->ni1[d][s]; f->ni2 = bdry->ni2[d][s];
      f->nj1 = bdry->nj1[d][s]; f->nj2 = bdry->nj2[d][s];
      f->nk1 = bdry->nk1[d][s]; f->nk2 = bdry->nk2[d][s];
      f->A = bdry->A[d][s]; f->B = bdry->B[d][s]; f->D = bdry->D[d][s];
      f->aux = bdry->auxvar[d][s].var;
    }

  if (src->total_number > 0) {
    p.src_n = src->total_number;
    p.src_max_nt = src->max_nt;
    p.src_max_stage = src->max_stage;
    p.src_force = src->force_actived;
    p.src_moment = src->moment_actived;
    p.src_spatial = src->itype_spatial_ext;
    p.src_ext_half = src->ext_half_npoint;
    p.src_ext_coef = src->ext_func_coef;
    p.src_surface_strict = src->is_surface_force_strict;
    p.src_n_surface_force = src->total_number_surface_force;
    p.src_si = src->si; p.src_sj = src->sj; p.src_sk = src->sk;
    p.src_si_inc = src->si_inc; p.src_sj_inc = src->sj_inc; p.src_sk_inc = src->sk_inc;
    p.src_it_begin = src->it_begin; p.src_it_end = src->it_end;
    p.Fx = src->Fx; p.Fy = src->Fy; p.Fz = src->Fz;
    p.Mxx = src->Mxx; p.Myy = src->Myy; p.Mzz = src->Mzz;
    p.Mxz = src->Mxz; p.Myz = src->Myz; p.Mxy = src->Mxy;
    if (src->total_number_surface_force > 0) {
      p.src_force_rate_indx = src->force_rate_indx;
      p.Fx_rate = src->Fx_rate; p.Fy_rate = src->Fy_rate; p.Fz_rate = src->Fz_rate;
    }
  }

  /* receivers: gather the per-station interpolation data, packed output */
  int nr = iorecv->total_number;
  float *rdijk = NULL, *rseis = NULL;
  int *ridx = NULL;
  if (nr > 0) {
    rdijk = (float *)malloc(sizeof(float) * 3 * nr);
    ridx = (int *)malloc(sizeof(int) * 8 * nr);
    rseis = (float *)calloc((size_t)nr * iorecv->ncmp * iorecv->max_nt, sizeof(float));
    if (!rdijk || !ridx || !rseis) unsupported("host memory for receivers");
    for (int r = 0; r < nr; r++) {
      iorecv_one_t *o = iorecv->recvone + r;
      rdijk[3 * r] = o->di; rdijk[3 * r + 1] = o->dj; rdijk[3 * r + 2] = o->dk;
      memcpy(ridx + 8 * r, o->indx1d, 8 * sizeof(int));
    }
    p.recv_n = nr;
    p.recv_max_nt = iorecv->max_nt;
    p.recv_ncmp = iorecv->ncmp;
    p.recv_dijk = rdijk;
    p.recv_indx1d = ridx;
    p.recv_seismo = rseis;
  }
  /* lines: concatenated */
  int nline = 0;
  for (int l = 0; l < ioline->num_of_lines; l++) nline += ioline->line_nr[l];
  int *liptr = NULL;
  float *lseis = NULL;
  if (nline > 0) {
    liptr = (int *)malloc(sizeof(int) * nline);
    lseis = (float *)calloc((size_t)nline * wav->ncmp * ioline->max_nt, sizeof(float));
    if (!liptr || !lseis) unsupported("host memory for receiver lines");
    int n = 0;
    for (int l = 0; l < ioline->num_of_lines; l++)
      for (int r = 0; r < ioline->line_nr[l]; r++) liptr[n++] = ioline->recv_iptr[l][r];
    p.line_n = nline;
    p.line_max_nt = ioline->max_nt;
    p.line_iptr = liptr;
    p.line_seismo = lseis;
  }

  p.ncmp = wav->ncmp;
  p.nlevel = wav->nlevel;
  p.wav = wav->v5d;
  p.dt = dt;
  p.t0 = t0;
  p.nt_total = nt_total;

  /* slice / snapshot writers of the reference */
  int nslice = ioslice->num_of_slice_x + ioslice->num_of_slice_y +
               ioslice->num_of_slice_z;
  int nsnap = iosnap->num_of_snap;
#ifdef CGFD_DROPIN_REFERENCE_HEADERS
  ioslice_nc_t ioslice_nc;
  iosnap_nc_t iosnap_nc;
  io_slice_nc_create(ioslice, wav->ncmp, wav->visco_type, wav->cmp_name, gd->ni,
                     gd->nj, gd->nk, mympi->topoid, &ioslice_nc);
  io_snap_nc_create(iosnap, &iosnap_nc, mympi->topoid);
#else
  if (nslice + nsnap > 0) {
    fprintf(stderr, "drv_rk_curv_col_allstep (GPU): built without the reference's "
                    "NetCDF writers, %d slices and %d snapshots skipped\n",
            nslice, nsnap);
    nslice = nsnap = 0;
  }
#endif
#ifndef CGFD_DROPIN_REFERENCE_HEADERS
  const int output_every = 0;
  (void)output_all;
#else
  const int output_every = output_all == 1;
#endif
  const int step_wise = nslice + nsnap > 0 || output_every;
  float *w_host = NULL, *w_buff = NULL;
  cgfd_box_t *box = NULL;
  if (step_wise) {
    size_t L = (size_t)wav->ncmp * gd->nx * gd->ny * gd->nz;
    w_host = (float *)calloc(L, sizeof(float));
    w_buff = (float *)calloc(L, sizeof(float));
    box = (cgfd_box_t *)malloc((size_t)(nslice + nsnap + 1) * sizeof(cgfd_box_t));
    if (!w_host || !w_buff || !box) unsupported("host memory for slice/snapshot output");
  }
  const int nslice_box = nslice > 0 ? slice_boxes(gd, ioslice, wav, box) : 0;

#ifdef CGFD_DROPIN_REFERENCE_HEADERS
  const out_ctx_t octx = {ioslice, &ioslice_nc, iosnap, &iosnap_nc, gd, md, wav,
                          w_host, w_buff, nt_total, output_every, dt, t0,
                          output_dir, mympi->topoid};
#define write_output(it_) write_step(&octx, (it_))
#else
#define write_output(it_) ((void)(it_))
#endif
  if (verbose > 0) fprintf(stdout, "GPU time loop: %d steps ...\n", nt_total);
  cgfd_solver_t *s = NULL;
  check(cgfd_solver_create(&p, &s), "solver setup");
  /* Steps are queued without waiting; the boxes of a step that writes are
   * packed behind it into one of two output slots, and written while the
   * device runs the next step. */
  int pend_it = -1, pend_slot = 0, slot = 0;
  for (int done = 0; done < nt_total;) {
    int n = nt_total - done;
    if (qc_check_nan_num_of_step > 0) {
      int to_qc = qc_check_nan_num_of_step - done % qc_check_nan_num_of_step;
      if (to_qc < n) n = to_qc;
    }
    if (step_wise) {   /* run through the next step that writes */
      int next = nslice > 0 || output_every ? done : next_snapshot(iosnap, nt_total, done);
      if (next - done + 1 < n) n = next - done + 1;
    }
    check(cgfd_solver_run_async(s, n), "time loop");
    done += n;
    const int it = done - 1;
    int nbox = 0, due = 0;
    if (step_wise) {
      nbox = nslice_box;
      for (int m = 0; m < nsnap; m++)
        if (snapshot_due(iosnap, m, nt_total, it)) nbox += snapshot_box(iosnap, m, box + nbox);
      due = nbox > 0 || output_every;
    }
    if (due && !output_every)
      check(cgfd_solver_pack_boxes_async(s, box, nbox, slot), "slices/snapshots");
    if (pend_it >= 0) {
      check(cgfd_solver_collect_boxes(s, pend_slot, w_host, NULL), "slices/snapshots");
      write_output(pend_it);
      pend_it = -1;
    }
    if (due && output_every) {
      check(cgfd_solver_fetch_state(s, w_host), "state for output");
      write_output(it);
    } else if (due) {
      pend_it = it;
      pend_slot = slot;
      slot ^= 1;
    }
    if (qc_check_nan_num_of_step > 0 && done % qc_check_nan_num_of_step == 0)
      check(cgfd_solver_check_finite(s), "wavefield check");
  }
  if (pend_it >= 0) {
    check(cgfd_solver_collect_boxes(s, pend_slot, w_host, NULL), "slices/snapshots");
    write_output(pend_it);
  }
  check(cgfd_solver_run(s, 0), "time loop");   /* waits, reads device errors */
  check(cgfd_solver_fetch(s), "fetch");
  if (p.free_top && bdry->matVx2Vz2)
    check(cgfd_solver_fetch_surface_matrices(s, bdry->matVx2Vz2, bdry->matVy2Vz2,
                                             bdry->matF2Vz2),
          "free-surface matrices");
  if (p.free_top && md->medium_type == CGFD_MEDIUM_VISCOELASTIC_ISO && bdry->matD)
    check(cgfd_solver_fetch_surface_rotation(s, bdry->matD), "free-surface rotation matrices");
#ifdef CGFD_DROPIN_REFERENCE_HEADERS
  if (p.free_top) {
    float *PG = (float *)calloc((size_t)15 * gd->nx * gd->ny, sizeof(float));
    if (!PG) unsupported("host memory for the peak-motion maps");
    check(cgfd_solver_fetch_pg(s, PG), "peak-motion maps");
    PG_slice_output(PG, gd, output_dir, output_fname_part, mympi->topoid);
    free(PG);
  }
  io_slice_nc_close(&ioslice_nc);
  io_snap_nc_close(&iosnap_nc);
#endif
  cgfd_solver_destroy(s);
  free(w_host);
  free(w_buff);
  free(box);

  /* scatter seismograms back into the reference's buffers */
  for (int r = 0; r < nr; r++) {
    size_t len = (size_t)iorecv->ncmp * iorecv->max_nt;
    memcpy(iorecv->recvone[r].seismo, rseis + r * len, len * sizeof(float));
  }
  int n = 0;
  for (int l = 0; l < ioline->num_of_lines; l++) {
    size_t len = (size_t)ioline->line_nr[l] * wav->ncmp * ioline->max_nt;
    memcpy(ioline->recv_seismo[l], lseis + (size_t)n * wav->ncmp * ioline->max_nt,
           len * sizeof(float));
    n += ioline->line_nr[l];
  }
  free(rdijk); free(ridx); free(rseis); free(liptr); free(lseis);
  free(dd_vi); free(dd_mij);
}
