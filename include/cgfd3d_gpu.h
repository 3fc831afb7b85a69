/*
 * cgfd3d_gpu.h -- C ABI of the GB300 (sm_103a) time-stepping library.
 *
 * This library replaces the time loop of CGFD3D:
 *
 *   void drv_rk_curv_col_allstep(fd_t*, gd_t*, gdcurv_metric_t*, md_t*,
 *        src_t*, bdry_t*, wav_t*, mympi_t*, iorecv_t*, ioline_t*,
 *        ioslice_t*, iosnap_t*, float dt, int nt_total, float t0, ...)
 *   (reference: forward/drv_rk_curv_col.h:17-37, forward/drv_rk_curv_col.c:27-556)
 *
 * Two layers are exported:
 *
 *   1. the drop-in `drv_rk_curv_col_allstep` itself, built from
 *      cgfd3d_gb300/csrc/dropin/drv_rk_curv_col_gpu.c against the reference's
 *      own struct headers; it unpacks the reference structs into a
 *      cgfd_problem_t and calls cgfd_allstep();
 *   2. the flat C ABI below: plain pointers and sizes, no reference types,
 *      so any FFI (ctypes, cgo, JNI) can bind it.
 *
 * Every array is a host array in the reference's layout: padded volume
 * nx*ny*nz (ni+6, nj+6, nk+6), index i + j*nx + k*nx*ny, k upward with the
 * free surface at k = nk2 (forward/gd_t.c:2856-2892); wavefield levels are
 * nlevel x ncmp x volume with component order Vx,Vy,Vz,Txx,Tyy,Tzz,Tyz,Txz,Txy
 * (forward/wav_t.c:93-136).  Errors are reported by return code (0 = ok) and
 * cgfd_last_error(); nothing in this ABI calls exit().
 */
#ifndef CGFD3D_GPU_H
#define CGFD3D_GPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CGFD_ABI_VERSION 6

/* medium types, same codes as forward/constants.h:24-29 */
#define CGFD_MEDIUM_ELASTIC_ISO 2
#define CGFD_MEDIUM_ELASTIC_VTI 3
#define CGFD_MEDIUM_ELASTIC_ANISO 4
#define CGFD_MEDIUM_VISCOELASTIC_ISO 5
#define CGFD_MAX_MAXWELL 8

/* source spatial types, forward/constants.h:36-38 */
#define CGFD_SRC_POINT 1
#define CGFD_SRC_GAUSSIAN 2

/* error codes */
#define CGFD_OK 0
#define CGFD_EINVAL 1      /* bad argument / unsupported configuration */
#define CGFD_ECUDA 2       /* CUDA runtime error */
#define CGFD_ENOMEM 3      /* device allocation failed */
#define CGFD_ENONFINITE 4  /* NaN/Inf found by the finiteness check */

/* One CFS-PML face: bdry_t.{ni1..nk2,A,B,D,auxvar}[idim][iside]
 * (forward/bdry_t.h:86-108, forward/bdry_t.c:115-327). */
typedef struct {
  int enabled;                       /* is_sides_pml[idim][iside] */
  int ni1, ni2, nj1, nj2, nk1, nk2;  /* face box, inclusive, padded indices */
  const float *A, *B, *D;            /* length = box extent along the normal */
  float *aux;  /* nlevel x ncmp x box volume, level order pre,tmp,rhs,end;
                  only level 0 (pre) is read, the final state is written
                  back to level 0 (nt_total even) or 3 (odd) like the
                  reference's pointer swap */
} cgfd_pml_face_t;

/* Everything drv_rk_curv_col_allstep reads and writes, flattened. */
typedef struct {
  /* grid: gd_t (forward/gd_t.h:27-125) */
  int ni, nj, nk, nx, ny, nz, ni1, ni2, nj1, nj2, nk1, nk2;

  /* metrics: gdcurv_metric_t (forward/gd_t.h:152-174), each nx*ny*nz */
  const float *jac, *xi_x, *xi_y, *xi_z, *eta_x, *eta_y, *eta_z,
              *zeta_x, *zeta_y, *zeta_z;

  /* media: md_t (forward/md_t.h:11-73); slw is 1/rho
   * (md_rho_to_slow, forward/md_t.c:601-623, applied before the call) */
  int medium_type;
  const float *slw, *lambda, *mu;                /* iso, visco */
  const float *c11, *c13, *c33, *c55, *c66;       /* vti */
  int nmaxwell;                                   /* visco GMB */
  const float *wl;                                /* nmaxwell */
  const float *Ylam[CGFD_MAX_MAXWELL], *Ymu[CGFD_MAX_MAXWELL];

  /* boundaries: bdry_t (forward/bdry_t.h:66-151) */
  int free_top;                      /* is_sides_free[2][1] */
  cgfd_pml_face_t pml[3][2];         /* [idim][iside] */

  /* sources: src_t (forward/src_t.h:21-128) */
  int src_n, src_max_nt, src_max_stage;
  int src_force, src_moment;         /* force_actived, moment_actived */
  int src_spatial;                   /* itype_spatial_ext */
  int src_ext_half;                  /* ext_half_npoint */
  float src_ext_coef;                /* ext_func_coef (Gaussian width) */
  int src_surface_strict;            /* is_surface_force_strict */
  int src_n_surface_force;           /* total_number_surface_force: force
                                        sources whose spread reaches the free
                                        surface (their rate tables below) */
  const int *src_si, *src_sj, *src_sk, *src_it_begin, *src_it_end;
  const float *src_si_inc, *src_sj_inc, *src_sk_inc;
  const float *Fx, *Fy, *Fz;                     /* [is][it][istage] */
  const float *Mxx, *Myy, *Mzz, *Mxz, *Myz, *Mxy;

  /* station receivers: iorecv_t (forward/io_funcs.h:17-39) */
  int recv_n, recv_max_nt, recv_ncmp;
  const float *recv_dijk;            /* 3 per receiver: di, dj, dk */
  const int *recv_indx1d;            /* 8 per receiver */
  float *recv_seismo;                /* [n][ncmp][max_nt], written */

  /* line receivers: ioline_t (forward/io_funcs.h:42-60), all lines
   * concatenated */
  int line_n, line_max_nt;
  const int *line_iptr;              /* line_n */
  float *line_seismo;                /* [line_n][ncmp][max_nt], written */

  /* wavefield: wav_t.v5d (forward/wav_t.h:15-67) */
  int ncmp, nlevel;
  float *wav;  /* nlevel x ncmp x volume; level 0 read, final state written
                  to level 0 or 3 as for the PML aux */

  float dt, t0;
  int nt_total;

  /* grid coordinates gd_t.x3d/y3d/z3d (forward/gd_t.h:62-67), each
   * nx*ny*nz; read only for the visco-elastic free surface, whose stress
   * rotation needs the grid's eta tangent at k = nk2
   * (forward/sv_curv_col_vis_iso.c:353-507).  May be NULL otherwise. */
  const float *x3d, *y3d, *z3d;

  /* surface force sources (forward/src_t.c:1021-1028, :1084-1090):
   * src_force_rate_indx[n] is the source index of the n-th surface force,
   * F*_rate its force-rate table [n][max_nt][max_stage].  Each stage they
   * give the surface traction and velocity-rate layers
   * (forward/src_t.c:153-314) used by the traction image and vlow. */
  const int *src_force_rate_indx;
  const float *Fx_rate, *Fy_rate, *Fz_rate;

  /* Graves Q attenuation of an elastic medium (visco_type graves_Qs,
   * forward/sv_curv_col_el.c:638-666, applied at drv_rk_curv_col.c:414-416):
   * after each step's last stage every component of every physical point is
   * multiplied by expf(-PI * qs_freq * dt / Qs).  Qs: nx*ny*nz. */
  int graves_qs;
  float qs_freq;
  const float *Qs;

  /* exponential sponge (ablexp, forward/bdry_t.c:513-890, applied after each
   * step at drv_rk_curv_col.c:484-486): every component of the points of the
   * enabled blocks is multiplied by min(Ex[i], Ey[j], Ez[k]).
   * ablexp_blk[n] = {enable, ni1, ni2, nj1, nj2, nk1, nk2} of
   * bdry_t.bdry_blk[n]; Ex/Ey/Ez: nx, ny, nz floats. */
  int ablexp;
  const float *ablexp_Ex, *ablexp_Ey, *ablexp_Ez;
  int ablexp_blk[6][7];

  /* fully anisotropic elastic medium (medium_type 4, md_t c11..c66,
   * forward/md_t.h): the 16 constants below together with c11, c13, c33,
   * c55, c66 above, nx*ny*nz each (forward/sv_curv_col_el_aniso.c) */
  const float *c12, *c14, *c15, *c16, *c22, *c23, *c24, *c25, *c26;
  const float *c34, *c35, *c36, *c44, *c45, *c46, *c56;

  /* distributed (dd) sources added at grid points (src_t dd_*,
   * forward/src_t.c:1182-1930, injected after the other sources by
   * sv_curv_col_el_rhs_srcdd, forward/sv_curv_col_el.c:487-590): dd_n points
   * at local indices (ghosts included) dd_si/sj/sk; per step and RK stage
   * dd_vi[dd_max_nt][4][dd_n][3] (added to the velocity rates times
   * slw/jac) and dd_mij[dd_max_nt][4][dd_n][6] (Mxx Myy Mzz Myz Mxz Mxy,
   * subtracted from the stress rates times 1/jac), either may be NULL; the
   * sources act while the step index is below dd_max_nt. */
  int dd_n, dd_max_nt;
  const int *dd_si, *dd_sj, *dd_sk;
  const float *dd_vi, *dd_mij;
} cgfd_problem_t;

/* Opaque device-resident solver. */
typedef struct cgfd_solver cgfd_solver_t;

/* Last error message of the calling thread ("" when none). */
const char *cgfd_last_error(void);

/* ABI version (CGFD_ABI_VERSION). */
int cgfd_abi_version(void);

/* Uploads every input of `p` into HBM, computes the free-surface conversion
 * matrices of the medium on the device (forward/sv_curv_col_el_iso.c:
 * 1258-1375, forward/sv_curv_col_el_vti.c:1085-1206,
 * forward/sv_curv_col_vis_iso.c:353-507) and returns a solver positioned at
 * step 0.  Media: elastic_iso, elastic_vti, viscoelastic_iso (GMB, 1 to 3
 * Maxwell bodies).  `p` must stay valid until
 * cgfd_solver_destroy (host output arrays are written by cgfd_solver_fetch). */
int cgfd_solver_create(const cgfd_problem_t *p, cgfd_solver_t **out);

/* Advances `nsteps` RK4 steps on the device (no host traffic). */
int cgfd_solver_run(cgfd_solver_t *s, int nsteps);

/* Copies the current wavefield (into p->wav level 0 or 3, as the reference
 * leaves it), PML aux and seismograms back into the host arrays of `p`. */
int cgfd_solver_fetch(cgfd_solver_t *s);

/* Only the receiver and line seismograms of cgfd_solver_fetch (callers that
 * need no wavefield, such as shot gathers). */
int cgfd_solver_fetch_seismograms(cgfd_solver_t *s);

/* Current step index. */
int cgfd_solver_step(const cgfd_solver_t *s);

/* Copies the free-surface conversion matrices (3 x nx*ny*9, layout of
 * bdry_t.matVx2Vz2/matVy2Vz2/matF2Vz2, forward/bdry_t.c:86-109) to the host
 * arrays given (NULL skips one). */
int cgfd_solver_fetch_surface_matrices(cgfd_solver_t *s, float *mVx, float *mVy,
                                       float *mF);

/* Copies the visco-elastic surface rotation matrices (nx*ny*9, layout of
 * bdry_t.matD, forward/sv_curv_col_vis_iso.c:487-501) to mD.  Only for a
 * visco-elastic medium with a free surface. */
int cgfd_solver_fetch_surface_rotation(cgfd_solver_t *s, float *mD);

/* Copies the surface peak-motion maps accumulated so far (15 x nx*ny, the
 * PG array of forward/drv_rk_curv_col.c:123-130, filled as PG_calcu does,
 * forward/wav_t.c:379-455).  Only with a free surface. */
int cgfd_solver_fetch_pg(cgfd_solver_t *s, float *pg);

/* Copies the current state (ncmp x nx*ny*nz, reference layout) to w without
 * touching the problem's arrays. */
int cgfd_solver_fetch_state(cgfd_solver_t *s, float *w);

/* A box of wavefield points for slice and snapshot output: components
 * c1..c2 and the points (i1 + a*di, j1 + b*dj, k1 + c*dk), a < ni, b < nj,
 * c < nk, in padded-array indices (ghosts included), as the reference's
 * ioslice_t / iosnap_t hold them (forward/io_funcs.h).  An x slice at i is
 * {i1 = i, ni = 1, j over nj1..nj2, k over nk1..nk2}; a snapshot is
 * {i1, ni, di, j1, nj, dj, k1, nk, dk} of iosnap_t. */
typedef struct {
  int c1, c2;
  int i1, ni, di;
  int j1, nj, dj;
  int k1, nk, dk;
} cgfd_box_t;

/* Floats that nbox boxes hold; 0 when a box has a count or stride below 1 or
 * c2 < c1. */
size_t cgfd_box_floats(const cgfd_box_t *box, int nbox);

/* Packs the boxes of the current state (the level cgfd_solver_fetch_state
 * copies) on the device and copies only them to the host: box after box,
 * component after component, then k, j, i (i fastest) -- the order in which
 * io_slice_nc_put and io_snap_pack_buff (forward/io_funcs.c:992-1111,
 * 1525-1557) pack slices and snapshots.  out holds cgfd_box_floats() floats.
 * A box outside the padded grid or the solver's components is CGFD_EINVAL. */
int cgfd_solver_pack_boxes(cgfd_solver_t *s, const cgfd_box_t *box, int nbox,
                           float *out);

/* The same boxes written into w (ncmp x nx*ny*nz, reference layout) at their
 * own positions; the other points of w are left untouched.  Replaces the
 * whole-state copy in front of the reference's slice/snapshot writers, which
 * read only these points (forward/drv_rk_curv_col.c:501-506). */
int cgfd_solver_fetch_boxes(cgfd_solver_t *s, const cgfd_box_t *box, int nbox,
                            float *w);

/* Output overlapped with the time loop.  cgfd_solver_run_async queues steps
 * and returns; cgfd_solver_pack_boxes_async queues the packing of boxes of
 * the state after the queued steps into output slot `slot`
 * (0..CGFD_OUT_SLOTS-1) and returns; cgfd_solver_collect_boxes waits for that
 * slot and hands the boxes out as cgfd_solver_fetch_boxes (into w) and/or
 * cgfd_solver_pack_boxes (into out) do -- either pointer may be NULL.  With
 * two slots a caller writes step n's slices while the device runs step n+1.
 * A slot must be collected before it is packed again.  Errors of queued work
 * surface at the next collect or blocking call. */
#define CGFD_OUT_SLOTS 2
int cgfd_solver_run_async(cgfd_solver_t *s, int nsteps);
int cgfd_solver_pack_boxes_async(cgfd_solver_t *s, const cgfd_box_t *box, int nbox,
                                 int slot);
int cgfd_solver_collect_boxes(cgfd_solver_t *s, int slot, float *w, float *out);

/* Checks the whole wavefield for NaN/Inf on the device.
 * Returns CGFD_OK or CGFD_ENONFINITE. */
int cgfd_solver_check_finite(cgfd_solver_t *s);

/* CUDA-event times of the last cgfd_solver_run, milliseconds:
 * out[0] = sum over the interior stage-kernel launches (timing on only),
 * out[1] = the whole run, out[2] = sum over the CFS-PML face launches;
 * count[0] stage launches, count[1] all launches, count[2] face launches. */
int cgfd_solver_kernel_times(const cgfd_solver_t *s, float out[3], int count[3]);

/* Record a CUDA event pair around every stage launch of later runs. */
int cgfd_solver_set_timing(cgfd_solver_t *s, int on);

/* No counterpart in the reference (its loop has no device waits).  Every
 * wait of the stage kernel on a bulk copy or a buffer release gives up after
 * `wait_limit` polls (0: the default, about half a second): it records
 * device error 1, the whole CTA leaves its loop, the producer waits for the
 * copies it issued, and the run returns CGFD_ECUDA ("device wait timed
 * out") with the device still usable.  Test hook: skip_plane >= 0 makes the
 * first CTA of every stage launch leave out the copy of that wavefield
 * plane of its k march, so a wait on it runs out (-1: off).  A solver that
 * has timed out keeps its error; destroy it. */
int cgfd_solver_set_wait_test(cgfd_solver_t *s, int wait_limit, int skip_plane);

/* Host<->device bytes moved so far (uploads at create, fetches). */
int cgfd_solver_transfer_bytes(const cgfd_solver_t *s, size_t *h2d, size_t *d2h);

void cgfd_solver_destroy(cgfd_solver_t *s);

/* One-shot equivalent of drv_rk_curv_col_allstep on flat arrays:
 * create + run(nt_total) + fetch + destroy. */
int cgfd_allstep(const cgfd_problem_t *p);

/* Grid metrics on the device, as the reference's gd_curv_metric_cal
 * (forward/gd_t.c:190-402): from the node coordinates x3d/y3d/z3d
 * (nx*ny*nz each, ghosts included, 3-ghost layout) into `metric` =
 * 10 x nx*ny*nz host floats in the order jac, xi_x, xi_y, xi_z, eta_x,
 * eta_y, eta_z, zeta_x, zeta_y, zeta_z, ghost layers mirrored.  A problem
 * whose jac is NULL but whose x3d/y3d/z3d are set gets its metrics computed
 * this way inside cgfd_solver_create. */
int cgfd_metric_calc(int nx, int ny, int nz, int ni1, int ni2, int nj1, int nj2,
                     int nk1, int nk2, const float *x3d, const float *y3d,
                     const float *z3d, float *metric);

/* ------------------------------------------------------------------------
 * Point location: stations and sources given by coordinates, located on a
 * curvilinear grid as the reference locates them
 * (gd_curv_coord_to_glob_indx, forward/gd_t.c:1917-1995, after
 * gd_curv_depth_to_axis, :2179-2297, for points given by depth), with the
 * same indices and shifts bit for bit.  The grid has 3 ghost layers per side
 * (ni = nx - 6, ...).
 * ------------------------------------------------------------------------ */
typedef struct cgfd_locator cgfd_locator_t;

/* Copies the padded coordinates (nx*ny*nz floats each) to the device and
 * computes the bounds the search uses (gd_curv_set_minmax,
 * forward/gd_t.c:1708-1880). */
int cgfd_locator_create(int nx, int ny, int nz, const float *x3d, const float *y3d,
                        const float *z3d, cgfd_locator_t **out);

/* Locates n points.  is_depth[q] != 0 (is_depth may be NULL): z[q] is a
 * depth below the surface, converted to z first.  Per point: found[q] (1 or
 * 0), index[3q..3q+2] the global physical indices (i, j, k counted from the
 * first physical point; -1000 when not found), shift[3q..3q+2] the offsets
 * inside the cell (what the reference returns in sx_inc, sy_inc, sz_inc) and
 * z_located[q] (may be NULL) the z that was located. */
int cgfd_locator_locate(cgfd_locator_t *loc, int n, const float *x, const float *y,
                        const float *z, const int *is_depth, int *found, int *index,
                        float *shift, float *z_located);

void cgfd_locator_destroy(cgfd_locator_t *loc);

/* An elastic isotropic layered model discretised on a curvilinear grid,
 * as media_layer2model_el_iso does (media/media_layer2model.cpp:140-190,
 * 422-560, 1334-1384, 1984-2190; called at
 * forward/main_curv_col_el_3d.c:328-334): NI interfaces on a uniform
 * NX x NY mesh from (MINX, MINY) with spacing DX, DY; rec holds
 * [NI][NY][NX][10] = elevation, rho, rho_grad, rho_pow, vp, vp_grad,
 * vp_pow, vs, vs_grad, vs_pow (the .md3lay record).  method is the
 * reference's equivalent_medium_method: "loc" (the value at each point),
 * "har" (harmonic kappa and mu, arithmetic rho over each cell that touches
 * two layers) or "ari" (arithmetic lambda, mu, rho there).  Writes lam, mu,
 * rho (host, nx*ny*nz each).  A point outside the mesh or with
 * vp <= sqrt(2) vs is CGFD_EINVAL (the reference exits there), and so is
 * another method, and so is a model with a power outside [0, 1] on a
 * non-zero gradient: cgfd_media_layer_pow_ok(nc, rec, NI*NX*NY) tells it
 * beforehand
 * (nc: the record width, 10 here, 19 for VTI), and callers then use the
 * reference's host routine. */
int cgfd_media_layer_pow_ok(int nc, const float *rec, size_t nrec);

/* An elastic isotropic 3-D grid model (.md3grd) discretised on a
 * curvilinear grid, as media_grid2model_el_iso does
 * (media/media_grid2model.cpp:133-189, 424-556, 1067-1126, 1269-1356,
 * 1819-2079; called at forward/main_curv_col_el_3d.c:394-403): NI grid
 * levels in NL layers of ngz[l] levels, on a uniform NX x NY mesh from
 * (MINX, MINY) with spacing DX, DY, as the reference's reader leaves it
 * after cropping to the grid's extent; rec [NI][NY][NX][4] = elevation, rho,
 * vp, vs.  Values are linear between the two levels around a point;
 * method "loc" ("har" and "ari" are CGFD_EINVAL here: their device kernel is
 * withdrawn, and callers use the reference's host routine for them).
 * Writes rho, lambda, mu (host, the reference's argument order).  A point
 * outside the mesh or with vp <= sqrt(2) vs is CGFD_EINVAL. */
int cgfd_media_grid_el_iso(int NI, int NL, const int *ngz, int NX, int NY, float MINX,
                           float MINY, float DX, float DY, const float *rec, int nx, int ny,
                           int nz, const float *x3d, const float *y3d, const float *z3d,
                           const char *method, float *rho, float *lam, float *mu);

/* An elastic VTI 3-D grid model (media_type CGFD_LAYER_VTI_*) with the
 * "loc" method, as media_grid2model_el_vti does (media/media_grid2model.cpp:
 * 190-249, 556-700, 1127-1184; called at forward/main_curv_col_el_3d.c:
 * 406-415): rec [NI][NY][NX][7] = elevation and the six parameters of the
 * type, linear between levels, then para2vti.  Writes c11 c33 c55 c66 c13
 * rho (host).  "har" and "ari" are CGFD_EINVAL. */
int cgfd_media_grid_el_vti(int media_type, int NI, int NL, const int *ngz, int NX, int NY,
                           float MINX, float MINY, float DX, float DY, const float *rec, int nx,
                           int ny, int nz, const float *x3d, const float *y3d, const float *z3d,
                           const char *method, float *c11, float *c33, float *c55, float *c66,
                           float *c13, float *rho);

int cgfd_media_layer_el_iso(int NI, int NX, int NY, float MINX, float MINY, float DX,
                            float DY, const float *rec, int nx, int ny, int nz,
                            const float *x3d, const float *y3d, const float *z3d,
                            const char *method, float *lam, float *mu, float *rho);

/* Media types of cgfd_media_layer_el_vti, numbered as the reference numbers
 * them (media/media_utility.hpp:41-43). */
#define CGFD_LAYER_VTI_PREM 22     /* rho vph vpv vsh vsv eta */
#define CGFD_LAYER_VTI_THOMSEN 23  /* rho vp0 vs0 epsilon delta gamma */
#define CGFD_LAYER_VTI_CIJ 24      /* rho c11 c33 c55 c66 c13 */

/* An elastic VTI layered model discretised on a curvilinear grid, as
 * media_layer2model_el_vti does (media/media_layer2model.cpp:192-247,
 * 560-780, 1386-1438, 2197-2436; called at forward/main_curv_col_el_3d.c:
 * 336-345): as cgfd_media_layer_el_iso, with rec [NI][NY][NX][19] =
 * elevation, then value, gradient and power of the six parameters of
 * media_type in the .md3lay order; the parameters become c11 c33 c55 c66 c13
 * rho as para2vti converts them (media/media_utility.cpp:827-882).  "har"
 * averages c11 c13 c33 c55 c66 harmonically and rho arithmetically, "ari"
 * all arithmetically.  Writes the six host volumes (nx*ny*nz each). */
int cgfd_media_layer_el_vti(int media_type, int NI, int NX, int NY, float MINX, float MINY,
                            float DX, float DY, const float *rec, int nx, int ny, int nz,
                            const float *x3d, const float *y3d, const float *z3d,
                            const char *method, float *c11, float *c33, float *c55,
                            float *c66, float *c13, float *rho);


/* A model given as binary volumes of float samples on a regular 3-D mesh,
 * described as the reference's par file describes it: order[i] is the axis
 * (0 x, 1 y, 2 z) of the i-th dimension of the files, fastest first;
 * size, spacing and origin per file dimension (the z spacing may be
 * negative). */
typedef struct {
  int order[3];
  int size[3];
  float spacing[3];
  float origin[3];
} cgfd_bin_model_t;

/* rho, lambda, mu interpolated from rho, vp, vs volumes (whole files in
 * their stored order, size[0]*size[1]*size[2] floats each) on a curvilinear
 * grid, as media_bin2model_el_iso does (media/media_bin2model.cpp:27-234;
 * called at forward/main_curv_col_el_3d.c:470-484): the volumes cropped to
 * the grid's [xmin, xmax] x [ymin, ymax], then trilinear interpolation at
 * every point (TrilinearInterpolation, media/media_utility.cpp:299-391),
 * points beyond the model taking its edge.  A model that misses the grid,
 * a bad order, or a crop with fewer than two samples along an axis is
 * CGFD_EINVAL. */
int cgfd_media_bin_el_iso(const cgfd_bin_model_t *model, float xmin, float xmax, float ymin,
                          float ymax, const float *rho_vol, const float *vp_vol,
                          const float *vs_vol, int nx, int ny, int nz, const float *x3d,
                          const float *y3d, const float *z3d, float *rho, float *lam,
                          float *mu);

/* Qp, Qs interpolated from Qp, Qs volumes the same way
 * (media_bin2model_vis_iso, media/media_bin2model.cpp:236-432). */
int cgfd_media_bin_vis_iso(const cgfd_bin_model_t *model, float xmin, float xmax, float ymin,
                           float ymax, const float *qp_vol, const float *qs_vol, int nx,
                           int ny, int nz, const float *x3d, const float *y3d,
                           const float *z3d, float *qp, float *qs);

/* A box of the binary files: first sample and sample count per file
 * dimension (the files' order, fastest first). */
typedef struct {
  int first[3];
  int count[3];
} cgfd_bin_box_t;

/* The box of the files the grid needs: the x/y crop to [xmin, xmax] x
 * [ymin, ymax] and every z sample, as media_bin2model reads them
 * (media/media_bin2model.cpp:44-158, which reads only that crop of each
 * file).  Errors as cgfd_media_bin_el_iso. */
int cgfd_media_bin_crop(const cgfd_bin_model_t *model, float xmin, float xmax, float ymin,
                        float ymax, int nx, int ny, int nz, const float *z3d,
                        cgfd_bin_box_t *box);

/* cgfd_media_bin_el_iso / _vis_iso on volumes that hold only a box of the
 * files (count[0] * count[1] * count[2] floats each, file order), for
 * callers that read just the box cgfd_media_bin_crop gives: host and device
 * memory then grow with the crop, not with the files.  A box that does not
 * hold the crop is CGFD_EINVAL. */
int cgfd_media_bin_el_iso_box(const cgfd_bin_model_t *model, const cgfd_bin_box_t *box,
                              float xmin, float xmax, float ymin, float ymax,
                              const float *rho_box, const float *vp_box, const float *vs_box,
                              int nx, int ny, int nz, const float *x3d, const float *y3d,
                              const float *z3d, float *rho, float *lam, float *mu);
int cgfd_media_bin_vis_iso_box(const cgfd_bin_model_t *model, const cgfd_bin_box_t *box,
                               float xmin, float xmax, float ymin, float ymax,
                               const float *qp_box, const float *qs_box, int nx, int ny, int nz,
                               const float *x3d, const float *y3d, const float *z3d, float *qp,
                               float *qs);

/* Bytes of HBM a solver for `p` allocates (wavefield, media, metrics, aux). */
size_t cgfd_device_bytes(const cgfd_problem_t *p);

/* ------------------------------------------------------------------------
 * Batched shots.  No counterpart in the reference (it runs one shot per
 * process).  Independent problems that share the medium type (isotropic or
 * VTI elastic), dt and nt_total step together: every RK stage of every shot
 * is one kernel launch over all shots' tiles, the receivers and peak-motion
 * maps one launch each, and whole 8-step cycles of the operator schedule
 * replay from one CUDA graph.  Each shot keeps the semantics of
 * cgfd_solver_* (its results equal a single-shot run of its problem).
 * ---------------------------------------------------------------------- */
typedef struct cgfd_batch cgfd_batch_t;

/* Uploads every shot (each as cgfd_solver_create) and builds the batch;
 * kchunk = k planes per CTA (<= 0: default 16). */
int cgfd_batch_create(const cgfd_problem_t *const *shots, int nshot, int kchunk,
                      cgfd_batch_t **out);

/* Advances every shot by nsteps RK4 steps. */
int cgfd_batch_run(cgfd_batch_t *b, int nsteps);

/* Device time (CUDA events) and kernel launches of the last cgfd_batch_run. */
int cgfd_batch_times(const cgfd_batch_t *b, float *ms, int *launches);

/* cgfd_solver_fetch for every shot (results into each shot's problem). */
int cgfd_batch_fetch(cgfd_batch_t *b);

/* cgfd_solver_fetch_seismograms for every shot. */
int cgfd_batch_fetch_seismograms(cgfd_batch_t *b);

/* Every shot back at step 0 with its problem's host inputs. */
int cgfd_batch_reset(cgfd_batch_t *b);

/* k planes per CTA of the batched stage kernel. */
int cgfd_batch_set_kchunk(cgfd_batch_t *b, int kchunk);

/* Times `steps` steps for each candidate kchunk (after one warm-up step),
 * resetting the shots after each, and keeps the fastest: ms[c] receives the
 * times, *best the kchunk chosen.  The shots are at step 0 afterwards. */
int cgfd_batch_autotune(cgfd_batch_t *b, const int *cand, int ncand, int steps,
                        float *ms, int *best);

/* Schedule of the batched stage launches: 0 (default) one CTA per (shot,
 * tile, k chunk) item; 1 persistent, one CTA per SM taking the items
 * largest first (most points x planes) from a device counter, re-using its
 * shared memory and barriers from item to item.  Results are the same. */
int cgfd_batch_set_schedule(cgfd_batch_t *b, int persistent);
int cgfd_batch_schedule(const cgfd_batch_t *b);   /* -1 for a null batch */

/* cgfd_batch_autotune over both schedules: ms[s * ncand + c] the time of
 * candidate c under schedule s; the fastest (kchunk, schedule) is kept. */
int cgfd_batch_autotune_schedule(cgfd_batch_t *b, const int *cand, int ncand, int steps,
                                 float *ms, int *best_kchunk, int *best_persistent);

/* The solver of shot k (for cgfd_solver_fetch_* on one shot), or NULL. */
cgfd_solver_t *cgfd_batch_shot(cgfd_batch_t *b, int k);

void cgfd_batch_destroy(cgfd_batch_t *b);

/* ------------------------------------------------------------------------
 * Learned seismogram surrogate (no counterpart in the reference, which runs
 * the solver for every shot).  Device building blocks of a small network
 * that predicts receiver seismograms from a source position and moment
 * tensor, trained on seismograms of the batched solver; the Python layer
 * (cgfd3d_gb300/surrogate.py) composes them.  All pointers are device
 * pointers; `stream` is a cudaStream_t (null: the legacy default stream);
 * d_err is a device int that a bounded wait which ran out sets (non-zero).
 * ---------------------------------------------------------------------- */

/* output modes and activations of cgfd_sg_gemm */
#define CGFD_SG_OUT_BF16 0       /* C (and Z) bf16, stored */
#define CGFD_SG_OUT_F32 1        /* C fp32, stored */
#define CGFD_SG_OUT_F32_ADD 2    /* C fp32, added atomically (split along K) */
#define CGFD_SG_ACT_NONE 0
#define CGFD_SG_ACT_GELU 1       /* tanh-form GELU */

/* C[M, N] = alpha A[M, K] B[N, K]^T (+ bias[N]) on the tcgen05 tensor cores:
 * A, B bf16 with K contiguous (row strides lda, ldb elements, multiples of
 * 8, operands 16-byte aligned), FP32 accumulation.  mode CGFD_SG_OUT_BF16
 * stores act(C) as bf16 and, when Z is not null, the pre-activation C as
 * bf16 (same ldc); CGFD_SG_OUT_F32 stores fp32; CGFD_SG_OUT_F32_ADD adds
 * fp32 atomically and may split K over `splits` CTAs. */
int cgfd_sg_gemm(const void *A, long long lda, const void *B, long long ldb, void *C,
                 long long ldc, int M, int N, int K, float alpha, const float *bias, int act,
                 int mode, void *Z, int splits, int *d_err, void *stream);

/* The other building blocks (bf16 arrays unless stated, row-major):
 *   features      pos [B][3] fp32 -> out [B][nfeat]: the 3 coordinates, then
 *                 per coordinate d and f = 1..nfreq sin and cos of pi f x_d,
 *                 zeros up to nfeat
 *   im2col_up     X [B][Tin][C] -> A [B][Tin up][ks C]: nearest up-sampling
 *                 by `up` and the ks-tap window over time (zero outside)
 *   col2im_up_gelu  adjoint of im2col_up, times GELU'(Z): dZ [B][Tin][C]
 *                 (Z null: no GELU factor)
 *   gelu_bwd      dZ = dH GELU'(Z) for n values
 *   contract      U [B][T][R] fp32 = scale sum_k M[b][k] G[b][t][k][R] for t < T
 *                 (G [B][Tg][6][R], M [B][6] fp32)
 *   contract_loss as contract against Utrue, err[b] += sum (U - Utrue)^2 and
 *                 dG of the loss (1/B) sum_b err[b] / norm[b]
 *   transpose     Y [cols][rows] (ld ldy) = X^T (ld ldx)
 *   colsum        out[c] += sum over rows of X[r][c] (fp32 out)
 *   adamw         one AdamW step on fp32 w (and its bf16 copy w16) with
 *                 gradient g and moments m, v, bias corrections of `step`
 *   to_bf16       y = bf16(x) for n fp32 values */
int cgfd_sg_features(const float *pos, int B, int nfreq, int nfeat, void *out, void *stream);
int cgfd_sg_im2col_up(const void *X, int B, int Tin, int C, int up, int ks, void *A,
                      void *stream);
int cgfd_sg_col2im_up_gelu(const void *dA, int B, int Tin, int C, int up, int ks,
                           const void *Z, void *dZ, void *stream);
int cgfd_sg_gelu_bwd(const void *dH, const void *Z, long long n, void *dZ, void *stream);
int cgfd_sg_contract(const void *G, const float *M, int B, int Tg, int T, int R, float scale,
                     float *U, void *stream);
int cgfd_sg_contract_loss(const void *G, const float *M, int B, int Tg, int T, int R,
                          float scale, const float *Utrue, const float *norm, float *err,
                          void *dG, void *stream);
int cgfd_sg_transpose(const void *X, int rows, int cols, long long ldx, void *Y,
                      long long ldy, void *stream);
int cgfd_sg_colsum(const void *X, long long rows, int cols, long long ld, float *out,
                   void *stream);
int cgfd_sg_adamw(float *w, void *w16, const float *g, float *m, float *v, long long n,
                  float lr, float b1, float b2, float eps, float wd, int step, void *stream);
int cgfd_sg_to_bf16(const float *x, long long n, void *y, void *stream);

/* A trained surrogate as one object, for callers without Python: shots
 * given as arrays of per-shot descriptors on the host (normalised source
 * position pos [n][3] in [-1, 1], moment tensor mt [n][6] in the network's
 * units, order Mxx Myy Mzz Myz Mxz Mxy as the training data), seismograms
 * u [n][nt][3 nrec] fp32 back on the host.  params: the flat fp32
 * parameter vector of cgfd3d_gb300/surrogate.py (per layer W (out x in),
 * then its bias; cgfd_sg_net_nparam values), scale: the seismograms'
 * amplitude in the network's units; nrec a multiple of 4.  Requests run in chunks of
 * CGFD_SG_NET_CHUNK shots, each chunk bit-identical to the Python layer's
 * prediction of the same shots as one batch.  An object holds its own
 * stream and work buffers (about 1.6 GB for 64 receivers): one call at a
 * time per object; predict returns when u is written. */
#define CGFD_SG_NET_CHUNK 256
typedef struct cgfd_sg_net cgfd_sg_net_t;
long long cgfd_sg_net_nparam(int nrec, int nt);   /* -1: no such layout */
int cgfd_sg_net_create(int nrec, int nt, const float *params, long long nparam, float scale,
                       cgfd_sg_net_t **out);
int cgfd_sg_net_predict(cgfd_sg_net_t *net, int nshot, const float *pos, const float *mt,
                        float *u);
void cgfd_sg_net_destroy(cgfd_sg_net_t *net);

/* No counterpart in the reference.  NaN/Inf test of a device array the
 * caller owns that allocates no device memory, for callers that cannot call
 * cudaMalloc (a process whose device memory belongs to another framework's
 * pool or sits under a hard cap, or a check issued between the launches of
 * a time loop where an allocation would synchronise the device).  Same test
 * as cgfd_solver_check_finite(); *nonfinite = 1 when any of the n floats at
 * d_data is NaN or Inf, else 0.  Scratch: a file-scope __device__ array of
 * CGFD_NOALLOC_MAX_BLOCKS + 1 ints that every GPU loading this library keeps
 * until exit; n above CGFD_NOALLOC_MAX_FLOATS is rejected (CGFD_EINVAL).
 * The first call in a device's context looks the scratch address up (again
 * after a cudaDeviceReset or when another context of the device is current)
 * and should come before any stream capture; calls that overlap on the GPU
 * race on the shared scratch.  Runs on the legacy default stream and
 * returns after the result is on the host.  The legacy default stream is
 * not ordered against the solver's own non-blocking stream: a caller that
 * checks arrays a solver is still writing (cgfd_solver_run_async) must wait
 * for that solver's work first (cgfd_solver_fetch_* or a device
 * synchronisation). */
#define CGFD_NOALLOC_MAX_BLOCKS 65536
#define CGFD_NOALLOC_MAX_FLOATS (65536ull * 256ull * 64ull)
int cgfd_check_finite_noalloc(const float *d_data, size_t n, int *nonfinite);

#ifdef __cplusplus
}
#endif
#endif
