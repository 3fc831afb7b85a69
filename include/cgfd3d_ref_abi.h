/*
 * cgfd3d_ref_abi.h -- the CGFD3D struct layouts the drop-in entry point reads.
 *
 * drv_rk_curv_col_allstep() receives the reference's own structs by pointer
 * (forward/drv_rk_curv_col.h:17-37).  These declarations restate their
 * layouts field for field, so that the drop-in adapter
 * (cgfd3d_gb300/csrc/dropin/drv_rk_curv_col_gpu.c) can be compiled and
 * tested without the reference tree.  When the adapter is built inside the
 * reference tree (CGFD_DROPIN_REFERENCE_HEADERS defined) the reference's
 * own headers are used instead; tests/test_ref_abi.py checks, wherever the
 * reference tree is present, that every offset below equals the reference's.
 *
 * Sources of each layout:
 *   fd_op_t, fd_t         forward/fd_t.h:55-175
 *   gd_t, gdcurv_metric_t forward/gd_t.h:27-174
 *   md_t                  forward/md_t.h:11-73
 *   src_t                 forward/src_t.h:21-128
 *   bdrypml_auxvar_t, bdry_block_t, bdry_t   forward/bdry_t.h:20-151
 *   wav_t                 forward/wav_t.h:15-67
 *   iorecv_one_t, iorecv_t, ioline_t, ioslice_t, iosnap_t
 *                         forward/io_funcs.h:17-110
 *   mympi_t               forward/mympi_t.h:13-55 (leading fields only: the
 *                         rest depends on the MPI implementation's handle
 *                         types and is never read here)
 */
#ifndef CGFD3D_REF_ABI_H
#define CGFD3D_REF_ABI_H

#include <stddef.h>
#include <stdio.h>

#define CGFD_REF_NDIM 3
#define CGFD_REF_NDIM_2 6
#define CGFD_REF_2_NDIM 8
#define CGFD_REF_MAX_STRLEN 1024
#define CGFD_REF_GD_TILE 4
#define CGFD_REF_VISCO_GMB 2 /* CONST_VISCO_GMB, forward/constants.h:30 */
#define CGFD_REF_VISCO_GRAVES_QS 1 /* CONST_VISCO_GRAVES_QS, forward/constants.h:29 */

typedef struct {
  int total_len;
  int half_len;
  int left_len;
  int right_len;
  int *indx;
  int *shift;
  float *coef;
} fd_op_t;

typedef struct {
  float CFL;
  int num_rk_stages;
  float *rk_a;
  float *rk_b;
  float *rk_rhs_time;
  int fdc_len;
  int fdc_half_len;
  int fdc_nghosts;
  int *fdc_indx;
  float *fdc_coef;
  int fdx_nghosts, fdy_nghosts, fdz_nghosts;
  int fdx_max_len, fdy_max_len, fdz_max_len;
  int fdx_max_half_len, fdy_max_half_len, fdz_max_half_len;
  int num_of_pairs;
  int num_of_fdx_op, num_of_fdy_op, num_of_fdz_op;
  fd_op_t ***pair_fdx_op;
  fd_op_t ***pair_fdy_op;
  fd_op_t ***pair_fdz_op;
} fd_t;

typedef struct {
  int type; /* gd_type_t */
  int ni, nj, nk, nx, ny, nz;
  int ni1, ni2, nj1, nj2, nk1, nk2;
  int npoint_ghosts;
  int fdx_nghosts, fdy_nghosts, fdz_nghosts;
  int gni1, gnj1, gnk1;
  int gni2, gnj2, gnk2;
  int ni1_to_glob_phys0, nj1_to_glob_phys0, nk1_to_glob_phys0;
  int ni2_to_glob_phys0, nj2_to_glob_phys0, nk2_to_glob_phys0;
  int n1, n2, n3, n4;
  int ncmp;
  float *v4d;
  float *x3d, *y3d, *z3d;
  float *x1d, *y1d, *z1d;
  float dx, dy, dz;
  float x0_glob, y0_glob, z0_glob;
  float xmin, xmax, ymin, ymax, zmin, zmax;
  float xmin_phy, xmax_phy, ymin_phy, ymax_phy, zmin_phy, zmax_phy;
  float *cell_xmin, *cell_xmax, *cell_ymin, *cell_ymax, *cell_zmin, *cell_zmax;
  int tile_istart[CGFD_REF_GD_TILE];
  int tile_iend[CGFD_REF_GD_TILE];
  int tile_jstart[CGFD_REF_GD_TILE];
  int tile_jend[CGFD_REF_GD_TILE];
  int tile_kstart[CGFD_REF_GD_TILE];
  int tile_kend[CGFD_REF_GD_TILE];
  float tile_xmin[CGFD_REF_GD_TILE][CGFD_REF_GD_TILE][CGFD_REF_GD_TILE];
  float tile_xmax[CGFD_REF_GD_TILE][CGFD_REF_GD_TILE][CGFD_REF_GD_TILE];
  float tile_ymin[CGFD_REF_GD_TILE][CGFD_REF_GD_TILE][CGFD_REF_GD_TILE];
  float tile_ymax[CGFD_REF_GD_TILE][CGFD_REF_GD_TILE][CGFD_REF_GD_TILE];
  float tile_zmin[CGFD_REF_GD_TILE][CGFD_REF_GD_TILE][CGFD_REF_GD_TILE];
  float tile_zmax[CGFD_REF_GD_TILE][CGFD_REF_GD_TILE][CGFD_REF_GD_TILE];
  size_t siz_iy, siz_iz, siz_icmp;
  size_t siz_line, siz_slice, siz_volume;
  size_t *cmp_pos;
  char **cmp_name;
  char **index_name;
} gd_t;

typedef struct {
  int n1, n2, n3, n4;
  int nx, ny, nz, ncmp;
  float *v4d;
  float *jac;
  float *xi_x, *xi_y, *xi_z;
  float *eta_x, *eta_y, *eta_z;
  float *zeta_x, *zeta_y, *zeta_z;
  size_t siz_iy, siz_iz, siz_icmp;
  size_t *cmp_pos;
  char **cmp_name;
} gdcurv_metric_t;

typedef struct {
  int n1, n2, n3, n4;
  int nx, ny, nz, ncmp;
  float *v4d;
  size_t siz_iy, siz_iz, siz_icmp;
  size_t *cmp_pos;
  char **cmp_name;
  int medium_type;
  float *rho;
  float *kappa;
  float *lambda;
  float *mu;
  int nmaxwell;
  float visco_GMB_freq;
  float visco_GMB_fmin;
  float visco_GMB_fmax;
  float *Qs;
  float *Qp;
  float **Ylam;
  float **Ymu;
  float *wl;
  float *c11, *c12, *c13, *c14, *c15, *c16;
  float *c22, *c23, *c24, *c25, *c26;
  float *c33, *c34, *c35, *c36;
  float *c44, *c45, *c46;
  float *c55, *c56;
  float *c66;
  int visco_type;
  float visco_Qs_freq;
} md_t;

typedef struct {
  int total_number;
  int max_nt;
  int max_stage;
  int it;
  int istage;
  char evtnm[CGFD_REF_MAX_STRLEN];
  int *si, *sj, *sk;
  float *si_inc, *sj_inc, *sk_inc;
  int *it_begin, *it_end;
  int is_surface_force_strict;
  int total_number_surface_force;
  int idx_next_surface_force;
  int itype_spatial_ext;
  int ext_half_npoint;
  int ext_length_npoint;
  int ext_size_npoint;
  float ext_func_coef;
  int force_actived;
  int moment_actived;
  float *Fx, *Fy, *Fz;
  float *Mxx, *Myy, *Mzz, *Mxz, *Myz, *Mxy;
  int *force_rate_indx;
  float *Fx_rate, *Fy_rate, *Fz_rate;
  float *TxSrc, *TySrc, *TzSrc;
  float *VxSrc, *VySrc, *VzSrc;
  int dd_is_valid;
  int dd_is_add_at_point;
  int dd_smo_hlen;
  int dd_vi_actived;
  int dd_mij_actived;
  int dd_total_number;
  int dd_max_nt;
  int dd_nt_per_read;
  int dd_nt_this_read;
  int dd_it_here;
  int *dd_si, *dd_sj, *dd_sk;
  size_t *dd_indx;
  float *dd_si_inc, *dd_sj_inc, *dd_sk_inc;
  FILE *fp_vi;
  FILE *fp_mij;
  float *dd_vi;
  float *dd_mij;
} src_t;

typedef struct {
  float *var;
  int nx, ny, nz, ncmp, nlevel;
  size_t siz_iy, siz_iz, siz_icmp, siz_ilevel;
  size_t *cmp_pos;
  char **cmp_name;
  size_t *level_pos;
  size_t Vx_pos, Vy_pos, Vz_pos, Txx_pos, Tyy_pos, Tzz_pos, Tyz_pos, Txz_pos, Txy_pos;
  float *cur, *pre, *rhs, *end, *tmp;
} bdrypml_auxvar_t;

typedef struct {
  int enable;
  int nx1, nx2, ny1, ny2, nz1, nz2, nx, ny, nz;
  int ni1, ni2, nj1, nj2, nk1, nk2, ni, nj, nk;
} bdry_block_t;

typedef struct {
  int is_sides_pml[CGFD_REF_NDIM][2];
  int is_sides_free[CGFD_REF_NDIM][2];
  int is_sides_mpml[CGFD_REF_NDIM][2];
  int is_sides_ablexp[CGFD_REF_NDIM][2];
  int is_enable_pml;
  int is_enable_free;
  int is_enable_mpml;
  int is_enable_ablexp;
  int nx, ny, nz;
  int num_of_layers[CGFD_REF_NDIM][2];
  int ni1[CGFD_REF_NDIM][2];
  int ni2[CGFD_REF_NDIM][2];
  int nj1[CGFD_REF_NDIM][2];
  int nj2[CGFD_REF_NDIM][2];
  int nk1[CGFD_REF_NDIM][2];
  int nk2[CGFD_REF_NDIM][2];
  float *A[CGFD_REF_NDIM][2];
  float *B[CGFD_REF_NDIM][2];
  float *D[CGFD_REF_NDIM][2];
  float *Am[CGFD_REF_NDIM][2];
  float *Bm[CGFD_REF_NDIM][2];
  float *Dm[CGFD_REF_NDIM][2];
  bdrypml_auxvar_t auxvar[CGFD_REF_NDIM][2];
  bdry_block_t bdry_blk[CGFD_REF_NDIM_2];
  float *ablexp_Ex, *ablexp_Ey, *ablexp_Ez;
  float *matVx2Vz2, *matVy2Vz2, *matD, *matF2Vz2;
  float *matVx2Vz1, *matVy2Vz1;
  float *matVy2Vx1, *matVz2Vx1;
  float *matVy2Vx2, *matVz2Vx2;
  float *matVx2Vy1, *matVz2Vy1;
  float *matVx2Vy2, *matVz2Vy2;
} bdry_t;

typedef struct {
  float *v5d;
  int n1, n2, n3, n4, n5;
  int nx, ny, nz, ncmp, nlevel, nmaxwell;
  int visco_type;
  size_t siz_iy, siz_iz, siz_icmp, siz_ilevel;
  size_t *cmp_pos;
  char **cmp_name;
  size_t *level_pos;
  size_t Vx_pos, Vy_pos, Vz_pos, Txx_pos, Tyy_pos, Tzz_pos, Tyz_pos, Txz_pos, Txy_pos;
  size_t Vx_seq, Vy_seq, Vz_seq, Txx_seq, Tyy_seq, Tzz_seq, Tyz_seq, Txz_seq, Txy_seq;
  size_t *Jxx_pos, *Jyy_pos, *Jzz_pos, *Jxy_pos, *Jxz_pos, *Jyz_pos;
  size_t *Jxx_seq, *Jyy_seq, *Jzz_seq, *Jxy_seq, *Jxz_seq, *Jyz_seq;
} wav_t;

typedef struct {
  float x, y, z;
  float di, dj, dk;
  int i, j, k;
  int indx1d[CGFD_REF_2_NDIM];
  float *seismo;
  char name[CGFD_REF_MAX_STRLEN];
} iorecv_one_t;

typedef struct {
  int total_number;
  int max_nt;
  int ncmp;
  iorecv_one_t *recvone;
} iorecv_t;

typedef struct {
  int num_of_lines;
  int max_nt;
  int ncmp;
  int *line_nr;
  int *line_seq;
  int **recv_seq;
  int **recv_iptr;
  float **recv_x;
  float **recv_y;
  float **recv_z;
  float **recv_seismo;
  char **line_name;
} ioline_t;

typedef struct {
  size_t siz_max_wrk;
  int num_of_slice_x;
  int *slice_x_indx;
  char **slice_x_fname;
  int num_of_slice_y;
  int *slice_y_indx;
  char **slice_y_fname;
  int num_of_slice_z;
  int *slice_z_indx;
  char **slice_z_fname;
} ioslice_t;

typedef struct {
  size_t siz_max_wrk;
  int num_of_snap;
  int *i1, *j1, *k1, *ni, *nj, *nk, *di, *dj, *dk;
  int *it1, *dit;
  int *out_vel, *out_stress, *out_strain;
  int *i1_to_glob, *j1_to_glob, *k1_to_glob;
  char **fname;
} iosnap_t;

typedef struct {
  int nprocx;
  int nprocy;
  int myid;
} mympi_t;

#endif
