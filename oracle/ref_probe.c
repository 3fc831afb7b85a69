/*
 * ref_probe.c -- calls single functions of the reference build on inputs
 * given in a file, to make golden vectors for the parts of the path that sit
 * beside the time loop.  TEST INFRASTRUCTURE ONLY: linked with the
 * reference's own objects (oracle/Makefile, target _ref/ref_probe); nothing
 * of the product links or runs it.
 *
 *   ref_probe sac <input> <out_dir>
 *       station and line seismograms written by the reference's SAC output:
 *       io_recv_output_sac, io_recv_output_sac_el_iso_strain and
 *       io_line_output_sac (forward/io_funcs.c:1648-1868, lib/sacLib.c).
 *       <input>, native little-endian:
 *         int nr, ncmp, nt, nl; float dt; char evtnm[16];
 *         nr x { char name[16]; float x, y, z, lambda, mu; }
 *         float seismo[nr][ncmp][nt];
 *         char line_name[16];
 *         nl x { int seq; float x, y, z; }
 *         float line_seismo[nl][ncmp][nt];
 *
 *   ref_probe locate <input> <output>
 *       points of a curvilinear grid located as the reference locates
 *       stations and sources given by coordinates: gd_curv_set_minmax, then
 *       per point gd_curv_depth_to_axis when the point's z is a depth and
 *       gd_curv_coord_to_glob_indx (forward/gd_t.c:1708-2171, 2179-2297).
 *       <input>:  int nx, ny, nz, n; float x3d, y3d, z3d [nz][ny][nx];
 *                 n x { float x, y, z; int is_depth; }
 *       <output>: n x { int is_here, si, sj, sk; float sx_inc, sy_inc,
 *                       sz_inc, z; }   (z after the depth conversion)
 *
 *   ref_probe layer <md3lay> <grid> <method> <output>
 *       an elastic isotropic layered model discretised on a curvilinear
 *       grid by media_layer2model_el_iso (media/media_layer2model.cpp:
 *       140-190) with the equivalent-medium method <method> (loc, har, ari).
 *       <grid>:   int nx, ny, nz; float x3d, y3d, z3d [nz][ny][nx]
 *       <output>: float lambda, mu, rho [nz][ny][nx]
 *
 *   ref_probe layer_vti <md3lay> <grid> <method> <output>
 *       an elastic VTI layered model (elastic_vti_prem, _thomsen or _cij)
 *       discretised by media_layer2model_el_vti (media/media_layer2model.cpp:
 *       192-247); <output>: float c11, c33, c55, c66, c13, rho [nz][ny][nx]
 *
 *   ref_probe layer_one <md3lay> <grid> <method> <output>
 *       a one-component layered model (Qp, Qs, ...) discretised by
 *       media_layer2model_onecmp (media/media_layer2model.cpp:47-88);
 *       <output>: float var [nz][ny][nx]
 *
 *   ref_probe grid <md3grd> <grid> <method> <ext> <output>
 *       an elastic isotropic 3-D grid model discretised by
 *       media_grid2model_el_iso (media/media_grid2model.cpp:133-189) with the
 *       grid's extent <ext> (float xmin, xmax, ymin, ymax);
 *       <output>: float rho, lambda, mu [nz][ny][nx]
 *
 *   ref_probe grid_vti <md3grd> <grid> <method> <ext> <output>
 *       an elastic VTI 3-D grid model by media_grid2model_el_vti
 *       (media/media_grid2model.cpp:190-249); <output>: float c11, c33, c55,
 *       c66, c13, rho [nz][ny][nx]
 *
 *   ref_probe layer_aniso <md3lay> <grid> <method> <output>
 *       a layered model through media_layer2model_el_aniso
 *       (media/media_layer2model.cpp:249-420); <output>: float rho, c11,
 *       c12, ..., c66 (the 21 in the reference's argument order) [nz][ny][nx]
 *
 *   ref_probe grid_aniso <md3grd> <grid> <method> <ext> <output>
 *       a 3-D grid model through media_grid2model_el_aniso
 *       (media/media_grid2model.cpp:250-420); <output>: the 22 volumes as
 *       layer_aniso
 *
 *   ref_probe bin <grid> <params> <rho> <vp> <vs> <output>
 *   ref_probe bin_vis <grid> <params> <Qp> <Qs> <output>
 *       a model given as binary volumes interpolated on a curvilinear grid
 *       by media_bin2model_el_iso / media_bin2model_vis_iso
 *       (media/media_bin2model.cpp:27-432).  <params>: int bin_order[3],
 *       bin_size[3]; float bin_spacing[3], bin_origin[3], xmin, xmax, ymin,
 *       ymax.  <output>: float rho, lambda, mu (bin) or Qp, Qs (bin_vis)
 *       [nz][ny][nx]
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "io_funcs.h"

/* the reference's layered-model discretisation (C linkage,
 * media/media_layer2model.hpp:63-76); grid type 3 is GRID_CURV
 * (media/media_utility.hpp:50) */
int media_layer2model_el_iso(float *lam3d, float *mu3d, float *rho3d,
                             const float *x3d, const float *y3d, const float *z3d,
                             size_t nx, size_t ny, size_t nz, int grid_type,
                             const char *in_3lay_file,
                             const char *equivalent_medium_method, int myid);
int media_layer2model_el_vti(float *rho, float *c11, float *c33, float *c55, float *c66,
                             float *c13, const float *x3d, const float *y3d,
                             const float *z3d, size_t nx, size_t ny, size_t nz,
                             int grid_type, const char *in_3lay_file,
                             const char *equivalent_medium_method, int myid);
int media_layer2model_onecmp(float *var3d, const float *x3d, const float *y3d,
                             const float *z3d, size_t nx, size_t ny, size_t nz, int grid_type,
                             const char *in_var_file, const char *average_method, int myid);
int media_bin2model_el_iso(float *rho3d, float *lam3d, float *mu3d, const float *x3d,
                           const float *y3d, const float *z3d, size_t nx, size_t ny, size_t nz,
                           float xmin, float xmax, float ymin, float ymax, int grid_type,
                           int *bin_order, int *bin_size, float *bin_spacing,
                           float *bin_origin, const char *bin_file_rho, const char *bin_file_vp,
                           const char *bin_file_vs);
int media_bin2model_vis_iso(float *Qp3d, float *Qs3d, const float *x3d, const float *y3d,
                            const float *z3d, size_t nx, size_t ny, size_t nz, float xmin,
                            float xmax, float ymin, float ymax, int grid_type, int *bin_order,
                            int *bin_size, float *bin_spacing, float *bin_origin,
                            const char *bin_file_Qp, const char *bin_file_Qs);
int media_grid2model_el_iso(float *rho3d, float *lam3d, float *mu3d, const float *x3d,
                            const float *y3d, const float *z3d, int nx, int ny, int nz,
                            float Xmin, float Xmax, float Ymin, float Ymax, int grid_type,
                            const char *in_media_file, const char *equivalent_medium_method,
                            int myid);
int media_grid2model_el_vti(float *rho, float *c11, float *c33, float *c55, float *c66,
                            float *c13, const float *x3d, const float *y3d, const float *z3d,
                            int nx, int ny, int nz, float Xmin, float Xmax, float Ymin,
                            float Ymax, int grid_type, const char *in_media_file,
                            const char *equivalent_medium_method, int myid);
int media_layer2model_el_aniso(float *rho, float *c11, float *c12, float *c13, float *c14,
                               float *c15, float *c16, float *c22, float *c23, float *c24,
                               float *c25, float *c26, float *c33, float *c34, float *c35,
                               float *c36, float *c44, float *c45, float *c46, float *c55,
                               float *c56, float *c66, const float *x3d, const float *y3d,
                               const float *z3d, size_t nx, size_t ny, size_t nz, int grid_type,
                               const char *in_3lay_file, const char *equivalent_medium_method,
                               int myid);
int media_grid2model_el_aniso(float *rho, float *c11, float *c12, float *c13, float *c14,
                              float *c15, float *c16, float *c22, float *c23, float *c24,
                              float *c25, float *c26, float *c33, float *c34, float *c35,
                              float *c36, float *c44, float *c45, float *c46, float *c55,
                              float *c56, float *c66, const float *x3d, const float *y3d,
                              const float *z3d, int nx, int ny, int nz, float Xmin, float Xmax,
                              float Ymin, float Ymax, int grid_type, const char *in_media_file,
                              const char *equivalent_medium_method, int myid);
#define PROBE_GRID_CURV 3

static void rd(void *p, size_t n, FILE *fp)
{
  if (fread(p, 1, n, fp) != n) {
    fprintf(stderr, "ref_probe: short input\n");
    exit(2);
  }
}

static int probe_sac(const char *in, char *out_dir)
{
  FILE *fp = fopen(in, "rb");
  if (!fp) return 2;
  int hdr[4];
  float dt;
  char evtnm[17] = {0};
  rd(hdr, sizeof hdr, fp);
  rd(&dt, sizeof dt, fp);
  rd(evtnm, 16, fp);
  const int nr = hdr[0], ncmp = hdr[1], nt = hdr[2], nl = hdr[3];

  static const char *names9[9] = {"Vx", "Vy", "Vz", "Txx", "Tyy", "Tzz",
                                  "Tyz", "Txz", "Txy"};
  char **cmp_name = malloc(ncmp * sizeof(char *));
  for (int c = 0; c < ncmp; c++) {
    cmp_name[c] = calloc(CONST_MAX_STRLEN, 1);
    snprintf(cmp_name[c], CONST_MAX_STRLEN, "%s", c < 9 ? names9[c] : "J");
  }

  iorecv_t rec = {0};
  rec.total_number = nr;
  rec.max_nt = nt;
  rec.ncmp = ncmp;
  rec.recvone = calloc(nr, sizeof(iorecv_one_t));
  float *lam = malloc(nr * sizeof(float)), *mu = malloc(nr * sizeof(float));
  for (int r = 0; r < nr; r++) {
    iorecv_one_t *o = rec.recvone + r;
    char name[17] = {0};
    float v[5];
    rd(name, 16, fp);
    rd(v, sizeof v, fp);
    snprintf(o->name, CONST_MAX_STRLEN, "%s", name);
    o->x = v[0]; o->y = v[1]; o->z = v[2];
    lam[r] = v[3]; mu[r] = v[4];
    o->indx1d[0] = r;          /* media are indexed by the receiver here */
  }
  for (int r = 0; r < nr; r++) {
    rec.recvone[r].seismo = malloc((size_t)ncmp * nt * sizeof(float));
    rd(rec.recvone[r].seismo, (size_t)ncmp * nt * sizeof(float), fp);
  }

  ioline_t line = {0};
  char lname[17] = {0};
  rd(lname, 16, fp);
  line.num_of_lines = nl > 0;
  line.max_nt = nt;
  line.ncmp = ncmp;
  int line_nr = nl, *seq = malloc((nl + 1) * sizeof(int));
  float *lx = malloc((nl + 1) * sizeof(float)), *ly = malloc((nl + 1) * sizeof(float));
  float *lz = malloc((nl + 1) * sizeof(float));
  float *lseis = malloc(((size_t)nl * ncmp * nt + 1) * sizeof(float));
  char *lnames[1] = {lname};
  for (int r = 0; r < nl; r++) {
    float v[3];
    rd(&seq[r], sizeof(int), fp);
    rd(v, sizeof v, fp);
    lx[r] = v[0]; ly[r] = v[1]; lz[r] = v[2];
  }
  rd(lseis, (size_t)nl * ncmp * nt * sizeof(float), fp);
  fclose(fp);
  line.line_nr = &line_nr;
  line.recv_seq = &seq;
  line.recv_x = &lx;
  line.recv_y = &ly;
  line.recv_z = &lz;
  line.recv_seismo = &lseis;
  line.line_name = lnames;
  int *iptr = calloc(nl + 1, sizeof(int));
  line.recv_iptr = &iptr;

  char err[CONST_MAX_STRLEN];
  io_recv_output_sac(&rec, dt, ncmp, 0, cmp_name, evtnm, out_dir, err);
  io_recv_output_sac_el_iso_strain(&rec, lam, mu, dt, evtnm, out_dir, err);
  if (nl > 0) io_line_output_sac(&line, dt, cmp_name, evtnm, out_dir);
  return 0;
}

static int probe_locate(const char *in, const char *out)
{
  FILE *fp = fopen(in, "rb");
  if (!fp) return 2;
  int hdr[4];
  rd(hdr, sizeof hdr, fp);
  gd_t gd;
  memset(&gd, 0, sizeof gd);
  gd.type = GD_TYPE_CURV;
  gd.nx = hdr[0]; gd.ny = hdr[1]; gd.nz = hdr[2];
  const int n = hdr[3];
  gd.npoint_ghosts = 3;
  gd.ni = gd.nx - 6; gd.nj = gd.ny - 6; gd.nk = gd.nz - 6;
  gd.ni1 = 3; gd.ni2 = gd.ni1 + gd.ni - 1;
  gd.nj1 = 3; gd.nj2 = gd.nj1 + gd.nj - 1;
  gd.nk1 = 3; gd.nk2 = gd.nk1 + gd.nk - 1;
  gd.ni1_to_glob_phys0 = 0; gd.ni2_to_glob_phys0 = gd.ni - 1;
  gd.nj1_to_glob_phys0 = 0; gd.nj2_to_glob_phys0 = gd.nj - 1;
  gd.nk1_to_glob_phys0 = 0; gd.nk2_to_glob_phys0 = gd.nk - 1;
  gd.gni1 = 0; gd.gnj1 = 0; gd.gnk1 = 0;
  gd.gni2 = gd.ni - 1; gd.gnj2 = gd.nj - 1; gd.gnk2 = gd.nk - 1;
  gd.siz_iy = gd.siz_line = gd.nx;
  gd.siz_iz = gd.siz_slice = (size_t)gd.nx * gd.ny;
  gd.siz_icmp = gd.siz_volume = gd.siz_slice * gd.nz;
  size_t vol = gd.siz_icmp;
  gd.x3d = malloc(vol * sizeof(float));
  gd.y3d = malloc(vol * sizeof(float));
  gd.z3d = malloc(vol * sizeof(float));
  rd(gd.x3d, vol * sizeof(float), fp);
  rd(gd.y3d, vol * sizeof(float), fp);
  rd(gd.z3d, vol * sizeof(float), fp);
  float **cells[6] = {&gd.cell_xmin, &gd.cell_xmax, &gd.cell_ymin, &gd.cell_ymax,
                      &gd.cell_zmin, &gd.cell_zmax};
  for (int c = 0; c < 6; c++) *cells[c] = calloc(vol, sizeof(float));
  gd_curv_set_minmax(&gd);

  FILE *fo = fopen(out, "wb");
  if (!fo) return 2;
  for (int q = 0; q < n; q++) {
    float v[3];
    int is_depth;
    rd(v, sizeof v, fp);
    rd(&is_depth, sizeof is_depth, fp);
    float sz = v[2];
    if (is_depth) gd_curv_depth_to_axis(&gd, v[0], v[1], &sz, MPI_COMM_WORLD, 0);
    int idx[4];
    float inc[4];
    idx[0] = gd_curv_coord_to_glob_indx(&gd, v[0], v[1], sz, MPI_COMM_WORLD, 0,
                                        &idx[1], &idx[2], &idx[3], &inc[0], &inc[1],
                                        &inc[2]);
    inc[3] = sz;
    fwrite(idx, sizeof idx, 1, fo);
    fwrite(inc, sizeof inc, 1, fo);
  }
  fclose(fo);
  fclose(fp);
  return 0;
}

static int probe_layer(const char *lay, const char *grid, const char *method,
                       const char *out)
{
  FILE *fp = fopen(grid, "rb");
  if (!fp) return 2;
  int d[3];
  rd(d, sizeof d, fp);
  size_t vol = (size_t)d[0] * d[1] * d[2];
  float *x = malloc(vol * 4), *y = malloc(vol * 4), *z = malloc(vol * 4);
  rd(x, vol * 4, fp);
  rd(y, vol * 4, fp);
  rd(z, vol * 4, fp);
  fclose(fp);
  float *lam = calloc(vol, 4), *mu = calloc(vol, 4), *rho = calloc(vol, 4);
  media_layer2model_el_iso(lam, mu, rho, x, y, z, d[0], d[1], d[2], PROBE_GRID_CURV, lay,
                           method, 0);
  FILE *fo = fopen(out, "wb");
  if (!fo) return 2;
  fwrite(lam, 4, vol, fo);
  fwrite(mu, 4, vol, fo);
  fwrite(rho, 4, vol, fo);
  fclose(fo);
  return 0;
}

static int probe_layer_vti(const char *lay, const char *grid, const char *method,
                           const char *out)
{
  FILE *fp = fopen(grid, "rb");
  if (!fp) return 2;
  int d[3];
  rd(d, sizeof d, fp);
  size_t vol = (size_t)d[0] * d[1] * d[2];
  float *x = malloc(vol * 4), *y = malloc(vol * 4), *z = malloc(vol * 4);
  rd(x, vol * 4, fp);
  rd(y, vol * 4, fp);
  rd(z, vol * 4, fp);
  fclose(fp);
  float *c[6];   /* c11 c33 c55 c66 c13 rho */
  for (int n = 0; n < 6; n++) c[n] = calloc(vol, 4);
  media_layer2model_el_vti(c[5], c[0], c[1], c[2], c[3], c[4], x, y, z, d[0], d[1], d[2],
                           PROBE_GRID_CURV, lay, method, 0);
  FILE *fo = fopen(out, "wb");
  if (!fo) return 2;
  for (int n = 0; n < 6; n++) fwrite(c[n], 4, vol, fo);
  fclose(fo);
  return 0;
}

static int probe_layer_one(const char *lay, const char *grid, const char *method,
                           const char *out)
{
  FILE *fp = fopen(grid, "rb");
  if (!fp) return 2;
  int d[3];
  rd(d, sizeof d, fp);
  size_t vol = (size_t)d[0] * d[1] * d[2];
  float *x = malloc(vol * 4), *y = malloc(vol * 4), *z = malloc(vol * 4);
  rd(x, vol * 4, fp);
  rd(y, vol * 4, fp);
  rd(z, vol * 4, fp);
  fclose(fp);
  float *v = calloc(vol, 4);
  media_layer2model_onecmp(v, x, y, z, d[0], d[1], d[2], PROBE_GRID_CURV, lay, method, 0);
  FILE *fo = fopen(out, "wb");
  if (!fo) return 2;
  fwrite(v, 4, vol, fo);
  fclose(fo);
  return 0;
}

static int probe_bin(int vis, const char *grid, const char *params, const char *const *files,
                     const char *out)
{
  FILE *fp = fopen(grid, "rb");
  if (!fp) return 2;
  int d[3];
  rd(d, sizeof d, fp);
  size_t vol = (size_t)d[0] * d[1] * d[2];
  float *x = malloc(vol * 4), *y = malloc(vol * 4), *z = malloc(vol * 4);
  rd(x, vol * 4, fp);
  rd(y, vol * 4, fp);
  rd(z, vol * 4, fp);
  fclose(fp);
  fp = fopen(params, "rb");
  if (!fp) return 2;
  int order[3], size[3];
  float spacing[3], origin[3], ext[4];
  rd(order, sizeof order, fp);
  rd(size, sizeof size, fp);
  rd(spacing, sizeof spacing, fp);
  rd(origin, sizeof origin, fp);
  rd(ext, sizeof ext, fp);
  fclose(fp);
  const int nout = vis ? 2 : 3;
  float *o[3];
  for (int n = 0; n < nout; n++) o[n] = calloc(vol, 4);
  if (vis)
    media_bin2model_vis_iso(o[0], o[1], x, y, z, d[0], d[1], d[2], ext[0], ext[1], ext[2],
                            ext[3], PROBE_GRID_CURV, order, size, spacing, origin, files[0],
                            files[1]);
  else
    media_bin2model_el_iso(o[0], o[1], o[2], x, y, z, d[0], d[1], d[2], ext[0], ext[1], ext[2],
                           ext[3], PROBE_GRID_CURV, order, size, spacing, origin, files[0],
                           files[1], files[2]);
  FILE *fo = fopen(out, "wb");
  if (!fo) return 2;
  for (int n = 0; n < nout; n++) fwrite(o[n], 4, vol, fo);
  fclose(fo);
  return 0;
}

static int probe_grid(int vti, const char *grd, const char *grid, const char *method,
                      const char *extf, const char *out)
{
  FILE *fp = fopen(grid, "rb");
  if (!fp) return 2;
  int d[3];
  rd(d, sizeof d, fp);
  size_t vol = (size_t)d[0] * d[1] * d[2];
  float *x = malloc(vol * 4), *y = malloc(vol * 4), *z = malloc(vol * 4);
  rd(x, vol * 4, fp);
  rd(y, vol * 4, fp);
  rd(z, vol * 4, fp);
  fclose(fp);
  float ext[4];
  fp = fopen(extf, "rb");
  if (!fp) return 2;
  rd(ext, sizeof ext, fp);
  fclose(fp);
  const int nout = vti ? 6 : 3;
  float *o[6];   /* rho lambda mu, or c11 c33 c55 c66 c13 rho */
  for (int n = 0; n < nout; n++) o[n] = calloc(vol, 4);
  if (vti)
    media_grid2model_el_vti(o[5], o[0], o[1], o[2], o[3], o[4], x, y, z, d[0], d[1], d[2],
                            ext[0], ext[1], ext[2], ext[3], PROBE_GRID_CURV, grd, method, 0);
  else
    media_grid2model_el_iso(o[0], o[1], o[2], x, y, z, d[0], d[1], d[2], ext[0], ext[1],
                            ext[2], ext[3], PROBE_GRID_CURV, grd, method, 0);
  FILE *fo = fopen(out, "wb");
  if (!fo) return 2;
  for (int n = 0; n < nout; n++) fwrite(o[n], 4, vol, fo);
  fclose(fo);
  return 0;
}

static int probe_layer_aniso(const char *lay, const char *grid, const char *method,
                             const char *out)
{
  FILE *fp = fopen(grid, "rb");
  if (!fp) return 2;
  int d[3];
  rd(d, sizeof d, fp);
  size_t vol = (size_t)d[0] * d[1] * d[2];
  float *x = malloc(vol * 4), *y = malloc(vol * 4), *z = malloc(vol * 4);
  rd(x, vol * 4, fp);
  rd(y, vol * 4, fp);
  rd(z, vol * 4, fp);
  fclose(fp);
  float *c[22];
  for (int n = 0; n < 22; n++) c[n] = calloc(vol, 4);
  media_layer2model_el_aniso(c[0], c[1], c[2], c[3], c[4], c[5], c[6], c[7], c[8], c[9], c[10],
                             c[11], c[12], c[13], c[14], c[15], c[16], c[17], c[18], c[19],
                             c[20], c[21], x, y, z, d[0], d[1], d[2], PROBE_GRID_CURV, lay,
                             method, 0);
  FILE *fo = fopen(out, "wb");
  if (!fo) return 2;
  for (int n = 0; n < 22; n++) fwrite(c[n], 4, vol, fo);
  fclose(fo);
  return 0;
}

static int probe_grid_aniso(const char *grd, const char *grid, const char *method,
                            const char *extf, const char *out)
{
  FILE *fp = fopen(grid, "rb");
  if (!fp) return 2;
  int d[3];
  rd(d, sizeof d, fp);
  size_t vol = (size_t)d[0] * d[1] * d[2];
  float *x = malloc(vol * 4), *y = malloc(vol * 4), *z = malloc(vol * 4);
  rd(x, vol * 4, fp);
  rd(y, vol * 4, fp);
  rd(z, vol * 4, fp);
  fclose(fp);
  float ext[4];
  fp = fopen(extf, "rb");
  if (!fp) return 2;
  rd(ext, sizeof ext, fp);
  fclose(fp);
  float *c[22];
  for (int n = 0; n < 22; n++) c[n] = calloc(vol, 4);
  media_grid2model_el_aniso(c[0], c[1], c[2], c[3], c[4], c[5], c[6], c[7], c[8], c[9], c[10],
                            c[11], c[12], c[13], c[14], c[15], c[16], c[17], c[18], c[19],
                            c[20], c[21], x, y, z, d[0], d[1], d[2], ext[0], ext[1], ext[2],
                            ext[3], PROBE_GRID_CURV, grd, method, 0);
  FILE *fo = fopen(out, "wb");
  if (!fo) return 2;
  for (int n = 0; n < 22; n++) fwrite(c[n], 4, vol, fo);
  fclose(fo);
  return 0;
}

int main(int argc, char **argv)
{
  if (argc == 4 && strcmp(argv[1], "sac") == 0) return probe_sac(argv[2], argv[3]);
  if (argc == 4 && strcmp(argv[1], "locate") == 0) return probe_locate(argv[2], argv[3]);
  if (argc == 6 && strcmp(argv[1], "layer") == 0)
    return probe_layer(argv[2], argv[3], argv[4], argv[5]);
  if (argc == 6 && strcmp(argv[1], "layer_vti") == 0)
    return probe_layer_vti(argv[2], argv[3], argv[4], argv[5]);
  if (argc == 6 && strcmp(argv[1], "layer_one") == 0)
    return probe_layer_one(argv[2], argv[3], argv[4], argv[5]);
  if (argc == 6 && strcmp(argv[1], "layer_aniso") == 0)
    return probe_layer_aniso(argv[2], argv[3], argv[4], argv[5]);
  if (argc == 7 && strcmp(argv[1], "grid_aniso") == 0)
    return probe_grid_aniso(argv[2], argv[3], argv[4], argv[5], argv[6]);
  if (argc == 7 && strcmp(argv[1], "grid") == 0)
    return probe_grid(0, argv[2], argv[3], argv[4], argv[5], argv[6]);
  if (argc == 7 && strcmp(argv[1], "grid_vti") == 0)
    return probe_grid(1, argv[2], argv[3], argv[4], argv[5], argv[6]);
  if (argc == 8 && strcmp(argv[1], "bin") == 0)
    return probe_bin(0, argv[2], argv[3], (const char *const *)argv + 4, argv[7]);
  if (argc == 7 && strcmp(argv[1], "bin_vis") == 0)
    return probe_bin(1, argv[2], argv[3], (const char *const *)argv + 4, argv[6]);
  fprintf(stderr, "usage: ref_probe sac|locate <input> <output> | "
                  "layer|layer_vti|layer_one <md3lay> <grid> <method> <output>\n");
  return 2;
}
