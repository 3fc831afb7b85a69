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
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "io_funcs.h"

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

int main(int argc, char **argv)
{
  if (argc == 4 && strcmp(argv[1], "sac") == 0) return probe_sac(argv[2], argv[3]);
  fprintf(stderr, "usage: ref_probe sac <input> <out_dir>\n");
  return 2;
}
