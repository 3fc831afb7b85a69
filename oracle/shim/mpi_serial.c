/*
 * Serial implementation of the MPI subset declared in shim/mpi.h.
 * TEST INFRASTRUCTURE ONLY (reference build for golden vectors).
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "mpi.h"

static size_t type_size(MPI_Datatype t)
{
  switch (t) {
    case MPI_CHAR: return 1;
    case MPI_INT: return 4;
    case MPI_FLOAT: return 4;
    case MPI_LONG: return 8;
    case MPI_DOUBLE: return 8;
    default:
      fprintf(stderr, "mpi shim: unsupported datatype %d in a copy\n", t);
      exit(3);
  }
}

int MPI_Init(int *argc, char ***argv) { (void)argc; (void)argv; return 0; }
int MPI_Finalize(void) { return 0; }
int MPI_Abort(MPI_Comm comm, int code)
{
  (void)comm;
  fprintf(stderr, "MPI_Abort(%d) called\n", code);
  fflush(stderr);
  exit(code == 0 ? 1 : code);
}
int MPI_Comm_size(MPI_Comm comm, int *size) { (void)comm; *size = 1; return 0; }
int MPI_Comm_rank(MPI_Comm comm, int *rank) { (void)comm; *rank = 0; return 0; }
int MPI_Get_processor_name(char *name, int *len)
{
  strcpy(name, "serial");
  *len = (int)strlen(name);
  return 0;
}
int MPI_Barrier(MPI_Comm comm) { (void)comm; return 0; }
int MPI_Bcast(void *buf, int count, MPI_Datatype t, int root, MPI_Comm comm)
{ (void)buf; (void)count; (void)t; (void)root; (void)comm; return 0; }
int MPI_Allreduce(const void *sbuf, void *rbuf, int count, MPI_Datatype t,
                  MPI_Op op, MPI_Comm comm)
{
  (void)op; (void)comm;
  if (sbuf != rbuf) memcpy(rbuf, sbuf, (size_t)count * type_size(t));
  return 0;
}
int MPI_Allgather(const void *sbuf, int scount, MPI_Datatype st,
                  void *rbuf, int rcount, MPI_Datatype rt, MPI_Comm comm)
{
  (void)rcount; (void)rt; (void)comm;
  if (sbuf != rbuf) memcpy(rbuf, sbuf, (size_t)scount * type_size(st));
  return 0;
}
int MPI_Cart_create(MPI_Comm old, int ndims, const int dims[],
                    const int periods[], int reorder, MPI_Comm *cart)
{
  (void)old; (void)periods; (void)reorder;
  for (int i = 0; i < ndims; i++) {
    if (dims[i] != 1) {
      fprintf(stderr, "mpi shim: only a 1x1 process grid is supported\n");
      exit(3);
    }
  }
  *cart = 2;
  return 0;
}
int MPI_Cart_coords(MPI_Comm comm, int rank, int maxdims, int coords[])
{
  (void)comm; (void)rank;
  for (int i = 0; i < maxdims; i++) coords[i] = 0;
  return 0;
}
int MPI_Cart_shift(MPI_Comm comm, int dir, int disp, int *src, int *dst)
{
  (void)comm; (void)dir; (void)disp;
  *src = MPI_PROC_NULL;
  *dst = MPI_PROC_NULL;
  return 0;
}
int MPI_Send_init(const void *buf, int count, MPI_Datatype t, int dest,
                  int tag, MPI_Comm comm, MPI_Request *req)
{ (void)buf; (void)count; (void)t; (void)dest; (void)tag; (void)comm; *req = 0; return 0; }
int MPI_Recv_init(void *buf, int count, MPI_Datatype t, int src,
                  int tag, MPI_Comm comm, MPI_Request *req)
{ (void)buf; (void)count; (void)t; (void)src; (void)tag; (void)comm; *req = 0; return 0; }
int MPI_Startall(int n, MPI_Request reqs[]) { (void)n; (void)reqs; return 0; }
int MPI_Waitall(int n, MPI_Request reqs[], MPI_Status st[])
{ (void)n; (void)reqs; (void)st; return 0; }
int MPI_Sendrecv(const void *sbuf, int scount, MPI_Datatype st, int dest,
                 int stag, void *rbuf, int rcount, MPI_Datatype rt, int src,
                 int rtag, MPI_Comm comm, MPI_Status *status)
{
  (void)sbuf; (void)scount; (void)st; (void)stag; (void)rbuf; (void)rcount;
  (void)rt; (void)rtag; (void)comm; (void)status;
  if (dest != MPI_PROC_NULL || src != MPI_PROC_NULL) {
    fprintf(stderr, "mpi shim: Sendrecv with a real neighbour\n");
    exit(3);
  }
  return 0;
}
int MPI_Type_vector(int count, int blocklen, int stride, MPI_Datatype old,
                    MPI_Datatype *newtype)
{ (void)count; (void)blocklen; (void)stride; (void)old; *newtype = 1000; return 0; }
int MPI_Type_commit(MPI_Datatype *t) { (void)t; return 0; }
