/*
 * Serial stand-in for the MPI interface, written for this project.
 *
 * TEST INFRASTRUCTURE ONLY: it lets the CGFD3D reference sources compile
 * and run as a single rank so their output can serve as golden vectors.
 * Nothing in the product links against it.
 *
 * One rank, no neighbours: MPI_Cart_shift answers MPI_PROC_NULL on both
 * sides (non-periodic 1x1 topology), so every halo exchange in the
 * reference becomes a no-op, exactly as on one GPU.  Collectives copy the
 * send buffer into the receive buffer.
 */
#ifndef CGFD_SHIM_MPI_H
#define CGFD_SHIM_MPI_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Request;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_SUCCESS 0
#define MPI_COMM_WORLD ((MPI_Comm)1)
#define MPI_COMM_NULL  ((MPI_Comm)0)
#define MPI_PROC_NULL  (-2)
#define MPI_REQUEST_NULL ((MPI_Request)0)
#define MPI_STATUS_IGNORE   ((MPI_Status *)0)
#define MPI_STATUSES_IGNORE ((MPI_Status *)0)
#define MPI_MAX_PROCESSOR_NAME 256

/* datatype handle = element size in bytes (derived types get 1000+) */
#define MPI_CHAR   ((MPI_Datatype)1)
#define MPI_INT    ((MPI_Datatype)4)
#define MPI_FLOAT  ((MPI_Datatype)104)
#define MPI_REAL   ((MPI_Datatype)104)
#define MPI_LONG   ((MPI_Datatype)8)
#define MPI_DOUBLE ((MPI_Datatype)108)

#define MPI_SUM ((MPI_Op)1)
#define MPI_MAX ((MPI_Op)2)
#define MPI_MIN ((MPI_Op)3)

int MPI_Init(int *argc, char ***argv);
int MPI_Finalize(void);
int MPI_Abort(MPI_Comm comm, int code);
int MPI_Comm_size(MPI_Comm comm, int *size);
int MPI_Comm_rank(MPI_Comm comm, int *rank);
int MPI_Get_processor_name(char *name, int *len);
int MPI_Barrier(MPI_Comm comm);
int MPI_Bcast(void *buf, int count, MPI_Datatype t, int root, MPI_Comm comm);
int MPI_Allreduce(const void *sbuf, void *rbuf, int count, MPI_Datatype t,
                  MPI_Op op, MPI_Comm comm);
int MPI_Allgather(const void *sbuf, int scount, MPI_Datatype st,
                  void *rbuf, int rcount, MPI_Datatype rt, MPI_Comm comm);
int MPI_Cart_create(MPI_Comm old, int ndims, const int dims[],
                    const int periods[], int reorder, MPI_Comm *cart);
int MPI_Cart_coords(MPI_Comm comm, int rank, int maxdims, int coords[]);
int MPI_Cart_shift(MPI_Comm comm, int dir, int disp, int *src, int *dst);
int MPI_Send_init(const void *buf, int count, MPI_Datatype t, int dest,
                  int tag, MPI_Comm comm, MPI_Request *req);
int MPI_Recv_init(void *buf, int count, MPI_Datatype t, int src,
                  int tag, MPI_Comm comm, MPI_Request *req);
int MPI_Startall(int n, MPI_Request reqs[]);
int MPI_Waitall(int n, MPI_Request reqs[], MPI_Status st[]);
int MPI_Sendrecv(const void *sbuf, int scount, MPI_Datatype st, int dest,
                 int stag, void *rbuf, int rcount, MPI_Datatype rt, int src,
                 int rtag, MPI_Comm comm, MPI_Status *status);
int MPI_Type_vector(int count, int blocklen, int stride, MPI_Datatype old,
                    MPI_Datatype *newtype);
int MPI_Type_commit(MPI_Datatype *t);

#ifdef __cplusplus
}
#endif
#endif
