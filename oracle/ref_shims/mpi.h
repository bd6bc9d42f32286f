/* Single-rank stand-in for the MPI API surface that AMCAFE's sources use.
 *
 * Test infrastructure only: it lets the reference sources (src/src-mpi/*.C)
 * compile and run as one MPI rank so that their own results can pin the oracle.
 * With one rank every collective is a copy (or nothing), and point-to-point
 * calls are never reached (Partition::PartitionGraph is not called and
 * PassInformation has no neighbour ranks). */
#ifndef CAFE_REF_SHIM_MPI_H
#define CAFE_REF_SHIM_MPI_H
#include <string.h>
#include <stdlib.h>
#include <stdio.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Request;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_CHAR 1
#define MPI_INT 4
#define MPI_DOUBLE 8
#define MPI_DOUBLE_INT 16
#define MPI_SUM 1
#define MPI_MAX 2
#define MPI_MINLOC 3
#define MPI_ANY_TAG (-1)
#define MPI_STATUS_IGNORE ((MPI_Status *)0)
#define MPI_SUCCESS 0

static inline size_t cafe_shim_type_size(MPI_Datatype t) { return (size_t)t; }

static inline int MPI_Init(int *, char ***) { return MPI_SUCCESS; }
static inline int MPI_Finalize(void) { return MPI_SUCCESS; }
static inline int MPI_Comm_size(MPI_Comm, int *n) { *n = 1; return MPI_SUCCESS; }
static inline int MPI_Comm_rank(MPI_Comm, int *r) { *r = 0; return MPI_SUCCESS; }
static inline int MPI_Barrier(MPI_Comm) { return MPI_SUCCESS; }
static inline int MPI_Bcast(void *, int, MPI_Datatype, int, MPI_Comm) { return MPI_SUCCESS; }
static inline int MPI_Allreduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op, MPI_Comm) {
  if (n > 0 && s != r) memmove(r, s, (size_t)n * cafe_shim_type_size(t));
  return MPI_SUCCESS;
}
static inline int MPI_Allgather(const void *s, int ns, MPI_Datatype ts, void *r, int, MPI_Datatype,
                                MPI_Comm) {
  if (ns > 0 && s != r) memmove(r, s, (size_t)ns * cafe_shim_type_size(ts));
  return MPI_SUCCESS;
}
static inline int cafe_shim_unreachable(const char *what) {
  fprintf(stderr, "mpi shim: %s reached with one rank\n", what);
  abort();
  return 1;
}
static inline int MPI_Send(const void *, int, MPI_Datatype, int, int, MPI_Comm) {
  return cafe_shim_unreachable("MPI_Send");
}
static inline int MPI_Recv(void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status *) {
  return cafe_shim_unreachable("MPI_Recv");
}
static inline int MPI_Sendrecv(const void *, int, MPI_Datatype, int, int, void *, int, MPI_Datatype,
                               int, int, MPI_Comm, MPI_Status *) {
  return cafe_shim_unreachable("MPI_Sendrecv");
}
#endif
