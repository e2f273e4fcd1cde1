/* Single-rank stand-in for the MPI API, used only to compile the GENESIS 1.3 v4
 * reference sources into a CPU checker (oracle/_ref). Every communicator has one
 * rank; collectives copy the send buffer to the receive buffer; point-to-point
 * calls are never reached with one rank and do nothing.
 *
 * This file is test infrastructure written for this project; it is not part of
 * the reference and ships no reference code. */
#ifndef G4REF_MPI_SHIM_H
#define G4REF_MPI_SHIM_H

#include <string.h>
#include <stdlib.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Info;
typedef int MPI_Errhandler;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_INFO_NULL 0
#define MPI_ERRORS_RETURN 0
#define MPI_SUCCESS 0
#define MPI_CHAR 1
#define MPI_INT 4
#define MPI_DOUBLE 8
#define MPI_UNSIGNED_LONG_LONG 9
#define MPI_SUM 0
#define MPI_MAX 1
#define MPI_MIN 2
#define MPI_LAND 3
#define MPI_STATUS_IGNORE ((MPI_Status *)0)

static inline size_t g4ref_mpi_size(MPI_Datatype t) {
  switch (t) {
    case MPI_CHAR: return 1;
    case MPI_INT: return sizeof(int);
    case MPI_DOUBLE: return sizeof(double);
    case MPI_UNSIGNED_LONG_LONG: return sizeof(unsigned long long);
    default: return 8;
  }
}

static inline int MPI_Init(int *, char ***) { return 0; }
static inline int MPI_Finalize(void) { return 0; }
static inline int MPI_Comm_rank(MPI_Comm, int *r) { *r = 0; return 0; }
static inline int MPI_Comm_size(MPI_Comm, int *s) { *s = 1; return 0; }
static inline int MPI_Barrier(MPI_Comm) { return 0; }
static inline int MPI_Abort(MPI_Comm, int code) { exit(code); return 0; }
static inline int MPI_Errhandler_set(MPI_Comm, MPI_Errhandler) { return 0; }
static inline int MPI_Allreduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op, MPI_Comm) {
  if (s != r) memmove(r, s, (size_t)n * g4ref_mpi_size(t));
  return 0;
}
static inline int MPI_Reduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op, int, MPI_Comm) {
  if (s != r) memmove(r, s, (size_t)n * g4ref_mpi_size(t));
  return 0;
}
static inline int MPI_Allgather(const void *s, int n, MPI_Datatype t, void *r, int, MPI_Datatype, MPI_Comm) {
  if (s != r) memmove(r, s, (size_t)n * g4ref_mpi_size(t));
  return 0;
}
static inline int MPI_Gather(const void *s, int n, MPI_Datatype t, void *r, int, MPI_Datatype, int, MPI_Comm) {
  if (s != r) memmove(r, s, (size_t)n * g4ref_mpi_size(t));
  return 0;
}
static inline int MPI_Bcast(void *, int, MPI_Datatype, int, MPI_Comm) { return 0; }
static inline int MPI_Send(const void *, int, MPI_Datatype, int, int, MPI_Comm) { return 0; }
static inline int MPI_Recv(void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status *) { return 0; }
#define MPI_PROC_NULL (-2)
#define MPI_STATUS_IGNORE ((MPI_Status *)0)
static inline int MPI_Sendrecv(const void *, int, MPI_Datatype, int, int, void *, int, MPI_Datatype, int, int,
                               MPI_Comm, MPI_Status *) { return 0; }

#endif
