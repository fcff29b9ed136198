/*
 * Single-process stand-in for the MPI header, used only to compile the
 * reference prover's own sources into the test oracle (oracle/_ref).
 *
 * Part of the test infrastructure: nothing in the product links it.
 *
 * The reference functions that the oracle drivers call (fft, pfft,
 * MT_commit_Blake, whir_*, Whir_Open, RS folds, Encode, distributed_MT,
 * the secret-sharing helpers) touch MPI only through MPI_Comm_rank and, in
 * distributed_MT, an all-to-all of zero bytes.  This header models a world
 * of exactly one rank: collectives deliver a rank's own block to itself, and
 * point-to-point calls, which would need a second rank, abort loudly so a
 * driver that strays into collaborative code fails instead of producing
 * made-up bytes.
 */
#pragma once
#include <cstddef>
#include <cstdio>
#include <cstdlib>
#include <cstring>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;
typedef int MPI_Request;
typedef int MPI_Op;

#define MPI_COMM_WORLD 0
#define MPI_UINT64_T 1
#define MPI_UINT8_T 2
#define MPI_INT 3
#define MPI_DOUBLE 4
#define MPI_BYTE 5
#define MPI_CHAR 6
#define MPI_UNSIGNED_LONG_LONG 7
#define MPI_SUM 1
#define MPI_ANY_SOURCE (-1)
#define MPI_ANY_TAG (-1)
#define MPI_SUCCESS 0
#define MPI_STATUS_IGNORE ((MPI_Status *)0)
#define MPI_STATUSES_IGNORE ((MPI_Status *)0)

static inline void oracle_mpi_abort_(const char *what) {
  std::fprintf(stderr, "oracle mpi stub: %s is not available with one rank\n", what);
  std::abort();
}
static inline int MPI_Init(int *, char ***) { return 0; }
static inline int MPI_Finalize() { return 0; }
static inline int MPI_Comm_rank(MPI_Comm, int *r) { *r = 0; return 0; }
static inline int MPI_Comm_size(MPI_Comm, int *s) { *s = 1; return 0; }
static inline int MPI_Barrier(MPI_Comm) { return 0; }
static inline double MPI_Wtime() { return 0.0; }
static inline int MPI_Abort(MPI_Comm, int c) { std::exit(c); }
static inline int MPI_Send(const void *, int, MPI_Datatype, int, int, MPI_Comm) { oracle_mpi_abort_("MPI_Send"); return 1; }
static inline int MPI_Recv(void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status *) { oracle_mpi_abort_("MPI_Recv"); return 1; }
static inline int MPI_Isend(const void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request *) { oracle_mpi_abort_("MPI_Isend"); return 1; }
static inline int MPI_Irecv(void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request *) { oracle_mpi_abort_("MPI_Irecv"); return 1; }
static inline int MPI_Wait(MPI_Request *, MPI_Status *) { return 0; }
static inline int MPI_Waitall(int, MPI_Request *, MPI_Status *) { return 0; }
static inline int MPI_Waitany(int, MPI_Request *, int *, MPI_Status *) { oracle_mpi_abort_("MPI_Waitany"); return 1; }
static inline int MPI_Bcast(void *, int, MPI_Datatype, int, MPI_Comm) { return 0; }
static inline size_t oracle_mpi_size_(MPI_Datatype t) {
  switch (t) {
    case MPI_UINT64_T: case MPI_DOUBLE: case MPI_UNSIGNED_LONG_LONG: return 8;
    case MPI_INT: return 4;
    default: return 1;
  }
}
// With one rank an all-to-all delivers the rank's own block to itself.
static inline int MPI_Alltoall(const void *s, int sc, MPI_Datatype st, void *r, int, MPI_Datatype, MPI_Comm) {
  std::memcpy(r, s, (size_t)sc * oracle_mpi_size_(st));
  return 0;
}
static inline int MPI_Ialltoall(const void *s, int sc, MPI_Datatype st, void *r, int rc, MPI_Datatype rt, MPI_Comm c, MPI_Request *) {
  return MPI_Alltoall(s, sc, st, r, rc, rt, c);
}
static inline int MPI_Gather(const void *, int, MPI_Datatype, void *, int, MPI_Datatype, int, MPI_Comm) { oracle_mpi_abort_("MPI_Gather"); return 1; }
static inline int MPI_Allreduce(const void *, void *, int, MPI_Datatype, MPI_Op, MPI_Comm) { oracle_mpi_abort_("MPI_Allreduce"); return 1; }
static inline int MPI_Reduce(const void *, void *, int, MPI_Datatype, MPI_Op, int, MPI_Comm) { oracle_mpi_abort_("MPI_Reduce"); return 1; }
