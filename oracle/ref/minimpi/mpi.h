/*
 * Interface of a minimal MPI for running the reference prover's own
 * multi-rank code as N processes on one host (minimpi.cpp).
 *
 * Test infrastructure only: the product never links it.  It exists because
 * no MPI implementation is installed here, and the reference's
 * collaborative paths (packed-Shamir sharing, the leader's aggregation of
 * round messages, per-party commitments) need N ranks to produce the bytes
 * that the one-device GPU path must reproduce.
 *
 * Only the calls and datatypes the reference uses are provided.  Handles
 * are plain integers; MPI_Request indexes a per-process request table.
 */
#pragma once
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Request;
typedef int MPI_Op;
typedef struct {
  int MPI_SOURCE, MPI_TAG, MPI_ERROR;
  size_t bytes_;
} MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_UINT64_T 1
#define MPI_UINT8_T 2
#define MPI_INT 3
#define MPI_DOUBLE 4
#define MPI_BYTE 5
#define MPI_CHAR 6
#define MPI_UNSIGNED_LONG_LONG 7
#define MPI_UINT32_T 8
#define MPI_SUM 1
#define MPI_ANY_SOURCE (-1)
#define MPI_ANY_TAG (-1)
#define MPI_SUCCESS 0
#define MPI_REQUEST_NULL (-1)
#define MPI_STATUS_IGNORE ((MPI_Status *)0)
#define MPI_STATUSES_IGNORE ((MPI_Status *)0)

int MPI_Init(int *argc, char ***argv);
int MPI_Finalize(void);
int MPI_Comm_rank(MPI_Comm comm, int *rank);
int MPI_Comm_size(MPI_Comm comm, int *size);
int MPI_Abort(MPI_Comm comm, int code);
double MPI_Wtime(void);
int MPI_Send(const void *buf, int count, MPI_Datatype type, int dest, int tag, MPI_Comm comm);
int MPI_Recv(void *buf, int count, MPI_Datatype type, int src, int tag, MPI_Comm comm, MPI_Status *st);
int MPI_Isend(const void *buf, int count, MPI_Datatype type, int dest, int tag, MPI_Comm comm, MPI_Request *req);
int MPI_Irecv(void *buf, int count, MPI_Datatype type, int src, int tag, MPI_Comm comm, MPI_Request *req);
int MPI_Wait(MPI_Request *req, MPI_Status *st);
int MPI_Waitall(int n, MPI_Request *reqs, MPI_Status *sts);
int MPI_Waitany(int n, MPI_Request *reqs, int *index, MPI_Status *st);
int MPI_Barrier(MPI_Comm comm);
int MPI_Bcast(void *buf, int count, MPI_Datatype type, int root, MPI_Comm comm);
int MPI_Alltoall(const void *sbuf, int scount, MPI_Datatype stype, void *rbuf, int rcount, MPI_Datatype rtype,
                 MPI_Comm comm);
int MPI_Ialltoall(const void *sbuf, int scount, MPI_Datatype stype, void *rbuf, int rcount, MPI_Datatype rtype,
                  MPI_Comm comm, MPI_Request *req);

#ifdef __cplusplus
}
#endif
