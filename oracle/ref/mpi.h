/*
 * Single-rank stand-in for <mpi.h>, project-written, used only to compile the
 * reference's CPU solver headers into the test oracle (oracle/_ref).
 *
 * With one rank the reference never posts a halo message (numCommunication_ == 0,
 * blockGrid.hpp:281-285), so point-to-point calls and derived datatypes are no-ops,
 * and every reduction or broadcast is a copy of the caller's own contribution.
 */
#ifndef PPS_ORACLE_MPI_STUB_H
#define PPS_ORACLE_MPI_STUB_H

#include <string.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Request;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_SUCCESS 0
#define MPI_FLOAT 4
#define MPI_DOUBLE 8
#define MPI_INT 104
#define MPI_SUM 1

static inline int pps_stub_type_size(MPI_Datatype t) { return t == MPI_INT ? (int)sizeof(int) : t; }

static inline int MPI_Init(int*, char***) { return MPI_SUCCESS; }
static inline int MPI_Finalize(void) { return MPI_SUCCESS; }
static inline int MPI_Comm_size(MPI_Comm, int* size) { *size = 1; return MPI_SUCCESS; }
static inline int MPI_Comm_rank(MPI_Comm, int* rank) { *rank = 0; return MPI_SUCCESS; }
static inline int MPI_Barrier(MPI_Comm) { return MPI_SUCCESS; }
static inline int MPI_Reduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op, int, MPI_Comm)
{
    if (s != r) memcpy(r, s, (size_t)n * (size_t)pps_stub_type_size(t));
    return MPI_SUCCESS;
}
static inline int MPI_Allreduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op, MPI_Comm)
{
    if (s != r) memcpy(r, s, (size_t)n * (size_t)pps_stub_type_size(t));
    return MPI_SUCCESS;
}
static inline int MPI_Bcast(void*, int, MPI_Datatype, int, MPI_Comm) { return MPI_SUCCESS; }
static inline int MPI_Isend(const void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request* q)
{
    *q = 0;
    return MPI_SUCCESS;
}
static inline int MPI_Irecv(void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request* q)
{
    *q = 0;
    return MPI_SUCCESS;
}
static inline int MPI_Waitall(int n, MPI_Request*, MPI_Status* st)
{
    for (int i = 0; i < n; i++) st[i].MPI_ERROR = MPI_SUCCESS;
    return MPI_SUCCESS;
}
static inline int MPI_Type_indexed(int, const int*, const int*, MPI_Datatype old, MPI_Datatype* nt)
{
    *nt = old;
    return MPI_SUCCESS;
}
static inline int MPI_Type_commit(MPI_Datatype*) { return MPI_SUCCESS; }

#endif
