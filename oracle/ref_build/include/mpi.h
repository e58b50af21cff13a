/*
 * Single-rank MPI stand-in used only to compile the reference solver's own
 * CPU path as a test oracle.  Written for this project; it is NOT an MPI
 * implementation.  With one rank every collective is a copy, every
 * point-to-point exchange with a valid peer is a copy to oneself, and a peer
 * of -1 (the reference's "no neighbour" marker, ParallelManager.h:50-52)
 * sends or receives nothing.
 *
 * The reference passes doubles as MPI_LONG_DOUBLE (ParallelManager.h:113,
 * 120,127,245); it only ever ran on MSVC where long double is 8 bytes, so the
 * stub sizes MPI_LONG_DOUBLE elements as 8 bytes to reproduce that platform.
 */
#ifndef ORACLE_SINGLE_RANK_MPI_H
#define ORACLE_SINGLE_RANK_MPI_H

#include <string.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_SUCCESS 0
#define MPI_PROC_NULL (-2)
#define MPI_COMM_WORLD 1
#define MPI_INT 1
#define MPI_DOUBLE 2
#define MPI_LONG_DOUBLE 3
#define MPI_SUM 1
#define MPI_MIN 2
#define MPI_MAX 3

static inline size_t oracle_mpi_type_size(MPI_Datatype t) {
    return t == MPI_INT ? sizeof(int) : sizeof(double);
}

static inline int MPI_Init(int*, char***) { return MPI_SUCCESS; }
static inline int MPI_Finalize() { return MPI_SUCCESS; }
static inline int MPI_Comm_size(MPI_Comm, int* n) { *n = 1; return MPI_SUCCESS; }
static inline int MPI_Comm_rank(MPI_Comm, int* r) { *r = 0; return MPI_SUCCESS; }
static inline int MPI_Barrier(MPI_Comm) { return MPI_SUCCESS; }

static inline int MPI_Dims_create(int, int ndims, int* dims) {
    for (int d = 0; d < ndims; ++d) if (dims[d] == 0) dims[d] = 1;
    return MPI_SUCCESS;
}
static inline int MPI_Cart_create(MPI_Comm c, int, const int*, const int*, int, MPI_Comm* out) {
    *out = c; return MPI_SUCCESS;
}
static inline int MPI_Cart_coords(MPI_Comm, int, int ndims, int* coords) {
    for (int d = 0; d < ndims; ++d) coords[d] = 0;
    return MPI_SUCCESS;
}
static inline int MPI_Cart_rank(MPI_Comm, const int*, int* rank) { *rank = 0; return MPI_SUCCESS; }

static inline int MPI_Allreduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op, MPI_Comm) {
    memcpy(r, s, (size_t)n * oracle_mpi_type_size(t)); return MPI_SUCCESS;
}
static inline int MPI_Gather(const void* s, int n, MPI_Datatype t, void* r, int, MPI_Datatype, int, MPI_Comm) {
    if (r) memcpy(r, s, (size_t)n * oracle_mpi_type_size(t));
    return MPI_SUCCESS;
}
static inline int MPI_Send(const void*, int, MPI_Datatype, int, int, MPI_Comm) { return MPI_SUCCESS; }
static inline int MPI_Recv(void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status*) { return MPI_SUCCESS; }
static inline int MPI_Sendrecv(const void* s, int ns, MPI_Datatype ts, int dest, int,
                               void* r, int nr, MPI_Datatype, int source, int, MPI_Comm, MPI_Status*) {
    if (dest >= 0 && source >= 0 && ns > 0 && nr > 0) {
        int n = ns < nr ? ns : nr;
        memcpy(r, s, (size_t)n * oracle_mpi_type_size(ts));
    }
    return MPI_SUCCESS;
}

#endif
