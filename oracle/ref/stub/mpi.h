/*
 * Single-rank stand-in for <mpi.h>, used only to compile the PIC++ reference
 * sources into the test oracle under oracle/_ref/.  Not product code.
 *
 * One process is the whole Cartesian communicator: every dimension is 1, the
 * rank is 0, reductions and self send/receive copy the buffer, and barriers,
 * broadcasts, plain sends and receives do nothing.  With cartDim == 1 the
 * reference takes its local periodic-copy branches (e.g. PIC++/mpi_util.cpp
 * 261-272), so no message ever needs to travel.
 */
#ifndef PICPP_ORACLE_MPI_STUB_H
#define PICPP_ORACLE_MPI_STUB_H
#include <string.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;   /* value = element size in bytes */
typedef int MPI_Op;
typedef struct { int source, tag, error; } MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_DOUBLE ((MPI_Datatype)sizeof(double))
#define MPI_INT ((MPI_Datatype)sizeof(int))
#define MPI_SUM 0

static inline int MPI_Init(int*, char***) { return 0; }
static inline int MPI_Finalize() { return 0; }
static inline int MPI_Barrier(MPI_Comm) { return 0; }
static inline int MPI_Comm_size(MPI_Comm, int* size) { *size = 1; return 0; }
static inline int MPI_Comm_rank(MPI_Comm, int* rank) { *rank = 0; return 0; }
static inline int MPI_Cart_create(MPI_Comm, int, const int*, const int*, int, MPI_Comm* out) { *out = 0; return 0; }
static inline int MPI_Cart_get(MPI_Comm, int ndims, int* dims, int* periods, int* coords) {
    for (int d = 0; d < ndims; ++d) { dims[d] = 1; periods[d] = 1; coords[d] = 0; }
    return 0;
}
static inline int MPI_Cart_rank(MPI_Comm, const int*, int* rank) { *rank = 0; return 0; }
static inline int MPI_Cart_sub(MPI_Comm, const int*, MPI_Comm* out) { *out = 0; return 0; }
static inline int MPI_Bcast(void*, int, MPI_Datatype, int, MPI_Comm) { return 0; }
static inline int MPI_Allreduce(const void* in, void* out, int n, MPI_Datatype t, MPI_Op, MPI_Comm) {
    if (in != out) memmove(out, in, (size_t)n * (size_t)t);
    return 0;
}
static inline int MPI_Reduce(const void* in, void* out, int n, MPI_Datatype t, MPI_Op, int, MPI_Comm) {
    if (out && in != out) memmove(out, in, (size_t)n * (size_t)t);
    return 0;
}
static inline int MPI_Send(const void*, int, MPI_Datatype, int, int, MPI_Comm) { return 0; }
static inline int MPI_Recv(void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status*) { return 0; }
static inline int MPI_Sendrecv(const void* sb, int sn, MPI_Datatype st, int, int,
                               void* rb, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status*) {
    if (sb != rb) memmove(rb, sb, (size_t)sn * (size_t)st);
    return 0;
}
#endif
