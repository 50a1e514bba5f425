/*
 * Single-rank MPI stand-in. Test infrastructure only: it lets the reference
 * C++ sources (mmhej/poissonsolver, c++/source) compile as a one-process CPU
 * oracle. With one rank every exchange in the reference is a self-copy
 * (communication/constructor.cpp marks the rank-to-itself entry nway = 0 and
 * map.cpp / push.cpp / pull.cpp take their self-copy branch), so the
 * point-to-point calls below are never reached; they report failure if they are.
 */
#ifndef ORACLE_MPI_STUB_H
#define ORACLE_MPI_STUB_H

#include <string.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef struct { int source, tag, error; } MPI_Status;

#define MPI_COMM_WORLD     0
#define MPI_DOUBLE         ((MPI_Datatype)sizeof(double))
#define MPI_INT            ((MPI_Datatype)sizeof(int))
#define MPI_SUM            0
#define MPI_STATUS_IGNORE  ((MPI_Status *)0)
#define MPI_SUCCESS        0

static inline int MPI_Init(int *, char ***) { return MPI_SUCCESS; }
static inline int MPI_Finalize(void) { return MPI_SUCCESS; }
static inline int MPI_Comm_size(MPI_Comm, int *n) { *n = 1; return MPI_SUCCESS; }
static inline int MPI_Comm_rank(MPI_Comm, int *r) { *r = 0; return MPI_SUCCESS; }
static inline int MPI_Barrier(MPI_Comm) { return MPI_SUCCESS; }
/* One rank: a reduction to rank 0 is a copy of the local contribution. */
static inline int MPI_Reduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op, int, MPI_Comm)
{
    memcpy(r, s, (size_t)n * (size_t)t);
    return MPI_SUCCESS;
}
static inline int MPI_Send(const void *, int, MPI_Datatype, int, int, MPI_Comm) { return 1; }
static inline int MPI_Recv(void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status *) { return 1; }
static inline int MPI_Sendrecv(const void *, int, MPI_Datatype, int, int, void *, int, MPI_Datatype,
                               int, int, MPI_Comm, MPI_Status *) { return 1; }

#endif
