/*
 * Single-process stand-in for the handful of MPI calls the reference Wilson
 * solver makes (test infrastructure only: it lets the reference's own sources
 * build and run as one rank so they can serve as the oracle).
 *
 * Semantics: rank 0 of a world of size 1.  Reduce copies send to receive,
 * Bcast and Barrier do nothing, Wtime reads a monotonic clock.  Point-to-point
 * calls are never reached when the sub-grid equals the whole lattice (the only
 * configuration the oracle runs), so they fail loudly if they are.
 */
#ifndef WD_ORACLE_MPI_SHIM_H
#define WD_ORACLE_MPI_SHIM_H

#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Request;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_DOUBLE 8
#define MPI_SUM 1
#define MPI_SUCCESS 0
#define MPI_STATUS_IGNORE ((MPI_Status *)0)

static inline int MPI_Init(int *, char ***) { return MPI_SUCCESS; }
static inline int MPI_Finalize(void) { return MPI_SUCCESS; }
static inline int MPI_Comm_rank(MPI_Comm, int *r) { *r = 0; return MPI_SUCCESS; }
static inline int MPI_Comm_size(MPI_Comm, int *s) { *s = 1; return MPI_SUCCESS; }
static inline int MPI_Barrier(MPI_Comm) { return MPI_SUCCESS; }
static inline int MPI_Bcast(void *, int, MPI_Datatype, int, MPI_Comm) { return MPI_SUCCESS; }
static inline int MPI_Reduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op, int, MPI_Comm)
{
    memcpy(r, s, (size_t)n * (size_t)t);
    return MPI_SUCCESS;
}
static inline double MPI_Wtime(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}
static inline int wd_shim_p2p_unreachable(const char *what)
{
    fprintf(stderr, "mpi shim: %s needs more than one rank\n", what);
    abort();
    return 1;
}
static inline int MPI_Isend(const void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request *)
{ return wd_shim_p2p_unreachable("MPI_Isend"); }
static inline int MPI_Irecv(void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request *)
{ return wd_shim_p2p_unreachable("MPI_Irecv"); }
static inline int MPI_Wait(MPI_Request *, MPI_Status *) { return wd_shim_p2p_unreachable("MPI_Wait"); }
static inline int MPI_Send(const void *, int, MPI_Datatype, int, int, MPI_Comm)
{ return wd_shim_p2p_unreachable("MPI_Send"); }
static inline int MPI_Recv(void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status *)
{ return wd_shim_p2p_unreachable("MPI_Recv"); }

#endif
