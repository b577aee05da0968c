/*
 * Single-rank stand-in for <mpi.h>, used only to compile the Muesli reference
 * headers (OpenMP build) as a CPU checker. Test infrastructure: nothing in the
 * product links it.
 *
 * With one rank every collective is a local copy and point-to-point calls are
 * never reached (the reference only sends to neighbour ranks, and rank 0 has
 * none). The symbols are the ones the reference uses: src/muesli_com.cpp:39-311,
 * src/muesli.cpp:63-158, include/timer.h:43-107.
 */
#ifndef MSL_ORACLE_MPI_STUB_H
#define MSL_ORACLE_MPI_STUB_H

#include <string.h>
#include <time.h>

#define MPI_VERSION 3
#define MPI_SUBVERSION 1

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Request;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR, count; } MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_BYTE 1
#define MPI_ANY_TAG (-1)
#define MPI_ANY_SOURCE (-2)
#define MPI_SUCCESS 0
#define MPI_STATUS_IGNORE ((MPI_Status *)0)
#define MPI_STATUSES_IGNORE ((MPI_Status *)0)

static inline int MPI_Init(int *, char ***) { return 0; }
static inline int MPI_Finalize(void) { return 0; }
static inline int MPI_Comm_size(MPI_Comm, int *n) { *n = 1; return 0; }
static inline int MPI_Comm_rank(MPI_Comm, int *r) { *r = 0; return 0; }
static inline int MPI_Barrier(MPI_Comm) { return 0; }
static inline double MPI_Wtime(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}
/* One rank: the broadcast root already holds the data. */
static inline int MPI_Bcast(void *, int, MPI_Datatype, int, MPI_Comm) { return 0; }
/* One rank: gather/allgather/scatter copy the rank's own block (MPI_BYTE only). */
static inline int MPI_Allgather(const void *s, int n, MPI_Datatype, void *r, int, MPI_Datatype, MPI_Comm) {
    if (s != r) memmove(r, s, (size_t)n);
    return 0;
}
static inline int MPI_Gather(const void *s, int n, MPI_Datatype, void *r, int, MPI_Datatype, int, MPI_Comm) {
    if (r && s != r) memmove(r, s, (size_t)n);
    return 0;
}
static inline int MPI_Scatter(const void *s, int n, MPI_Datatype, void *r, int, MPI_Datatype, int, MPI_Comm) {
    if (s != r) memmove(r, s, (size_t)n);
    return 0;
}
/* Point-to-point: unreachable with one rank; kept as no-ops so the code links. */
static inline int MPI_Send(const void *, int, MPI_Datatype, int, int, MPI_Comm) { return 0; }
static inline int MPI_Isend(const void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request *q) { *q = 0; return 0; }
static inline int MPI_Recv(void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status *) { return 0; }
static inline int MPI_Irecv(void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request *q) { *q = 0; return 0; }
static inline int MPI_Wait(MPI_Request *, MPI_Status *) { return 0; }
static inline int MPI_Waitall(int, MPI_Request *, MPI_Status *) { return 0; }
static inline int MPI_Probe(int, int, MPI_Comm, MPI_Status *s) { if (s) s->count = 0; return 0; }
static inline int MPI_Get_count(const MPI_Status *s, MPI_Datatype, int *n) { *n = s ? s->count : 0; return 0; }

#endif
