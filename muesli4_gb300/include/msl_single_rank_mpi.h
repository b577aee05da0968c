// msl_single_rank_mpi.h -- the MPI names reference programs use, for one
// process.
//
// Programs written against the reference include "muesli.h" and receive the
// MPI API through it (the reference's include/muesli.h:36-38 pulls in
// <mpi.h>); its examples call MPI_Wtime directly for their timings (e.g.
// examples/gameoflife.cpp:71, examples/da_test.cpp:102). The GB300 front end
// runs one process on one device, so these names describe a world of one
// rank: rank 0 of size 1, barriers return at once, and a collective leaves
// (or copies) the calling rank's own data. No MPI library is involved.
//
// When a real <mpi.h> was included first (MPI_VERSION defined), this header
// declares nothing and the program keeps its MPI library.
#pragma once

#ifndef MPI_VERSION

#include <chrono>
#include <cstring>

typedef int MPI_Comm;
typedef int MPI_Datatype;  // the element size in bytes
typedef int MPI_Op;
typedef int MPI_Request;
typedef struct {
    int MPI_SOURCE, MPI_TAG, MPI_ERROR, count;
} MPI_Status;

#define MPI_COMM_WORLD ((MPI_Comm)0)
#define MPI_COMM_SELF ((MPI_Comm)1)
#define MPI_SUCCESS 0
#define MPI_ANY_TAG (-1)
#define MPI_ANY_SOURCE (-2)
#define MPI_IN_PLACE ((void *)-1)
#define MPI_STATUS_IGNORE ((MPI_Status *)0)
#define MPI_STATUSES_IGNORE ((MPI_Status *)0)
#define MPI_BYTE ((MPI_Datatype)1)
#define MPI_CHAR ((MPI_Datatype)sizeof(char))
#define MPI_INT ((MPI_Datatype)sizeof(int))
#define MPI_LONG ((MPI_Datatype)sizeof(long))
#define MPI_LONG_LONG ((MPI_Datatype)sizeof(long long))
#define MPI_FLOAT ((MPI_Datatype)sizeof(float))
#define MPI_DOUBLE ((MPI_Datatype)sizeof(double))
#define MPI_SUM ((MPI_Op)0)
#define MPI_MAX ((MPI_Op)1)
#define MPI_MIN ((MPI_Op)2)
#define MPI_PROD ((MPI_Op)3)

namespace msl {
namespace detail {
// Data of the one rank: a copy from send to receive buffer unless they are
// the same buffer (or the receive side is MPI_IN_PLACE).
inline void single_rank_copy(const void *send, void *recv, int count, MPI_Datatype type) {
    if (send && recv && send != recv && send != MPI_IN_PLACE && count > 0)
        std::memmove(recv, send, (size_t)count * (size_t)type);
}
}  // namespace detail
}  // namespace msl

inline int MPI_Init(int *, char ***) { return MPI_SUCCESS; }
inline int MPI_Initialized(int *flag) {
    if (flag) *flag = 1;
    return MPI_SUCCESS;
}
inline int MPI_Finalize(void) { return MPI_SUCCESS; }
inline int MPI_Abort(MPI_Comm, int code) {
    std::exit(code);
    return MPI_SUCCESS;
}
inline int MPI_Comm_size(MPI_Comm, int *size) {
    *size = 1;
    return MPI_SUCCESS;
}
inline int MPI_Comm_rank(MPI_Comm, int *rank) {
    *rank = 0;
    return MPI_SUCCESS;
}
inline int MPI_Barrier(MPI_Comm) { return MPI_SUCCESS; }
// Wall-clock seconds from a monotonic clock.
inline double MPI_Wtime(void) {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}
inline double MPI_Wtick(void) { return 1e-9; }
inline int MPI_Bcast(void *, int, MPI_Datatype, int, MPI_Comm) { return MPI_SUCCESS; }
inline int MPI_Reduce(const void *send, void *recv, int count, MPI_Datatype type, MPI_Op, int, MPI_Comm) {
    msl::detail::single_rank_copy(send, recv, count, type);
    return MPI_SUCCESS;
}
inline int MPI_Allreduce(const void *send, void *recv, int count, MPI_Datatype type, MPI_Op, MPI_Comm) {
    msl::detail::single_rank_copy(send, recv, count, type);
    return MPI_SUCCESS;
}
inline int MPI_Gather(const void *send, int count, MPI_Datatype type, void *recv, int, MPI_Datatype, int, MPI_Comm) {
    msl::detail::single_rank_copy(send, recv, count, type);
    return MPI_SUCCESS;
}
inline int MPI_Allgather(const void *send, int count, MPI_Datatype type, void *recv, int, MPI_Datatype, MPI_Comm) {
    msl::detail::single_rank_copy(send, recv, count, type);
    return MPI_SUCCESS;
}
inline int MPI_Scatter(const void *send, int count, MPI_Datatype type, void *recv, int, MPI_Datatype, int, MPI_Comm) {
    msl::detail::single_rank_copy(send, recv, count, type);
    return MPI_SUCCESS;
}

#endif  // MPI_VERSION
