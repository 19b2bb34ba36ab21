/*
 * Single-rank MPI stand-in used ONLY to compile the reference's own C++
 * translation units into the CPU oracle (oracle/_ref).  It is test
 * infrastructure: nothing in the product links it.
 *
 * With one rank and no overlap control points (isb == 0, which is what
 * InputParaGriddata sets up for a single rank, module/data_io.cpp:114-123),
 * every collective in the reference degenerates to a local copy:
 *   - MPI_Allreduce      (module/solver/solver.cpp:59, module/material_point.cpp:185)
 *   - MPI_Allgather      (module/solver/crsmat.cpp:256)
 * and the point-to-point halo exchange in NodeVarComm (module/mpi_data.h:36)
 * is never reached because isb == 0.
 */
#pragma once
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <chrono>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Request;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_COMM_SELF 1
#define MPI_INT 1
#define MPI_DOUBLE 2
#define MPI_CHAR 3
#define MPI_LONG 4
#define MPI_LONG_LONG 5
#define MPI_FLOAT 6
#define MPI_BYTE 7
#define MPI_SUM 1
#define MPI_MAX 2
#define MPI_MIN 3
#define MPI_IN_PLACE ((void *)1)
#define MPI_STATUS_IGNORE ((MPI_Status *)0)
#define MPI_STATUSES_IGNORE ((MPI_Status *)0)
#define MPI_SUCCESS 0

static inline size_t mpi_stub_type_size(MPI_Datatype t) {
    switch (t) {
    case MPI_INT: return sizeof(int);
    case MPI_DOUBLE: return sizeof(double);
    case MPI_CHAR: return 1;
    case MPI_LONG: return sizeof(long);
    case MPI_LONG_LONG: return sizeof(long long);
    case MPI_FLOAT: return sizeof(float);
    case MPI_BYTE: return 1;
    default: return 0;
    }
}

static inline int MPI_Init(int *, char ***) { return 0; }
static inline int MPI_Finalize() { return 0; }
static inline int MPI_Comm_size(MPI_Comm, int *n) { *n = 1; return 0; }
static inline int MPI_Comm_rank(MPI_Comm, int *r) { *r = 0; return 0; }
static inline int MPI_Barrier(MPI_Comm) { return 0; }
static inline double MPI_Wtime() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}
static inline int MPI_Allreduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op, MPI_Comm) {
    if (s != MPI_IN_PLACE && s != r) std::memcpy(r, s, (size_t)n * mpi_stub_type_size(t));
    return 0;
}
static inline int MPI_Reduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op, int, MPI_Comm) {
    if (s != MPI_IN_PLACE && s != r) std::memcpy(r, s, (size_t)n * mpi_stub_type_size(t));
    return 0;
}
static inline int MPI_Bcast(void *, int, MPI_Datatype, int, MPI_Comm) { return 0; }
static inline int MPI_Allgather(const void *s, int n, MPI_Datatype t, void *r, int, MPI_Datatype, MPI_Comm) {
    if (s != MPI_IN_PLACE && s != r) std::memcpy(r, s, (size_t)n * mpi_stub_type_size(t));
    return 0;
}
static inline int MPI_Abort(MPI_Comm, int code) {
    std::fprintf(stderr, "oracle: reference called MPI_Abort(%d)\n", code);
    std::exit(3);
    return 0;
}
static inline int mpi_stub_unreachable(const char *what) {
    std::fprintf(stderr, "oracle: single-rank stub reached %s\n", what);
    std::abort();
    return 0;
}
static inline int MPI_Isend(const void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request *) {
    return mpi_stub_unreachable("MPI_Isend");
}
static inline int MPI_Irecv(void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request *) {
    return mpi_stub_unreachable("MPI_Irecv");
}
static inline int MPI_Send(const void *, int, MPI_Datatype, int, int, MPI_Comm) { return mpi_stub_unreachable("MPI_Send"); }
static inline int MPI_Recv(void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status *) {
    return mpi_stub_unreachable("MPI_Recv");
}
static inline int MPI_Wait(MPI_Request *, MPI_Status *) { return 0; }
static inline int MPI_Waitall(int, MPI_Request *, MPI_Status *) { return 0; }
static inline int MPI_Sendrecv(const void *, int, MPI_Datatype, int, int, void *, int, MPI_Datatype, int, int, MPI_Comm,
                               MPI_Status *) {
    return mpi_stub_unreachable("MPI_Sendrecv");
}
