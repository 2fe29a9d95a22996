// Single-rank stand-in for <mpi.h>, used only to compile the reference's
// exafac/cpp_ext headers on a machine without MPI (oracle/_ref build).
//
// Test infrastructure: nothing in the product links this file.
//
// Semantics: exactly one rank (rank 0, size 1).  Every collective is the
// identity on that rank: data is copied from the send buffer to the receive
// buffer (or left alone for MPI_IN_PLACE); Cartesian/sub-communicators alias
// their parent.  These are the semantics an MPI library gives a job of size 1,
// which is the configuration the single-GPU build replaces.
#pragma once

#include <chrono>
#include <cstdint>
#include <cstring>

typedef int MPI_Comm;
typedef int MPI_Group;
typedef int MPI_Datatype;
typedef int MPI_Op;
struct MPI_Status {
    int MPI_SOURCE;
    int MPI_TAG;
    int MPI_ERROR;
};

#define MPI_COMM_WORLD 0
#define MPI_STATUS_IGNORE ((MPI_Status*)0)
#define MPI_IN_PLACE ((void*)1)

#define MPI_SUM 1
#define MPI_MIN 2
#define MPI_MAX 3

#define MPI_DOUBLE 1
#define MPI_FLOAT 2
#define MPI_INT 3
#define MPI_INT32_T 4
#define MPI_INT64_T 5
#define MPI_UINT32_T 6
#define MPI_UINT64_T 7

static inline size_t oracle_mpi_type_size(MPI_Datatype t) {
    switch (t) {
        case MPI_DOUBLE: return 8;
        case MPI_FLOAT: return 4;
        case MPI_INT: return sizeof(int);
        case MPI_INT32_T: return 4;
        case MPI_INT64_T: return 8;
        case MPI_UINT32_T: return 4;
        case MPI_UINT64_T: return 8;
        default: return 1;
    }
}

static inline void oracle_mpi_copy(void* dst, const void* src, long count, MPI_Datatype t) {
    if (src == MPI_IN_PLACE || dst == src || count <= 0) return;
    std::memmove(dst, src, (size_t)count * oracle_mpi_type_size(t));
}

static inline int MPI_Comm_size(MPI_Comm, int* s) { *s = 1; return 0; }
static inline int MPI_Comm_rank(MPI_Comm, int* r) { *r = 0; return 0; }
static inline int MPI_Barrier(MPI_Comm) { return 0; }
static inline int MPI_Bcast(void*, int, MPI_Datatype, int, MPI_Comm) { return 0; }

static inline int MPI_Allreduce(const void* s, void* r, int count, MPI_Datatype t, MPI_Op, MPI_Comm) {
    oracle_mpi_copy(r, s, count, t);
    return 0;
}
static inline int MPI_Allgather(const void* s, int scount, MPI_Datatype st, void* r, int, MPI_Datatype, MPI_Comm) {
    oracle_mpi_copy(r, s, scount, st);
    return 0;
}
static inline int MPI_Allgatherv(const void* s, int scount, MPI_Datatype st, void* r, const int*,
                                 const int* displs, MPI_Datatype, MPI_Comm) {
    oracle_mpi_copy((char*)r + (size_t)displs[0] * oracle_mpi_type_size(st), s, scount, st);
    return 0;
}
static inline int MPI_Alltoall(const void* s, int scount, MPI_Datatype st, void* r, int, MPI_Datatype, MPI_Comm) {
    oracle_mpi_copy(r, s, scount, st);
    return 0;
}
static inline int MPI_Alltoallv(const void* s, const int* scounts, const int* sdispls, MPI_Datatype st, void* r,
                                const int*, const int* rdispls, MPI_Datatype, MPI_Comm) {
    size_t es = oracle_mpi_type_size(st);
    oracle_mpi_copy((char*)r + (size_t)rdispls[0] * es, (const char*)s + (size_t)sdispls[0] * es, scounts[0], st);
    return 0;
}
static inline int MPI_Reduce_scatter_block(const void* s, void* r, int count, MPI_Datatype t, MPI_Op, MPI_Comm) {
    oracle_mpi_copy(r, s, count, t);
    return 0;
}
static inline int MPI_Sendrecv(const void* s, int scount, MPI_Datatype st, int, int, void* r, int, MPI_Datatype, int,
                               int, MPI_Comm, MPI_Status*) {
    oracle_mpi_copy(r, s, scount, st);
    return 0;
}
static inline int MPI_Cart_create(MPI_Comm c, int, const int*, const int*, int, MPI_Comm* out) { *out = c; return 0; }
static inline int MPI_Cart_get(MPI_Comm, int n, int* dims, int* periods, int* coords) {
    for (int i = 0; i < n; i++) { dims[i] = 1; periods[i] = 0; coords[i] = 0; }
    return 0;
}
static inline int MPI_Cart_sub(MPI_Comm c, const int*, MPI_Comm* out) { *out = c; return 0; }
static inline int MPI_Comm_group(MPI_Comm, MPI_Group* g) { *g = 0; return 0; }
static inline int MPI_Group_incl(MPI_Group, int, const int*, MPI_Group* g) { *g = 0; return 0; }
static inline int MPI_Comm_create_group(MPI_Comm c, MPI_Group, int, MPI_Comm* out) { *out = c; return 0; }
static inline double MPI_Wtime() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}
