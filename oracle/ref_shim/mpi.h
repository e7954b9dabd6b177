/*
 * Single-rank stand-in for <mpi.h>, used ONLY to compile the reference's
 * src/tet.cpp, src/volume.cpp and src/dense.cpp unmodified as a test oracle.
 * It is test infrastructure: nothing in the product links against it.
 *
 * Semantics are those of MPI with one rank: reductions copy the send buffer
 * to the receive buffer; point-to-point and MPI-IO calls are no-ops that
 * report success.  MPI_Reduce additionally records its last operands so the
 * oracle driver can read the statistics that dense_stats() reduces
 * (src/dense.cpp:1298-1300: max_dense, tot_mass, check_mass).
 */
#ifndef TESS_ORACLE_SHIM_MPI_H
#define TESS_ORACLE_SHIM_MPI_H

#include <string.h>
#include <stdio.h>
#include <stdlib.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Info;
typedef int MPI_File;
typedef int MPI_Request;
typedef struct { int count; } MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_SUCCESS 0
#define MPI_INT 4
#define MPI_FLOAT 5
#define MPI_DOUBLE 8
#define MPI_MIN 1
#define MPI_MAX 2
#define MPI_SUM 3
#define MPI_ORDER_C 0
#define MPI_MODE_WRONLY 1
#define MPI_MODE_CREATE 2
#define MPI_INFO_NULL 0
#define MPI_MAX_ERROR_STRING 64
#define MPI_ANY_SOURCE (-1)
#define MPI_STATUS_IGNORE ((MPI_Status*)0)
#define MPI_STATUSES_IGNORE ((MPI_Status*)0)

static inline size_t tess_shim_type_size(MPI_Datatype t)
{
    return t == MPI_DOUBLE ? 8 : 4;
}

/* last three MPI_Reduce calls, read back by the oracle driver */
struct tess_shim_reduce_log { double value[3]; int n; };
extern struct tess_shim_reduce_log tess_shim_reduce_record;

static inline int MPI_Init(int*, char***) { return 0; }
static inline int MPI_Finalize() { return 0; }
static inline int MPI_Comm_rank(MPI_Comm, int* r) { *r = 0; return 0; }
static inline int MPI_Comm_size(MPI_Comm, int* s) { *s = 1; return 0; }
static inline int MPI_Barrier(MPI_Comm) { return 0; }
static inline double MPI_Wtime() { return 0.0; }
static inline int MPI_Allreduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op, MPI_Comm)
{
    memmove(r, s, (size_t)n * tess_shim_type_size(t));
    return 0;
}
static inline int MPI_Reduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op, int, MPI_Comm)
{
    memmove(r, s, (size_t)n * tess_shim_type_size(t));
    if (n == 1 && tess_shim_reduce_record.n < 3)
    {
        double v = (t == MPI_DOUBLE) ? *(const double*)s
                 : (t == MPI_FLOAT) ? (double)*(const float*)s : (double)*(const int*)s;
        tess_shim_reduce_record.value[tess_shim_reduce_record.n++] = v;
    }
    return 0;
}
static inline int MPI_File_open(MPI_Comm, char*, int, MPI_Info, MPI_File* f) { *f = 0; return 0; }
static inline int MPI_File_set_size(MPI_File, long long) { return 0; }
static inline int MPI_File_set_view(MPI_File, long long, MPI_Datatype, MPI_Datatype, char*, MPI_Info) { return 0; }
static inline int MPI_File_write_all(MPI_File, const void*, int n, MPI_Datatype, MPI_Status* st)
{
    if (st) st->count = n;
    return 0;
}
static inline int MPI_File_close(MPI_File*) { return 0; }
static inline int MPI_Get_count(const MPI_Status* st, MPI_Datatype, int* c) { *c = st ? st->count : 0; return 0; }
static inline int MPI_Type_create_subarray(int, const int*, const int*, const int*, int, MPI_Datatype, MPI_Datatype* t) { *t = 0; return 0; }
static inline int MPI_Type_commit(MPI_Datatype*) { return 0; }
static inline int MPI_Type_free(MPI_Datatype*) { return 0; }
static inline int MPI_Isend(const void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request* r) { *r = 0; return 0; }
static inline int MPI_Recv(void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status*) { return 0; }
static inline int MPI_Waitall(int, MPI_Request*, MPI_Status*) { return 0; }
static inline int MPI_Error_string(int, char* s, int* len) { s[0] = 0; *len = 0; return 0; }
static inline int MPI_Abort(MPI_Comm, int code) { fprintf(stderr, "MPI_Abort(%d)\n", code); abort(); return 0; }

#endif
