/*
 * Single-rank stand-in for <mpi.h>, used ONLY to compile the reference's
 * src/tet.cpp, src/volume.cpp and src/dense.cpp unmodified as a test oracle.
 * It is test infrastructure: nothing in the product links against it.
 *
 * Semantics are those of MPI with one rank: reductions copy the send buffer
 * to the receive buffer; point-to-point calls are no-ops that report success
 * (with one rank, ProjectGrid never takes its send/receive branch).
 * MPI_Reduce additionally records its last operands so the oracle driver can
 * read the statistics that dense_stats() reduces (src/dense.cpp:1298-1300:
 * max_dense, tot_mass, check_mass).
 *
 * The MPI-IO calls WriteGrid makes (src/dense.cpp:751-870) do write the file:
 * MPI_File_open / set_size / close map to POSIX open / ftruncate / close, a
 * subarray filetype (MPI_Type_create_subarray, C order, up to 3 dimensions)
 * set as the view places each element of MPI_File_write_all at its offset in
 * the global array, and a plain MPI_FLOAT view writes nothing for count 0.
 */
#ifndef TESS_ORACLE_SHIM_MPI_H
#define TESS_ORACLE_SHIM_MPI_H

#include <string.h>
#include <stdio.h>
#include <stdlib.h>
#include <fcntl.h>
#include <unistd.h>

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
#define MPI_IN_PLACE ((void*)1)
static inline int MPI_Allreduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op, MPI_Comm)
{
    if (s != MPI_IN_PLACE)
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
/* subarray filetypes: handles 100 + slot */
struct tess_shim_subarray { int used, ndims, sizes[3], subsizes[3], starts[3]; };
static struct tess_shim_subarray tess_shim_types[16];
/* the one open file's view */
static int tess_shim_view = 0;
static long long tess_shim_disp = 0;

static inline int MPI_File_open(MPI_Comm, char* path, int, MPI_Info, MPI_File* f)
{
    *f = open(path, O_WRONLY | O_CREAT, 0644);
    tess_shim_view = 0;
    tess_shim_disp = 0;
    return *f >= 0 ? 0 : 1;
}
static inline int MPI_File_set_size(MPI_File f, long long n) { return ftruncate(f, (off_t)n) == 0 ? 0 : 1; }
static inline int MPI_File_set_view(MPI_File, long long disp, MPI_Datatype, MPI_Datatype filetype, char*, MPI_Info)
{
    tess_shim_view = filetype;
    tess_shim_disp = disp;
    return 0;
}
static inline int MPI_File_write_all(MPI_File f, const void* buf, int n, MPI_Datatype t, MPI_Status* st)
{
    const size_t es = tess_shim_type_size(t);
    if (st) st->count = n;
    if (n == 0) return 0;
    if (tess_shim_view < 100 || tess_shim_view >= 116 || !tess_shim_types[tess_shim_view - 100].used)
        return pwrite(f, buf, (size_t)n * es, (off_t)tess_shim_disp) == (ssize_t)((size_t)n * es) ? 0 : 1;
    const struct tess_shim_subarray* a = &tess_shim_types[tess_shim_view - 100];
    /* pad to 3 dimensions, slowest first (MPI_ORDER_C) */
    int sz[3] = { 1, 1, 1 }, sub[3] = { 1, 1, 1 }, st0[3] = { 0, 0, 0 };
    for (int i = 0; i < a->ndims; ++i)
    {
        sz[3 - a->ndims + i] = a->sizes[i];
        sub[3 - a->ndims + i] = a->subsizes[i];
        st0[3 - a->ndims + i] = a->starts[i];
    }
    const char* p = (const char*)buf;
    int done = 0;
    for (int i = 0; i < sub[0] && done < n; ++i)
        for (int j = 0; j < sub[1] && done < n; ++j)
        {
            int run = sub[2] < n - done ? sub[2] : n - done;
            long long off = (((long long)(st0[0] + i) * sz[1] + (st0[1] + j)) * sz[2] + st0[2]) * (long long)es;
            if (pwrite(f, p, (size_t)run * es, (off_t)(tess_shim_disp + off)) != (ssize_t)((size_t)run * es))
                return 1;
            p += (size_t)run * es;
            done += run;
        }
    return 0;
}
static inline int MPI_File_close(MPI_File* f) { int r = close(*f); *f = -1; return r == 0 ? 0 : 1; }
static inline int MPI_Get_count(const MPI_Status* st, MPI_Datatype, int* c) { *c = st ? st->count : 0; return 0; }
static inline int MPI_Type_create_subarray(int nd, const int* sizes, const int* subsizes, const int* starts, int,
                                           MPI_Datatype, MPI_Datatype* t)
{
    for (int k = 0; k < 16; ++k)
        if (!tess_shim_types[k].used && nd >= 1 && nd <= 3)
        {
            tess_shim_types[k].used = 1;
            tess_shim_types[k].ndims = nd;
            for (int i = 0; i < nd; ++i)
            {
                tess_shim_types[k].sizes[i] = sizes[i];
                tess_shim_types[k].subsizes[i] = subsizes[i];
                tess_shim_types[k].starts[i] = starts[i];
            }
            *t = 100 + k;
            return 0;
        }
    *t = 0;
    return 1;
}
static inline int MPI_Type_commit(MPI_Datatype*) { return 0; }
static inline int MPI_Type_free(MPI_Datatype* t)
{
    if (*t >= 100 && *t < 116) tess_shim_types[*t - 100].used = 0;
    *t = 0;
    return 0;
}
static inline int MPI_Isend(const void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request* r) { *r = 0; return 0; }
static inline int MPI_Recv(void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status*) { return 0; }
static inline int MPI_Waitall(int, MPI_Request*, MPI_Status*) { return 0; }
static inline int MPI_Error_string(int, char* s, int* len) { s[0] = 0; *len = 0; return 0; }
static inline int MPI_Abort(MPI_Comm, int code) { fprintf(stderr, "MPI_Abort(%d)\n", code); abort(); return 0; }

#endif
