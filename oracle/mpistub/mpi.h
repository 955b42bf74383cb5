/* Single-rank MPI stand-in used only to compile the reference's header
 * templates for the oracle.  It is test infrastructure: no product code
 * includes it.  Every communicator has exactly one rank, so each collective
 * or point-to-point exchange degenerates to a copy of the caller's own
 * buffer, and window/file/request calls are no-ops.  Only the subset of the
 * MPI-3 C API named by the reference's headers is provided.               */
#ifndef GBC_ORACLE_MPI_STUB_H
#define GBC_ORACLE_MPI_STUB_H

#include <stddef.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int MPI_Comm;
typedef int MPI_Group;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Win;
typedef int MPI_File;
typedef int MPI_Info;
typedef int MPI_Request;
typedef int64_t MPI_Aint;
typedef int64_t MPI_Offset;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; int count; } MPI_Status;
typedef void (MPI_User_function)(void *, void *, int *, MPI_Datatype *);

#define MPI_SUCCESS 0
#define MPI_COMM_WORLD 1
#define MPI_COMM_SELF 2
#define MPI_COMM_NULL 0
#define MPI_GROUP_NULL 0
#define MPI_REQUEST_NULL 0
#define MPI_INFO_NULL 0
#define MPI_OP_NULL 0
#define MPI_DATATYPE_NULL 0
#define MPI_IDENT 0
#define MPI_CONGRUENT 1
#define MPI_SIMILAR 2
#define MPI_UNEQUAL 3
#define MPI_MAX_ERROR_STRING 256
#define MPI_LOCK_SHARED 1
#define MPI_LOCK_EXCLUSIVE 2
#define MPI_MODE_NOCHECK 1
#define MPI_MODE_NOSTORE 2
#define MPI_MODE_NOPUT 4
#define MPI_MODE_NOPRECEDE 8
#define MPI_MODE_NOSUCCEED 16
#define MPI_MODE_RDONLY 2
#define MPI_MODE_WRONLY 4
#define MPI_MODE_CREATE 1
#define MPI_THREAD_SINGLE 0
#define MPI_THREAD_FUNNELED 1
#define MPI_THREAD_SERIALIZED 2
#define MPI_THREAD_MULTIPLE 3
#define MPI_ANY_SOURCE (-1)
#define MPI_ANY_TAG (-1)
#define MPI_UNDEFINED (-32766)
#define MPI_STATUS_IGNORE ((MPI_Status *)0)
#define MPI_STATUSES_IGNORE ((MPI_Status *)0)
#define MPI_IN_PLACE ((void *)1)

/* operations (the single rank never combines anything) */
#define MPI_MAX 1
#define MPI_MIN 2
#define MPI_SUM 3
#define MPI_PROD 4
#define MPI_LAND 5
#define MPI_BAND 6
#define MPI_LOR 7
#define MPI_BOR 8
#define MPI_LXOR 9
#define MPI_BXOR 10

/* predefined datatypes: the handle indexes a size table */
#define MPI_CHAR 1
#define MPI_SHORT 2
#define MPI_INT 3
#define MPI_LONG 4
#define MPI_LONG_LONG_INT 5
#define MPI_LONG_LONG 5
#define MPI_UNSIGNED_CHAR 6
#define MPI_UNSIGNED_SHORT 7
#define MPI_UNSIGNED 8
#define MPI_UNSIGNED_LONG 9
#define MPI_UNSIGNED_LONG_LONG 10
#define MPI_FLOAT 11
#define MPI_DOUBLE 12
#define MPI_LONG_DOUBLE 13
#define MPI_BYTE 14
#define MPI_C_BOOL 15
#define MPI_CXX_BOOL 15
#define MPI_INT8_T 16
#define MPI_INT16_T 17
#define MPI_INT32_T 18
#define MPI_INT64_T 19
#define MPI_UINT8_T 20
#define MPI_UINT16_T 21
#define MPI_UINT32_T 22
#define MPI_UINT64_T 23
#define MPI_SIGNED_CHAR 24
#define MPI_WCHAR 25
#define MPI_DOUBLE_INT 26
#define MPI_2INT 27
#define MPI_FLOAT_INT 28
#define MPI_LONG_INT 29
#define MPI_SHORT_INT 30
#define MPI_LONG_DOUBLE_INT 31
#define GBC_STUB_NTYPES 4096

__attribute__((weak)) size_t *gbc_stub_type_table(void)
{
    static size_t sizes[GBC_STUB_NTYPES];
    static int next = 64;
    static int init = 0;
    if (!init) {
        init = 1;
        sizes[MPI_CHAR] = 1; sizes[MPI_SHORT] = sizeof(short); sizes[MPI_INT] = sizeof(int);
        sizes[MPI_LONG] = sizeof(long); sizes[MPI_LONG_LONG] = sizeof(long long);
        sizes[MPI_UNSIGNED_CHAR] = 1; sizes[MPI_UNSIGNED_SHORT] = sizeof(unsigned short);
        sizes[MPI_UNSIGNED] = sizeof(unsigned); sizes[MPI_UNSIGNED_LONG] = sizeof(unsigned long);
        sizes[MPI_UNSIGNED_LONG_LONG] = sizeof(unsigned long long); sizes[MPI_FLOAT] = sizeof(float);
        sizes[MPI_DOUBLE] = sizeof(double); sizes[MPI_LONG_DOUBLE] = sizeof(long double);
        sizes[MPI_BYTE] = 1; sizes[MPI_C_BOOL] = 1; sizes[MPI_INT8_T] = 1; sizes[MPI_INT16_T] = 2;
        sizes[MPI_INT32_T] = 4; sizes[MPI_INT64_T] = 8; sizes[MPI_UINT8_T] = 1; sizes[MPI_UINT16_T] = 2;
        sizes[MPI_UINT32_T] = 4; sizes[MPI_UINT64_T] = 8; sizes[MPI_SIGNED_CHAR] = 1; sizes[MPI_WCHAR] = 4;
        sizes[MPI_DOUBLE_INT] = 16; sizes[MPI_2INT] = 8; sizes[MPI_FLOAT_INT] = 8; sizes[MPI_LONG_INT] = 16; sizes[MPI_SHORT_INT] = 8; sizes[MPI_LONG_DOUBLE_INT] = 32;
        sizes[0] = (size_t)next; /* slot 0 keeps the next free handle */
    }
    return sizes;
}
static inline size_t gbc_stub_tsize(MPI_Datatype t)
{
    size_t *s = gbc_stub_type_table();
    if (t <= 0 || t >= GBC_STUB_NTYPES || s[t] == 0) {
        fprintf(stderr, "mpi stub: unknown datatype %d\n", t);
        abort();
    }
    return s[t];
}
static inline void gbc_stub_copy(const void *src, void *dst, long long count, MPI_Datatype t)
{
    if (src == MPI_IN_PLACE || dst == MPI_IN_PLACE || src == dst || count <= 0) return;
    memmove(dst, src, (size_t)count * gbc_stub_tsize(t));
}

static inline int MPI_Init(int *argc, char ***argv) { (void)argc; (void)argv; return 0; }
static inline int MPI_Init_thread(int *argc, char ***argv, int req, int *prov) { (void)argc; (void)argv; *prov = req; return 0; }
static inline int MPI_Finalize(void) { return 0; }
static inline int MPI_Finalized(int *flag) { *flag = 0; return 0; }
static inline int MPI_Initialized(int *flag) { *flag = 1; return 0; }
static inline int MPI_Abort(MPI_Comm c, int code) { (void)c; fprintf(stderr, "MPI_Abort(%d)\n", code); exit(code ? code : 1); }
static inline double MPI_Wtime(void) { struct timespec ts; clock_gettime(CLOCK_MONOTONIC, &ts); return ts.tv_sec + 1e-9 * ts.tv_nsec; }
static inline int MPI_Error_string(int code, char *s, int *len) { *len = snprintf(s, MPI_MAX_ERROR_STRING, "mpi stub error %d", code); return 0; }
static inline int MPI_Pcontrol(const int level, ...) { (void)level; return 0; }

static inline int MPI_Comm_rank(MPI_Comm c, int *r) { (void)c; *r = 0; return 0; }
static inline int MPI_Comm_size(MPI_Comm c, int *s) { (void)c; *s = 1; return 0; }
static inline int MPI_Comm_split(MPI_Comm c, int color, int key, MPI_Comm *out) { (void)c; (void)color; (void)key; *out = MPI_COMM_SELF; return 0; }
static inline int MPI_Comm_dup(MPI_Comm c, MPI_Comm *out) { *out = c; return 0; }
static inline int MPI_Comm_free(MPI_Comm *c) { *c = MPI_COMM_NULL; return 0; }
static inline int MPI_Comm_compare(MPI_Comm a, MPI_Comm b, int *res) { (void)a; (void)b; *res = MPI_CONGRUENT; return 0; }
static inline int MPI_Comm_group(MPI_Comm c, MPI_Group *g) { (void)c; *g = 1; return 0; }
static inline int MPI_Comm_create(MPI_Comm c, MPI_Group g, MPI_Comm *out) { (void)g; *out = c; return 0; }
static inline int MPI_Group_incl(MPI_Group g, int n, const int *r, MPI_Group *out) { (void)n; (void)r; *out = g; return 0; }
static inline int MPI_Group_excl(MPI_Group g, int n, const int *r, MPI_Group *out) { (void)n; (void)r; *out = g; return 0; }
static inline int MPI_Group_free(MPI_Group *g) { *g = MPI_GROUP_NULL; return 0; }
static inline int MPI_Barrier(MPI_Comm c) { (void)c; return 0; }

static inline int MPI_Type_contiguous(int count, MPI_Datatype old, MPI_Datatype *out)
{
    size_t *s = gbc_stub_type_table();
    int h = (int)s[0];
    if (h >= GBC_STUB_NTYPES) { fprintf(stderr, "mpi stub: too many datatypes\n"); abort(); }
    s[h] = (size_t)count * gbc_stub_tsize(old);
    s[0] = (size_t)(h + 1);
    *out = h;
    return 0;
}
static inline int MPI_Type_create_struct(int n, const int *bl, const MPI_Aint *disp, const MPI_Datatype *types, MPI_Datatype *out)
{
    /* size = end of the furthest block; enough for the reference's struct types */
    size_t *s = gbc_stub_type_table();
    size_t end = 0;
    for (int i = 0; i < n; ++i) { size_t e = (size_t)disp[i] + (size_t)bl[i] * gbc_stub_tsize(types[i]); if (e > end) end = e; }
    int h = (int)s[0];
    s[h] = end; s[0] = (size_t)(h + 1); *out = h;
    return 0;
}
static inline int MPI_Type_commit(MPI_Datatype *t) { (void)t; return 0; }
static inline int MPI_Type_free(MPI_Datatype *t) { *t = MPI_DATATYPE_NULL; return 0; }
static inline int MPI_Type_size(MPI_Datatype t, int *sz) { *sz = (int)gbc_stub_tsize(t); return 0; }
static inline int MPI_Get_count(const MPI_Status *st, MPI_Datatype t, int *c) { (void)t; *c = st ? st->count : 0; return 0; }
static inline int MPI_Op_create(MPI_User_function *f, int commute, MPI_Op *op) { (void)f; (void)commute; *op = 100; return 0; }
static inline int MPI_Op_free(MPI_Op *op) { *op = MPI_OP_NULL; return 0; }

static inline int MPI_Bcast(void *b, int n, MPI_Datatype t, int root, MPI_Comm c) { (void)b; (void)n; (void)t; (void)root; (void)c; return 0; }
static inline int MPI_Ibcast(void *b, int n, MPI_Datatype t, int root, MPI_Comm c, MPI_Request *r) { (void)b; (void)n; (void)t; (void)root; (void)c; *r = 0; return 0; }
static inline int MPI_Reduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op op, int root, MPI_Comm c) { (void)op; (void)root; (void)c; gbc_stub_copy(s, r, n, t); return 0; }
static inline int MPI_Allreduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op op, MPI_Comm c) { (void)op; (void)c; gbc_stub_copy(s, r, n, t); return 0; }
static inline int MPI_Scan(const void *s, void *r, int n, MPI_Datatype t, MPI_Op op, MPI_Comm c) { (void)op; (void)c; gbc_stub_copy(s, r, n, t); return 0; }
static inline int MPI_Exscan(const void *s, void *r, int n, MPI_Datatype t, MPI_Op op, MPI_Comm c) { (void)s; (void)r; (void)n; (void)t; (void)op; (void)c; return 0; }
static inline int MPI_Reduce_scatter(const void *s, void *r, const int *counts, MPI_Datatype t, MPI_Op op, MPI_Comm c) { (void)op; (void)c; gbc_stub_copy(s, r, counts[0], t); return 0; }
static inline int MPI_Allgather(const void *s, int sn, MPI_Datatype st, void *r, int rn, MPI_Datatype rt, MPI_Comm c) { (void)rn; (void)rt; (void)c; gbc_stub_copy(s, r, sn, st); return 0; }
static inline int MPI_Allgatherv(const void *s, int sn, MPI_Datatype st, void *r, const int *rc, const int *rd, MPI_Datatype rt, MPI_Comm c)
{ (void)rc; (void)c; if (s != MPI_IN_PLACE) gbc_stub_copy(s, (char *)r + (size_t)rd[0] * gbc_stub_tsize(rt), sn, st); return 0; }
static inline int MPI_Gather(const void *s, int sn, MPI_Datatype st, void *r, int rn, MPI_Datatype rt, int root, MPI_Comm c) { (void)rn; (void)rt; (void)root; (void)c; gbc_stub_copy(s, r, sn, st); return 0; }
static inline int MPI_Gatherv(const void *s, int sn, MPI_Datatype st, void *r, const int *rc, const int *rd, MPI_Datatype rt, int root, MPI_Comm c)
{ (void)rc; (void)root; (void)c; if (s != MPI_IN_PLACE) gbc_stub_copy(s, (char *)r + (size_t)rd[0] * gbc_stub_tsize(rt), sn, st); return 0; }
static inline int MPI_Scatter(const void *s, int sn, MPI_Datatype st, void *r, int rn, MPI_Datatype rt, int root, MPI_Comm c) { (void)sn; (void)st; (void)root; (void)c; if (r != MPI_IN_PLACE) gbc_stub_copy(s, r, rn, rt); return 0; }
static inline int MPI_Scatterv(const void *s, const int *sc, const int *sd, MPI_Datatype st, void *r, int rn, MPI_Datatype rt, int root, MPI_Comm c)
{ (void)sc; (void)root; (void)c; if (r != MPI_IN_PLACE) gbc_stub_copy((const char *)s + (size_t)sd[0] * gbc_stub_tsize(st), r, rn, rt); return 0; }
static inline int MPI_Alltoall(const void *s, int sn, MPI_Datatype st, void *r, int rn, MPI_Datatype rt, MPI_Comm c) { (void)rn; (void)rt; (void)c; gbc_stub_copy(s, r, sn, st); return 0; }
static inline int MPI_Alltoallv(const void *s, const int *sc, const int *sd, MPI_Datatype st, void *r, const int *rc, const int *rd, MPI_Datatype rt, MPI_Comm c)
{
    (void)rc; (void)c;
    if (s == MPI_IN_PLACE) return 0;
    gbc_stub_copy((const char *)s + (size_t)sd[0] * gbc_stub_tsize(st), (char *)r + (size_t)rd[0] * gbc_stub_tsize(rt), sc[0], st);
    return 0;
}
static inline int MPI_Sendrecv(const void *s, int sn, MPI_Datatype st, int dest, int stag, void *r, int rn, MPI_Datatype rt, int src, int rtag, MPI_Comm c, MPI_Status *status)
{
    (void)dest; (void)stag; (void)rn; (void)rt; (void)src; (void)rtag; (void)c;
    gbc_stub_copy(s, r, sn, st);
    if (status) status->count = sn;
    return 0;
}
/* A single rank never sends to anyone but itself; the reference's 1x1 paths
 * never reach these, so a call means the stub is being used beyond its scope. */
static inline int gbc_stub_p2p(const char *what) { fprintf(stderr, "mpi stub: %s is not supported with one rank\n", what); abort(); }
static inline int MPI_Send(const void *b, int n, MPI_Datatype t, int d, int tag, MPI_Comm c) { (void)b; (void)n; (void)t; (void)d; (void)tag; (void)c; return gbc_stub_p2p("MPI_Send"); }
static inline int MPI_Recv(void *b, int n, MPI_Datatype t, int s, int tag, MPI_Comm c, MPI_Status *st) { (void)b; (void)n; (void)t; (void)s; (void)tag; (void)c; (void)st; return gbc_stub_p2p("MPI_Recv"); }
static inline int MPI_Isend(const void *b, int n, MPI_Datatype t, int d, int tag, MPI_Comm c, MPI_Request *r) { (void)b; (void)n; (void)t; (void)d; (void)tag; (void)c; (void)r; return gbc_stub_p2p("MPI_Isend"); }
static inline int MPI_Irecv(void *b, int n, MPI_Datatype t, int s, int tag, MPI_Comm c, MPI_Request *r) { (void)b; (void)n; (void)t; (void)s; (void)tag; (void)c; (void)r; return gbc_stub_p2p("MPI_Irecv"); }
static inline int MPI_Wait(MPI_Request *r, MPI_Status *s) { (void)r; (void)s; return 0; }
static inline int MPI_Test(MPI_Request *r, int *flag, MPI_Status *s) { (void)r; (void)s; *flag = 1; return 0; }
static inline int MPI_Waitall(int n, MPI_Request *r, MPI_Status *s) { (void)n; (void)r; (void)s; return 0; }

static inline int MPI_Win_create(void *b, MPI_Aint sz, int du, MPI_Info i, MPI_Comm c, MPI_Win *w) { (void)b; (void)sz; (void)du; (void)i; (void)c; *w = 1; return 0; }
static inline int MPI_Win_free(MPI_Win *w) { *w = 0; return 0; }
static inline int MPI_Win_fence(int a, MPI_Win w) { (void)a; (void)w; return 0; }
static inline int MPI_Win_lock(int lt, int r, int a, MPI_Win w) { (void)lt; (void)r; (void)a; (void)w; return 0; }
static inline int MPI_Win_unlock(int r, MPI_Win w) { (void)r; (void)w; return 0; }
static inline int MPI_Win_start(MPI_Group g, int a, MPI_Win w) { (void)g; (void)a; (void)w; return 0; }
static inline int MPI_Win_post(MPI_Group g, int a, MPI_Win w) { (void)g; (void)a; (void)w; return 0; }
static inline int MPI_Win_complete(MPI_Win w) { (void)w; return 0; }
static inline int MPI_Win_wait(MPI_Win w) { (void)w; return 0; }
static inline int MPI_Put(const void *o, int oc, MPI_Datatype ot, int tr, MPI_Aint td, int tc, MPI_Datatype tt, MPI_Win w) { (void)o; (void)oc; (void)ot; (void)tr; (void)td; (void)tc; (void)tt; (void)w; return gbc_stub_p2p("MPI_Put"); }
static inline int MPI_Get(void *o, int oc, MPI_Datatype ot, int tr, MPI_Aint td, int tc, MPI_Datatype tt, MPI_Win w) { (void)o; (void)oc; (void)ot; (void)tr; (void)td; (void)tc; (void)tt; (void)w; return gbc_stub_p2p("MPI_Get"); }
static inline int MPI_Info_create(MPI_Info *i) { *i = 1; return 0; }
static inline int MPI_Info_set(MPI_Info i, const char *k, const char *v) { (void)i; (void)k; (void)v; return 0; }
static inline int MPI_Info_free(MPI_Info *i) { *i = 0; return 0; }
static inline int MPI_File_open(MPI_Comm c, const char *n, int m, MPI_Info i, MPI_File *f) { (void)c; (void)n; (void)m; (void)i; (void)f; return gbc_stub_p2p("MPI_File_open"); }
static inline int MPI_File_close(MPI_File *f) { (void)f; return 0; }
static inline int MPI_File_set_view(MPI_File f, MPI_Offset d, MPI_Datatype e, MPI_Datatype ft, const char *rep, MPI_Info i) { (void)f; (void)d; (void)e; (void)ft; (void)rep; (void)i; return 0; }
static inline int MPI_File_write(MPI_File f, const void *b, int n, MPI_Datatype t, MPI_Status *s) { (void)f; (void)b; (void)n; (void)t; (void)s; return 0; }
static inline int MPI_File_write_all(MPI_File f, const void *b, int n, MPI_Datatype t, MPI_Status *s) { (void)f; (void)b; (void)n; (void)t; (void)s; return 0; }
static inline int MPI_File_read_at(MPI_File f, MPI_Offset o, void *b, int n, MPI_Datatype t, MPI_Status *s) { (void)f; (void)o; (void)b; (void)n; (void)t; (void)s; return 0; }

#ifdef __cplusplus
}
#endif
#endif
