/*
 * Single-rank MPI stand-in used only to compile the heFFTe reference (stock
 * backend) as a CPU oracle.  Test infrastructure: nothing in the product links
 * against it.
 *
 * It models exactly one process (rank 0 of a world of size 1).  Collectives
 * degenerate to local copies; point-to-point calls are only meaningful as
 * self-messages, which the single-rank heFFTe plans never issue
 * (heffte_reshape3d.h:512-528 builds no communicating reshape when the input
 * and output boxes of the only rank match).
 */
#ifndef GB300_ORACLE_MPI_SHIM_H
#define GB300_ORACLE_MPI_SHIM_H

#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int MPI_Comm;
typedef int MPI_Group;
typedef int MPI_Request;
typedef int MPI_Datatype; /* value = size of one element in bytes */
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_SUCCESS 0
#define MPI_COMM_WORLD 1
#define MPI_COMM_SELF 2
#define MPI_COMM_NULL 0
#define MPI_GROUP_NULL 0
#define MPI_STATUS_IGNORE ((MPI_Status*)0)
#define MPI_STATUSES_IGNORE ((MPI_Status*)0)
#define MPI_UNDEFINED (-32766)
#define MPI_REQUEST_NULL 0

#define MPI_BYTE 1
#define MPI_CHAR 1
#define MPI_INT 4
#define MPI_FLOAT 5           /* distinct tag; size resolved below */
#define MPI_DOUBLE 8
#define MPI_LONG_LONG 9
#define MPI_C_COMPLEX 10
#define MPI_C_DOUBLE_COMPLEX 16

#define MPI_SUM 0
#define MPI_MAX 1
#define MPI_MIN 2
typedef int MPI_Op;

static inline size_t gb300_shim_type_size(MPI_Datatype t){
    switch(t){
        case MPI_BYTE: return 1;
        case MPI_INT: return 4;
        case MPI_FLOAT: return 4;
        case MPI_DOUBLE: return 8;
        case MPI_LONG_LONG: return 8;
        case MPI_C_COMPLEX: return 8;
        case MPI_C_DOUBLE_COMPLEX: return 16;
        default: return (size_t)t;
    }
}

static inline int MPI_Init(int *argc, char ***argv){ (void)argc; (void)argv; return MPI_SUCCESS; }
static inline int MPI_Finalize(void){ return MPI_SUCCESS; }
static inline int MPI_Comm_rank(MPI_Comm c, int *r){ (void)c; *r = 0; return MPI_SUCCESS; }
static inline int MPI_Comm_size(MPI_Comm c, int *s){ (void)c; *s = 1; return MPI_SUCCESS; }
static inline int MPI_Comm_group(MPI_Comm c, MPI_Group *g){ (void)c; *g = 1; return MPI_SUCCESS; }
static inline int MPI_Group_incl(MPI_Group g, int n, const int *r, MPI_Group *ng){ (void)g; (void)r; *ng = (n > 0) ? 1 : 0; return MPI_SUCCESS; }
static inline int MPI_Comm_create(MPI_Comm c, MPI_Group g, MPI_Comm *nc){ (void)c; *nc = (g != 0) ? MPI_COMM_SELF : MPI_COMM_NULL; return MPI_SUCCESS; }
static inline int MPI_Group_free(MPI_Group *g){ *g = 0; return MPI_SUCCESS; }
static inline int MPI_Comm_free(MPI_Comm *c){ *c = MPI_COMM_NULL; return MPI_SUCCESS; }
static inline int MPI_Barrier(MPI_Comm c){ (void)c; return MPI_SUCCESS; }

static inline double MPI_Wtime(void){
    struct timespec ts; clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1.e-9 * (double)ts.tv_nsec;
}

static inline int MPI_Allgather(const void *s, int sc, MPI_Datatype st, void *r, int rc, MPI_Datatype rt, MPI_Comm c){
    (void)rc; (void)rt; (void)c;
    memcpy(r, s, (size_t)sc * gb300_shim_type_size(st));
    return MPI_SUCCESS;
}
static inline int MPI_Alltoall(const void *s, int sc, MPI_Datatype st, void *r, int rc, MPI_Datatype rt, MPI_Comm c){
    (void)rc; (void)rt; (void)c;
    memcpy(r, s, (size_t)sc * gb300_shim_type_size(st));
    return MPI_SUCCESS;
}
static inline int MPI_Alltoallv(const void *s, const int *sc, const int *sd, MPI_Datatype st,
                                void *r, const int *rc, const int *rd, MPI_Datatype rt, MPI_Comm c){
    (void)rc; (void)rt; (void)c;
    size_t es = gb300_shim_type_size(st);
    memcpy((char*)r + (size_t)rd[0] * es, (const char*)s + (size_t)sd[0] * es, (size_t)sc[0] * es);
    return MPI_SUCCESS;
}
static inline int MPI_Allreduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op op, MPI_Comm c){
    (void)op; (void)c;
    if (s != r) memcpy(r, s, (size_t)n * gb300_shim_type_size(t));
    return MPI_SUCCESS;
}
static inline int MPI_Reduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op op, int root, MPI_Comm c){
    (void)root; return MPI_Allreduce(s, r, n, t, op, c);
}
static inline void gb300_shim_p2p_abort(const char *name){
    fprintf(stderr, "single-rank MPI stand-in: %s is not available\n", name);
    abort();
}
static inline int MPI_Send(const void *b, int n, MPI_Datatype t, int d, int tag, MPI_Comm c){
    (void)b; (void)n; (void)t; (void)d; (void)tag; (void)c; gb300_shim_p2p_abort("MPI_Send"); return 1;
}
static inline int MPI_Isend(const void *b, int n, MPI_Datatype t, int d, int tag, MPI_Comm c, MPI_Request *q){
    (void)b; (void)n; (void)t; (void)d; (void)tag; (void)c; (void)q; gb300_shim_p2p_abort("MPI_Isend"); return 1;
}
static inline int MPI_Irecv(void *b, int n, MPI_Datatype t, int s, int tag, MPI_Comm c, MPI_Request *q){
    (void)b; (void)n; (void)t; (void)s; (void)tag; (void)c; (void)q; gb300_shim_p2p_abort("MPI_Irecv"); return 1;
}
static inline int MPI_Waitany(int n, MPI_Request *q, int *i, MPI_Status *st){
    (void)n; (void)q; (void)i; (void)st; gb300_shim_p2p_abort("MPI_Waitany"); return 1;
}
static inline int MPI_Waitall(int n, MPI_Request *q, MPI_Status *st){
    (void)n; (void)q; (void)st; return MPI_SUCCESS;
}

#ifdef __cplusplus
}
#endif

#endif
