/* Test infrastructure (oracle build only).
 *
 * A single-rank stand-in for the MPI calls that the reference's solver and
 * loader make, so that its own sources compile and run in one process with
 * OpenMP only.  Semantics for one rank:
 *   - Comm_rank = 0, Comm_size = 1, Wtime = omp_get_wtime;
 *   - (I)Allreduce with MPI_IN_PLACE leaves the buffer as is (sum over one rank);
 *     with a separate send buffer it copies count elements;
 *   - (I)Allgatherv copies the send buffer to recvbuf + displs[0] (memmove);
 *   - Wait / Waitsome / Isend / Irecv / Barrier do nothing.
 * Every Allgatherv also calls an optional hook with its send pointer; the
 * oracle's driver uses it to follow which shift is the seed (the reference
 * gathers the seed's search vector once per iteration and after a switch,
 * src/solver_dynamic.c:115,230,352) without touching the reference's code.
 */
#ifndef HBICG_ORACLE_MPI_SHIM_H
#define HBICG_ORACLE_MPI_SHIM_H

#include <string.h>
#include <omp.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Request;
typedef struct { int MPI_SOURCE; int MPI_TAG; int MPI_ERROR; } MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_DOUBLE 8
#define MPI_INT 4
#define MPI_CHAR 1
#define MPI_SUM 0
#define MPI_IN_PLACE ((void *)1)
#define MPI_STATUS_IGNORE ((MPI_Status *)0)
#define MPI_THREAD_FUNNELED 1
#define MPI_MAX_PROCESSOR_NAME 64
#define MPI_SUCCESS 0

/* Hook called on every Allgatherv/Iallgatherv with the send pointer. */
extern void (*hbicg_shim_gather_hook)(const void *sendbuf, int count);

static inline int MPI_Comm_rank(MPI_Comm c, int *r) { (void)c; *r = 0; return 0; }
static inline int MPI_Comm_size(MPI_Comm c, int *s) { (void)c; *s = 1; return 0; }
static inline double MPI_Wtime(void) { return omp_get_wtime(); }
static inline int MPI_Barrier(MPI_Comm c) { (void)c; return 0; }
static inline int MPI_Init(int *argc, char ***argv) { (void)argc; (void)argv; return 0; }
static inline int MPI_Init_thread(int *argc, char ***argv, int req, int *prov) {
    (void)argc; (void)argv; *prov = req; return 0;
}
static inline int MPI_Finalize(void) { return 0; }
static inline int MPI_Get_processor_name(char *name, int *len) {
    strcpy(name, "oracle"); *len = 6; return 0;
}

static inline int MPI_Allreduce(const void *s, void *r, int count, MPI_Datatype t, MPI_Op op, MPI_Comm c) {
    (void)op; (void)c;
    if (s != MPI_IN_PLACE) memmove(r, s, (size_t)count * (size_t)t);
    return 0;
}
static inline int MPI_Iallreduce(const void *s, void *r, int count, MPI_Datatype t, MPI_Op op, MPI_Comm c,
                                 MPI_Request *req) {
    *req = 0;
    return MPI_Allreduce(s, r, count, t, op, c);
}
static inline int MPI_Allgatherv(const void *s, int scount, MPI_Datatype st, void *r, const int *rcounts,
                                 const int *displs, MPI_Datatype rt, MPI_Comm c) {
    (void)rcounts; (void)rt; (void)c;
    if (hbicg_shim_gather_hook) hbicg_shim_gather_hook(s, scount);
    memmove((char *)r + (size_t)displs[0] * (size_t)st, s, (size_t)scount * (size_t)st);
    return 0;
}
static inline int MPI_Iallgatherv(const void *s, int scount, MPI_Datatype st, void *r, const int *rcounts,
                                  const int *displs, MPI_Datatype rt, MPI_Comm c, MPI_Request *req) {
    *req = 0;
    return MPI_Allgatherv(s, scount, st, r, rcounts, displs, rt, c);
}
static inline int MPI_Gather(const void *s, int sc, MPI_Datatype st, void *r, int rc, MPI_Datatype rt, int root,
                             MPI_Comm c) {
    (void)rc; (void)rt; (void)root; (void)c;
    memmove(r, s, (size_t)sc * (size_t)st);
    return 0;
}
static inline int MPI_Wait(MPI_Request *req, MPI_Status *st) { (void)req; (void)st; return 0; }
static inline int MPI_Waitsome(int n, MPI_Request *reqs, int *done, int *idx, MPI_Status *st) {
    (void)reqs; (void)idx; (void)st; *done = n; return 0;
}
static inline int MPI_Isend(const void *b, int n, MPI_Datatype t, int dst, int tag, MPI_Comm c, MPI_Request *r) {
    (void)b; (void)n; (void)t; (void)dst; (void)tag; (void)c; *r = 0; return 0;
}
static inline int MPI_Irecv(void *b, int n, MPI_Datatype t, int src, int tag, MPI_Comm c, MPI_Request *r) {
    (void)b; (void)n; (void)t; (void)src; (void)tag; (void)c; *r = 0; return 0;
}

#endif
