/* Single-rank MPI stand-in (see mpi.h).  Oracle build only. */
#include "mpi.h"

#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

static size_t tsize(MPI_Datatype t) { return (size_t)(t / 16); }

static void cp(void* dst, const void* src, size_t n)
{
    if (src == MPI_IN_PLACE || src == NULL || dst == NULL || dst == src || n == 0) return;
    memmove(dst, src, n);
}

int MPI_Init(int* argc, char*** argv) { (void)argc; (void)argv; return 0; }
int MPI_Finalize(void) { return 0; }
int MPI_Comm_size(MPI_Comm comm, int* size) { (void)comm; *size = 1; return 0; }
int MPI_Comm_rank(MPI_Comm comm, int* rank) { (void)comm; *rank = 0; return 0; }
int MPI_Comm_split(MPI_Comm comm, int color, int key, MPI_Comm* newcomm)
{
    (void)color; (void)key; *newcomm = comm; return 0;
}
int MPI_Comm_free(MPI_Comm* comm) { *comm = MPI_COMM_NULL; return 0; }
int MPI_Barrier(MPI_Comm comm) { (void)comm; return 0; }
int MPI_Bcast(void* buf, int count, MPI_Datatype t, int root, MPI_Comm comm)
{
    (void)buf; (void)count; (void)t; (void)root; (void)comm; return 0;
}
int MPI_Reduce(const void* s, void* r, int count, MPI_Datatype t, MPI_Op op, int root, MPI_Comm comm)
{
    (void)op; (void)root; (void)comm; cp(r, s, (size_t)count * tsize(t)); return 0;
}
int MPI_Allreduce(const void* s, void* r, int count, MPI_Datatype t, MPI_Op op, MPI_Comm comm)
{
    (void)op; (void)comm; cp(r, s, (size_t)count * tsize(t)); return 0;
}
int MPI_Gather(const void* s, int sc, MPI_Datatype st, void* r, int rc, MPI_Datatype rt, int root, MPI_Comm comm)
{
    (void)rc; (void)rt; (void)root; (void)comm; cp(r, s, (size_t)sc * tsize(st)); return 0;
}
int MPI_Gatherv(const void* s, int sc, MPI_Datatype st, void* r, const int* rcs, const int* displs,
                MPI_Datatype rt, int root, MPI_Comm comm)
{
    (void)rcs; (void)root; (void)comm;
    if (r) cp((char*)r + (size_t)displs[0] * tsize(rt), s, (size_t)sc * tsize(st));
    return 0;
}
int MPI_Scatter(const void* s, int sc, MPI_Datatype st, void* r, int rc, MPI_Datatype rt, int root, MPI_Comm comm)
{
    (void)rc; (void)rt; (void)root; (void)comm; cp(r, s, (size_t)sc * tsize(st)); return 0;
}
int MPI_Scatterv(const void* s, const int* scs, const int* displs, MPI_Datatype st, void* r, int rc,
                 MPI_Datatype rt, int root, MPI_Comm comm)
{
    (void)rc; (void)rt; (void)root; (void)comm;
    if (s) cp(r, (const char*)s + (size_t)displs[0] * tsize(st), (size_t)scs[0] * tsize(st));
    return 0;
}
int MPI_Allgather(const void* s, int sc, MPI_Datatype st, void* r, int rc, MPI_Datatype rt, MPI_Comm comm)
{
    (void)rc; (void)rt; (void)comm; cp(r, s, (size_t)sc * tsize(st)); return 0;
}
int MPI_Allgatherv(const void* s, int sc, MPI_Datatype st, void* r, const int* rcs, const int* displs,
                   MPI_Datatype rt, MPI_Comm comm)
{
    (void)rcs; (void)comm; cp((char*)r + (size_t)displs[0] * tsize(rt), s, (size_t)sc * tsize(st)); return 0;
}
int MPI_Alltoallv(const void* s, const int* scs, const int* sdispls, MPI_Datatype st, void* r, const int* rcs,
                  const int* rdispls, MPI_Datatype rt, MPI_Comm comm)
{
    (void)rcs; (void)comm;
    cp((char*)r + (size_t)rdispls[0] * tsize(rt), (const char*)s + (size_t)sdispls[0] * tsize(st),
       (size_t)scs[0] * tsize(st));
    return 0;
}
double MPI_Wtime(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}
int MPI_Abort(MPI_Comm comm, int code)
{
    (void)comm;
    fprintf(stderr, "MPI_Abort(%d)\n", code);
    exit(code ? code : 1);
}
int MPI_Error_string(int code, char* str, int* len)
{
    *len = snprintf(str, MPI_MAX_ERROR_STRING, "single-rank MPI stand-in error %d", code);
    return 0;
}
