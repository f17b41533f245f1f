/* Single-rank MPI stand-in (see mpi.h).  Oracle build only. */
#include "mpi.h"

#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

static size_t tsize(MPI_Datatype t) { return (size_t)(t / 16); }

/* Derived datatypes: a vector of `count` blocks of `blocklen` base elements,
 * blocks `stride` base extents apart, optionally resized to `extent` bytes.
 * A message of n items of a type is the ordered list of its basic elements;
 * single-rank collectives copy that list from the send to the receive side. */
struct dtype
{
    int used, kind; /* kind 1 vector, 2 resized */
    MPI_Datatype base;
    int count, blocklen, stride;
    long extent;
};
static struct dtype dtab[64];

static long textent(MPI_Datatype t)
{
    if (t >= 0) return (long)tsize(t);
    const struct dtype* d = &dtab[-t - 1];
    if (d->kind == 2) return d->extent;
    return ((long)(d->count - 1) * d->stride + d->blocklen) * textent(d->base);
}

/* append the byte offsets (relative to off) of the basic elements of one item */
static void telems(MPI_Datatype t, long off, long** list, size_t* n, size_t* cap, size_t* esz)
{
    if (t >= 0)
    {
        if (*n == *cap)
        {
            *cap = *cap ? 2 * *cap : 1024;
            *list = realloc(*list, *cap * sizeof(long));
        }
        (*list)[(*n)++] = off;
        *esz = tsize(t);
        return;
    }
    const struct dtype* d = &dtab[-t - 1];
    if (d->kind == 2)
    {
        telems(d->base, off, list, n, cap, esz);
        return;
    }
    const long be = textent(d->base);
    for (int c = 0; c < d->count; ++c)
        for (int b = 0; b < d->blocklen; ++b) telems(d->base, off + ((long)c * d->stride + b) * be, list, n, cap, esz);
}

static void typed_copy(void* r, long roff, int rn, MPI_Datatype rt, const void* s, long soff, int sn, MPI_Datatype st)
{
    long *ls = NULL, *lr = NULL;
    size_t ns = 0, cs = 0, nr = 0, cr = 0, es = 0, er = 0;
    for (int j = 0; j < sn; ++j) telems(st, soff + j * textent(st), &ls, &ns, &cs, &es);
    for (int j = 0; j < rn; ++j) telems(rt, roff + j * textent(rt), &lr, &nr, &cr, &er);
    size_t n = ns < nr ? ns : nr;
    for (size_t i = 0; i < n; ++i) memcpy((char*)r + lr[i], (const char*)s + ls[i], es);
    free(ls);
    free(lr);
}

int MPI_Type_vector(int count, int blocklength, int stride, MPI_Datatype oldtype, MPI_Datatype* newtype)
{
    for (int i = 0; i < 64; ++i)
        if (!dtab[i].used)
        {
            dtab[i] = (struct dtype){1, 1, oldtype, count, blocklength, stride, 0};
            *newtype = -(i + 1);
            return 0;
        }
    return 1;
}
int MPI_Type_create_resized(MPI_Datatype oldtype, MPI_Aint lb, MPI_Aint extent, MPI_Datatype* newtype)
{
    (void)lb;
    for (int i = 0; i < 64; ++i)
        if (!dtab[i].used)
        {
            dtab[i] = (struct dtype){1, 2, oldtype, 0, 0, 0, (long)extent};
            *newtype = -(i + 1);
            return 0;
        }
    return 1;
}
int MPI_Type_commit(MPI_Datatype* datatype) { (void)datatype; return 0; }
int MPI_Type_free(MPI_Datatype* datatype)
{
    if (*datatype < 0) dtab[-*datatype - 1].used = 0;
    *datatype = 0;
    return 0;
}

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
    (void)root; (void)comm;
    if (st < 0 || rt < 0)
    {
        if (r) typed_copy(r, (long)displs[0] * textent(rt), rcs[0], rt, s, 0, sc, st);
        return 0;
    }
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
    (void)root; (void)comm;
    if (st < 0 || rt < 0)
    {
        if (s) typed_copy(r, 0, rc, rt, s, (long)displs[0] * textent(st), scs[0], st);
        return 0;
    }
    (void)rc; (void)rt;
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

int MPI_File_open(MPI_Comm comm, const char* filename, int amode, MPI_Info info, MPI_File* fh)
{
    (void)comm; (void)info;
    if (amode != MPI_MODE_RDONLY) return 1;
    FILE* f = fopen(filename, "rb");
    *fh = f;
    return f ? MPI_SUCCESS : 1;
}
int MPI_File_read_at_all(MPI_File fh, MPI_Offset offset, void* buf, int count, MPI_Datatype t, MPI_Status* status)
{
    (void)status;
    FILE* f = (FILE*)fh;
    if (fseek(f, (long)offset, SEEK_SET)) return 1;
    const size_t n = (size_t)count * tsize(t);
    return fread(buf, 1, n, f) == n ? MPI_SUCCESS : 1;
}
int MPI_File_close(MPI_File* fh)
{
    int e = fclose((FILE*)*fh);
    *fh = NULL;
    return e ? 1 : MPI_SUCCESS;
}
