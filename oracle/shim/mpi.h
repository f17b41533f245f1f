/* Single-rank stand-in for the MPI API, written from the MPI standard's
 * signatures.  It lets the reference's hot-path sources compile and run as
 * one process (nkpool = nqpool = 1, one plane-wave rank).  Collectives
 * degenerate to copies from the send to the receive buffer.
 * Oracle build only: test infrastructure, never linked into the product. */
#pragma once
#include <stddef.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;

#define MPI_SUCCESS 0
#define MPI_MAX_ERROR_STRING 256
#define MPI_COMM_WORLD ((MPI_Comm)1)
#define MPI_COMM_NULL ((MPI_Comm)0)
#define MPI_IN_PLACE ((void*)1)
#define MPI_THREAD_FUNNELED 1

/* datatype code = 16 * size_in_bytes + id */
#define MPI_INT ((MPI_Datatype)(16 * 4 + 1))
#define MPI_LONG_LONG_INT ((MPI_Datatype)(16 * 8 + 2))
#define MPI_LONG_LONG MPI_LONG_LONG_INT
#define MPI_DOUBLE ((MPI_Datatype)(16 * 8 + 3))
#define MPI_FLOAT ((MPI_Datatype)(16 * 4 + 4))
#define MPI_C_DOUBLE_COMPLEX ((MPI_Datatype)(16 * 16 + 5))
#define MPI_C_FLOAT_COMPLEX ((MPI_Datatype)(16 * 8 + 6))
#define MPI_C_BOOL ((MPI_Datatype)(16 * 1 + 7))
#define MPI_CHAR ((MPI_Datatype)(16 * 1 + 8))

#define MPI_SUM ((MPI_Op)1)
#define MPI_MAX ((MPI_Op)2)
#define MPI_MIN ((MPI_Op)3)
#define MPI_LOR ((MPI_Op)4)
#define MPI_LAND ((MPI_Op)5)

typedef long MPI_Aint;
/* derived datatypes (vector, resized) get negative handles */
int MPI_Type_vector(int count, int blocklength, int stride, MPI_Datatype oldtype, MPI_Datatype* newtype);
int MPI_Type_create_resized(MPI_Datatype oldtype, MPI_Aint lb, MPI_Aint extent, MPI_Datatype* newtype);
int MPI_Type_commit(MPI_Datatype* datatype);
int MPI_Type_free(MPI_Datatype* datatype);

int MPI_Init(int* argc, char*** argv);
int MPI_Finalize(void);
int MPI_Comm_size(MPI_Comm comm, int* size);
int MPI_Comm_rank(MPI_Comm comm, int* rank);
int MPI_Comm_split(MPI_Comm comm, int color, int key, MPI_Comm* newcomm);
int MPI_Comm_free(MPI_Comm* comm);
int MPI_Barrier(MPI_Comm comm);
int MPI_Bcast(void* buf, int count, MPI_Datatype t, int root, MPI_Comm comm);
int MPI_Reduce(const void* s, void* r, int count, MPI_Datatype t, MPI_Op op, int root, MPI_Comm comm);
int MPI_Allreduce(const void* s, void* r, int count, MPI_Datatype t, MPI_Op op, MPI_Comm comm);
int MPI_Gather(const void* s, int sc, MPI_Datatype st, void* r, int rc, MPI_Datatype rt, int root, MPI_Comm comm);
int MPI_Gatherv(const void* s, int sc, MPI_Datatype st, void* r, const int* rcs, const int* displs,
                MPI_Datatype rt, int root, MPI_Comm comm);
int MPI_Scatter(const void* s, int sc, MPI_Datatype st, void* r, int rc, MPI_Datatype rt, int root, MPI_Comm comm);
int MPI_Scatterv(const void* s, const int* scs, const int* displs, MPI_Datatype st, void* r, int rc,
                 MPI_Datatype rt, int root, MPI_Comm comm);
int MPI_Allgather(const void* s, int sc, MPI_Datatype st, void* r, int rc, MPI_Datatype rt, MPI_Comm comm);
int MPI_Allgatherv(const void* s, int sc, MPI_Datatype st, void* r, const int* rcs, const int* displs,
                   MPI_Datatype rt, MPI_Comm comm);
int MPI_Alltoallv(const void* s, const int* scs, const int* sdispls, MPI_Datatype st, void* r, const int* rcs,
                  const int* rdispls, MPI_Datatype rt, MPI_Comm comm);
double MPI_Wtime(void);
int MPI_Abort(MPI_Comm comm, int code);
int MPI_Error_string(int code, char* str, int* len);

/* MPI-IO: a rank's file view is the whole file (one process) */
typedef struct
{
    int source, tag, error;
} MPI_Status;
typedef int MPI_Info;
typedef void* MPI_File;
typedef long long MPI_Offset;
#define MPI_STATUS_IGNORE ((MPI_Status*)0)
#define MPI_INFO_NULL ((MPI_Info)0)
#define MPI_MODE_RDONLY 2
int MPI_File_open(MPI_Comm comm, const char* filename, int amode, MPI_Info info, MPI_File* fh);
int MPI_File_read_at_all(MPI_File fh, MPI_Offset offset, void* buf, int count, MPI_Datatype t, MPI_Status* status);
int MPI_File_close(MPI_File* fh);
