/*
 * Single-rank MPI shim -- TEST INFRASTRUCTURE ONLY (part of the oracle).
 *
 * The reference solver (ark-cpp-mpi, source/main.cpp) talks to its neighbours only
 * through MPI: blocking MPI_Sendrecv halo exchanges (main.cpp:603-801, 1049-1631),
 * one MPI_Allreduce(MIN) for dt (main.cpp:412) and MPI-IO for its VTK writer.  No
 * MPI is installed in this image, so the oracle compiles the reference sources
 * unmodified against this header.
 *
 * Semantics for one rank:
 *   - a datatype handle is its size in bytes (MPI_DOUBLE == 8, MPI_CHAR == 1);
 *   - MPI_Sendrecv with source == MPI_PROC_NULL leaves the receive buffer untouched
 *     (as MPI does); with source == the calling rank it copies the send buffer into
 *     the receive buffer.  The oracle harness points the x and z neighbours at rank 0
 *     itself, which turns every exchange along those axes into a periodic copy
 *     (right edge -> left ghost, left edge -> right ghost), and the y neighbours at
 *     MPI_PROC_NULL (walls);
 *   - reductions over one rank copy the input to the output;
 *   - MPI-IO calls write through stdio so the VTK writer still produces a file.
 */
#ifndef ARK_ORACLE_MPI_SHIM_H
#define ARK_ORACLE_MPI_SHIM_H

#include <stdio.h>
#include <string.h>
#include <time.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Info;
typedef long long MPI_Offset;
typedef FILE *MPI_File;
typedef struct { int source, tag, error; } MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_PROC_NULL (-2)
#define MPI_STATUS_IGNORE ((MPI_Status *)0)
#define MPI_INFO_NULL 0
#define MPI_SUCCESS 0

#define MPI_CHAR 1
#define MPI_INT 4
#define MPI_DOUBLE 8

#define MPI_MIN 1
#define MPI_MAX 2
#define MPI_SUM 3

#define MPI_MODE_CREATE 1
#define MPI_MODE_WRONLY 2

static inline int MPI_Init(int *argc, char ***argv) { (void)argc; (void)argv; return 0; }
static inline int MPI_Finalize(void) { return 0; }
static inline int MPI_Comm_size(MPI_Comm c, int *n) { (void)c; *n = 1; return 0; }
static inline int MPI_Comm_rank(MPI_Comm c, int *r) { (void)c; *r = 0; return 0; }

static inline int MPI_Dims_create(int nnodes, int ndims, int *dims) {
    for (int d = 0; d < ndims; ++d)
        if (dims[d] == 0) dims[d] = 1;
    (void)nnodes;
    return 0;
}

static inline int MPI_Cart_create(MPI_Comm old, int ndims, const int *dims, const int *periods,
                                  int reorder, MPI_Comm *cart) {
    (void)old; (void)ndims; (void)dims; (void)periods; (void)reorder;
    *cart = 0;
    return 0;
}

static inline int MPI_Cart_coords(MPI_Comm c, int rank, int maxdims, int *coords) {
    (void)c; (void)rank;
    for (int d = 0; d < maxdims; ++d) coords[d] = 0;
    return 0;
}

/* One rank, non-periodic topology (the reference's own main() asks for periods
 * false, main.cpp:55): both neighbours are MPI_PROC_NULL.  The oracle harness
 * overrides the neighbour globals itself to select periodic axes. */
static inline int MPI_Cart_shift(MPI_Comm c, int dir, int disp, int *src, int *dst) {
    (void)c; (void)dir; (void)disp;
    *src = MPI_PROC_NULL;
    *dst = MPI_PROC_NULL;
    return 0;
}

static inline int MPI_Sendrecv(const void *sendbuf, int sendcount, MPI_Datatype sendtype,
                               int dest, int sendtag, void *recvbuf, int recvcount,
                               MPI_Datatype recvtype, int source, int recvtag, MPI_Comm comm,
                               MPI_Status *status) {
    (void)dest; (void)sendtag; (void)recvtag; (void)comm; (void)recvtype;
    if (status) { status->source = source; status->tag = recvtag; status->error = 0; }
    if (source == MPI_PROC_NULL) return 0;
    /* source is this rank: the message it sent (to itself) arrives here */
    size_t n = (size_t)(sendcount < recvcount ? sendcount : recvcount) * (size_t)sendtype;
    memmove(recvbuf, sendbuf, n);
    return 0;
}

static inline int MPI_Allreduce(const void *in, void *out, int count, MPI_Datatype t, MPI_Op op,
                                MPI_Comm c) {
    (void)op; (void)c;
    memmove(out, in, (size_t)count * (size_t)t);
    return 0;
}

static inline int MPI_Reduce(const void *in, void *out, int count, MPI_Datatype t, MPI_Op op,
                             int root, MPI_Comm c) {
    (void)op; (void)root; (void)c;
    memmove(out, in, (size_t)count * (size_t)t);
    return 0;
}

static inline int MPI_Bcast(void *buf, int count, MPI_Datatype t, int root, MPI_Comm c) {
    (void)buf; (void)count; (void)t; (void)root; (void)c;
    return 0;
}

static inline double MPI_Wtime(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

static inline int MPI_File_open(MPI_Comm c, const char *name, int mode, MPI_Info info,
                                MPI_File *fh) {
    (void)c; (void)mode; (void)info;
    *fh = fopen(name, "wb");
    return *fh ? 0 : 1;
}

static inline int MPI_File_write_at(MPI_File fh, MPI_Offset off, const void *buf, int count,
                                    MPI_Datatype t, MPI_Status *status) {
    (void)status;
    if (!fh) return 1;
    fseek(fh, (long)off, SEEK_SET);
    fwrite(buf, (size_t)t, (size_t)count, fh);
    return 0;
}

static inline int MPI_File_close(MPI_File *fh) {
    if (*fh) fclose(*fh);
    *fh = 0;
    return 0;
}

#endif
