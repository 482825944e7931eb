/*
 * mpi.h -- single-rank MPI stub for building the reference's own CUDA program
 * (src/main.cu) on one GPU.
 *
 * TEST AND BENCHMARK INFRASTRUCTURE ONLY: used by oracle/build.py to build
 * oracle/_ref/lbm_ref_cuda, the reference's unmodified step timed beside the
 * product.  Never linked into the product.
 *
 * One rank, periodic Cartesian topology: rank 0 is its own top and bottom
 * neighbour.  Irecv records the receive buffer under its tag, Send copies into
 * the buffer recorded under the same tag, Wait does nothing; with one rank this
 * is exactly the exchange of src/mpiupdate*.c:34-41 (TAG1: bot_snd -> top_rcv,
 * TAG2: top_snd -> bot_rcv), i.e. periodic wrap in z.  Reduce copies, Bcast
 * does nothing, Abort exits.
 */
#ifndef LBM_MPI_STUB_H
#define LBM_MPI_STUB_H

#include <stdio.h>
#include <stdlib.h>
#include <string.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Request;
typedef struct {
    int MPI_SOURCE, MPI_TAG, MPI_ERROR;
} MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_INT 1
#define MPI_FLOAT 2
#define MPI_MAX 1
#define MPI_SUM 2

static void *lbm_mpi_stub_recv[16];

static inline size_t lbm_mpi_stub_size(MPI_Datatype t) { return t == MPI_INT ? sizeof(int) : sizeof(float); }

static inline int MPI_Init(int *, char ***) { return 0; }
static inline int MPI_Finalize(void) { return 0; }
static inline int MPI_Abort(MPI_Comm, int code)
{
    fprintf(stderr, "MPI_Abort(%d)\n", code);
    exit(1);
}
static inline int MPI_Comm_size(MPI_Comm, int *n) { *n = 1; return 0; }
static inline int MPI_Comm_rank(MPI_Comm, int *r) { *r = 0; return 0; }
static inline int MPI_Bcast(void *, int, MPI_Datatype, int, MPI_Comm) { return 0; }
static inline int MPI_Cart_create(MPI_Comm, int, int *, int *, int, MPI_Comm *c) { *c = 0; return 0; }
static inline int MPI_Cart_coords(MPI_Comm, int, int, int *coords) { coords[0] = 0; return 0; }
static inline int MPI_Cart_shift(MPI_Comm, int, int, int *src, int *dst) { *src = 0; *dst = 0; return 0; }
static inline int MPI_Reduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op, int, MPI_Comm)
{
    memcpy(r, s, (size_t)n * lbm_mpi_stub_size(t));
    return 0;
}
static inline int MPI_Irecv(void *buf, int, MPI_Datatype, int, int tag, MPI_Comm, MPI_Request *req)
{
    lbm_mpi_stub_recv[tag & 15] = buf;
    *req = tag;
    return 0;
}
static inline int MPI_Send(const void *buf, int n, MPI_Datatype t, int, int tag, MPI_Comm)
{
    void *dst = lbm_mpi_stub_recv[tag & 15];
    if (!dst) {
        fprintf(stderr, "MPI stub: Send with tag %d has no matching Irecv\n", tag);
        exit(1);
    }
    memcpy(dst, buf, (size_t)n * lbm_mpi_stub_size(t));
    return 0;
}
static inline int MPI_Wait(MPI_Request *, MPI_Status *) { return 0; }

#endif
