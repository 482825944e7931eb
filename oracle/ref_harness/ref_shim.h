/*
 * ref_shim.h -- lets the reference's CUDA-C sources compile as host C++.
 *
 * TEST INFRASTRUCTURE ONLY (builds oracle/_ref, the reference's own step
 * kernels run on the CPU).  Force-included before the reference sources by
 * oracle/build.py.
 *
 * - CUDA qualifiers become no-ops; blockIdx / threadIdx / blockDim become
 *   thread-local variables set by the launch emulation in zsc_ref_cpu.cpp.
 * - MPI is a single-rank stub: Irecv records its buffer by tag, Send copies
 *   into the buffer recorded under the same tag (top = bot = self), Reduce
 *   copies, Bcast and Wait do nothing.  With one rank this is exactly what
 *   src/mpiupdate*.c:34-41 exchange (TAG1: bot_snd -> top_rcv, TAG2:
 *   top_snd -> bot_rcv), i.e. periodic wrap in z.
 */
#pragma once
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>

#define __global__
#define __device__
#define __constant__
#define __host__

struct zr_dim3 { int x, y, z; };
extern thread_local zr_dim3 blockIdx, threadIdx, blockDim;

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef struct { int src, tag; } MPI_Status;
typedef int MPI_Request;

#define MPI_COMM_WORLD 0
#define MPI_INT 1
#define MPI_FLOAT 2
#define MPI_MAX 1
#define MPI_SUM 2

static inline size_t zr_mpi_size(MPI_Datatype t) { return t == MPI_INT ? sizeof(int) : sizeof(float); }

/* tag -> receive buffer of the pending Irecv */
extern void *zr_mpi_recv_buf[8];

static inline int MPI_Init(int *, char ***) { return 0; }
static inline int MPI_Finalize(void) { return 0; }
static inline int MPI_Abort(MPI_Comm, int code) { fprintf(stderr, "MPI_Abort(%d)\n", code); exit(1); }
static inline int MPI_Comm_size(MPI_Comm, int *n) { *n = 1; return 0; }
static inline int MPI_Comm_rank(MPI_Comm, int *r) { *r = 0; return 0; }
static inline int MPI_Bcast(void *, int, MPI_Datatype, int, MPI_Comm) { return 0; }
static inline int MPI_Cart_create(MPI_Comm, int, int *, int *, int, MPI_Comm *c) { *c = 0; return 0; }
static inline int MPI_Cart_coords(MPI_Comm, int, int, int *coords) { coords[0] = 0; return 0; }
static inline int MPI_Cart_shift(MPI_Comm, int, int, int *src, int *dst) { *src = 0; *dst = 0; return 0; }
static inline int MPI_Reduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op, int, MPI_Comm)
{
    memcpy(r, s, (size_t)n * zr_mpi_size(t));
    return 0;
}
static inline int MPI_Irecv(void *buf, int, MPI_Datatype, int, int tag, MPI_Comm, MPI_Request *req)
{
    zr_mpi_recv_buf[tag & 7] = buf;
    *req = tag;
    return 0;
}
static inline int MPI_Send(const void *buf, int n, MPI_Datatype t, int, int tag, MPI_Comm)
{
    memcpy(zr_mpi_recv_buf[tag & 7], buf, (size_t)n * zr_mpi_size(t));
    return 0;
}
static inline int MPI_Wait(MPI_Request *, MPI_Status *) { return 0; }
