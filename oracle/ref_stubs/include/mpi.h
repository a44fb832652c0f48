/*
 * Single-rank MPI stand-in used only to compile the reference's SRC/orth.c and
 * SRC/util.c as a CPU oracle (test infrastructure, never shipped).
 *
 * It provides exactly the MPI surface those two files touch:
 *   MPI_Comm_rank / MPI_Comm_size  (SRC/orth.c:65-66, SRC/util.c:25,49)
 *   MPI_Allreduce SUM on doubles   (SRC/orth.c:113,132,187,196,277,286,...)
 *   MPI_Barrier                    (SRC/util.c:28,33)
 * With one rank an allreduce-SUM is a copy from sendbuf to recvbuf.
 */
#ifndef ORACLE_STUB_MPI_H
#define ORACLE_STUB_MPI_H

#include <string.h>
#include <time.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;

#define MPI_COMM_WORLD 0
#define MPI_DOUBLE 1
#define MPI_INT 2
#define MPI_SUM 1
#define MPI_MAX 2
#define MPI_SUCCESS 0

#ifdef __cplusplus
extern "C" {
#endif

static inline int oracle_mpi_type_size(MPI_Datatype t) {
    return t == MPI_DOUBLE ? (int)sizeof(double) : (int)sizeof(int);
}

static inline int MPI_Init(int *argc, char ***argv) { (void)argc; (void)argv; return MPI_SUCCESS; }
static inline int MPI_Finalize(void) { return MPI_SUCCESS; }
static inline int MPI_Comm_rank(MPI_Comm c, int *r) { (void)c; *r = 0; return MPI_SUCCESS; }
static inline int MPI_Comm_size(MPI_Comm c, int *n) { (void)c; *n = 1; return MPI_SUCCESS; }
static inline int MPI_Barrier(MPI_Comm c) { (void)c; return MPI_SUCCESS; }

static inline int MPI_Allreduce(const void *send, void *recv, int count,
                                MPI_Datatype t, MPI_Op op, MPI_Comm c) {
    (void)op; (void)c;
    if (send != recv && count > 0)
        memmove(recv, send, (size_t)count * (size_t)oracle_mpi_type_size(t));
    return MPI_SUCCESS;
}

static inline int MPI_Reduce(const void *send, void *recv, int count,
                             MPI_Datatype t, MPI_Op op, int root, MPI_Comm c) {
    (void)root;
    return MPI_Allreduce(send, recv, count, t, op, c);
}

static inline double MPI_Wtime(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

#ifdef __cplusplus
}
#endif
#endif
