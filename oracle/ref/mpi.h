/*
 * mpi.h -- single-rank stand-in for the MPI calls made by the reference's
 * MPIEngine (include/fiuncho/MPIEngine.h:33-45, 143-174) and CLI
 * (app/main.cpp:143-167).  TEST INFRASTRUCTURE ONLY: lets the reference's
 * own headers compile in the oracle build, with one rank (size 1, rank 0);
 * the gathers copy the send buffer to the receive buffer.
 */
#ifndef ORACLE_MPI_SHIM_H
#define ORACLE_MPI_SHIM_H

#include <cstdlib>
#include <cstring>
#include <ctime>

typedef int MPI_Comm;
typedef int MPI_Datatype;
#define MPI_COMM_WORLD 0
#define MPI_INT 1
#define MPI_BYTE 2

static inline int MPI_Init(int *, char ***) { return 0; }
static inline int MPI_Finalize() { return 0; }
static inline int MPI_Abort(MPI_Comm, int code) { std::exit(code); }
static inline int MPI_Comm_size(MPI_Comm, int *size) { *size = 1; return 0; }
static inline int MPI_Comm_rank(MPI_Comm, int *rank) { *rank = 0; return 0; }
static inline double MPI_Wtime()
{
    timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return ts.tv_sec + ts.tv_nsec * 1e-9;
}
static inline size_t oracle_mpi_size(MPI_Datatype t) { return t == MPI_INT ? sizeof(int) : 1; }
static inline int MPI_Gather(const void *send, int count, MPI_Datatype t, void *recv, int, MPI_Datatype, int,
                             MPI_Comm)
{
    if (recv) std::memcpy(recv, send, count * oracle_mpi_size(t));
    return 0;
}
static inline int MPI_Gatherv(const void *send, int count, MPI_Datatype t, void *recv, const int *, const int *displs,
                              MPI_Datatype, int, MPI_Comm)
{
    if (recv && count) std::memcpy((char *)recv + (displs ? displs[0] : 0), send, count * oracle_mpi_size(t));
    return 0;
}

#endif
