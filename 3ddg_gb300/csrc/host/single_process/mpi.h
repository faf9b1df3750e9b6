// A single-process stand-in for the handful of MPI calls the reference's
// driver makes (cppsrc/driver.cpp:73-84, 236-289).  In this package every
// block of the mesh lives in one GPU's memory and inter-block faces are read
// on the device, so the driver runs as one process: rank 0 of 1.  Put this
// directory on the include path to build the reference's driver against this
// package on a host without MPI; with an MPI installation, build with mpicxx
// and run one rank.
#pragma once

#include <chrono>

typedef int MPI_Comm;
typedef int MPI_Errhandler;
#define MPI_COMM_WORLD 0
#define MPI_ERRORS_RETURN 0
#define MPI_SUCCESS 0

inline int MPI_Init(int*, char***) { return MPI_SUCCESS; }
inline int MPI_Finalize() { return MPI_SUCCESS; }
inline int MPI_Comm_set_errhandler(MPI_Comm, MPI_Errhandler) { return MPI_SUCCESS; }
inline int MPI_Comm_rank(MPI_Comm, int* rank)
{
    *rank = 0;
    return MPI_SUCCESS;
}
inline int MPI_Comm_size(MPI_Comm, int* size)
{
    *size = 1;
    return MPI_SUCCESS;
}
inline int MPI_Barrier(MPI_Comm) { return MPI_SUCCESS; }
inline double MPI_Wtime()
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}
