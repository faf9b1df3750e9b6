/* Single-rank stand-in for <mpi.h>, used only to compile the reference sources
 * as a one-process CPU oracle (test infrastructure; never part of the product).
 *
 * Rank 0 of a world of size 1.  With NUM_BLOCKS = 1 1 1 the reference never
 * sends or receives (cppsrc/Grid.cpp:490-493 takes the periodicSelf branch), so
 * the point-to-point calls below abort loudly if they are ever reached.
 */
#ifndef DG_REFSHIM_MPI_H
#define DG_REFSHIM_MPI_H
#include <cstdio>
#include <cstdlib>
#include <sys/time.h>

typedef int MPI_Comm;
typedef int MPI_Request;
typedef int MPI_Datatype;
typedef int MPI_Errhandler;
typedef struct { int source, tag, error; } MPI_Status;
#define MPI_COMM_WORLD 0
#define MPI_ERRORS_RETURN 0
#define MPI_FLOAT 0

static inline int MPI_Init(int*, char***) { return 0; }
static inline int MPI_Finalize() { return 0; }
static inline int MPI_Comm_set_errhandler(MPI_Comm, MPI_Errhandler) { return 0; }
static inline int MPI_Comm_rank(MPI_Comm, int* r) { *r = 0; return 0; }
static inline int MPI_Comm_size(MPI_Comm, int* s) { *s = 1; return 0; }
static inline int MPI_Barrier(MPI_Comm) { return 0; }
static inline double MPI_Wtime()
{
    struct timeval tv;
    gettimeofday(&tv, 0);
    return (double)tv.tv_sec + 1e-6 * (double)tv.tv_usec;
}
static inline int MPI_Isend(const void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request*)
{
    std::fprintf(stderr, "single-rank MPI stand-in: MPI_Isend reached (use NUM_BLOCKS = 1 1 1)\n");
    std::abort();
}
static inline int MPI_Recv(void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status*)
{
    std::fprintf(stderr, "single-rank MPI stand-in: MPI_Recv reached (use NUM_BLOCKS = 1 1 1)\n");
    std::abort();
}
#endif
