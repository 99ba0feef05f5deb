/* Minimal stand-in for <mpi.h> so the reference's single-process hot path
 * compiles without an MPI installation.  Only the names that the hot-path
 * translation units mention are provided; the one collective they reach
 * (an all-gather used by temporal halo finding, which the oracle disables)
 * copies the caller's buffer, which is what a one-rank communicator does. */
#ifndef ORACLE_STUB_MPI_H
#define ORACLE_STUB_MPI_H
#include <string.h>
typedef int MPI_Datatype;
typedef int MPI_Comm;
#define MPI_CHAR 1
#define MPI_COMM_WORLD 0
static inline int MPI_Allgather(const void *sbuf, int scount, MPI_Datatype st,
                                void *rbuf, int rcount, MPI_Datatype rt,
                                MPI_Comm c) {
    (void)st; (void)rcount; (void)rt; (void)c;
    memmove(rbuf, sbuf, (size_t)scount);
    return 0;
}
#endif
