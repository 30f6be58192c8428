/*
 * mpi.h -- a stand-in for the MPI header with just the names the ch9/MPI
 * sources' headers mention (Field::updateBoundaries), so that the single-
 * process pieces of that variant (its particle source) compile for the
 * golden vectors.  TEST INFRASTRUCTURE ONLY: no message is ever sent; the
 * harness runs as the one rank whose k index is 0.
 */
#ifndef ESPIC_MPI_STUB_H
#define ESPIC_MPI_STUB_H
typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef struct {
    int unused;
} MPI_Status;
#define MPI_COMM_WORLD 0
#define MPI_DOUBLE 1
#define MPI_STATUS_IGNORE ((MPI_Status *)0)
static inline int MPI_Sendrecv(const void *, int, MPI_Datatype, int, int, void *, int, MPI_Datatype, int, int,
                               MPI_Comm, MPI_Status *) {
    return 1; /* never called by the source sampler */
}
#endif
