/*
 * ORACLE — test infrastructure only.  A world-size-one stand-in for the few
 * MPI calls that the reference's CIC header makes, so that its loops can be
 * compiled from the reference's own source into oracle/_ref/ and the
 * oracle checked against them.  Nothing in the product includes this file.
 *
 * One process is the whole communicator: size 1, rank 0.  A datatype is its
 * size in bytes; MPI_Alltoall and MPI_Alltoallv copy the rank's own block
 * from the send to the receive buffer, which is what MPI does at world size
 * one.
 */
#ifndef JLD_ORACLE_MPI_STUB_H
#define JLD_ORACLE_MPI_STUB_H

#include <stddef.h>
#include <string.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;

#define MPI_COMM_WORLD ((MPI_Comm)0)
#define MPI_INT ((MPI_Datatype)sizeof(int))
#define MPI_FLOAT ((MPI_Datatype)sizeof(float))
#define MPI_DOUBLE ((MPI_Datatype)sizeof(double))
#define MPI_SUCCESS 0

static inline int MPI_Comm_size(MPI_Comm, int* size) { *size = 1; return MPI_SUCCESS; }
static inline int MPI_Comm_rank(MPI_Comm, int* rank) { *rank = 0; return MPI_SUCCESS; }

static inline int MPI_Type_contiguous(int count, MPI_Datatype old, MPI_Datatype* out) {
  *out = count * old;
  return MPI_SUCCESS;
}
static inline int MPI_Type_commit(MPI_Datatype*) { return MPI_SUCCESS; }
static inline int MPI_Type_free(MPI_Datatype*) { return MPI_SUCCESS; }

static inline int MPI_Alltoall(const void* send, int scount, MPI_Datatype stype, void* recv, int,
                               MPI_Datatype, MPI_Comm) {
  memmove(recv, send, (size_t)scount * (size_t)stype);
  return MPI_SUCCESS;
}

static inline int MPI_Alltoallv(const void* send, const int* scounts, const int* sdispl,
                                MPI_Datatype stype, void* recv, const int*, const int* rdispl,
                                MPI_Datatype, MPI_Comm) {
  if (scounts[0] > 0)
    memmove((char*)recv + (size_t)rdispl[0] * (size_t)stype,
            (const char*)send + (size_t)sdispl[0] * (size_t)stype,
            (size_t)scounts[0] * (size_t)stype);
  return MPI_SUCCESS;
}

#endif
