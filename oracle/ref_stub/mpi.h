/*
 * Sequential MPI stand-in (one process) -- TEST INFRASTRUCTURE ONLY.
 * Lets the reference's get_cluster.h / mpi_range.cxx compile and run unmodified on
 * one rank, for pinning the oracle. Collectives reduce to copies; MPI_Exscan leaves
 * rank 0's receive buffer untouched, as MPI specifies it undefined there and common
 * implementations leave it as is (the reference zero-fills it first,
 * 2d/get_cluster.h:223-226).
 */
#ifndef PRBF_REF_STUB_MPI_H
#define PRBF_REF_STUB_MPI_H
#include <cstring>
typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
#define MPI_INT 1
#define MPI_DOUBLE 2
#define MPI_SUM 1
static inline int MPI_Comm_size(MPI_Comm, int* n) { *n = 1; return 0; }
static inline int MPI_Comm_rank(MPI_Comm, int* r) { *r = 0; return 0; }
static inline int stub_mpi_size(MPI_Datatype t) { return t == MPI_DOUBLE ? 8 : 4; }
static inline int MPI_Exscan(const void*, void*, int, MPI_Datatype, MPI_Op, MPI_Comm) { return 0; }
static inline int MPI_Allreduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op, MPI_Comm) {
  std::memmove(r, s, (size_t)n * stub_mpi_size(t));
  return 0;
}
#endif
