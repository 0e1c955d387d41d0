// Single-process stand-in for the MPI names the tbslas headers use: one rank
// (rank 0 of 1).  Collectives copy the caller's data.  A datatype handle is
// the element size in bytes (pvfmm::par::Mpi_datatype<T>::value() returns
// sizeof(T)), so the copies know their lengths.
//
// TEST INFRASTRUCTURE ONLY: compiled with the reference's own headers into
// oracle/_ref (the build recipe is oracle/build_ref.py).
#pragma once
#include <cstddef>
#include <cstring>

typedef int MPI_Comm;
typedef size_t MPI_Datatype;
typedef int MPI_Op;
#define MPI_COMM_WORLD 0
#define MPI_COMM_SELF 1
#define MPI_INT sizeof(int)
#define MPI_DOUBLE sizeof(double)
#define MPI_MAX 1
#define MPI_SUM 2

inline int MPI_Comm_rank(MPI_Comm, int* r) { *r = 0; return 0; }
inline int MPI_Comm_size(MPI_Comm, int* s) { *s = 1; return 0; }
inline int MPI_Allgather(const void* s, int n, MPI_Datatype t, void* r, int, MPI_Datatype,
                         MPI_Comm) {
  std::memmove(r, s, n * t);
  return 0;
}
inline int MPI_Gather(const void* s, int n, MPI_Datatype t, void* r, int, MPI_Datatype, int,
                      MPI_Comm) {
  std::memmove(r, s, n * t);
  return 0;
}
inline int MPI_Allreduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op, MPI_Comm) {
  std::memmove(r, s, n * t);
  return 0;
}
inline int MPI_Reduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op, int, MPI_Comm) {
  std::memmove(r, s, n * t);
  return 0;
}
inline int MPI_Barrier(MPI_Comm) { return 0; }
