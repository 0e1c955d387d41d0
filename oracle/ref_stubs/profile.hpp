// Stand-in for pvfmm::Profile (timers and FLOP counters): no-ops.
// TEST INFRASTRUCTURE ONLY (oracle/_ref).
#pragma once
#include <mpi.h>

namespace pvfmm {
struct Profile {
  static void Tic(const char*, const MPI_Comm* = nullptr, bool = false, int = 0) {}
  static void Toc() {}
  static void Add_FLOP(long long) {}
  static void Add_MEM(long long) {}
  static void Enable(bool) {}
  static void print(const MPI_Comm* = nullptr) {}
};
}  // namespace pvfmm
