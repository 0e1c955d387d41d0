// Drives the C++ drop-in layer (include/tbslas_gb300.hpp) the way a tbslas
// advection driver does: build the velocity and concentration trees, evaluate
// the velocity functor, backtrace points with ComputeTrajRK2 and advance the
// concentration with SolveSemilagInSitu.  Input / output are raw float64
// files written / read by tests/test_cpp_shim.py.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "tbslas_gb300.hpp"

namespace tg = tbslas_gb300;

static std::vector<double> read_f64(FILE* f, size_t n) {
  std::vector<double> v(n);
  if (fread(v.data(), sizeof(double), n, f) != n) { fprintf(stderr, "short read\n"); exit(2); }
  return v;
}

int main(int argc, char** argv) {
  if (argc != 3) { fprintf(stderr, "usage: shim_demo in.bin out.bin\n"); return 2; }
  FILE* f = fopen(argv[1], "rb");
  std::vector<double> hdr = read_f64(f, 6);  // L, q, npts, dt, bc, steps
  const long L = (long)hdr[0];
  const int q = (int)hdr[1];
  const long npts = (long)hdr[2];
  const double dt = hdr[3];
  const tg::BoundaryType bc = hdr[4] != 0 ? tg::Periodic : tg::FreeSpace;
  const int steps = (int)hdr[5];
  const long nc = (long)(q + 1) * (q + 2) * (q + 3) / 6;
  std::vector<double> anchor = read_f64(f, 3 * L);
  std::vector<double> depth_d = read_f64(f, L);
  std::vector<double> vc = read_f64(f, L * 3 * nc);
  std::vector<double> cc = read_f64(f, L * nc);
  std::vector<double> pts = read_f64(f, 3 * npts);
  fclose(f);
  std::vector<int32_t> depth(depth_d.begin(), depth_d.end());

  try {
    tg::Context ctx(0);
    tg::Tree tvel(ctx, anchor, depth, q, 3);
    tg::Tree tcon(ctx, anchor, depth, q, 1);
    tvel.SetChebData(vc);
    tcon.SetChebData(cc);
    tg::NodeFieldFunctor<double> tvel_func(&tvel, bc);

    std::vector<double> v(3 * npts);
    tvel_func(pts.data(), (int)npts, v.data());
    std::vector<double> xdep;
    tg::ComputeTrajRK2(tvel_func, pts, 0.0, -dt, 1, xdep);
    for (int timestep = 1; timestep <= steps; ++timestep)
      tg::SolveSemilagInSitu(tvel_func, tcon, timestep, dt, 1);
    std::vector<double> out = tcon.ChebData();

    FILE* g = fopen(argv[2], "wb");
    fwrite(v.data(), sizeof(double), v.size(), g);
    fwrite(xdep.data(), sizeof(double), xdep.size(), g);
    fwrite(out.data(), sizeof(double), out.size(), g);
    fclose(g);
  } catch (const tg::Error& e) {
    fprintf(stderr, "%s\n", e.what());
    return 1;
  }
  return 0;
}
