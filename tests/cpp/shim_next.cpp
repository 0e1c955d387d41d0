// Drives the C++ layer's time-dependent functors, BDF2 step and re-meshing
// the way the reference's drivers call them (advtv.cpp: FieldSetFunctor +
// SolveSemilagInSitu; advtvextrap.cpp: the two-functor SolveSemilagInSitu;
// advdiff-ss.cpp: the BDF2 step; advection.cpp: RefineTree + Balance21 after
// a step).  Input / output are raw float64 files written / read by
// tests/test_cpp_shim.py.
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

static void write_f64(FILE* g, const std::vector<double>& v) {
  fwrite(v.data(), sizeof(double), v.size(), g);
}

int main(int argc, char** argv) {
  if (argc != 3) { fprintf(stderr, "usage: shim_next in.bin out.bin\n"); return 2; }
  FILE* f = fopen(argv[1], "rb");
  std::vector<double> hdr = read_f64(f, 5);  // L, q, dt, tol, max_depth
  const long L = (long)hdr[0];
  const int q = (int)hdr[1];
  const double dt = hdr[2], tol = hdr[3];
  const int max_depth = (int)hdr[4];
  const long nc = (long)(q + 1) * (q + 2) * (q + 3) / 6;
  std::vector<double> anchor = read_f64(f, 3 * L);
  std::vector<double> depth_d = read_f64(f, L);
  std::vector<std::vector<double>> vc(4);
  for (auto& v : vc) v = read_f64(f, L * 3 * nc);
  std::vector<double> cc = read_f64(f, L * nc), cp = read_f64(f, L * nc);
  fclose(f);
  std::vector<int32_t> depth(depth_d.begin(), depth_d.end());
  try {
    tg::Context ctx(0);
    std::vector<tg::Tree*> tv;
    for (int k = 0; k < 4; ++k) {
      tv.push_back(new tg::Tree(ctx, anchor, depth, q, 3));
      tv.back()->SetChebData(vc[k]);
    }
    FILE* g = fopen(argv[2], "wb");
    // FieldSetFunctor, times 0, dt, 2dt, 3dt; step 2 queries [dt, 2dt]
    tg::FieldSetFunctor<double> fs({tv[0], tv[1], tv[2], tv[3]}, {0.0, dt, 2 * dt, 3 * dt});
    tg::Tree t1(ctx, anchor, depth, q, 1);
    t1.SetChebData(cc);
    tg::SolveSemilagInSitu(fs, t1, 2, dt, 1);
    write_f64(g, t1.ChebData());
    // the two-functor form: v_n = tv[1] at X, 1.5 tv[1] - 0.5 tv[0] at X*
    tg::NodeFieldFunctor<double> vn(tv[1]);
    tg::FieldExtrapFunctor<double> ex(tv[0], tv[1]);
    tg::Tree t2(ctx, anchor, depth, q, 1);
    t2.SetChebData(cc);
    tg::SolveSemilagInSitu(vn, ex, t2, 2, dt, 1);
    write_f64(g, t2.ChebData());
    // BDF2 at tcurr = 2 dt through tv[0]
    tg::NodeFieldFunctor<double> v0(tv[0]);
    tg::Tree tp(ctx, anchor, depth, q, 1), tc(ctx, anchor, depth, q, 1), tn(ctx, anchor, depth, q, 1);
    tp.SetChebData(cp);
    tc.SetChebData(cc);
    tg::SemilagBDF2(v0, tp, tc, tn, 2 * dt, dt, 1);
    write_f64(g, tn.ChebData());
    // re-mesh the BDF2 result
    tn.Remesh(tol, 0, max_depth, tg::FreeSpace);
    std::vector<double> a2;
    std::vector<int32_t> d2;
    tn.Leaves(a2, d2);
    const double nl = (double)d2.size();
    fwrite(&nl, sizeof(double), 1, g);
    write_f64(g, a2);
    write_f64(g, std::vector<double>(d2.begin(), d2.end()));
    write_f64(g, tn.ChebData());
    fclose(g);
    for (auto* t : tv) delete t;
  } catch (const tg::Error& e) {
    fprintf(stderr, "%s\n", e.what());
    return 1;
  }
  return 0;
}
