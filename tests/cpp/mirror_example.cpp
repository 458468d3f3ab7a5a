// Exercises the C++ front-end (include/illum_gb300.hpp) the way the
// reference's illum_cli.cpp drives illum_context / thermal_model
// (src/cpp/illum_cli.cpp:305-456): horizons, form factors, one step of
// direct insolation + radiosity + conduction. Mesh in: argv[1] holds
// "nv nt" then nv*3 floats and nt*3 ints (text). Prints the surface
// temperatures after the step, one per line.
#include <cstdio>
#include <fstream>
#include <iostream>
#include <vector>

#include "illum_gb300.hpp"

int main(int argc, char** argv) {
  if (argc < 2) return 2;
  std::ifstream in(argv[1]);
  int nv, nt;
  in >> nv >> nt;
  std::vector<float> v(3 * (size_t)nv);
  std::vector<int32_t> f(3 * (size_t)nt);
  for (auto& x : v) in >> x;
  for (auto& x : f) in >> x;
  try {
    illum_gb300::illum_context ctx(v, f);
    ctx.make_horizons(16, 1e-3, 1e-5);
    auto F = ctx.compute_F(0.1);
    std::vector<double> disk;
    illum_gb300::fib_spiral(disk, 100);
    std::vector<double> sun = {2.2e8, 1.0e7, 3.0e7};
    auto E = ctx.get_direct_radiosity(sun, disk);
    auto rad = ctx.radiosity(E, 1e-10, 200);
    std::vector<double> z(20);
    for (int k = 0; k < 20; ++k) z[k] = 0.001 * (k + 1) * (k + 1);
    illum_gb300::thermal_model tm(ctx, z, 300.0, 1.05e6, 233.0);
    tm.step(600.0, rad);
    auto T = tm.T();
    std::printf("%zu\n", F.n_nonzero());
    for (int i = 0; i < ctx.get_num_faces(); ++i) std::printf("%.17g\n", T[(size_t)i * (tm.nz + 1)]);
  } catch (const std::exception& e) {
    std::cerr << e.what() << "\n";
    return 1;
  }
  return 0;
}
