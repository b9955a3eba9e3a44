// Exercises include/amrs_cns.hpp the way a C++ caller of the reference's CNS
// class would: compute_rhs on a ghost-filled state, then advance steps.
//   cns_adapter_main <in.bin> <rhs_out.bin> <state_out.bin> n nsteps dt mu
// in.bin: ghosted initial state (5, n+6, n+6, n+6) float64, periodic box of
// edge 2*pi; outputs: dSdt of the initial state (valid cells) and the valid
// state after nsteps SSPRK3 steps.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "amrs_cns.hpp"

int main(int argc, char** argv) {
  if (argc < 8) return 2;
  const int n = std::atoi(argv[4]), nsteps = std::atoi(argv[5]);
  const double dt = std::atof(argv[6]), mu = std::atof(argv[7]);
  const size_t ng = (size_t)5 * (n + 6) * (n + 6) * (n + 6), nv = (size_t)5 * n * n * n;
  std::vector<double> U(ng), R(nv);
  FILE* f = std::fopen(argv[1], "rb");
  if (!f || std::fread(U.data(), 8, ng, f) != ng) return 3;
  std::fclose(f);
  amrs::Geometry geom;
  geom.domain = amrs::Box{{0, 0, 0}, {n - 1, n - 1, n - 1}};
  for (int d = 0; d < 3; ++d) geom.dx[d] = 2.0 * 3.14159265358979323846 / n;
  amrs_scheme sc{1, 1, 1, 4, 0};
  // R = 1 gas, constant mu, k = cp mu / Pr (Pr = 0.71)
  const double gamma = 1.4, cv = 1.0 / (gamma - 1.0), cp = gamma / (gamma - 1.0);
  amrs_closures cl{gamma, cv, cp, 1.0, 0, 0, mu, 110.4, cp * mu / 0.71, 194.0, 1.0, 0.01};
  try {
    amrs::CNS lev(geom, sc, cl, 3, 3, 0);
    amrs::MultiFab& S = lev.get_new_data();
    cudaMemcpy(S.fab(0).dataPtr(), U.data(), ng * 8, cudaMemcpyHostToDevice);
    lev.FillPatch(S);
    amrs::MultiFab dSdt(std::vector<amrs::Box>{geom.domain}, 5, 0);
    lev.compute_rhs(S, dSdt, dt);
    cudaMemcpy(R.data(), dSdt.fab(0).dataPtr(), nv * 8, cudaMemcpyDeviceToHost);
    for (int s = 0; s < nsteps; ++s) lev.advance(lev.curTime(), dt, 1, 1);
    cudaMemcpy(U.data(), lev.get_new_data().fab(0).dataPtr(), ng * 8, cudaMemcpyDeviceToHost);
    amrs::check(amrs_sync_check(lev.handle(), nullptr), "sync");
  } catch (const amrs::Error& e) {
    std::fprintf(stderr, "%s\n", e.what());
    return 4;
  }
  f = std::fopen(argv[2], "wb");
  std::fwrite(R.data(), 8, nv, f);
  std::fclose(f);
  // valid cells of the final state
  std::vector<double> V(nv);
  size_t t = 0;
  for (int c = 0; c < 5; ++c)
    for (int k = 3; k < n + 3; ++k)
      for (int j = 3; j < n + 3; ++j)
        for (int i = 3; i < n + 3; ++i) V[t++] = U[(((size_t)c * (n + 6) + k) * (n + 6) + j) * (n + 6) + i];
  f = std::fopen(argv[3], "wb");
  std::fwrite(V.data(), 8, nv, f);
  std::fclose(f);
  return 0;
}
