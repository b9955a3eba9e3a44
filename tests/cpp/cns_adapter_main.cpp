// Exercises include/amrs_cns.hpp the way a C++ caller of the reference's CNS
// class would: compute_rhs on a ghost-filled state, then advance steps.
//   cns_adapter_main <in.bin> <rhs_out.bin> <state_out.bin> n nsteps dt mu [m [run]]
// in.bin: ghosted initial state (5, n+6, n+6, n+6) float64, periodic box of
// edge 2*pi; the level is split into m boxes per direction (cuts at
// floor(i*n/m), default m = 1); outputs: dSdt of the initial state (valid
// cells) and the valid state after nsteps SSPRK3 steps.
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "amrs_cns.hpp"

namespace {

// Copy between the global ghosted host array (n+6)^3 and one box's device
// FAB (ghosted or valid-only), box cells only or with its ghosts.
void copy_box(std::vector<double>& G, int n, int gg, const amrs::FArrayBox& fab, int fg, bool to_device,
              int ncells_g) {
  const amrs::Box& b = fab.box();
  const int nx = b.length(0) + 2 * fg, ny = b.length(1) + 2 * fg, nz = b.length(2) + 2 * fg;
  std::vector<double> B((size_t)5 * nx * ny * nz);
  const int N = n + 2 * gg;
  auto gi = [&](int c, int k, int j, int i) {
    return (((size_t)c * N + (k + gg)) * N + (j + gg)) * N + (i + gg);
  };
  const int w = ncells_g;  // ghost layers to copy (0: valid cells only)
  if (!to_device && cudaMemcpy(B.data(), fab.dataPtr(), B.size() * 8, cudaMemcpyDeviceToHost) != cudaSuccess)
    throw amrs::Error(AMRS_ERR_CUDA, "copy_box");
  for (int c = 0; c < 5; ++c)
    for (int k = b.lo[2] - w; k <= b.hi[2] + w; ++k)
      for (int j = b.lo[1] - w; j <= b.hi[1] + w; ++j)
        for (int i = b.lo[0] - w; i <= b.hi[0] + w; ++i) {
          const size_t bi = (((size_t)c * nz + (k - b.lo[2] + fg)) * ny + (j - b.lo[1] + fg)) * nx + (i - b.lo[0] + fg);
          if (to_device) B[bi] = G[gi(c, k, j, i)];
          else G[gi(c, k, j, i)] = B[bi];
        }
  if (to_device && cudaMemcpy(fab.dataPtr(), B.data(), B.size() * 8, cudaMemcpyHostToDevice) != cudaSuccess)
    throw amrs::Error(AMRS_ERR_CUDA, "copy_box");
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 8) return 2;
  const int n = std::atoi(argv[4]), nsteps = std::atoi(argv[5]);
  const double dt = std::atof(argv[6]), mu = std::atof(argv[7]);
  const int m = argc > 8 ? std::atoi(argv[8]) : 1;
  const size_t ng = (size_t)5 * (n + 6) * (n + 6) * (n + 6), nv = (size_t)5 * n * n * n;
  std::vector<double> U(ng), R(nv), V(nv);
  FILE* f = std::fopen(argv[1], "rb");
  if (!f || std::fread(U.data(), 8, ng, f) != ng) return 3;
  std::fclose(f);
  amrs::Geometry geom;
  geom.domain = amrs::Box{{0, 0, 0}, {n - 1, n - 1, n - 1}};
  for (int d = 0; d < 3; ++d) geom.dx[d] = 2.0 * 3.14159265358979323846 / n;
  std::vector<amrs::Box> grids;
  for (int c = 0; c < m; ++c)
    for (int b = 0; b < m; ++b)
      for (int a = 0; a < m; ++a)
        grids.push_back(amrs::Box{{a * n / m, b * n / m, c * n / m},
                                  {(a + 1) * n / m - 1, (b + 1) * n / m - 1, (c + 1) * n / m - 1}});
  amrs_scheme sc{1, 1, 1, 4, 0, 0};
  // R = 1 gas, constant mu, k = cp mu / Pr (Pr = 0.71)
  const double gamma = 1.4, cv = 1.0 / (gamma - 1.0), cp = gamma / (gamma - 1.0);
  amrs_closures cl{gamma, cv, cp, 1.0, 0, 0, mu, 110.4, cp * mu / 0.71, 194.0, 1.0, 0.01};
  try {
    // optional x body force (cns.rhs_source with the channel problem's user_source form)
    const double fx = argc > 10 ? std::atof(argv[10]) : 0.0;
    const double bf[3] = {fx, 0.0, 0.0};
    amrs::CNS lev(geom, grids, sc, cl, 3, 3, 0, fx != 0.0 ? bf : nullptr);
    amrs::MultiFab& S = lev.get_new_data();
    for (int b = 0; b < S.size(); ++b) copy_box(U, n, 3, S.fab(b), 3, true, 3);
    lev.FillPatch(S);
    amrs::MultiFab dSdt(grids, 5, 0);
    lev.compute_rhs(S, dSdt, dt);
    std::vector<double> Rg((size_t)5 * n * n * n);
    for (int b = 0; b < dSdt.size(); ++b) copy_box(Rg, n, 0, dSdt.fab(b), 0, false, 0);
    R = Rg;
    if (argc > 9 && std::string(argv[9]) == "run") {
      // the whole loop as one device launch, fixed dt
      if (lev.run(1e30, nsteps, 0.0, dt) != nsteps) return 5;
    } else {
      for (int s = 0; s < nsteps; ++s) lev.advance(lev.curTime(), dt, 1, 1);
    }
    amrs::MultiFab& F = lev.get_new_data();
    for (int b = 0; b < F.size(); ++b) copy_box(V, n, 0, F.fab(b), 3, false, 0);
    amrs::check(amrs_sync_check(lev.handle(), nullptr), "sync");
  } catch (const amrs::Error& e) {
    std::fprintf(stderr, "%s\n", e.what());
    return 4;
  }
  f = std::fopen(argv[2], "wb");
  std::fwrite(R.data(), 8, nv, f);
  std::fclose(f);
  f = std::fopen(argv[3], "wb");
  std::fwrite(V.data(), 8, nv, f);
  std::fclose(f);
  return 0;
}
