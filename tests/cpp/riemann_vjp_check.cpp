// CPU check of the two-shock solver's reverse (riemann_vjp.cuh, the code
// the MUSCL-Riemann adjoint kernel runs) against forward-mode dual numbers
// through the oracle's riemann_prob: for random Riemann problems (density
// and pressure ratios up to e^+-4, velocities up to twice the sound speed,
// no floored state), J^T fb from the reverse equals the ten dual
// directional derivatives contracted with fb.  Prints the worst relative
// difference and the number of cases over 1e-9.
#include "../../oracle/cns_oracle.cpp"
#include "../../amrsolver_gb300/csrc/riemann_vjp.cuh"

#include <cstdio>
#include <cstdlib>
#include <random>

int main(int argc, char** argv) {
  const int ncase = argc > 1 ? std::atoi(argv[1]) : 100000;
  std::mt19937_64 rng(12345);
  std::normal_distribution<double> N(0.0, 1.0);
  const double g = 1.4;
  double worst = 0.0;
  int nbad = 0;
  for (int t = 0; t < ncase; ++t) {
    const double sc = (t % 3 == 0) ? 0.1 : ((t % 3 == 1) ? 0.7 : 1.5);
    double in[10];
    const double rl = std::exp(sc * N(rng)), pl = std::exp(sc * N(rng));
    const double rr = std::exp(sc * N(rng)), pr = std::exp(sc * N(rng));
    in[0] = rl; in[1] = sc * N(rng) * std::sqrt(g * pl / rl); in[2] = pl; in[3] = N(rng); in[4] = N(rng);
    in[5] = rr; in[6] = sc * N(rng) * std::sqrt(g * pr / rr); in[7] = pr; in[8] = N(rng); in[9] = N(rng);
    double fb[5];
    for (double& x : fb) x = N(rng);
    double ib[10];
    amrs::rpvjp::riemann_prob_vjp(g, 1e-40, in, fb, ib);
    double num = 0.0, den = 0.0;
    for (int a = 0; a < 10; ++a) {
      orc::Dual d[10], f[5];
      for (int b = 0; b < 10; ++b) d[b] = orc::Dual(in[b], a == b ? 1.0 : 0.0);
      orc::riemann_prob<orc::Dual>(orc::Dual(g), orc::Dual(1e-40), d[0], d[1], d[2], d[3], d[4], d[5], d[6], d[7],
                                   d[8], d[9], f[0], f[1], f[2], f[3], f[4]);
      double jt = 0.0;
      for (int n = 0; n < 5; ++n) jt += f[n].d * fb[n];
      num = std::max(num, std::fabs(jt - ib[a]));
      den = std::max(den, std::fabs(jt));
    }
    const double rel = num / (den + 1e-300);
    if (rel > 1e-9) ++nbad;
    worst = std::max(worst, rel);
  }
  std::printf("%.6e %d\n", worst, nbad);
  return 0;
}
