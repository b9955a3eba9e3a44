// Host check of amrs::ddiv_rn (amrsolver_gb300/csrc/ddiv.cuh) against the
// host's IEEE double division: random operands from several distributions
// plus hand-picked edge cases; prints "mismatches N checked M" and exits
// non-zero on any difference in the bits.
//   ddiv_check <count> <seed>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cmath>

#include "../../amrsolver_gb300/csrc/ddiv.cuh"

static uint64_t s_state;
static uint64_t rnd() {  // splitmix64
  uint64_t z = (s_state += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
static double from_bits(uint64_t u) { double x; memcpy(&x, &u, 8); return x; }
static uint64_t to_bits(double x) { uint64_t u; memcpy(&u, &x, 8); return u; }
static double unif() { return (rnd() >> 11) * (1.0 / 9007199254740992.0); }

static long long bad = 0, checked = 0;
static void check(double a, double b) {
  const double ref = a / b, got = amrs::ddiv_rn(a, b);
  ++checked;
  if (to_bits(ref) != to_bits(got) && !(std::isnan(ref) && std::isnan(got))) {
    if (bad < 10) printf("MISMATCH a=%a b=%a ref=%a got=%a\n", a, b, ref, got);
    ++bad;
  }
}

int main(int argc, char** argv) {
  const long long n = argc > 1 ? atoll(argv[1]) : 1000000;
  s_state = argc > 2 ? strtoull(argv[2], nullptr, 10) : 1;
  const double num[4] = {0.1, 0.6, 0.3, 1.0};
  for (long long i = 0; i < n; ++i) {
    const int kind = (int)(i % 6);
    double a, b;
    if (kind == 0) {  // the WENO weights: c_k / (eps + beta)^2
      const double e = 1e-40 + std::pow(10.0, -60.0 + 120.0 * unif());
      a = num[rnd() & 3];
      b = e * e;
    } else if (kind == 1) {  // 1 / (alpha0 + alpha1 + alpha2)
      a = 1.0;
      b = std::pow(10.0, -40.0 + 130.0 * unif());
    } else if (kind == 2) {  // arbitrary bits, any sign, exponent anywhere
      a = from_bits(rnd());
      b = from_bits(rnd());
    } else if (kind == 3) {  // random significands, moderate exponents
      a = from_bits((rnd() & 0x800FFFFFFFFFFFFFull) | ((uint64_t)(900 + rnd() % 250) << 52));
      b = from_bits((rnd() & 0x800FFFFFFFFFFFFFull) | ((uint64_t)(900 + rnd() % 250) << 52));
    } else if (kind == 4) {  // significands near all-ones / power of two
      const uint64_t fa = (rnd() & 1) ? (0xFFFFFFFFFFFFFull - (rnd() & 0xFFFFFF)) : (rnd() & 0xFFFFFF);
      const uint64_t fb = (rnd() & 1) ? (0xFFFFFFFFFFFFFull - (rnd() & 0xFFFFFF)) : (rnd() & 0xFFFFFF);
      a = from_bits(fa | ((uint64_t)(1000 + rnd() % 40) << 52));
      b = from_bits(fb | ((uint64_t)(1000 + rnd() % 40) << 52));
    } else {  // quotients landing next to the rounding boundaries: a = q b +- a few ulps
      b = from_bits((rnd() & 0xFFFFFFFFFFFFFull) | (1023ull << 52));
      const double q = from_bits((rnd() & 0xFFFFFFFFFFFFFull) | ((uint64_t)(1020 + rnd() % 8) << 52));
      const double p = q * b;
      a = from_bits(to_bits(p) + (int64_t)(rnd() % 5) - 2);
    }
    check(a, b);
  }
  // edge cases: powers of two, extremes of the domain, special values
  const double edges[] = {1.0, 2.0, 0.5, 3.0, 1.5, 0.1, 1e-40, 1e-80, 1e300, 1e-300, 2.2250738585072014e-308,
                          4.9e-324, 1.7976931348623157e308, 0.0, -0.0, INFINITY, -INFINITY, NAN, -1.0, 7.0};
  for (double a : edges)
    for (double b : edges) check(a, b);
  printf("mismatches %lld checked %lld\n", bad, checked);
  return bad ? 1 : 0;
}
