// Host check of amrs::dsqrt_rn (amrsolver_gb300/csrc/ddiv.cuh) against the
// host's IEEE square root: random operands (arbitrary bits, positive
// doubles over the whole exponent range, significands near powers of two,
// squares of random doubles and their neighbours) and special values.
//   dsqrt_check <count> <seed>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "../../amrsolver_gb300/csrc/ddiv.cuh"

static uint64_t s_state;
static uint64_t rnd() {
  uint64_t z = (s_state += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
static double from_bits(uint64_t u) { double x; memcpy(&x, &u, 8); return x; }
static uint64_t to_bits(double x) { uint64_t u; memcpy(&u, &x, 8); return u; }

static long long bad = 0, checked = 0;
static void check(double x) {
  const double ref = std::sqrt(x), got = amrs::dsqrt_rn(x);
  ++checked;
  if (to_bits(ref) != to_bits(got) && !(std::isnan(ref) && std::isnan(got))) {
    if (bad < 10) printf("MISMATCH x=%a ref=%a got=%a\n", x, ref, got);
    ++bad;
  }
}

int main(int argc, char** argv) {
  const long long n = argc > 1 ? atoll(argv[1]) : 1000000;
  s_state = argc > 2 ? strtoull(argv[2], nullptr, 10) : 1;
  for (long long i = 0; i < n; ++i) {
    const int kind = (int)(i % 4);
    double x;
    if (kind == 0) x = from_bits(rnd());
    else if (kind == 1) x = from_bits(rnd() & 0x7FFFFFFFFFFFFFFFull);
    else if (kind == 2) {
      const uint64_t f = (rnd() & 1) ? (0xFFFFFFFFFFFFFull - (rnd() & 0xFFFFFF)) : (rnd() & 0xFFFFFF);
      x = from_bits(f | ((uint64_t)(1 + rnd() % 2046) << 52));
    } else {
      const double r = from_bits((rnd() & 0xFFFFFFFFFFFFFull) | ((uint64_t)(600 + rnd() % 800) << 52));
      x = from_bits(to_bits(r * r) + (int64_t)(rnd() % 5) - 2);
    }
    check(x);
  }
  const double edges[] = {0.0, -0.0, 1.0, 2.0, 4.0, 0.25, 3.0, 1e-300, 1e300, 2.2250738585072014e-308, 4.9e-324,
                          1.7976931348623157e308, INFINITY, -INFINITY, NAN, -1.0, 1.4 * 0.71};
  for (double x : edges) check(x);
  printf("mismatches %lld checked %lld\n", bad, checked);
  return bad ? 1 : 0;
}
