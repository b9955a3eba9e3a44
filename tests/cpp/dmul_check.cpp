// Host check of amrs::dmul_rn (amrsolver_gb300/csrc/ddiv.cuh) against the
// host's IEEE double multiplication: random operands from several
// distributions (arbitrary bits, moderate exponents, significands near
// all-ones and powers of two, short significands whose products fall on
// rounding ties, exponents at the edges of the integer path's domain) plus
// hand-picked edge cases; prints "mismatches N checked M" and exits non-zero
// on any difference in the bits.
//   dmul_check <count> <seed>
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

static long long bad = 0, checked = 0;
static void check(double a, double b) {
  volatile double va = a, vb = b;
  const double ref = va * vb, got = amrs::dmul_rn(a, b);
  ++checked;
  if (to_bits(ref) != to_bits(got) && !(std::isnan(ref) && std::isnan(got))) {
    if (bad < 10) printf("MISMATCH a=%a b=%a ref=%a got=%a\n", a, b, ref, got);
    ++bad;
  }
}

static uint64_t sign() { return (rnd() & 1) ? (1ull << 63) : 0ull; }

int main(int argc, char** argv) {
  const long long n = argc > 1 ? atoll(argv[1]) : 1000000;
  s_state = argc > 2 ? strtoull(argv[2], nullptr, 10) : 1;
  for (long long i = 0; i < n; ++i) {
    const int kind = (int)(i % 6);
    double a, b;
    if (kind == 0) {  // arbitrary bits, any sign, exponent anywhere
      a = from_bits(rnd());
      b = from_bits(rnd());
    } else if (kind == 1) {  // random significands and signs, moderate exponents
      a = from_bits((rnd() & 0x800FFFFFFFFFFFFFull) | ((uint64_t)(900 + rnd() % 250) << 52));
      b = from_bits((rnd() & 0x800FFFFFFFFFFFFFull) | ((uint64_t)(900 + rnd() % 250) << 52));
    } else if (kind == 2) {  // significands near all-ones / power of two
      const uint64_t fa = (rnd() & 1) ? (0xFFFFFFFFFFFFFull - (rnd() & 0xFFFFFF)) : (rnd() & 0xFFFFFF);
      const uint64_t fb = (rnd() & 1) ? (0xFFFFFFFFFFFFFull - (rnd() & 0xFFFFFF)) : (rnd() & 0xFFFFFF);
      a = from_bits(sign() | fa | ((uint64_t)(1000 + rnd() % 40) << 52));
      b = from_bits(sign() | fb | ((uint64_t)(1000 + rnd() % 40) << 52));
    } else if (kind == 3) {  // short significands: 53- or 54-bit products, ties to even
      const int wa = 20 + (int)(rnd() % 14), wb = 54 - wa + (int)(rnd() % 3) - 1;
      const uint64_t sa = ((rnd() & ((1ull << (wa - 1)) - 1)) | (1ull << (wa - 1))) << (53 - wa);
      const uint64_t sb = ((rnd() & ((1ull << (wb - 1)) - 1)) | (1ull << (wb - 1))) << (53 - wb);
      a = from_bits(sign() | (sa & 0xFFFFFFFFFFFFFull) | ((uint64_t)(1000 + rnd() % 40) << 52));
      b = from_bits(sign() | (sb & 0xFFFFFFFFFFFFFull) | ((uint64_t)(1000 + rnd() % 40) << 52));
    } else if (kind == 4) {  // exponent sums at the edges of the domain (underflow, overflow)
      const int ea = 1 + (int)(rnd() % 2046);
      const int target = (rnd() & 1) ? (int)(rnd() % 6) - 3 : 2043 + (int)(rnd() % 6);
      int eb = target - ea + 1023;
      if (eb < 0) eb = 0;
      if (eb > 2046) eb = 2046;
      a = from_bits(sign() | (rnd() & 0xFFFFFFFFFFFFFull) | ((uint64_t)ea << 52));
      b = from_bits(sign() | (rnd() & 0xFFFFFFFFFFFFFull) | ((uint64_t)eb << 52));
    } else {  // zeros, subnormals and specials against random values
      const uint64_t sp[6] = {0ull, 1ull << 63, 0x7FF0000000000000ull, 0x7FF8000000000000ull, rnd() & 0xFFFFFFFFFFFFFull,
                              rnd() & 0x800FFFFFFFFFFFFFull};
      a = from_bits(sp[rnd() % 6]);
      b = from_bits((rnd() & 0x800FFFFFFFFFFFFFull) | ((uint64_t)(rnd() % 2048) << 52));
      if (rnd() & 1) { const double t = a; a = b; b = t; }
    }
    check(a, b);
  }
  const double edges[] = {1.0, 2.0, 0.5, 3.0, 1.5, 0.1, 1e-40, 1e-80, 1e300, 1e-300, 2.2250738585072014e-308,
                          4.9e-324, 1.7976931348623157e308, 0.0, -0.0, INFINITY, -INFINITY, NAN, -1.0, 7.0,
                          1.0000000000000002, 0.99999999999999989, 1.4142135623730951, 1e154, 1e-154};
  for (double a : edges)
    for (double b : edges) check(a, b);
  printf("mismatches %lld checked %lld\n", bad, checked);
  return bad ? 1 : 0;
}
