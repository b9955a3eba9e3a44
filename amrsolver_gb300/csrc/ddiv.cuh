// Correctly rounded FP64 division a / b, multiplication a * b and square
// root sqrt(x) (IEEE round to nearest, ties to even) computed on the integer
// pipe.
//
// Why: on this GPU the FP64 pipe issues 2 lanes per clock per SM and every
// kernel of the path is bound by it; a hardware-style FP64 division
// (reciprocal seed plus Newton steps in DFMA) costs several FP64 issue slots.
// The same correctly rounded quotient can be formed from the operands' bits
// with 32/64-bit integer multiplies, which run on a unit with far more lanes
// and overlap with the FP64 work of other warps.  The quotient is the same
// number (IEEE division is correctly rounded, so any correct method gives the
// same bits): kernels that must match the reference bit for bit may use it.
//
// Method (long division by a fixed-point reciprocal with Newton-Raphson
// refinement and an exact remainder correction, as in integer division by
// invariant divisors, Granlund & Montgomery 1994, Moller & Granlund 2011):
//   significands ma, mb in [2^52, 2^53); d = mb * 2^11 in [2^63, 2^64)
//   y0  ~ 2^127 / d from a correctly rounded FP32 reciprocal of d's top 24
//       bits (relative error < 2^-22)
//   y  <- y + y (2^127 - d y) / 2^127, twice (error squares each time; the
//       truncations leave |y - 2^127/d| <= 4 units, relative < 2^-61)
//   Q~ = floor((ma * 2^11) y / 2^74), within 1 of Q = floor(ma 2^53 / mb)
//   R  = ma 2^53 - Q~ mb (exact in 64 bits since |R| < 2^54), one
//       correction step each way gives Q and 0 <= R < mb
//   Q in [2^53, 2^54): 54 quotient bits, the last one is the rounding bit and
//       R != 0 the sticky bit; Q in [2^52, 2^53): 53 bits, rounding decided
//       by comparing 2R with mb.
// Domain: b normal and finite, and either a = +-0 (result +-0) or a normal
// and finite with a result exponent that is normal with room for a rounding
// carry; anything else (b zero, subnormal, infinite or NaN, a subnormal,
// infinite or NaN, results that overflow or underflow) takes the hardware
// division, so the function equals a / b for every input.
#pragma once
#include <stdint.h>

#ifdef __CUDACC__
#define AMRS_HD __host__ __device__ __forceinline__
#else
#include <math.h>
#include <string.h>
#define AMRS_HD inline
#endif

namespace amrs {

AMRS_HD uint64_t ddiv_mulhi(uint64_t a, uint64_t b) {
#ifdef __CUDA_ARCH__
  return __umul64hi(a, b);
#else
  return (uint64_t)(((unsigned __int128)a * b) >> 64);
#endif
}

// The bits of x.  On the device an opaque move: the compiler would otherwise
// turn integer tests on a reinterpreted double (an exponent field equal to
// 0x7FF, (bits << 1) == 0) back into FP64 compares, each of which takes an
// FP64 issue slot -- the very resource these functions exist to spare
// (measured: 1 FP64 instruction per division and 4 per multiplication with a
// plain reinterpretation, none with the move).
AMRS_HD uint64_t ddiv_bits(double x) {
#ifdef __CUDA_ARCH__
  uint64_t u;
  asm("mov.b64 %0, %1;" : "=l"(u) : "d"(x));
  return u;
#else
  uint64_t u;
  memcpy(&u, &x, 8);
  return u;
#endif
}

AMRS_HD double ddiv_from_bits(uint64_t u) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)u);
#else
  double x;
  memcpy(&x, &u, 8);
  return x;
#endif
}

// The hardware operations for inputs outside the integer paths' domains, out
// of line: a call is a real branch taken only by lanes that need it, where an
// inlined fallback is predicated by the compiler and issues its FP64
// instruction on every call.
#ifdef __CUDA_ARCH__
static __device__ __noinline__ double ddiv_hw(double a, double b) { return a / b; }
static __device__ __noinline__ double dmul_hw(double a, double b) { return __dmul_rn(a, b); }
static __device__ __noinline__ double dsqrt_hw(double x) { return sqrt(x); }
#else
inline double ddiv_hw(double a, double b) { return a / b; }
inline double dmul_hw(double a, double b) { return a * b; }
inline double dsqrt_hw(double x) { return ::sqrt(x); }
#endif

// Seeds of the Newton iterations.  They need about 22 correct bits, not
// correct rounding: on the device the approximate FP32 reciprocal and
// reciprocal square root (rcp.approx / rsqrt.approx, within 1 ulp and
// 2^-22.9 relative), which run on the special-function unit and use no FP64
// slot.  The host build perturbs the correctly rounded value by up to
// +-2 ulps, so the host checks cover seeds at least that far off.
AMRS_HD uint32_t ddiv_seed_perturb(uint32_t rb, uint32_t v) {
#ifdef __CUDA_ARCH__
  (void)v;
  return rb;
#else
  return rb + (uint32_t)((int)((v ^ (v >> 7) ^ (v >> 13)) % 5u) - 2);
#endif
}

// Reciprocal of a float holding an integer dt in [2^23, 2^24) (relative
// error below 2^-22.5), returned as its bits.
AMRS_HD uint32_t ddiv_rcp_bits(uint32_t dt) {
  const uint32_t fb = 0x4B000000u | (dt & 0x7FFFFFu);  // the float equal to dt
#ifdef __CUDA_ARCH__
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(__uint_as_float(fb)));
  return __float_as_uint(r);
#else
  float f, r;
  memcpy(&f, &fb, 4);
  r = 1.0f / f;
  uint32_t rb;
  memcpy(&rb, &r, 4);
  return ddiv_seed_perturb(rb, dt);
#endif
}

// One Newton-Raphson step of y ~ 2^127 / d (d in [2^63, 2^64)).
AMRS_HD uint64_t ddiv_newton(uint64_t d, uint64_t y) {
  const uint64_t plo = d * y, phi = ddiv_mulhi(d, y);
  // e = 2^127 - d y as (ehi * 2^64 + elo), elo dropped: |ehi| < 2^43 here
  const int64_t ehi = (int64_t)((1ull << 63) - phi - (plo != 0 ? 1ull : 0ull));
  const uint64_t m = ehi < 0 ? (uint64_t)(-ehi) : (uint64_t)ehi;
  const uint64_t lo = y * m, hi = ddiv_mulhi(y, m);
  const uint64_t corr = (hi << 1) | (lo >> 63);  // y |e| / 2^127
  if (ehi < 0) return y - corr;
  const uint64_t s = y + corr;
  return s < y ? ~0ull : s;  // 2^127 / d <= 2^64: clamp a carry
}

// a / b, correctly rounded; the integer path where its domain holds.
AMRS_HD double ddiv_rn(double a, double b) {
  const uint64_t ua = ddiv_bits(a), ub = ddiv_bits(b);
  const int ea = (int)((ua >> 52) & 0x7FF), eb = (int)((ub >> 52) & 0x7FF);
  const int E = ea - eb + 1023;  // biased exponent of the quotient when ma >= mb
  const bool azero = (ua << 1) == 0;
  if (eb == 0 || eb == 0x7FF || (!azero && (ea == 0 || ea == 0x7FF || E < 2 || E > 2045))) return ddiv_hw(a, b);
  const uint64_t FRAC = (1ull << 52) - 1, HID = 1ull << 52;
  const uint64_t ma = (ua & FRAC) | HID, mb = (ub & FRAC) | HID;
  const uint64_t d = mb << 11;
  // seed: y0 = r * 2^87 with r ~ 1/dt, dt = d >> 40: r = m 2^(er - 23) gives
  // y0 = m << (er + 64); r lies near (2^-24, 2^-23], an approximate r may sit
  // just outside, and a y0 of 2^64 or more is clamped
  const uint32_t rb = ddiv_rcp_bits((uint32_t)(d >> 40));
  const int rsh = (int)((rb >> 23) & 0xFFu) - 127 + 64;
  const uint64_t y0 = rsh >= 41 ? ~0ull : ((uint64_t)((rb & 0x7FFFFFu) | 0x800000u) << rsh);
  const uint64_t y = ddiv_newton(d, ddiv_newton(d, y0));
  // quotient of X = ma 2^53 by mb
  uint64_t q = ddiv_mulhi(ma << 11, y) >> 10;
  int64_t r = (int64_t)((ma << 53) - q * mb);
  if (r < 0) {
    q -= 1;
    r += (int64_t)mb;
  } else if (r >= (int64_t)mb) {
    q += 1;
    r -= (int64_t)mb;
  }
  uint64_t sig, inc;
  int ebias;
  if (q >= (1ull << 53)) {
    sig = q >> 1;
    const uint64_t round = q & 1ull, sticky = r != 0 ? 1ull : 0ull;
    inc = round & (sticky | (sig & 1ull));
    ebias = E;
  } else {
    sig = q;
    const uint64_t twor = (uint64_t)r << 1;
    inc = (twor > mb || (twor == mb && (sig & 1ull))) ? 1ull : 0ull;
    ebias = E - 1;
  }
  // (ebias - 1) << 52 plus the 53-bit significand (hidden bit included);
  // a rounding carry to 2^53 moves into the exponent by itself
  const uint64_t mag = azero ? 0ull : ((uint64_t)(ebias - 1) << 52) + sig + inc;
  return ddiv_from_bits(mag | ((ua ^ ub) & (1ull << 63)));
}

// a * b, correctly rounded (IEEE round to nearest, ties to even), computed on
// the integer pipe.  Significands ma, mb in [2^52, 2^53): the exact product
// P = ma mb lies in [2^104, 2^106); (ma 2^11)(mb 2) = P 2^12 is formed as a
// 128-bit integer whose high word is floor(P / 2^52) in [2^52, 2^54) and
// whose low word holds the remaining bits of P.  A high word of 2^53 or more
// gives the 53-bit significand P >> 53 with bit 52 of P as the rounding bit;
// otherwise P >> 52 with bit 51; the bits below are the sticky bit.
// Domain: a and b normal and finite with a normal result exponent, or either
// one +-0 and the other finite (result +-0); anything else (subnormal,
// infinite or NaN operands, products that underflow) takes the hardware
// multiplication, so the function equals a * b for every input.  A product
// that rounds up past the largest finite number becomes +-inf, as IEEE
// rounding to nearest gives.
AMRS_HD double dmul_rn(double a, double b) {
  const uint64_t ua = ddiv_bits(a), ub = ddiv_bits(b);
  const int ea = (int)((ua >> 52) & 0x7FF), eb = (int)((ub >> 52) & 0x7FF);
  const int E = ea + eb - 1023;  // biased exponent of the product when P < 2^105
  const bool fin = ea != 0x7FF && eb != 0x7FF;
  const bool zero = fin && ((ua << 1) == 0 || (ub << 1) == 0);
  if (!zero && (ea == 0 || eb == 0 || !fin || E < 1 || E > 2045)) return dmul_hw(a, b);
  const uint64_t X = (ua << 11) | (1ull << 63);                     // ma 2^11
  const uint64_t Y = ((ub << 1) & ((1ull << 53) - 2)) | (1ull << 53);  // mb 2
  const uint64_t hi = ddiv_mulhi(X, Y), lo = X * Y;
  const bool top = (hi >> 53) != 0;
  const uint64_t sig = top ? (hi >> 1) : hi;
  const uint64_t round = top ? (hi & 1ull) : (lo >> 63);
  const uint64_t sticky = (top ? lo : (lo << 1)) != 0 ? 1ull : 0ull;
  const uint64_t inc = round & (sticky | (sig & 1ull));
  const int eres = top ? E + 1 : E;
  const uint64_t mag = zero ? 0ull : ((uint64_t)(eres - 1) << 52) + sig + inc;
  return ddiv_from_bits(mag | ((ua ^ ub) & (1ull << 63)));
}

// Reciprocal square root of a float holding an integer v in [2^22, 2^24)
// (relative error below 2^-22.5), returned as its bits.
AMRS_HD uint32_t dsqrt_rsqrt_bits(uint32_t v) {
  // v as a float without a conversion instruction: 2^23 + low bits, or
  // 2^22 + low bits for v below 2^23
  const uint32_t fb = (v >> 23) ? (0x4B000000u | (v & 0x7FFFFFu)) : (0x4A800000u | ((v << 1) & 0x7FFFFFu));
#ifdef __CUDA_ARCH__
  float r;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(__uint_as_float(fb)));
  return __float_as_uint(r);
#else
  float f;
  memcpy(&f, &fb, 4);
  const float r = (float)(1.0 / sqrt((double)f));
  uint32_t rb;
  memcpy(&rb, &r, 4);
  return ddiv_seed_perturb(rb, v);
#endif
}

// One Newton-Raphson step of y ~ 2^95 / sqrt(n) (n in [2^62, 2^64)):
// y <- y + y (1 - n y^2 / 2^190) / 2.
AMRS_HD uint64_t dsqrt_newton(uint64_t n, uint64_t y) {
  const uint64_t t = ddiv_mulhi(y, y);             // y^2 / 2^64
  const uint64_t u = ddiv_mulhi(n, t);             // n y^2 / 2^128, ~2^62
  const int64_t e = (int64_t)((1ull << 62) - u);   // 2^62 (1 - n y^2 / 2^190)
  const uint64_t m = e < 0 ? (uint64_t)(-e) : (uint64_t)e;
  const uint64_t lo = y * m, hi = ddiv_mulhi(y, m);
  const uint64_t corr = (hi << 1) | (lo >> 63);    // y |e| / 2^63
  if (e < 0) return y - corr;
  const uint64_t s = y + corr;
  return s < y ? ~0ull : s;
}

// sqrt(x), correctly rounded (IEEE round to nearest even), computed on the
// integer pipe for positive normal x (and +-0); anything else takes the
// hardware square root, so the function equals sqrt(x) for every input.
// Method: x = M 2^(2k) with N = M 2^104 an integer in [2^104, 2^106); a
// fixed-point reciprocal square root y ~ 2^95 / sqrt(N / 2^42) from a
// correctly rounded FP32 rsqrt seed and two Newton-Raphson steps (relative
// error < 2^-60); S~ = floor(sqrt(N)) within 1 from (N / 2^42) y / 2^74; the
// exact remainder R = N - S^2 (|R| < 2^55, exact in 64-bit arithmetic) fixes
// S and decides the rounding: up iff R > S (N is an integer, so it never
// equals (S + 1/2)^2).
AMRS_HD double dsqrt_rn(double x) {
  const uint64_t ux = ddiv_bits(x);
  const int ex = (int)(ux >> 52);  // sign bit included: negative x lands above 0x7FF
  if ((ux << 1) == 0) return x;     // +-0
  if (ex == 0 || ex >= 0x7FF) return dsqrt_hw(x);
  const int e = ex - 1023;
  const uint64_t mx = (ux & ((1ull << 52) - 1)) | (1ull << 52);
  const uint64_t N_lo = (e & 1) ? (mx << 53) : (mx << 52);  // N mod 2^64
  const uint64_t n64 = (e & 1) ? (mx << 11) : (mx << 10);   // N / 2^42, in [2^62, 2^64)
  const uint32_t rb = dsqrt_rsqrt_bits((uint32_t)(n64 >> 40));
  // y0 = rsqrt * 2^75 = m << (er + 52) for rsqrt = m 2^(er - 23) near (2^-12, 2^-11];
  // an approximate value may sit just outside, and 2^64 or more is clamped
  const int rsh = (int)((rb >> 23) & 0xFFu) - 127 + 52;
  const uint64_t y0 = rsh >= 41 ? ~0ull : ((uint64_t)((rb & 0x7FFFFFu) | 0x800000u) << rsh);
  const uint64_t y = dsqrt_newton(n64, dsqrt_newton(n64, y0));
  uint64_t S = ddiv_mulhi(n64, y) >> 10;
  int64_t R = (int64_t)(N_lo - S * S);
  if (R < 0) {
    S -= 1;
    R += (int64_t)(2 * S + 1);
  } else if (R > (int64_t)(2 * S)) {
    R -= (int64_t)(2 * S + 1);
    S += 1;
  }
  const uint64_t inc = R > (int64_t)S ? 1ull : 0ull;
  const int eb = (e >> 1) + 1023;  // floor(e / 2), biased
  return ddiv_from_bits(((uint64_t)(eb - 1) << 52) + S + inc);
}

}  // namespace amrs
