// CPU oracle for amrsolver's compressible RHS + SSP-RK stage path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the checker: only tests/, the smoke
// check in __graft_entry__.py and bench.py's CPU-baseline / reference arm may
// load the library built from it.  The GPU product never links or calls it.
//
// It restates, operation by operation and in the same floating-point order,
// the reference functions listed beside each template below (paths are inside
// the Monal-Patel/amrsolver tree).  The restatement is templated on the scalar
// type so the same source yields
//   * double      : the oracle proper (built with -ffp-contract=off),
//   * Cnt         : an operation-counting scalar (algorithmic flop counts),
//   * Dual        : forward-mode dual numbers (Jacobian-vector products).
//
// Parity pin: oracle/build_ref.sh compiles the reference's own headers and
// src/tim/CNS_advance.cpp (unmodified, against a from-scratch stand-in for the
// few AMReX types they use) into oracle/_ref/libcnsref.so; tests compare this
// restatement with that build bit for bit, and tests/golden/*.npz hold
// vectors produced by that build so the pin also holds where the reference
// sources are absent.
// WENO5-Riemann (the riemann_weno extension, flux code 3 here) has no
// reference counterpart: for it this file is the specification, and its
// parity is unpinned against the reference.
//
// Layout of every field (Array4 convention): component-major, i fastest,
// ghost-inclusive.  A box [lo,hi] with g ghosts is stored as
// (ncomp, nz+2g, ny+2g, nx+2g) in C order.

#include <cmath>
#include <cstdint>
#include <cstring>
#include <cstdio>
#include <limits>
#include <vector>
#include <algorithm>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace orc {

// ---------------------------------------------------------------- scalars --
struct OpCounts { long long add = 0, mul = 0, div = 0, sqrt = 0, cmp = 0; };
// phases of compute_rhs: 0 cons2prim, 1 Euler face fluxes, 2 JST,
// 3 viscous cell fluxes, 4 viscous face averages, 5 flux divergence
constexpr int NPHASE = 6;
static thread_local OpCounts g_cntp[NPHASE];
static thread_local int g_phase = 0;
#define g_cnt g_cntp[g_phase]

// Operation-counting scalar.  +,-,* and / each count 1 in their bucket;
// sqrt counts 1; comparisons (max/min/branches) count in cmp; unary minus,
// abs and copysign are sign-bit operations and count nothing.
struct Cnt {
  double v;
  Cnt(double x = 0.0) : v(x) {}
};
inline Cnt operator+(Cnt a, Cnt b) { g_cnt.add++; return Cnt(a.v + b.v); }
inline Cnt operator-(Cnt a, Cnt b) { g_cnt.add++; return Cnt(a.v - b.v); }
inline Cnt operator*(Cnt a, Cnt b) { g_cnt.mul++; return Cnt(a.v * b.v); }
inline Cnt operator/(Cnt a, Cnt b) { g_cnt.div++; return Cnt(a.v / b.v); }
inline Cnt operator-(Cnt a) { return Cnt(-a.v); }
inline Cnt& operator+=(Cnt& a, Cnt b) { a = a + b; return a; }
inline Cnt& operator-=(Cnt& a, Cnt b) { a = a - b; return a; }
inline bool operator<(Cnt a, Cnt b) { g_cnt.cmp++; return a.v < b.v; }
inline bool operator>(Cnt a, Cnt b) { g_cnt.cmp++; return a.v > b.v; }
inline bool operator>=(Cnt a, Cnt b) { g_cnt.cmp++; return a.v >= b.v; }
inline Cnt sqrt(Cnt a) { g_cnt.sqrt++; return Cnt(std::sqrt(a.v)); }
inline Cnt fabs(Cnt a) { return Cnt(std::fabs(a.v)); }
inline Cnt copysign(Cnt a, Cnt b) { return Cnt(std::copysign(a.v, b.v)); }
inline double val(Cnt a) { return a.v; }

// Forward-mode dual number: value v and one tangent d.
// max/min/abs/branches follow the value (subgradient of the taken branch).
struct Dual {
  double v, d;
  Dual(double x = 0.0, double dx = 0.0) : v(x), d(dx) {}
};
inline Dual operator+(Dual a, Dual b) { return Dual(a.v + b.v, a.d + b.d); }
inline Dual operator-(Dual a, Dual b) { return Dual(a.v - b.v, a.d - b.d); }
inline Dual operator*(Dual a, Dual b) { return Dual(a.v * b.v, a.d * b.v + a.v * b.d); }
inline Dual operator/(Dual a, Dual b) {
  double q = a.v / b.v;
  return Dual(q, (a.d - q * b.d) / b.v);
}
inline Dual operator-(Dual a) { return Dual(-a.v, -a.d); }
inline Dual& operator+=(Dual& a, Dual b) { a = a + b; return a; }
inline Dual& operator-=(Dual& a, Dual b) { a = a - b; return a; }
inline bool operator<(Dual a, Dual b) { return a.v < b.v; }
inline bool operator>(Dual a, Dual b) { return a.v > b.v; }
inline bool operator>=(Dual a, Dual b) { return a.v >= b.v; }
inline Dual sqrt(Dual a) {
  double s = std::sqrt(a.v);
  return Dual(s, a.d / (2.0 * s));
}
inline Dual fabs(Dual a) { return a.v < 0 ? Dual(-a.v, -a.d) : a; }
inline Dual copysign(Dual a, Dual b) {
  double r = std::copysign(a.v, b.v);
  return Dual(r, (r == a.v) ? a.d : -a.d);
}
inline double val(Dual a) { return a.v; }

inline double val(double a) { return a; }
using std::sqrt;
using std::fabs;
using std::copysign;

// std::max / std::min semantics (what the reference's amrex::max/min use).
template <class R> inline R rmax(const R& a, const R& b) { return (a < b) ? b : a; }
template <class R> inline R rmin(const R& a, const R& b) { return (b < a) ? b : a; }
template <class R> inline R rmax3(const R& a, const R& b, const R& c) { return rmax(rmax(a, b), c); }

// pow(x, 2) as the reference evaluates it (std::pow with an int exponent
// promotes to pow(double,double)); the other scalars square directly.
inline double pow2(double x) { return std::pow(x, 2.0); }
inline Cnt pow2(Cnt x) { return x * x; }
inline Dual pow2(Dual x) { return x * x; }

// ------------------------------------------------------------------ layout --
constexpr int URHO = 0, UMX = 1, UMY = 2, UMZ = 3, UET = 4, NCONS = 5;
constexpr int QRHO = 0, QU = 1, QV = 2, QW = 3, QT = 4, QPRES = 5, NPRIM = 6;
constexpr int NGHOST = 3;

struct Box {
  int lo[3], hi[3];
  int n(int d) const { return hi[d] - lo[d] + 1; }
  long long cells() const { return (long long)n(0) * n(1) * n(2); }
};

// Array4-like view: p points at (blo, n=0).
template <class R> struct Arr {
  R* p = nullptr;
  long long js = 0, ks = 0, ns = 0;
  int b0 = 0, b1 = 0, b2 = 0;
  R& operator()(int i, int j, int k, int n = 0) const {
    return p[(i - b0) + (j - b1) * js + (k - b2) * ks + n * ns];
  }
};

template <class R> Arr<R> make_arr(R* p, const Box& b, int g) {
  Arr<R> a;
  a.p = p;
  int nx = b.n(0) + 2 * g, ny = b.n(1) + 2 * g, nz = b.n(2) + 2 * g;
  a.js = nx;
  a.ks = (long long)nx * ny;
  a.ns = (long long)nx * ny * nz;
  a.b0 = b.lo[0] - g;
  a.b1 = b.lo[1] - g;
  a.b2 = b.lo[2] - g;
  return a;
}

// Nodal (face) array in direction d over [lo,hi] with hi+1 in d.
template <class R> Arr<R> make_face_arr(R* p, const Box& b, int d) {
  Arr<R> a;
  a.p = p;
  int nx = b.n(0) + (d == 0), ny = b.n(1) + (d == 1), nz = b.n(2) + (d == 2);
  a.js = nx;
  a.ks = (long long)nx * ny;
  a.ns = (long long)nx * ny * nz;
  a.b0 = b.lo[0];
  a.b1 = b.lo[1];
  a.b2 = b.lo[2];
  return a;
}

// ---------------------------------------------------------------- closures --
// Ideal gas + transport, src/cls/Closures.h:72-166.  visc_law 0 = constant
// (visc_const_t, :103-110), 1 = Sutherland (visc_suth_t, :112-120);
// cond_law 0 = constant (cond_const_t, :130-143), 1 = Sutherland
// (cond_suth_t, :155-166).  Cshock/Cdamp: closures_derived_t, :172-182.
struct Closures {
  double gamma, cv, cp, Rspec;
  int visc_law;
  double visc_ref, Tvisc_ref;
  int cond_law;
  double cond_ref, Tcond_ref;
  double Cshock, Cdamp;
  template <class R> R visc(const R& T) const {
    if (visc_law == 0) return R(visc_ref);
    return R(visc_ref) * T * sqrt(T) / (R(Tvisc_ref) + T);
  }
  template <class R> R cond(const R& T) const {
    if (cond_law == 0) return R(cond_ref);
    return R(cond_ref) * T * sqrt(T) / (R(Tcond_ref) + T);
  }
};

// Scheme switches, the reference's cns.* run-time keys (src/CNS.cpp:85-136).
struct Scheme {
  int rhs_euler;   // cns.rhs_euler
  int rhs_visc;    // cns.rhs_visc
  int flux_euler;  // 1 = KEEP, 2 = WENO5-JS LLF, 3 = WENO5-Riemann (extension), other = MUSCL + Riemann
  int order_keep;  // 2, 4, 6
  int art_diss;    // JST artificial dissipation
  int rhs_source;  // cns.rhs_source, with the body-force source below
  double force[3]; // body force per unit mass of the source term
};

// KEEP coefficients, CPU branch of the reference (src/CNS.cpp:241-252).
inline void keep_coeffs(int order, double c[3]) {
  if (order == 6) {
    c[0] = 6.0 / 4; c[1] = -6.0 / 20; c[2] = 2.0 / 60;
  } else if (order == 4) {
    c[0] = 4.0 / 3; c[1] = -2.0 / 12; c[2] = 0.0;
  } else {
    c[0] = 1.0; c[1] = 0.0; c[2] = 0.0;
  }
}

// ---------------------------------------------------------- point kernels --
// cons2prim: src/rhs/CNS_hydro_K.h:15-34.
template <class R>
inline void cons2prim(int i, int j, int k, const Arr<R>& u, const Arr<R>& q, const Closures& cl) {
  R rho = u(i, j, k, URHO);
  rho = rmax(R(1e-40), rho);
  R rhoinv = R(1.0) / rho;
  R ux = u(i, j, k, UMX) * rhoinv;
  R uy = u(i, j, k, UMY) * rhoinv;
  R uz = u(i, j, k, UMZ) * rhoinv;
  R rhoke = R(0.5) * rho * (ux * ux + uy * uy + uz * uz);
  R rhoei = (u(i, j, k, UET) - rhoke);
  R p = (R(cl.gamma) - R(1.0)) * rhoei;
  q(i, j, k, QRHO) = rho;
  q(i, j, k, QU) = ux;
  q(i, j, k, QV) = uy;
  q(i, j, k, QW) = uz;
  q(i, j, k, QPRES) = p;
  q(i, j, k, QT) = p / (rho * R(cl.Rspec));
}

// KEEP split-form flux at the d-face below (i,j,k): src/rhs/CentralKEEP.h:19-36
// (fDiv, fgDiv, fgQuad, fghCubic) and :40-145 (KEEP), one direction at a time.
// The three direction blocks of the reference differ only in which velocity
// is normal; argument orders of every helper are kept.
template <class R>
inline void keep_face(int i, int j, int k, int d, int halfsten, const double* coeffs,
                      const Arr<R>& q, R F[NCONS], const Closures& cl) {
  const int di = (d == 0), dj = (d == 1), dk = (d == 2);
  const int QN = QU + d;  // normal velocity
  for (int n = 0; n < NCONS; ++n) F[n] = R(0.0);
  for (int l = 1; l <= halfsten; l++) {
    for (int m = 0; m <= l - 1; m++) {
      const int o1 = m, o2 = m - l;
      const int i1 = i + o1 * di, j1 = j + o1 * dj, k1 = k + o1 * dk;
      const int i2 = i + o2 * di, j2 = j + o2 * dj, k2 = k + o2 * dk;
      R rho1 = q(i1, j1, k1, QRHO), ux1 = q(i1, j1, k1, QU), uy1 = q(i1, j1, k1, QV),
        uz1 = q(i1, j1, k1, QW), ie1 = R(cl.cv) * q(i1, j1, k1, QT), p1 = q(i1, j1, k1, QPRES);
      R rho2 = q(i2, j2, k2, QRHO), ux2 = q(i2, j2, k2, QU), uy2 = q(i2, j2, k2, QV),
        uz2 = q(i2, j2, k2, QW), ie2 = R(cl.cv) * q(i2, j2, k2, QT), p2 = q(i2, j2, k2, QPRES);
      R un1 = q(i1, j1, k1, QN), un2 = q(i2, j2, k2, QN);
      const R c = R(coeffs[l - 1]);
      // fgQuad(rho1,rho2,un1,un2) = 0.25*(f+fl)*(g+gl)
      R massflx = R(0.25) * (rho1 + rho2) * (un1 + un2);
      R ke = R(0.5) * (ux1 * ux2 + uy1 * uy2 + uz1 * uz2);
      // fghCubic(f,fl,g,gl,h,hl) = 0.125*(f+fl)*(g+gl)*(h+hl)
      auto cubic = [&](const R& h1, const R& h2) {
        return R(0.1250) * (rho1 + rho2) * (un1 + un2) * (h1 + h2);
      };
      R fdiv = R(0.5) * (p1 + p2);                 // fDiv(p1,p2)
      R fgdiv = R(0.5) * (p1 * un2 + p2 * un1);    // fgDiv(p1,p2,un1,un2)
      F[URHO] += c * massflx;
      F[UMX] += c * (d == 0 ? (cubic(ux1, ux2) + fdiv) : cubic(ux1, ux2));
      F[UMY] += c * (d == 1 ? (cubic(uy1, uy2) + fdiv) : cubic(uy1, uy2));
      F[UMZ] += c * (d == 2 ? (cubic(uz1, uz2) + fdiv) : cubic(uz1, uz2));
      F[UET] += c * (massflx * ke + cubic(ie1, ie2) + fgdiv);
    }
  }
}

// Physical Euler fluxes and max eigenvalue: src/rhs/High_resolution.h:83-121.
template <class R>
inline void cons2eulerflux_lambda(int i, int j, int k, const Arr<R>& u, const Arr<R> pf[3],
                                  const Arr<R>& lam, const Closures& cl) {
  R rhoinv = R(1.0) / u(i, j, k, URHO);
  R momx = u(i, j, k, UMX), momy = u(i, j, k, UMY), momz = u(i, j, k, UMZ), rhoet = u(i, j, k, UET);
  R ux = momx * rhoinv, uy = momy * rhoinv, uz = momz * rhoinv;
  R rhoekin = R(0.5) * rhoinv * (momx * momx + momy * momy + momz * momz);
  R rhoeint = rhoet - rhoekin;
  R P = (R(cl.gamma) - R(1.0)) * rhoeint;
  pf[0](i, j, k, URHO) = momx;
  pf[0](i, j, k, UMX) = momx * ux + P;
  pf[0](i, j, k, UMY) = momy * ux;
  pf[0](i, j, k, UMZ) = momz * ux;
  pf[0](i, j, k, UET) = (rhoet + P) * ux;
  pf[1](i, j, k, URHO) = momy;
  pf[1](i, j, k, UMX) = momx * uy;
  pf[1](i, j, k, UMY) = momy * uy + P;
  pf[1](i, j, k, UMZ) = momz * uy;
  pf[1](i, j, k, UET) = (rhoet + P) * uy;
  pf[2](i, j, k, URHO) = momz;
  pf[2](i, j, k, UMX) = momx * uz;
  pf[2](i, j, k, UMY) = momy * uz;
  pf[2](i, j, k, UMZ) = momz * uz + P;
  pf[2](i, j, k, UET) = (rhoet + P) * uz;
  R cs = sqrt(R(cl.gamma) * P * rhoinv);
  lam(i, j, k, 0) = fabs(rmax3(ux + cs, ux - cs, ux));
  lam(i, j, k, 1) = fabs(rmax3(uy + cs, uy - cs, uy));
  lam(i, j, k, 2) = fabs(rmax3(uz + cs, uz - cs, uz));
}

// WENO5-JS upwind-biased face value: src/rhs/High_resolution.h:124-159
// (including the fourth-power smoothness term of beta[1]).
template <class R> inline R weno5js(const R s[5]) {
  const R eps = R(1e-40);
  R beta0 = R(13.0 / 12.0) * (s[0] - R(2.0) * s[1] + s[2]) * (s[0] - R(2.0) * s[1] + s[2]) +
            R(0.25) * (s[0] - R(4.0) * s[1] + R(3.0) * s[2]) * (s[0] - R(4.0) * s[1] + R(3.0) * s[2]);
  R beta1 = R(13.0 / 12.0) * (s[1] - R(2.0) * s[2] + s[3]) * (s[1] - R(2.0) * s[2] + s[3]) +
            R(0.25) * (s[1] - s[3]) * (s[1] - s[3]) * (s[1] - s[3]) * (s[1] - s[3]);
  R beta2 = R(13.0 / 12.0) * (s[2] - R(2.0) * s[3] + s[4]) * (s[2] - R(2.0) * s[3] + s[4]) +
            R(0.25) * (R(3.0) * s[2] - R(4.0) * s[3] + s[4]) * (R(3.0) * s[2] - R(4.0) * s[3] + s[4]);
  R alpha0 = R(0.1) / pow2(eps + beta0);
  R alpha1 = R(0.6) / pow2(eps + beta1);
  R alpha2 = R(0.3) / pow2(eps + beta2);
  R sum = R(1.0) / (alpha0 + alpha1 + alpha2);
  R vl0 = R(2.0) * s[0] - R(7.0) * s[1] + R(11.0) * s[2];
  R vl1 = -s[1] + R(5.0) * s[2] + R(2.0) * s[3];
  R vl2 = R(2.0) * s[2] + R(5.0) * s[3] - s[4];
  return R(1.0 / 6.0) * sum * (alpha0 * vl0 + alpha1 * vl1 + alpha2 * vl2);
}

// Local Lax-Friedrichs split WENO flux at the d-face below (i,j,k), comp n:
// src/rhs/High_resolution.h:162-246.
template <class R>
inline R weno_llf_face(int i, int j, int k, int n, int d, const Arr<R>& u, const Arr<R>& pf,
                       const Arr<R>& lam) {
  const int di = (d == 0), dj = (d == 1), dk = (d == 2);
  auto L = [&](int o) { return lam(i + o * di, j + o * dj, k + o * dk, d); };
  auto U = [&](int o) { return u(i + o * di, j + o * dj, k + o * dk, n); };
  auto P = [&](int o) { return pf(i + o * di, j + o * dj, k + o * dk, n); };
  R maxeigen = rmax(rmax(rmax(rmax(rmax(L(-3), L(-2)), L(-1)), L(0)), L(1)), L(2));
  R df[6];
  for (int q = 0; q < 6; ++q) df[q] = maxeigen * U(q - 3);
  R sten[5];
  for (int q = 0; q < 5; ++q) sten[q] = R(0.5) * (P(q - 3) + df[q]);
  R flx = weno5js(sten);
  sten[4] = R(0.5) * (P(-2) - df[1]);
  sten[3] = R(0.5) * (P(-1) - df[2]);
  sten[2] = R(0.5) * (P(0) - df[3]);
  sten[1] = R(0.5) * (P(1) - df[4]);
  sten[0] = R(0.5) * (P(2) - df[5]);
  flx += weno5js(sten);
  return flx;
}

// MC limiter: src/rhs/Riemann.h:9-17.
template <class R> inline R limiter(R dlft, R drgt) {
  R dcen = R(0.5) * (dlft + drgt);
  R dsgn = copysign(R(1.0), dcen);
  R slop = R(2.0) * rmin(fabs(dlft), fabs(drgt));
  R dlim = (dlft * drgt >= R(0.0)) ? slop : R(0.0);
  return dsgn * rmin(dlim, fabs(dcen));
}

// Characteristic slopes in direction d: src/rhs/Riemann.h:19-120
// (cns_slope_x adds 2e-40 to the sound speed, y and z add 1e-40).
template <class R>
inline void cns_slope(int i, int j, int k, int d, const Arr<R>& dq, const Arr<R>& q, const Closures& cl) {
  const int di = (d == 0), dj = (d == 1), dk = (d == 2);
  const int QN = QU + d;
  const int QT1 = (d == 0) ? QV : QU;
  const int QT2 = (d == 2) ? QV : QW;
  const int im = i - di, jm = j - dj, km = k - dk, ip = i + di, jp = j + dj, kp = k + dk;
  R cspeed = sqrt(R(cl.gamma) * R(cl.Rspec) * q(i, j, k, QT)) + R(d == 0 ? 2.e-40 : 1.e-40);
  R dlft = R(0.5) * (q(i, j, k, QPRES) - q(im, jm, km, QPRES)) / cspeed -
           R(0.5) * q(i, j, k, QRHO) * (q(i, j, k, QN) - q(im, jm, km, QN));
  R drgt = R(0.5) * (q(ip, jp, kp, QPRES) - q(i, j, k, QPRES)) / cspeed -
           R(0.5) * q(i, j, k, QRHO) * (q(ip, jp, kp, QN) - q(i, j, k, QN));
  R d0 = limiter(dlft, drgt);
  R cs2 = cspeed * cspeed;
  dlft = (q(i, j, k, QRHO) - q(im, jm, km, QRHO)) - (q(i, j, k, QPRES) - q(im, jm, km, QPRES)) / cs2;
  drgt = (q(ip, jp, kp, QRHO) - q(i, j, k, QRHO)) - (q(ip, jp, kp, QPRES) - q(i, j, k, QPRES)) / cs2;
  R d1 = limiter(dlft, drgt);
  dlft = R(0.5) * (q(i, j, k, QPRES) - q(im, jm, km, QPRES)) / cspeed +
         R(0.5) * q(i, j, k, QRHO) * (q(i, j, k, QN) - q(im, jm, km, QN));
  drgt = R(0.5) * (q(ip, jp, kp, QPRES) - q(i, j, k, QPRES)) / cspeed +
         R(0.5) * q(i, j, k, QRHO) * (q(ip, jp, kp, QN) - q(i, j, k, QN));
  R d2 = limiter(dlft, drgt);
  dlft = q(i, j, k, QT1) - q(im, jm, km, QT1);
  drgt = q(ip, jp, kp, QT1) - q(i, j, k, QT1);
  R d3 = limiter(dlft, drgt);
  dlft = q(i, j, k, QT2) - q(im, jm, km, QT2);
  drgt = q(ip, jp, kp, QT2) - q(i, j, k, QT2);
  R d4 = limiter(dlft, drgt);
  dq(i, j, k, 0) = d0;
  dq(i, j, k, 1) = d1;
  dq(i, j, k, 2) = d2;
  dq(i, j, k, 3) = d3;
  dq(i, j, k, 4) = d4;
}

// Two-shock approximate Riemann solver: src/rhs/Riemann.h:123-249.
template <class R>
inline void riemann_prob(const R gamma, const R smallp, const R rl, const R ul, const R pl,
                         const R ut1l, const R ut2l, const R rr, const R ur, const R pr,
                         const R ut1r, const R ut2r, R& flxrho, R& flxu, R& flxut, R& flxutt,
                         R& flxe) {
  const R weakwv = R(1.e-3);
  const R small = R(1.e-6);
  R clsql = gamma * pl * rl;
  R clsqr = gamma * pr * rr;
  R wl = sqrt(clsql);
  R wr = sqrt(clsqr);
  R cleft = wl / rl;
  R cright = wr / rr;
  R ccsmall = small * (cleft + cright);
  R pstar = (wl * pr + wr * pl - wr * wl * (ur - ul)) / (wl + wr);
  pstar = rmax(pstar, smallp);
  R pstnm1 = pstar;
  R wlsq = (R(0.5) * (gamma - R(1.)) * (pstar + pl) + pstar) * rl;
  R wrsq = (R(0.5) * (gamma - R(1.)) * (pstar + pr) + pstar) * rr;
  wl = sqrt(wlsq);
  wr = sqrt(wrsq);
  R ustarp = ul - (pstar - pl) / wl;
  R ustarm = ur + (pstar - pr) / wr;
  pstar = (wl * pr + wr * pl - wr * wl * (ur - ul)) / (wl + wr);
  pstar = rmax(pstar, smallp);
  R ustar = R(0.0);
  for (int iter = 0; iter < 3; ++iter) {
    wlsq = (R(0.5) * (gamma - R(1.)) * (pstar + pl) + pstar) * rl;
    wrsq = (R(0.5) * (gamma - R(1.)) * (pstar + pr) + pstar) * rr;
    wl = R(1.) / sqrt(wlsq);
    wr = R(1.) / sqrt(wrsq);
    R ustnm1 = ustarm;
    R ustnp1 = ustarp;
    ustarm = ur - (pr - pstar) * wr;
    ustarp = ul + (pl - pstar) * wl;
    R dpditer = fabs(pstnm1 - pstar);
    R zp = fabs(ustarp - ustnp1);
    if (zp - weakwv * cleft < R(0.0)) zp = dpditer * wl;
    R zm = fabs(ustarm - ustnm1);
    if (zm - weakwv * cright < R(0.0)) zm = dpditer * wr;
    R zz = zp + zm;
    R denom = dpditer / rmax(zz, ccsmall);
    pstnm1 = pstar;
    pstar = pstar - denom * (ustarm - ustarp);
    pstar = rmax(pstar, smallp);
    ustar = R(0.5) * (ustarm + ustarp);
  }
  R ro, uo, po, sgnm, utrans1, utrans2;
  if (ustar > R(0.)) {
    ro = rl; uo = ul; po = pl; sgnm = R(1.); utrans1 = ut1l; utrans2 = ut2l;
  } else if (ustar < R(0.)) {
    ro = rr; uo = ur; po = pr; sgnm = R(-1.); utrans1 = ut1r; utrans2 = ut2r;
  } else {
    uo = R(0.5) * (ur + ul);
    po = R(0.5) * (pr + pl);
    ro = R(2.) * (rl * rr) / (rl + rr);
    sgnm = R(1.);
    utrans1 = R(0.5) * (ut1l + ut1r);
    utrans2 = R(0.5) * (ut2l + ut2r);
  }
  R wosq = (R(0.5) * (gamma - R(1.)) * (pstar + po) + pstar) * ro;
  R co = sqrt(gamma * po / ro);
  R wo = sqrt(wosq);
  R dpjmp = pstar - po;
  R rstar = ro / (R(1.) - ro * dpjmp / wosq);
  R cstar = sqrt(gamma * pstar / rstar);
  R spout = co - sgnm * uo;
  R spin = cstar - sgnm * uo;
  if (pstar >= po) {
    spin = wo / ro - sgnm * uo;
    spout = spin;
  }
  R ss = rmax(spout - spin, spout + spin);
  R frac = R(0.5) * (R(1.) + (spin + spout) / rmax(ss, ccsmall));
  R rgdnv, ugdnv, pgdnv;
  if (spout < R(0.)) {
    rgdnv = ro; ugdnv = uo; pgdnv = po;
  } else if (spin >= R(0.)) {
    rgdnv = rstar; ugdnv = ustar; pgdnv = pstar;
  } else {
    rgdnv = frac * rstar + (R(1.) - frac) * ro;
    ugdnv = frac * ustar + (R(1.) - frac) * uo;
    pgdnv = frac * pstar + (R(1.) - frac) * po;
  }
  flxrho = rgdnv * ugdnv;
  flxu = rgdnv * ugdnv * ugdnv + pgdnv;
  flxut = rgdnv * ugdnv * utrans1;
  flxutt = rgdnv * ugdnv * utrans2;
  flxe = ugdnv * (R(0.5) * rgdnv * (ugdnv * ugdnv + utrans1 * utrans1 + utrans2 * utrans2) +
                  pgdnv / (gamma - R(1.)) + pgdnv);
}

// MUSCL face states + Riemann flux at the d-face below (i,j,k):
// src/rhs/Riemann.h:251-337 (cns_riemann_z takes the left sound speed from
// q(i,j,k+1,QT), reproduced here).
template <class R>
inline void cns_riemann(int i, int j, int k, int d, const Arr<R>& f, const Arr<R>& dq,
                        const Arr<R>& q, const Closures& cl) {
  const int di = (d == 0), dj = (d == 1), dk = (d == 2);
  const int QN = QU + d;
  const int QT1 = (d == 0) ? QV : QU;
  const int QT2 = (d == 2) ? QV : QW;
  const int UN = UMX + d;
  const int UT1 = (d == 0) ? UMY : UMX;
  const int UT2 = (d == 2) ? UMY : UMZ;
  const int im = i - di, jm = j - dj, km = k - dk;
  const R g = R(cl.gamma), Rs = R(cl.Rspec);
  R cspeed = (d == 2) ? sqrt(g * Rs * q(i, j, k + 1, QT)) + R(1.e-40)
                      : sqrt(g * Rs * q(im, jm, km, QT)) + R(1.e-40);
  R rl = q(im, jm, km, QRHO) + R(0.5) * ((dq(im, jm, km, 0) + dq(im, jm, km, 2)) / cspeed + dq(im, jm, km, 1));
  rl = rmax(rl, R(1.0e-40));
  R ul = q(im, jm, km, QN) + R(0.5) * ((dq(im, jm, km, 2) - dq(im, jm, km, 0)) / q(im, jm, km, QRHO));
  R pl = q(im, jm, km, QPRES) + R(0.5) * (dq(im, jm, km, 0) + dq(im, jm, km, 2)) * cspeed;
  pl = rmax(pl, R(1.0e-40));
  R ut1l = q(im, jm, km, QT1) + R(0.5) * dq(im, jm, km, 3);
  R ut2l = q(im, jm, km, QT2) + R(0.5) * dq(im, jm, km, 4);
  cspeed = sqrt(g * Rs * q(i, j, k, QT)) + R(1.e-40);
  R rr = q(i, j, k, QRHO) - R(0.5) * ((dq(i, j, k, 0) + dq(i, j, k, 2)) / cspeed + dq(i, j, k, 1));
  rr = rmax(rr, R(1.0e-40));
  R ur = q(i, j, k, QN) - R(0.5) * ((dq(i, j, k, 2) - dq(i, j, k, 0)) / q(i, j, k, QRHO));
  R pr = q(i, j, k, QPRES) - R(0.5) * (dq(i, j, k, 0) + dq(i, j, k, 2)) * cspeed;
  pr = rmax(pr, R(1.0e-40));
  R ut1r = q(i, j, k, QT1) - R(0.5) * dq(i, j, k, 3);
  R ut2r = q(i, j, k, QT2) - R(0.5) * dq(i, j, k, 4);
  R frho, fu, fut, futt, fe;
  riemann_prob(g, R(1.0e-40), rl, ul, pl, ut1l, ut2l, rr, ur, pr, ut1r, ut2r, frho, fu, fut, futt, fe);
  f(i, j, k, URHO) = frho;
  f(i, j, k, UN) = fu;
  f(i, j, k, UT1) = fut;
  f(i, j, k, UT2) = futt;
  f(i, j, k, UET) = fe;
}

// WENO5-Riemann (flux code 3: the riemann_weno extension), with no
// counterpart in the reference: the reference pairs WENO5 only with the
// local Lax-Friedrichs split (flux_euler = 2) and the two-shock solver only
// with MUSCL (its Riemann path).  Here rho, u_n, p, u_t1, u_t2 are reconstructed to the
// d-face below (i,j,k) from each side with weno5js (left state: cells
// i-3..i+1; right state: the mirror i+2..i-2), density and pressure floored
// at 1e-40 as the MUSCL states are (src/rhs/Riemann.h:260-272), and the
// states go to riemann_prob.
template <class R>
inline void weno_riemann_face(int i, int j, int k, int d, const Arr<R>& f, const Arr<R>& q, const Closures& cl) {
  const int di = (d == 0), dj = (d == 1), dk = (d == 2);
  const int QN = QU + d;
  const int QT1 = (d == 0) ? QV : QU;
  const int QT2 = (d == 2) ? QV : QW;
  const int UN = UMX + d;
  const int UT1 = (d == 0) ? UMY : UMX;
  const int UT2 = (d == 2) ? UMY : UMZ;
  const int comp[5] = {QRHO, QN, QPRES, QT1, QT2};
  R lft[5], rgt[5];
  for (int m = 0; m < 5; ++m) {
    R s[5];
    for (int o = 0; o < 5; ++o) s[o] = q(i + (o - 3) * di, j + (o - 3) * dj, k + (o - 3) * dk, comp[m]);
    lft[m] = weno5js(s);
    for (int o = 0; o < 5; ++o) s[o] = q(i + (2 - o) * di, j + (2 - o) * dj, k + (2 - o) * dk, comp[m]);
    rgt[m] = weno5js(s);
  }
  const R rl = rmax(lft[0], R(1.0e-40)), pl = rmax(lft[2], R(1.0e-40));
  const R rr = rmax(rgt[0], R(1.0e-40)), pr = rmax(rgt[2], R(1.0e-40));
  R frho, fu, fut, futt, fe;
  riemann_prob(R(cl.gamma), R(1.0e-40), rl, lft[1], pl, lft[3], lft[4], rr, rgt[1], pr, rgt[3], rgt[4], frho, fu,
               fut, futt, fe);
  f(i, j, k, URHO) = frho;
  f(i, j, k, UN) = fu;
  f(i, j, k, UT1) = fut;
  f(i, j, k, UT2) = futt;
  f(i, j, k, UET) = fe;
}

// Cell-centred viscous fluxes: src/rhs/CNS_hydro_K.h:108-172.
template <class R>
inline void viscous_fluxes(int i, int j, int k, const Arr<R>& q, const Arr<R> pf[3], const double dxinv[3],
                           const Closures& cl, int loc = -1) {
  // loc -1: ViscousFluxes (src/rhs/CNS_hydro_K.h:108-172); loc 0 / 1:
  // ViscousWallFluxes at the ghost row of a lower / upper y wall (:177-251),
  // one-sided second-order y derivatives
  R ux = q(i, j, k, QU);
  R dudx = (q(i + 1, j, k, QU) - q(i - 1, j, k, QU)) * R(0.5) * R(dxinv[0]);
  R dvdx = (q(i + 1, j, k, QV) - q(i - 1, j, k, QV)) * R(0.5) * R(dxinv[0]);
  R dwdx = (q(i + 1, j, k, QW) - q(i - 1, j, k, QW)) * R(0.5) * R(dxinv[0]);
  R dTdx = (q(i + 1, j, k, QT) - q(i - 1, j, k, QT)) * R(0.5) * R(dxinv[0]);
  R uy = q(i, j, k, QV);
  R dudy, dvdy, dwdy, dTdy;
  if (loc == 0) {
    dudy = (-q(i, j + 2, k, QU) + R(4) * q(i, j + 1, k, QU) - R(3) * q(i, j, k, QU)) * R(0.5) * R(dxinv[1]);
    dvdy = (-q(i, j + 2, k, QV) + R(4) * q(i, j + 1, k, QV) - R(3) * q(i, j, k, QV)) * R(0.5) * R(dxinv[1]);
    dwdy = (-q(i, j + 2, k, QW) + R(4) * q(i, j + 1, k, QW) - R(3) * q(i, j, k, QW)) * R(0.5) * R(dxinv[1]);
    dTdy = (-q(i, j + 2, k, QT) + R(4) * q(i, j + 1, k, QT) - R(3) * q(i, j, k, QT)) * R(0.5) * R(dxinv[1]);
  } else if (loc == 1) {
    dudy = (R(3) * q(i, j, k, QU) - R(4) * q(i, j - 1, k, QU) + q(i, j - 2, k, QU)) * R(0.5) * R(dxinv[1]);
    dvdy = (R(3) * q(i, j, k, QV) - R(4) * q(i, j - 1, k, QV) + q(i, j - 2, k, QV)) * R(0.5) * R(dxinv[1]);
    dwdy = (R(3) * q(i, j, k, QW) - R(4) * q(i, j - 1, k, QW) + q(i, j - 2, k, QW)) * R(0.5) * R(dxinv[1]);
    dTdy = (R(3) * q(i, j, k, QT) - R(4) * q(i, j - 1, k, QT) + q(i, j - 2, k, QT)) * R(0.5) * R(dxinv[1]);
  } else {
    dudy = (q(i, j + 1, k, QU) - q(i, j - 1, k, QU)) * R(0.5) * R(dxinv[1]);
    dvdy = (q(i, j + 1, k, QV) - q(i, j - 1, k, QV)) * R(0.5) * R(dxinv[1]);
    dwdy = (q(i, j + 1, k, QW) - q(i, j - 1, k, QW)) * R(0.5) * R(dxinv[1]);
    dTdy = (q(i, j + 1, k, QT) - q(i, j - 1, k, QT)) * R(0.5) * R(dxinv[1]);
  }
  R uz = q(i, j, k, QW);
  R dudz = (q(i, j, k + 1, QU) - q(i, j, k - 1, QU)) * R(0.5) * R(dxinv[2]);
  R dvdz = (q(i, j, k + 1, QV) - q(i, j, k - 1, QV)) * R(0.5) * R(dxinv[2]);
  R dwdz = (q(i, j, k + 1, QW) - q(i, j, k - 1, QW)) * R(0.5) * R(dxinv[2]);
  R dTdz = (q(i, j, k + 1, QT) - q(i, j, k - 1, QT)) * R(0.5) * R(dxinv[2]);
  R div = dudx + dvdy + dwdz;
  R mu = cl.visc(q(i, j, k, QT));
  R lambda = cl.cond(q(i, j, k, QT));
  R r1_3 = R(1.0) / R(3.0);
  R tauxx = R(2.0) * mu * (dudx - r1_3 * div);
  R tauxy = mu * (dudy + dvdx);
  R tauxz = mu * (dudz + dwdx);
  R tauyy = R(2.0) * mu * (dvdy - r1_3 * div);
  R tauyz = mu * (dvdz + dwdy);
  R tauzz = R(2.0) * mu * (dwdz - r1_3 * div);
  const Arr<R>& fx = pf[0];
  const Arr<R>& fy = pf[1];
  const Arr<R>& fz = pf[2];
  fx(i, j, k, URHO) = R(0.0);
  fx(i, j, k, UMX) = -tauxx;
  fx(i, j, k, UMY) = -tauxy;
  fx(i, j, k, UMZ) = -tauxz;
  fx(i, j, k, UET) = -lambda * dTdx - tauxx * ux - tauxy * uy - tauxz * uz;
  fy(i, j, k, URHO) = R(0.0);
  fy(i, j, k, UMX) = -tauxy;
  fy(i, j, k, UMY) = -tauyy;
  fy(i, j, k, UMZ) = -tauyz;
  fy(i, j, k, UET) = -lambda * dTdy - tauxy * ux - tauyy * uy - tauyz * uz;
  fz(i, j, k, URHO) = R(0.0);
  fz(i, j, k, UMX) = -tauxz;
  fz(i, j, k, UMY) = -tauyz;
  fz(i, j, k, UMZ) = -tauzz;
  fz(i, j, k, UET) = -lambda * dTdz - tauxz * ux - tauyz * uy - tauzz * uz;
}

// JST sensor: src/rhs/CNS_hydro_K.h:39-44; sensor + spectral radius :46-75.
template <class R> inline R discon_sensor(R pp, R pl, R pr) {
  R pjst = pr + R(2.0) * pp + pl;
  R ptvd = fabs(pr - pp) + fabs(pp - pl);
  return fabs(R(2.0) * (pr - R(2.0) * pp + pl) / (pjst + ptvd + R(1.0e-40)));
}

template <class R>
inline void sensor_lambda(int i, int j, int k, const Arr<R>& q, const Arr<R>& lam, const Arr<R>& sen,
                          const Closures& cl) {
  R pp = q(i, j, k, QPRES);
  sen(i, j, k, 0) = discon_sensor(pp, q(i - 1, j, k, QPRES), q(i + 1, j, k, QPRES));
  sen(i, j, k, 1) = discon_sensor(pp, q(i, j - 1, k, QPRES), q(i, j + 1, k, QPRES));
  sen(i, j, k, 2) = discon_sensor(pp, q(i, j, k - 1, QPRES), q(i, j, k + 1, QPRES));
  R ux = q(i, j, k, QU), uy = q(i, j, k, QV), uz = q(i, j, k, QW);
  R cs = sqrt(R(cl.gamma) * q(i, j, k, QPRES) / q(i, j, k, QRHO));
  lam(i, j, k, 0) = fabs(ux) + cs;
  lam(i, j, k, 1) = fabs(uy) + cs;
  lam(i, j, k, 2) = fabs(uz) + cs;
}

// JST dissipation subtracted from the three face fluxes at (i,j,k), comp n:
// src/rhs/CNS_hydro_K.h:78-104.  The y and z blocks read component 0 of the
// sensor and of lambda, and the z fourth difference uses k-1 three times;
// both are reproduced.
template <class R>
inline void jst_flux(int i, int j, int k, int n, const Arr<R>& lam, const Arr<R>& sen, const Arr<R>& u,
                     R& fx, R& fy, R& fz, const Closures& cl) {
  R dw, s, rr, fdamp;
  R u_ijk = u(i, j, k, n);
  const R Cs = R(cl.Cshock), Cd = R(cl.Cdamp);
  dw = (u_ijk - u(i - 1, j, k, n));
  s = Cs * rmax(sen(i - 1, j, k, 0), sen(i, j, k, 0));
  rr = rmax(lam(i - 1, j, k, 0), lam(i, j, k, 0));
  fdamp = u(i + 1, j, k, n) - R(3.0) * u(i, j, k, n) + R(3.0) * u(i - 1, j, k, n) - u(i - 2, j, k, n);
  fx -= (s * dw - rmax(R(0.0), Cd - s) * fdamp) * rr;
  dw = (u_ijk - u(i, j - 1, k, n));
  s = Cs * rmax(sen(i, j - 1, k, 0), sen(i, j, k, 0));
  rr = rmax(lam(i, j - 1, k, 0), lam(i, j, k, 0));
  fdamp = u(i, j + 1, k, n) - R(3.0) * u(i, j, k, n) + R(3.0) * u(i, j - 1, k, n) - u(i, j - 2, k, n);
  fy -= (s * dw - rmax(R(0.0), Cd - s) * fdamp) * rr;
  dw = (u_ijk - u(i, j, k - 1, n));
  s = Cs * rmax(sen(i, j, k - 1, 0), sen(i, j, k, 0));
  rr = rmax(lam(i, j, k - 1, 0), lam(i, j, k, 0));
  fdamp = u(i, j, k - 1, n) - R(3.0) * u(i, j, k, n) + R(3.0) * u(i, j, k - 1, n) - u(i, j, k - 1, n);
  fz -= (s * dw - rmax(R(0.0), Cd - s) * fdamp) * rr;
}

inline void set_phase(int p) { g_phase = p; }

// Grow-only per-thread scratch fields, reused across calls the way the
// reference allocates its level scratch MultiFabs once (src/CNS.cpp:432-467).
template <class R> R* pool(int slot, size_t n) {
  static thread_local std::vector<R> p[16];
  if (p[slot].size() < n) p[slot].resize(n);
  return p[slot].data();
}

// ------------------------------------------------------------ compute_rhs --
// CNS::compute_rhs for one box: src/tim/CNS_advance.cpp:186-391.
// u: ghosted (NGHOST) conserved state; dsdt: valid-only output.
// Only faces the divergence reads are evaluated (the reference also computes
// x-fluxes on j,k = hi+1 etc., which never reach dsdt).
// y walls of the domain with boundary code 6 (user-defined, ext_dir): the
// reference's wall treatment for boxes that touch them.
struct Walls {
  int lo, hi;          // code 6 on the lower / upper y side
  int dom_lo, dom_hi;  // the domain's y extent
};

template <class R>
void compute_rhs_box(const Scheme& sc, const Closures& cl, const Box& bx, const double dxinv[3],
                     const R* uptr, R* dsdt, int nthreads, const Walls* walls = nullptr) {
  const int g = NGHOST;
  const long long ncg = (long long)(bx.n(0) + 2 * g) * (bx.n(1) + 2 * g) * (bx.n(2) + 2 * g);
  Arr<R> u = make_arr<R>(const_cast<R*>(uptr), bx, g);
  Arr<R> q = make_arr<R>(pool<R>(0, ncg * NPRIM), bx, g);
  const int lo0 = bx.lo[0], lo1 = bx.lo[1], lo2 = bx.lo[2];
  const int hi0 = bx.hi[0], hi1 = bx.hi[1], hi2 = bx.hi[2];
  (void)nthreads;
#ifdef _OPENMP
  const int nt = nthreads > 0 ? nthreads : 1;
#endif

  set_phase(0);
  // 1. cons -> prims over the grown box (:200-208)
#ifdef _OPENMP
#pragma omp parallel for num_threads(nt) schedule(static)
#endif
  for (int k = lo2 - g; k <= hi2 + g; ++k)
    for (int j = lo1 - g; j <= hi1 + g; ++j)
      for (int i = lo0 - g; i <= hi0 + g; ++i) cons2prim(i, j, k, u, q, cl);

  // face fluxes, one array per direction, nodal in that direction
  Arr<R> F[3];
  for (int d = 0; d < 3; ++d) {
    const long long nf = (long long)(bx.n(0) + (d == 0)) * (bx.n(1) + (d == 1)) * (bx.n(2) + (d == 2));
    R* fp = pool<R>(1 + d, nf * NCONS);
    F[d] = make_face_arr<R>(fp, bx, d);
    if (!sc.rhs_euler) {  // every face is written by the Euler fluxes otherwise
#ifdef _OPENMP
#pragma omp parallel for num_threads(nt) schedule(static)
#endif
      for (long long t = 0; t < nf * NCONS; ++t) fp[t] = R(0.0);
    }
  }

  // 2. Euler fluxes (:221-224)
  set_phase(1);
  if (sc.rhs_euler) {
    if (sc.flux_euler == 1) {
      double coeffs[3];
      keep_coeffs(sc.order_keep, coeffs);
      const int halfsten = sc.order_keep / 2;
      for (int d = 0; d < 3; ++d) {
#ifdef _OPENMP
#pragma omp parallel for num_threads(nt) schedule(static)
#endif
        for (int k = lo2; k <= hi2 + (d == 2); ++k)
          for (int j = lo1; j <= hi1 + (d == 1); ++j)
            for (int i = lo0; i <= hi0 + (d == 0); ++i) {
              R f[NCONS];
              keep_face(i, j, k, d, halfsten, coeffs, q, f, cl);
              for (int n = 0; n < NCONS; ++n) F[d](i, j, k, n) = f[n];
            }
      }
    } else if (sc.flux_euler == 2) {
      Arr<R> PF[3];
      for (int d = 0; d < 3; ++d) PF[d] = make_arr<R>(pool<R>(4 + d, ncg * NCONS), bx, g);
      Arr<R> lam = make_arr<R>(pool<R>(7, ncg * 3), bx, g);
#ifdef _OPENMP
#pragma omp parallel for num_threads(nt) schedule(static)
#endif
      for (int k = lo2 - g; k <= hi2 + g; ++k)
        for (int j = lo1 - g; j <= hi1 + g; ++j)
          for (int i = lo0 - g; i <= hi0 + g; ++i) cons2eulerflux_lambda(i, j, k, u, PF, lam, cl);
      for (int d = 0; d < 3; ++d) {
#ifdef _OPENMP
#pragma omp parallel for num_threads(nt) schedule(static)
#endif
        for (int k = lo2; k <= hi2 + (d == 2); ++k)
          for (int j = lo1; j <= hi1 + (d == 1); ++j)
            for (int i = lo0; i <= hi0 + (d == 0); ++i)
              for (int n = 0; n < NCONS; ++n) F[d](i, j, k, n) = weno_llf_face(i, j, k, n, d, u, PF[d], lam);
      }
    } else if (sc.flux_euler == 3) {
      for (int d = 0; d < 3; ++d) {
#ifdef _OPENMP
#pragma omp parallel for num_threads(nt) schedule(static)
#endif
        for (int k = lo2; k <= hi2 + (d == 2); ++k)
          for (int j = lo1; j <= hi1 + (d == 1); ++j)
            for (int i = lo0; i <= hi0 + (d == 0); ++i) weno_riemann_face(i, j, k, d, F[d], q, cl);
      }
    } else {
      // MUSCL + Riemann (src/rhs/Riemann.h:339-408); slope temp on grow(bx,1)
      Box b1 = bx;
      for (int d = 0; d < 3; ++d) { b1.lo[d] -= 1; b1.hi[d] += 1; }
      Arr<R> dq = make_arr<R>(pool<R>(8, b1.cells() * NCONS), b1, 0);
      for (int d = 0; d < 3; ++d) {
        const int di = (d == 0), dj = (d == 1), dk = (d == 2);
#ifdef _OPENMP
#pragma omp parallel for num_threads(nt) schedule(static)
#endif
        for (int k = lo2 - dk; k <= hi2 + dk; ++k)
          for (int j = lo1 - dj; j <= hi1 + dj; ++j)
            for (int i = lo0 - di; i <= hi0 + di; ++i) cns_slope(i, j, k, d, dq, q, cl);
#ifdef _OPENMP
#pragma omp parallel for num_threads(nt) schedule(static)
#endif
        for (int k = lo2; k <= hi2 + dk; ++k)
          for (int j = lo1; j <= hi1 + dj; ++j)
            for (int i = lo0; i <= hi0 + di; ++i) cns_riemann(i, j, k, d, F[d], dq, q, cl);
      }
    }

    // Order reduction next to y walls (:226-229, Flux_2nd_Order_KEEP in
    // src/rhs/CentralKEEP.h:232-287): KEEPy with halfsten 1 and coefficient
    // 1 overwrites the y faces j in [lo, lo+H-1] of a box on a lower wall and
    // [hi-H+1, hi] (not the wall face hi+1) of a box on an upper wall.
    if (sc.flux_euler == 1 && sc.order_keep != 2 && walls) {
      const double c2[3] = {1.0, 0.0, 0.0};
      const int H = sc.order_keep / 2;
      for (int side = 0; side < 2; ++side) {
        int j0, j1;
        if (side == 0) {
          if (!(walls->lo && lo1 == walls->dom_lo)) continue;
          j0 = lo1; j1 = lo1 + H - 1;
        } else {
          if (!(walls->hi && hi1 == walls->dom_hi)) continue;
          j0 = hi1 - H + 1; j1 = hi1;
        }
        for (int k = lo2; k <= hi2; ++k)
          for (int j = j0; j <= j1; ++j)
            for (int i = lo0; i <= hi0; ++i) {
              R f[NCONS];
              keep_face(i, j, k, 1, 1, c2, q, f, cl);
              for (int n = 0; n < NCONS; ++n) F[1](i, j, k, n) = f[n];
            }
      }
    }

    // JST artificial dissipation (:235-265): sensor/lambda on the valid box,
    // zero elsewhere, then subtracted on every face.
    if (sc.art_diss == 1) {
      set_phase(2);
      R* lb = pool<R>(9, ncg * 3);
      R* sb = pool<R>(10, ncg * 3);
      for (long long t = 0; t < ncg * 3; ++t) { lb[t] = R(0.0); sb[t] = R(0.0); }
      Arr<R> lam = make_arr<R>(lb, bx, g), sen = make_arr<R>(sb, bx, g);
      for (int k = lo2; k <= hi2; ++k)
        for (int j = lo1; j <= hi1; ++j)
          for (int i = lo0; i <= hi0; ++i) sensor_lambda(i, j, k, q, lam, sen, cl);
      // The reference loops over the all-direction nodal box and updates the
      // three face fluxes of each node together; only faces the divergence
      // reads are kept here, each updated exactly once.
      for (int k = lo2; k <= hi2 + 1; ++k)
        for (int j = lo1; j <= hi1 + 1; ++j)
          for (int i = lo0; i <= hi0 + 1; ++i)
            for (int n = 0; n < NCONS; ++n) {
              R dummy[3] = {R(0.0), R(0.0), R(0.0)};
              const bool vx = (j <= hi1 && k <= hi2), vy = (i <= hi0 && k <= hi2), vz = (i <= hi0 && j <= hi1);
              R& fx = vx ? F[0](i, j, k, n) : dummy[0];
              R& fy = vy ? F[1](i, j, k, n) : dummy[1];
              R& fz = vz ? F[2](i, j, k, n) : dummy[2];
              jst_flux(i, j, k, n, lam, sen, u, fx, fy, fz, cl);
            }
    }
  }

  // 3. viscous fluxes (:276-353): cell fluxes on grow(bx,1), face averages added
  if (sc.rhs_visc) {
    set_phase(3);
    Box b1 = bx;
    for (int d = 0; d < 3; ++d) { b1.lo[d] -= 1; b1.hi[d] += 1; }
    Arr<R> VF[3];
    for (int d = 0; d < 3; ++d) VF[d] = make_arr<R>(pool<R>(11 + d, b1.cells() * NCONS), b1, 0);
#ifdef _OPENMP
#pragma omp parallel for num_threads(nt) schedule(static)
#endif
    for (int k = lo2 - 1; k <= hi2 + 1; ++k)
      for (int j = lo1 - 1; j <= hi1 + 1; ++j)
        for (int i = lo0 - 1; i <= hi0 + 1; ++i) {
          // wall rows (:300-333): the ghost row below a lower / above an
          // upper y wall of a box that touches it
          int loc = -1;
          if (walls && walls->lo && lo1 == walls->dom_lo && j == lo1 - 1) loc = 0;
          if (walls && walls->hi && hi1 == walls->dom_hi && j == hi1 + 1) loc = 1;
          viscous_fluxes(i, j, k, q, VF, dxinv, cl, loc);
        }
    // ViscousNumericalFluxes: src/rhs/CNS_hydro_K.h:254-261
    set_phase(4);
    for (int d = 0; d < 3; ++d) {
      const int di = (d == 0), dj = (d == 1), dk = (d == 2);
#ifdef _OPENMP
#pragma omp parallel for num_threads(nt) schedule(static)
#endif
      for (int k = lo2; k <= hi2 + dk; ++k)
        for (int j = lo1; j <= hi1 + dj; ++j)
          for (int i = lo0; i <= hi0 + di; ++i)
            for (int n = 0; n < NCONS; ++n)
              F[d](i, j, k, n) += R(0.5) * (VF[d](i - di, j - dj, k - dk, n) + VF[d](i, j, k, n));
    }
  }

  // 4. flux divergence (:376-391)
  set_phase(5);
  Arr<R> ds = make_arr<R>(dsdt, bx, 0);
#ifdef _OPENMP
#pragma omp parallel for num_threads(nt) schedule(static)
#endif
  for (int k = lo2; k <= hi2; ++k)
    for (int n = 0; n < NCONS; ++n)
      for (int j = lo1; j <= hi1; ++j)
        for (int i = lo0; i <= hi0; ++i)
          ds(i, j, k, n) = R(dxinv[0]) * (F[0](i, j, k, n) - F[0](i + 1, j, k, n)) +
                           R(dxinv[1]) * (F[1](i, j, k, n) - F[1](i, j + 1, k, n)) +
                           R(dxinv[2]) * (F[2](i, j, k, n) - F[2](i, j, k + 1, n));

  // 5. source term (:396-407): the channel problem's user_source
  //    (exm/Channel/prob.h:189-193: rhs(UMX) += rho fx, rhs(UET) += m_x fx)
  //    for a body force f per unit mass, each direction with f_d != 0 in
  //    x, y, z order
  if (sc.rhs_source) {
    for (int k = lo2; k <= hi2; ++k)
      for (int j = lo1; j <= hi1; ++j)
        for (int i = lo0; i <= hi0; ++i)
          for (int d = 0; d < 3; ++d) {
            if (sc.force[d] == 0.0) continue;
            ds(i, j, k, UMX + d) = ds(i, j, k, UMX + d) + u(i, j, k, URHO) * R(sc.force[d]);
            ds(i, j, k, UET) = ds(i, j, k, UET) + u(i, j, k, UMX + d) * R(sc.force[d]);
          }
  }
}

// -------------------------------------------------------------- halo fill --
// Single-level FillPatch semantics for one box that spans the whole domain:
// periodic images in periodic directions, then the physical BC types of
// src/set/CNS_setup.cpp:18-31 applied direction by direction (x, then y,
// then z) over the whole ghost region.  bc code per side: -1 periodic,
// 2 outflow (foextrap), 3/4 symmetry/slip wall (reflect_even, normal
// velocity reflect_odd), 5 no-slip (reflect_even, all velocities reflect_odd).
// Codes 1 and 6 (ext_dir through the problem's bcnormal) leave the cells
// beyond those sides, corners included, as the caller stored them.
enum BCT { BC_INT = 0, BC_FOEXTRAP = 2, BC_EVEN = 3, BC_ODD = 4 };

inline int comp_bc_type(int phys, int comp, int dir) {
  // scalar_bc / norm_vel_bc / tang_vel_bc tables (src/set/CNS_setup.cpp:18-31)
  const bool normal = (comp == UMX + dir);
  const bool vel = (comp >= UMX && comp <= UMZ);
  switch (phys) {
    case 2: return BC_FOEXTRAP;
    case 3:
    case 4: return (vel && normal) ? BC_ODD : BC_EVEN;
    case 5: return vel ? BC_ODD : BC_EVEN;
    default: return BC_INT;
  }
}

template <class R>
void fill_halo_box(const Box& dom, const int bc_lo[3], const int bc_hi[3], R* uptr, int ncomp) {
  const int g = NGHOST;
  Arr<R> u = make_arr<R>(uptr, dom, g);
  int glo[3], ghi[3];
  for (int d = 0; d < 3; ++d) { glo[d] = dom.lo[d] - g; ghi[d] = dom.hi[d] + g; }
  // cells beyond an ext_dir side (codes 1, 6: the problem's bcnormal fills
  // them, src/set/bcs.cpp) are the caller's and are not touched here
  auto ext_dir = [&](const int c[3]) {
    for (int d = 0; d < 3; ++d) {
      if (c[d] < dom.lo[d] && (bc_lo[d] == 1 || bc_lo[d] == 6)) return true;
      if (c[d] > dom.hi[d] && (bc_hi[d] == 1 || bc_hi[d] == 6)) return true;
    }
    return false;
  };
  // periodic directions: image of every ghost cell whose other coordinates are
  // inside the domain or already filled; applying directions in order and
  // sweeping the full ghost extent of earlier directions reproduces the corner
  // fill of FillBoundary for an all-periodic single box.
  for (int d = 0; d < 3; ++d) {
    if (!(bc_lo[d] == -1 && bc_hi[d] == -1)) continue;
    const int n = dom.n(d);
#ifdef _OPENMP
    #pragma omp parallel for schedule(static) if (u.ns > 100000)
#endif
    for (int k = glo[2]; k <= ghi[2]; ++k)
      for (int j = glo[1]; j <= ghi[1]; ++j)
        for (int i = glo[0]; i <= ghi[0]; ++i) {
          int c[3] = {i, j, k};
          if (c[d] >= dom.lo[d] && c[d] <= dom.hi[d]) continue;
          if (ext_dir(c)) continue;
          int s[3] = {i, j, k};
          s[d] = (c[d] < dom.lo[d]) ? c[d] + n : c[d] - n;
          for (int m = 0; m < ncomp; ++m) u(i, j, k, m) = u(s[0], s[1], s[2], m);
        }
  }
  for (int d = 0; d < 3; ++d) {
    for (int side = 0; side < 2; ++side) {
      const int phys = side ? bc_hi[d] : bc_lo[d];
      if (phys == -1 || phys == 0 || phys == 1 || phys == 6) continue;
#ifdef _OPENMP
      #pragma omp parallel for schedule(static) if (u.ns > 100000)
#endif
      for (int k = glo[2]; k <= ghi[2]; ++k)
        for (int j = glo[1]; j <= ghi[1]; ++j)
          for (int i = glo[0]; i <= ghi[0]; ++i) {
            int c[3] = {i, j, k};
            const bool outside = side ? (c[d] > dom.hi[d]) : (c[d] < dom.lo[d]);
            if (!outside || ext_dir(c)) continue;
            for (int m = 0; m < ncomp; ++m) {
              const int t = comp_bc_type(phys, m, d);
              int s[3] = {i, j, k};
              if (t == BC_FOEXTRAP) {
                s[d] = side ? dom.hi[d] : dom.lo[d];
                u(i, j, k, m) = u(s[0], s[1], s[2], m);
              } else if (t == BC_EVEN || t == BC_ODD) {
                s[d] = side ? 2 * dom.hi[d] - c[d] + 1 : 2 * dom.lo[d] - c[d] - 1;
                R v = u(s[0], s[1], s[2], m);
                u(i, j, k, m) = (t == BC_ODD) ? -v : v;
              }
            }
          }
    }
  }
}

// -------------------------------------------------------------------- dt --
// cns_estdt (src/cls/CNS_K.h:12-47; z-velocity read from UMY as there).
inline double cns_estdt(const Box& bx, const double* uptr, const double dx[3], const Closures& cl, int g) {
  Arr<double> s = make_arr<double>(const_cast<double*>(uptr), bx, g);
  double dt = std::numeric_limits<double>::max();
  for (int k = bx.lo[2]; k <= bx.hi[2]; ++k)
    for (int j = bx.lo[1]; j <= bx.hi[1]; ++j)
      for (int i = bx.lo[0]; i <= bx.hi[0]; ++i) {
        double rho = s(i, j, k, URHO), mx = s(i, j, k, UMX), my = s(i, j, k, UMY), mz = s(i, j, k, UMY);
        double rhoinv = 1.0 / rmax(rho, 1.0e-40);
        double vx = mx * rhoinv, vy = my * rhoinv, vz = mz * rhoinv;
        double ke = 0.5 * rho * (vx * vx + vy * vy + vz * vz);
        double rhoei = (s(i, j, k, UET) - ke);
        double p = (cl.gamma - 1.0) * rhoei;
        double cs = std::sqrt(cl.gamma * p * rhoinv);
        double dtx = dx[0] / (std::fabs(vx) + cs);
        double dty = dx[1] / (std::fabs(vy) + cs);
        double dtz = dx[2] / (std::fabs(vz) + cs);
        dt = rmin(dt, rmin(dtx, rmin(dty, dtz)));
      }
  return dt;
}

// ------------------------------------------------------------- RK stages --
// CNS::advance stage sequences (src/tim/CNS_advance.cpp:51-183) written as
// AMReX BLAS-1 programs.  Registers: S1 (old state), S2 (new state), dS
// (the RHS).  LinComb(dst,a,x,b,y): dst = a*x + b*y; Saxpy(dst,a,x):
// dst += a*x; Xpay(dst,a,x): dst = x + a*dst; Copy(dst,x).
enum Reg { RS1 = 0, RS2 = 1, RDS = 2 };
enum OpK { OP_LINCOMB = 0, OP_SAXPY = 1, OP_XPAY = 2, OP_COPY = 3 };
struct Op { int kind, dst, x, y; double a, b; };
struct StageProg {
  int src;  // which state FillPatch reads: 0 = S1 (old), 1 = S2 (new)
  int nops;
  Op ops[3];
};

inline int rk_program(int order_rk, int stages_rk, double dt, StageProg* st) {
  auto op = [](int kind, int dst, int x, int y, double a, double b) { Op o{kind, dst, x, y, a, b}; return o; };
  if (order_rk == -2) {  // :51-70
    st[0] = {0, 1, {op(OP_LINCOMB, RS2, RS1, RDS, 1.0, dt)}};
    st[1] = {1, 2, {op(OP_LINCOMB, RS2, RS2, RS1, 0.5, 0.5), op(OP_SAXPY, RS2, RDS, 0, 0.5 * dt, 0)}};
    return 2;
  }
  if (order_rk == 0) {  // :71-75
    st[0] = {0, 1, {op(OP_COPY, RS2, RDS, 0, 0, 0)}};
    return 1;
  }
  if (order_rk == 1) {  // :76-80
    st[0] = {0, 1, {op(OP_LINCOMB, RS2, RS1, RDS, 1.0, dt)}};
    return 1;
  }
  if (order_rk == 2) {  // :81-114, SSPRK(m,2); stage 1 reads S2 = copy of S1
    const int m = stages_rk;
    for (int i = 1; i <= m - 1; ++i) st[i - 1] = {i == 1 ? 0 : 1, 1, {op(OP_SAXPY, RS2, RDS, 0, dt / double(m - 1), 0)}};
    st[m - 1] = {m == 1 ? 0 : 1, 2, {op(OP_LINCOMB, RS2, RS2, RDS, double(m - 1), dt),
                                      op(OP_LINCOMB, RS2, RS1, RS2, 1.0 / m, 1.0 / m)}};
    return m;
  }
  if (order_rk == 3 && stages_rk == 3) {  // :118-139
    st[0] = {0, 1, {op(OP_LINCOMB, RS2, RS1, RDS, 1.0, dt)}};
    st[1] = {1, 2, {op(OP_XPAY, RDS, RS2, 0, dt, 0), op(OP_LINCOMB, RS2, RS1, RDS, 3.0 / 4, 1.0 / 4)}};
    st[2] = {1, 2, {op(OP_XPAY, RDS, RS2, 0, dt, 0), op(OP_LINCOMB, RS2, RS1, RDS, 1.0 / 3, 2.0 / 3)}};
    return 3;
  }
  if (order_rk == 3 && stages_rk == 4) {  // :141-166
    st[0] = {0, 1, {op(OP_LINCOMB, RS2, RS1, RDS, 1.0, dt / 2)}};
    st[1] = {1, 1, {op(OP_SAXPY, RS2, RDS, 0, dt / 2, 0)}};
    st[2] = {1, 2, {op(OP_LINCOMB, RS2, RS1, RS2, 2.0 / 3, 1.0 / 3), op(OP_SAXPY, RS2, RDS, 0, dt / 6, 0)}};
    st[3] = {1, 1, {op(OP_SAXPY, RS2, RDS, 0, dt / 2, 0)}};
    return 4;
  }
  return -1;
}

template <class R> inline void apply_ops(const StageProg& p, R reg[3]) {
  for (int o = 0; o < p.nops; ++o) {
    const Op& q = p.ops[o];
    if (q.kind == OP_LINCOMB) reg[q.dst] = R(q.a) * reg[q.x] + R(q.b) * reg[q.y];
    else if (q.kind == OP_SAXPY) reg[q.dst] = reg[q.dst] + R(q.a) * reg[q.x];
    else if (q.kind == OP_XPAY) reg[q.dst] = reg[q.x] + R(q.a) * reg[q.dst];
    else reg[q.dst] = reg[q.x];
  }
}

}  // namespace orc

// ================================================================= C API ==
using namespace orc;

struct OrcClosures {
  double gamma, cv, cp, Rspec;
  int32_t visc_law, cond_law;
  double visc_ref, Tvisc_ref, cond_ref, Tcond_ref, Cshock, Cdamp;
};
struct OrcScheme {
  int32_t rhs_euler, rhs_visc, flux_euler, order_keep, art_diss, rhs_source;
  double force[3];
};

static Closures to_cl(const OrcClosures* c) {
  Closures cl;
  cl.gamma = c->gamma; cl.cv = c->cv; cl.cp = c->cp; cl.Rspec = c->Rspec;
  cl.visc_law = c->visc_law; cl.visc_ref = c->visc_ref; cl.Tvisc_ref = c->Tvisc_ref;
  cl.cond_law = c->cond_law; cl.cond_ref = c->cond_ref; cl.Tcond_ref = c->Tcond_ref;
  cl.Cshock = c->Cshock; cl.Cdamp = c->Cdamp;
  return cl;
}
static Scheme to_sc(const OrcScheme* s) {
  Scheme sc;
  sc.rhs_euler = s->rhs_euler; sc.rhs_visc = s->rhs_visc; sc.flux_euler = s->flux_euler;
  sc.order_keep = s->order_keep; sc.art_diss = s->art_diss;
  sc.rhs_source = s->rhs_source;
  for (int d = 0; d < 3; ++d) sc.force[d] = s->force[d];
  return sc;
}
static Box to_box(const int* lo, const int* hi) {
  Box b;
  for (int d = 0; d < 3; ++d) { b.lo[d] = lo[d]; b.hi[d] = hi[d]; }
  return b;
}
static long long ghosted(const Box& b) {
  return (long long)(b.n(0) + 2 * NGHOST) * (b.n(1) + 2 * NGHOST) * (b.n(2) + 2 * NGHOST);
}

extern "C" {

int orc_version(void) { return 1; }

// dS/dt of one ghost-filled box (CNS::compute_rhs for one box).
int orc_compute_rhs(const OrcScheme* s, const OrcClosures* c, const int* lo, const int* hi,
                    const double* dxinv, const double* U, double* dSdt, int nthreads) {
  if (!s || !c || !lo || !hi || !dxinv || !U || !dSdt) return 1;
  Box b = to_box(lo, hi);
  for (int d = 0; d < 3; ++d) if (b.n(d) < 1) return 2;
  compute_rhs_box<double>(to_sc(s), to_cl(c), b, dxinv, U, dSdt, nthreads);
  return 0;
}

// dS/dt of one ghost-filled box of a domain whose y sides may be code-6
// walls: walls4 = {wall_lo, wall_hi, dom_lo_y, dom_hi_y}.
int orc_compute_rhs_walls(const OrcScheme* s, const OrcClosures* c, const int* lo, const int* hi,
                          const double* dxinv, const double* U, double* dSdt, int nthreads, const int* walls4) {
  if (!s || !c || !lo || !hi || !dxinv || !U || !dSdt || !walls4) return 1;
  Box b = to_box(lo, hi);
  for (int d = 0; d < 3; ++d) if (b.n(d) < 1) return 2;
  Walls w{walls4[0], walls4[1], walls4[2], walls4[3]};
  compute_rhs_box<double>(to_sc(s), to_cl(c), b, dxinv, U, dSdt, nthreads, &w);
  return 0;
}

// The same on a box of a domain with code-6 y walls (walls4 as for
// orc_compute_rhs_walls).
int orc_compute_rhs_jvp_walls(const OrcScheme* s, const OrcClosures* c, const int* lo, const int* hi,
                              const double* dxinv, const double* U, const double* W, double* R, double* JW,
                              int nthreads, const int* walls4) {
  if (!s || !c || !lo || !hi || !dxinv || !U || !W || !R || !JW || !walls4) return 1;
  Box b = to_box(lo, hi);
  const long long ng = ghosted(b) * NCONS, nv = b.cells() * NCONS;
  std::vector<Dual> ud(ng), rd(nv);
  for (long long t = 0; t < ng; ++t) ud[t] = Dual(U[t], W[t]);
  Walls w{walls4[0], walls4[1], walls4[2], walls4[3]};
  compute_rhs_box<Dual>(to_sc(s), to_cl(c), b, dxinv, ud.data(), rd.data(), nthreads, &w);
  for (long long t = 0; t < nv; ++t) { R[t] = rd[t].v; JW[t] = rd[t].d; }
  return 0;
}

// Jacobian-vector product: R = dS/dt(U), JW = d(dS/dt)/dU . W (dual numbers).
int orc_compute_rhs_jvp(const OrcScheme* s, const OrcClosures* c, const int* lo, const int* hi,
                        const double* dxinv, const double* U, const double* W, double* R, double* JW,
                        int nthreads) {
  if (!s || !c || !lo || !hi || !dxinv || !U || !W || !R || !JW) return 1;
  Box b = to_box(lo, hi);
  const long long ng = ghosted(b) * NCONS, nv = b.cells() * NCONS;
  std::vector<Dual> ud(ng), rd(nv);
  for (long long t = 0; t < ng; ++t) ud[t] = Dual(U[t], W[t]);
  compute_rhs_box<Dual>(to_sc(s), to_cl(c), b, dxinv, ud.data(), rd.data(), nthreads);
  for (long long t = 0; t < nv; ++t) { R[t] = rd[t].v; JW[t] = rd[t].d; }
  return 0;
}

// Algorithmic operation counts of one RHS evaluation of one box, per phase
// (cons2prim, Euler faces, JST, viscous cells, viscous faces, divergence):
// counts[5*phase + {0..4}] = {add, mul, div, sqrt, cmp}.
int orc_compute_rhs_count(const OrcScheme* s, const OrcClosures* c, const int* lo, const int* hi,
                          const double* dxinv, const double* U, long long* counts) {
  if (!s || !c || !lo || !hi || !dxinv || !U || !counts) return 1;
  Box b = to_box(lo, hi);
  const long long ng = ghosted(b) * NCONS, nv = b.cells() * NCONS;
  std::vector<Cnt> uc(ng), rc(nv);
  for (long long t = 0; t < ng; ++t) uc[t] = Cnt(U[t]);
  for (int p = 0; p < NPHASE; ++p) g_cntp[p] = OpCounts();
  compute_rhs_box<Cnt>(to_sc(s), to_cl(c), b, dxinv, uc.data(), rc.data(), 1);
  g_phase = 0;
  for (int p = 0; p < NPHASE; ++p) {
    counts[5 * p + 0] = g_cntp[p].add; counts[5 * p + 1] = g_cntp[p].mul; counts[5 * p + 2] = g_cntp[p].div;
    counts[5 * p + 3] = g_cntp[p].sqrt; counts[5 * p + 4] = g_cntp[p].cmp;
  }
  return 0;
}

// Ghost fill of a single box covering the domain (bc codes as cns.lo_bc/hi_bc).
int orc_fill_halo(const int* lo, const int* hi, const int* bc_lo, const int* bc_hi, double* U, int ncomp) {
  if (!lo || !hi || !bc_lo || !bc_hi || !U) return 1;
  for (int d = 0; d < 3; ++d) {
    if ((bc_lo[d] == -1) != (bc_hi[d] == -1)) return 3;
    for (int s = 0; s < 2; ++s) {
      int p = s ? bc_hi[d] : bc_lo[d];
      if (p < -1 || p > 6) return 4;  // 1, 6: ext_dir, cells left to the caller
    }
  }
  fill_halo_box<double>(to_box(lo, hi), bc_lo, bc_hi, U, ncomp);
  return 0;
}

// The channel problem's bcnormal (exm/Channel/prob.h:158-186) as cns_bcfill
// calls it (src/set/bcs.cpp:40-100) for every ghost cell beyond a code-6 y
// side, after the fill above: s_int = the column's first interior cell,
// dratio = de/di from prob_lo, prob_hi and dx, no-slip velocity, the
// interior pressure, T = max(Tw + dratio (Tw - T_int), Tmin), rho = p/(R T).
struct OrcBcNormal {
  int32_t kind;
  double Tw, Tmin;
  double prob_lo[3], prob_hi[3], dx[3];
};

int orc_fill_halo_bcnormal(const int* lo, const int* hi, const int* bc_lo, const int* bc_hi, double* U,
                           const OrcClosures* c, const OrcBcNormal* bn) {
  if (int rc = orc_fill_halo(lo, hi, bc_lo, bc_hi, U, NCONS)) return rc;
  if (!c || !bn) return 1;
  if (bn->kind != 1) return 0;
  const Box b = to_box(lo, hi);
  Arr<double> u = make_arr<double>(U, b, NGHOST);
  const double gamma = c->gamma, Rs = c->Rspec;
  for (int side = 0; side < 2; ++side) {
    if ((side ? bc_hi[1] : bc_lo[1]) != 6) continue;
    const int jf = side ? hi[1] : lo[1];
    for (int g = 1; g <= NGHOST; ++g) {
      const int j = side ? jf + g : jf - g;
      for (int k = lo[2] - NGHOST; k <= hi[2] + NGHOST; ++k)
        for (int i = lo[0] - NGHOST; i <= hi[0] + NGHOST; ++i) {
          const double rho = u(i, jf, k, URHO), mx = u(i, jf, k, UMX), my = u(i, jf, k, UMY);
          const double mz = u(i, jf, k, UMZ), et = u(i, jf, k, UET);
          const double ue = -mx / rho, ve = -my / rho, we = -mz / rho;
          const double eint = (et - 0.5 * (mx * mx + my * my + mz * mz) / rho) / rho;
          const double p = (gamma - 1.0) * rho * eint;
          const double Tint = p / (Rs * rho);
          const double x = bn->prob_lo[1] + (double)(j + 0.5) * bn->dx[1];
          const double di = side ? bn->prob_hi[1] - (double)(jf + 0.5) * bn->dx[1]
                                 : (double)(jf + 0.5) * bn->dx[1] - bn->prob_lo[1];
          const double de = side ? x - bn->prob_hi[1] : bn->prob_lo[1] - x;
          const double dratio = de / di;
          const double t = bn->Tw + dratio * (bn->Tw - Tint);
          const double Te = (t < bn->Tmin) ? bn->Tmin : t;
          const double re = p / (Rs * Te);
          const double ekin = 0.5 * (ue * ue + ve * ve + we * we);
          const double eint_e = p / (re * (gamma - 1.0));
          u(i, j, k, URHO) = re;
          u(i, j, k, UMX) = re * ue;
          u(i, j, k, UMY) = re * ve;
          u(i, j, k, UMZ) = re * we;
          u(i, j, k, UET) = re * (eint_e + ekin);
        }
    }
  }
  return 0;
}

// cfl * min over the valid box of dx/(|u|+c): CNS::estTimeStep (src/CNS.cpp:380-395).
double orc_est_timestep(const OrcClosures* c, const int* lo, const int* hi, const double* dx,
                        const double* U, int nghost, double cfl) {
  return cns_estdt(to_box(lo, hi), U, dx, to_cl(c), nghost) * cfl;
}

// CNS::printTotal's primitive extrema and convective CFL table
// (src/CNS.cpp:532-611) of one ghosted box: cons2prim over the valid cells,
// min/max of each primitive (rho, u, v, w, T, p), and pointCFL
// (src/cls/CNS_K.h:49-59) cell by cell in k, j, i order from a zeroed table:
// row d = (max |u_d + c|, max |u_d - c|, CFL_d), c = sqrt(gamma Rspec T),
// CFL_d = max(row d's first two) * dt / dx_d.  out: min[6], max[6], table[9].
int orc_prim_stats(const OrcClosures* c, const int* lo, const int* hi, const double* dx, const double* U,
                   double dt, double* out) {
  if (!c || !lo || !hi || !dx || !U || !out) return 1;
  const Box b = to_box(lo, hi);
  const Closures cl = to_cl(c);
  Arr<double> u = make_arr<double>(const_cast<double*>(U), b, NGHOST);
  std::vector<double> qv((size_t)b.cells() * NPRIM);
  Arr<double> q = make_arr<double>(qv.data(), b, 0);
  for (int k = b.lo[2]; k <= b.hi[2]; ++k)
    for (int j = b.lo[1]; j <= b.hi[1]; ++j)
      for (int i = b.lo[0]; i <= b.hi[0]; ++i) cons2prim(i, j, k, u, q, cl);
  for (int n = 0; n < NPRIM; ++n) {
    double mn = q(b.lo[0], b.lo[1], b.lo[2], n), mx = mn;
    for (int k = b.lo[2]; k <= b.hi[2]; ++k)
      for (int j = b.lo[1]; j <= b.hi[1]; ++j)
        for (int i = b.lo[0]; i <= b.hi[0]; ++i) {
          mn = rmin(mn, q(i, j, k, n));
          mx = rmax(mx, q(i, j, k, n));
        }
    out[n] = mn;
    out[NPRIM + n] = mx;
  }
  double t[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  for (int k = b.lo[2]; k <= b.hi[2]; ++k)
    for (int j = b.lo[1]; j <= b.hi[1]; ++j)
      for (int i = b.lo[0]; i <= b.hi[0]; ++i) {
        const double sos = std::sqrt(cl.gamma * cl.Rspec * q(i, j, k, QT));
        for (int d = 0; d < 3; ++d) {
          t[d][0] = rmax(t[d][0], std::fabs(q(i, j, k, QU + d) + sos));
          t[d][1] = rmax(t[d][1], std::fabs(q(i, j, k, QU + d) - sos));
          t[d][2] = rmax(t[d][0], t[d][1]) * dt / dx[d];
        }
      }
  for (int d = 0; d < 3; ++d)
    for (int e = 0; e < 3; ++e) out[2 * NPRIM + 3 * d + e] = t[d][e];
  return 0;
}

// The derived plot variables of CNS::writePlotFile (src/set/CNS_setup.cpp:
// 153-176) over the valid cells of one ghosted box, in the operation order
// of derpres, dertemp and dervel (src/cls/CNS_K.h:76-129).  out (valid box,
// 5 components): pressure, temperature, x, y, z velocity.
int orc_plot_derive(const OrcClosures* c, const int* lo, const int* hi, const double* U, double* out) {
  if (!c || !lo || !hi || !U || !out) return 1;
  const Box b = to_box(lo, hi);
  Arr<double> u = make_arr<double>(const_cast<double*>(U), b, NGHOST);
  Arr<double> o = make_arr<double>(out, b, 0);
  const double gamma = c->gamma, cv = c->cv;
  for (int k = b.lo[2]; k <= b.hi[2]; ++k)
    for (int j = b.lo[1]; j <= b.hi[1]; ++j)
      for (int i = b.lo[0]; i <= b.hi[0]; ++i) {
        const double rhoinv = 1.0 / u(i, j, k, URHO);
        const double mx = u(i, j, k, UMX), my = u(i, j, k, UMY), mz = u(i, j, k, UMZ);
        const double rhoeint = u(i, j, k, UET) - 0.5 * rhoinv * (mx * mx + my * my + mz * mz);
        o(i, j, k, 0) = (gamma - 1.0) * rhoeint;
        o(i, j, k, 1) = (rhoeint * rhoinv) / cv;
        o(i, j, k, 2) = u(i, j, k, UMX) / u(i, j, k, URHO);
        o(i, j, k, 3) = u(i, j, k, UMY) / u(i, j, k, URHO);
        o(i, j, k, 4) = u(i, j, k, UMZ) / u(i, j, k, URHO);
      }
  return 0;
}

// Number of stages of an RK variant, or -1 if the reference rejects it.
int orc_rk_nstages(int order_rk, int stages_rk) {
  StageProg st[8];
  if (order_rk == 2 && (stages_rk < 2 || stages_rk > 8)) return -1;
  return rk_program(order_rk, stages_rk, 1.0, st);
}

// One CNS::advance step of a single-box domain.  S1 (in, ghosted) holds U^n;
// S2 (out, ghosted) receives U^{n+1} on its valid cells.  Halo: orc_fill_halo.
int orc_advance(const OrcScheme* s, const OrcClosures* c, const int* lo, const int* hi,
                const double* dxinv, const int* bc_lo, const int* bc_hi, int order_rk,
                int stages_rk, double dt, double* S1, double* S2, int nthreads) {
  if (!s || !c || !lo || !hi || !dxinv || !S1 || !S2) return 1;
  StageProg st[8];
  if (order_rk == 2 && (stages_rk < 2 || stages_rk > 8)) return 5;
  const int ns = rk_program(order_rk, stages_rk, dt, st);
  if (ns < 0) return 5;
  Box b = to_box(lo, hi);
  const long long ng = ghosted(b), nv = b.cells();
  double* sborder_p = pool<double>(14, ng * NCONS);
  double* ds_p = pool<double>(15, nv * NCONS);
  struct { double* p; double* data() const { return p; } } sborder{sborder_p}, ds{ds_p};
  Arr<double> a1 = make_arr<double>(S1, b, NGHOST), a2 = make_arr<double>(S2, b, NGHOST);
  Arr<double> ab = make_arr<double>(sborder.data(), b, NGHOST), ad = make_arr<double>(ds.data(), b, 0);
  const Scheme sc = to_sc(s);
  const Closures cl = to_cl(c);
  if (order_rk == 2) {  // MultiFab::Copy(S2,S1) before the stages
    for (int n = 0; n < NCONS; ++n)
      for (int k = b.lo[2]; k <= b.hi[2]; ++k)
        for (int j = b.lo[1]; j <= b.hi[1]; ++j)
          for (int i = b.lo[0]; i <= b.hi[0]; ++i) a2(i, j, k, n) = a1(i, j, k, n);
  }
  for (int is = 0; is < ns; ++is) {
    // FillPatch: copy the source state (ghost cells beyond ext_dir sides, the
    // caller's, come with it), then fill the other ghosts
    std::memcpy(sborder.data(), st[is].src ? S2 : S1, sizeof(double) * ng * NCONS);
    int rc = orc_fill_halo(lo, hi, bc_lo, bc_hi, sborder.data(), NCONS);
    if (rc) return rc;
    // code-6 y sides of this single-box domain are walls
    Walls w{bc_lo && bc_lo[1] == 6, bc_hi && bc_hi[1] == 6, b.lo[1], b.hi[1]};
    compute_rhs_box<double>(sc, cl, b, dxinv, sborder.data(), ds.data(), nthreads, &w);
#ifdef _OPENMP
#pragma omp parallel for collapse(2) num_threads(nthreads > 0 ? nthreads : 1) schedule(static)
#endif
    for (int n = 0; n < NCONS; ++n)
      for (int k = b.lo[2]; k <= b.hi[2]; ++k)
        for (int j = b.lo[1]; j <= b.hi[1]; ++j)
          for (int i = b.lo[0]; i <= b.hi[0]; ++i) {
            double reg[3] = {a1(i, j, k, n), a2(i, j, k, n), ad(i, j, k, n)};
            apply_ops(st[is], reg);
            a2(i, j, k, n) = reg[RS2];
            ad(i, j, k, n) = reg[RDS];
          }
  }
  return 0;
}

}  // extern "C"
