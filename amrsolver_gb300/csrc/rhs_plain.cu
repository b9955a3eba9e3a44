// Face-array RHS path: the reference's kernel sequence, one kernel per
// sub-operation, flattened over a box list.  It carries the schemes that
// have no fused kernel yet (WENO5-JS LLF, MUSCL + Riemann, JST dissipation)
// and a KEEP variant kept as the "plain per-box" baseline.
//
//   Euler face fluxes  -> FaceRec::f[d]   (KEEP / WENO / Riemann)
//   JST dissipation    -> subtracted from f[d]
//   viscous averages   -> added to f[d]   (cell fluxes from visc_cell_kernel)
//   divergence + RK stage program -> output slot
//
// Operation order follows the cited reference functions and the file is
// built with -fmad=false, so results match the reference's CPU build
// (WENO5 squares its smoothness terms directly, where the reference calls
// pow(x, 2); the two can differ in the last bit).  The default WENO5 face
// kernel instead forms the nonlinear weights over a common denominator
// with explicit fused multiply-adds (weno5js_cd): the same function in
// exact arithmetic, a quarter of the divisions, rounding differences only.
#include "amrs_kernels.h"
#include "ddiv.cuh"

namespace amrs {

// face index -> (box, direction, i, j, k) over faces nodal in d
struct FaceIdx {
  int b, d, i, j, k;
};

__device__ __forceinline__ bool decode_face(const BoxTable& tb, const FaceTable& ft, long long g, FaceIdx& f) {
  long long base = 0;
  for (int d = 0; d < 3; ++d) {
    const long long tot = ft.fpre[d][tb.n];
    if (g < base + tot) {
      const long long l = g - base;
      const int b = find_box_ll(ft.fpre[d], tb.n, l);
      const BoxRec& R = tb.box[b];
      const int loc = (int)(l - ft.fpre[d][b]);
      const int nx = R.hi[0] - R.lo[0] + 1 + (d == 0), ny = R.hi[1] - R.lo[1] + 1 + (d == 1);
      f.b = b;
      f.d = d;
      f.i = loc % nx + R.lo[0];
      const int t = loc / nx;
      f.j = t % ny + R.lo[1];
      f.k = t / ny + R.lo[2];
      return true;
    }
    base += tot;
  }
  return false;
}

__device__ __forceinline__ void decode_cell(const BoxRec& R, int loc, int g, int& i, int& j, int& k) {
  const int nx = R.hi[0] - R.lo[0] + 1 + 2 * g, ny = R.hi[1] - R.lo[1] + 1 + 2 * g;
  i = loc % nx + R.lo[0] - g;
  const int t = loc / nx;
  j = t % ny + R.lo[1] - g;
  k = t / ny + R.lo[2] - g;
}

static int grid_for(long long n, int nsm) {
  long long blocks = (n + 255) / 256;
  const long long cap = (long long)nsm * 8;
  return (int)(blocks < cap ? (blocks < 1 ? 1 : blocks) : cap);
}

// ------------------------------------------------------- KEEP, plain ----
// src/rhs/CentralKEEP.h:40-145, one face per thread, pairs summed in the
// reference's (l, m) order without sharing between faces.
template <int ORDER>
__global__ void __launch_bounds__(256) keep_faces_plain_kernel(BoxTable tb, FaceTable ft, long long total) {
  if (list_idle(tb)) return;
  constexpr int H = ORDER / 2;
  double coef[3];
  if (ORDER == 6) { coef[0] = 6.0 / 4; coef[1] = -6.0 / 20; coef[2] = 2.0 / 60; }
  else if (ORDER == 4) { coef[0] = 4.0 / 3; coef[1] = -2.0 / 12; coef[2] = 0.0; }
  else { coef[0] = 1.0; coef[1] = 0.0; coef[2] = 0.0; }
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < total;
       g += (long long)gridDim.x * blockDim.x) {
    FaceIdx f;
    if (!decode_face(tb, ft, g, f)) continue;
    const BoxRec& R = tb.box[f.b];
    const DArr Q = R.q;
    const int di = f.d == 0, dj = f.d == 1, dk = f.d == 2;
    // y faces next to a code-6 wall: second-order KEEP, coefficient 1
    // (Flux_2nd_Order_KEEP, src/rhs/CentralKEEP.h:232-287)
    const bool red = f.d == 1 && R.walls && (f.j <= R.red_lo || (f.j >= R.red_hi && f.j <= R.hi[1]));
    const int hs = red ? 1 : H;
    double F[5] = {0, 0, 0, 0, 0};
#pragma unroll
    for (int l = 1; l <= H; ++l)
#pragma unroll
      for (int m = 0; m < l; ++m) {
        if (l > hs) continue;
        double q1[NQ], q2[NQ], T[5];
        const long long o1 = Q.off(f.i + m * di, f.j + m * dj, f.k + m * dk);
        const long long o2 = Q.off(f.i + (m - l) * di, f.j + (m - l) * dj, f.k + (m - l) * dk);
#pragma unroll
        for (int n = 0; n < NQ; ++n) { q1[n] = Q.p[o1 + n * Q.ns]; q2[n] = Q.p[o2 + n * Q.ns]; }
        const double c = red ? 1.0 : coef[l - 1];
        if (f.d == 0) keep_pair<0>(q1, q2, c, T);
        else if (f.d == 1) keep_pair<1>(q1, q2, c, T);
        else keep_pair<2>(q1, q2, c, T);
#pragma unroll
        for (int n = 0; n < 5; ++n) F[n] = F[n] + T[n];
      }
    const DArr Fd = ft.fr[f.b].f[f.d];
    const long long of = Fd.off(f.i, f.j, f.k);
#pragma unroll
    for (int n = 0; n < 5; ++n) Fd.p[of + n * Fd.ns] = F[n];
  }
}

// ------------------------------------------------------------- WENO5 ----
// Physical Euler fluxes + max eigenvalue: src/rhs/High_resolution.h:83-121.
#ifndef AMRS_WPF_IMUL
#define AMRS_WPF_IMUL 0x0B
#endif
__global__ void __launch_bounds__(256) weno_flux_lambda_kernel(BoxTable tb, FaceTable ft, int s_in, long long total) {
  if (list_idle(tb)) return;
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < total;
       g += (long long)gridDim.x * blockDim.x) {
    const int b = find_box_ll(ft.gpre, tb.n, g);
    const BoxRec& R = tb.box[b];
    const FaceRec& FR = ft.fr[b];
    int i, j, k;
    decode_cell(R, (int)(g - ft.gpre[b]), NGHOST, i, j, k);
    const DArr U = R.slot[s_in];
    const long long o = U.off(i, j, k);
    const double gam = tb.cls[R.cl].gamma;
    const double rhoinv = ddiv_rn(1.0, U.p[o]);
    const double momx = U.p[o + U.ns], momy = U.p[o + 2 * U.ns], momz = U.p[o + 3 * U.ns];
    const double rhoet = U.p[o + 4 * U.ns];
    // products on the integer pipe (kmul), by bit of AMRS_WPF_IMUL: 0 the
    // velocities, 1 the kinetic energy, 2 the pressure, 3 the fluxes, 4 the
    // sound speed's argument
    constexpr int M = AMRS_WPF_IMUL;
    constexpr bool M0 = M & 1, M1 = (M >> 1) & 1, M2 = (M >> 2) & 1, M3 = (M >> 3) & 1, M4 = (M >> 4) & 1;
    const double ux = kmul<M0>(momx, rhoinv), uy = kmul<M0>(momy, rhoinv), uz = kmul<M0>(momz, rhoinv);
    const double rhoekin = kmul<M1>(kmul<M1>(0.5, rhoinv), kmul<M1>(momx, momx) + kmul<M1>(momy, momy) +
                                                               kmul<M1>(momz, momz));
    const double rhoeint = rhoet - rhoekin;
    const double P = kmul<M2>(gam - 1.0, rhoeint);
    const long long op = FR.pf[0].off(i, j, k);
    const long long ns = FR.pf[0].ns;
    double* fx = FR.pf[0].p + op;
    double* fy = FR.pf[1].p + op;
    double* fz = FR.pf[2].p + op;
    const double rhoh = rhoet + P;
    fx[0] = momx; fx[ns] = kmul<M3>(momx, ux) + P; fx[2 * ns] = kmul<M3>(momy, ux); fx[3 * ns] = kmul<M3>(momz, ux);
    fx[4 * ns] = kmul<M3>(rhoh, ux);
    fy[0] = momy; fy[ns] = kmul<M3>(momx, uy); fy[2 * ns] = kmul<M3>(momy, uy) + P; fy[3 * ns] = kmul<M3>(momz, uy);
    fy[4 * ns] = kmul<M3>(rhoh, uy);
    fz[0] = momz; fz[ns] = kmul<M3>(momx, uz); fz[2 * ns] = kmul<M3>(momy, uz); fz[3 * ns] = kmul<M3>(momz, uz) + P;
    fz[4 * ns] = kmul<M3>(rhoh, uz);
    const double cs = dsqrt_rn(kmul<M4>(kmul<M4>(gam, P), rhoinv));
    const long long ol = FR.lam.off(i, j, k);
    // |max(max(u + c, u - c), u)| of the reference: with c >= 0 and rounding
    // monotonic, fl(u + c) >= u >= fl(u - c), so the maximum is u + c itself
    // (a NaN c gives NaN either way)
    FR.lam.p[ol] = fabs(ux + cs);
    FR.lam.p[ol + FR.lam.ns] = fabs(uy + cs);
    FR.lam.p[ol + 2 * FR.lam.ns] = fabs(uz + cs);
  }
}

// WENO5-JS (src/rhs/High_resolution.h:124-159), beta[1] with the fourth power.
// Operation order of the reference; a sum x + 2^k*y (power-of-two factor,
// exact product) is one fma, which rounds exactly like the reference's
// separate multiply and add.  The four divisions are correctly rounded on
// the integer pipe (ddiv_rn): the same quotients as the reference's, at a
// fraction of the FP64 issue slots.
// Products formed on the integer pipe (kmul), by bit: 0 the shared 3 s2,
// 1 the (13/12) x^2 terms, 2 the quarter-scaled squares b^2 and f^2, 3 the
// fourth power of beta1, 4 the squares of eps + beta, 5 the stencil
// coefficients 7, 11, 5, 6 the final scaling, 7 the weight products,
// 8 the LLF halves (0.5 me) U of the face kernel; bit 9 takes the maximum
// wave speed of the face kernel as an integer maximum of the bit patterns.
#ifndef AMRS_WENO_IMUL
#define AMRS_WENO_IMUL 0x263
#endif
// The same for the reconstructions of the WENO5-Riemann face kernel, whose
// serial solver leaves less room on the integer pipe.
#ifndef AMRS_WRREC_IMUL
#define AMRS_WRREC_IMUL 0x001
#endif
template <int M = AMRS_WENO_IMUL>
__device__ __forceinline__ double weno5js(const double s0, const double s1, const double s2, const double s3,
                                          const double s4) {
  constexpr bool M0 = M & 1, M1 = (M >> 1) & 1, M2 = (M >> 2) & 1, M3 = (M >> 3) & 1, M4 = (M >> 4) & 1,
                 M5 = (M >> 5) & 1, M6 = (M >> 6) & 1, M7 = (M >> 7) & 1;
  const double eps = 1e-40;
  const double s2x3 = kmul<M0>(3.0, s2);
  const double a = fma(-2.0, s1, s0) + s2;         // s0 - 2 s1 + s2
  const double b = fma(-4.0, s1, s0) + s2x3;       // s0 - 4 s1 + 3 s2
  const double c = fma(-2.0, s2, s1) + s3;         // s1 - 2 s2 + s3
  const double g = s1 - s3;
  const double d = fma(-2.0, s3, s2) + s4;         // s2 - 2 s3 + s4
  const double f = fma(-4.0, s3, s2x3) + s4;       // 3 s2 - 4 s3 + s4
  // 0.25*b*b == 0.25*(b*b) and 0.25*g*g*g*g == 0.25*(((g*g)*g)*g): the
  // quarter scales exactly, so x + 0.25*y is one fma(0.25, y, x) (normal range)
  constexpr double c1312 = 13.0 / 12.0;
  const double beta0 = fma(0.25, kmul<M2>(b, b), kmul<M1>(kmul<M1>(c1312, a), a));
  const double beta1 = fma(0.25, kmul<M3>(kmul<M3>(kmul<M3>(g, g), g), g), kmul<M1>(kmul<M1>(c1312, c), c));
  const double beta2 = fma(0.25, kmul<M2>(f, f), kmul<M1>(kmul<M1>(c1312, d), d));
  const double e0 = eps + beta0, e1 = eps + beta1, e2 = eps + beta2;
  const double alpha0 = ddiv_rn(0.1, kmul<M4>(e0, e0));
  const double alpha1 = ddiv_rn(0.6, kmul<M4>(e1, e1));
  const double alpha2 = ddiv_rn(0.3, kmul<M4>(e2, e2));
  const double sum = ddiv_rn(1.0, alpha0 + alpha1 + alpha2);
  const double vl0 = fma(2.0, s0, -kmul<M5>(7.0, s1)) + kmul<M5>(11.0, s2);  // 2 s0 - 7 s1 + 11 s2
  const double vl1 = fma(2.0, s3, -s1 + kmul<M5>(5.0, s2));                  // -s1 + 5 s2 + 2 s3
  const double vl2 = fma(2.0, s2, kmul<M5>(5.0, s3)) - s4;                   // 2 s2 + 5 s3 - s4
  return kmul<M6>(kmul<M6>(1.0 / 6.0, sum),
                  kmul<M7>(alpha0, vl0) + kmul<M7>(alpha1, vl1) + kmul<M7>(alpha2, vl2));
}

// The same reconstruction with its weights over a common denominator, for
// inputs t = 2s (the LLF halves are folded into the caller):
//   w_k = a_k / (a0+a1+a2),  a_k = c_k / e_k^2,  e_k = beta_k + eps
//   sum_k w_k v_k / 6 = (sum_k c_k v_k P_k) / (6 sum_k c_k P_k),  P_k = prod_{j!=k} e_j^2.
// 4 beta(s) is evaluated from t and eps becomes 4 eps, so the weights are
// unchanged in exact arithmetic; the 1/6 and the final 1/2 go into the v_k coefficients.
// One division instead of four; every product and sum is a fused
// multiply-add where one fits.  Range: the products P_k stay finite for
// |t| up to about 1e38 and normal for eps = 4e-40 (P_k >= 2.6e-158).
__device__ __forceinline__ double weno5js_cd(const double t0, const double t1, const double t2, const double t3,
                                             const double t4) {
  constexpr double eps4 = 4e-40;
  constexpr double c1312 = 13.0 / 12.0;
  // beta_0: (13/12) d1^2 + (1/4) d2^2
  const double d1 = fma(-2.0, t1, t0) + t2;
  const double d2 = fma(3.0, t2, fma(-4.0, t1, t0));
  const double e0 = fma(c1312 * d1, d1, fma(0.25 * d2, d2, eps4));
  // beta_1: (13/12) d3^2 + (1/4) (s1 - s3)^4; its fourth-power term is not
  // homogeneous of degree 2, so in t = 2s: 4 beta_1 = (13/12) d3^2 + (1/16) g^4
  const double d3 = fma(-2.0, t2, t1) + t3;
  const double g = t1 - t3;
  const double g2 = g * g;
  const double e1 = fma(c1312 * d3, d3, fma(0.0625 * g2, g2, eps4));
  // beta_2: (13/12) d4^2 + (1/4) d5^2
  const double d4 = fma(-2.0, t3, t2) + t4;
  const double d5 = fma(-4.0, t3, fma(3.0, t2, t4));
  const double e2 = fma(c1312 * d4, d4, fma(0.25 * d5, d5, eps4));
  const double E0 = e0 * e0, E1 = e1 * e1, E2 = e2 * e2;
  const double P0 = E1 * E2, P1 = E0 * E2, P2 = E0 * E1;
  const double den = fma(0.1, P0, fma(0.6, P1, 0.3 * P2));
  // c_k v_k / 12 with v0 = 2t0 - 7t1 + 11t2, v1 = -t1 + 5t2 + 2t3, v2 = 2t2 + 5t3 - t4
  constexpr double k0 = 0.1 / 12.0, k1 = 0.6 / 12.0, k2 = 0.3 / 12.0;
  const double v0 = fma(11.0 * k0, t2, fma(-7.0 * k0, t1, (2.0 * k0) * t0));
  const double v1 = fma(2.0 * k1, t3, fma(5.0 * k1, t2, -k1 * t1));
  const double v2 = fma(-k2, t4, fma(5.0 * k2, t3, (2.0 * k2) * t2));
  const double num = fma(v0, P0, fma(v1, P1, v2 * P2));
  return num / den;
}

// LLF-split WENO face flux for all components (src/rhs/High_resolution.h:162-246).
// REF_ORDER: the reference's operation order; otherwise the split halves
// 0.5 (f +- alpha U) enter weno5js_cd doubled as fma(+-alpha, U, f).
template <bool REF_ORDER>
__global__ void __launch_bounds__(256) weno_face_kernel(BoxTable tb, FaceTable ft, int s_in, long long total) {
  if (list_idle(tb)) return;
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < total;
       g += (long long)gridDim.x * blockDim.x) {
    FaceIdx f;
    if (!decode_face(tb, ft, g, f)) continue;
    const BoxRec& R = tb.box[f.b];
    const FaceRec& FR = ft.fr[f.b];
    const DArr U = R.slot[s_in];
    const DArr PF = FR.pf[f.d];
    const DArr L = FR.lam;
    const long long st = (f.d == 0) ? 1 : (f.d == 1 ? L.js : L.ks);
    const long long su = (f.d == 0) ? 1 : (f.d == 1 ? U.js : U.ks);
    const long long ol = L.off(f.i, f.j, f.k) + f.d * L.ns;
    double me;
    if (REF_ORDER && !((AMRS_WENO_IMUL >> 9) & 1)) {
      me = rmax(L.p[ol - 3 * st], L.p[ol - 2 * st]);
      me = rmax(me, L.p[ol - st]);
      me = rmax(me, L.p[ol]);
      me = rmax(me, L.p[ol + st]);
      me = rmax(me, L.p[ol + 2 * st]);
    } else {
      // lambda = |u| + c > 0: the integer order of the bit patterns is the
      // order of the values, and the maximum (the same value as the
      // reference's chain of rmax) needs no FP64 instruction
      long long m = __double_as_longlong(L.p[ol - 3 * st]);
#pragma unroll
      for (int q = -2; q <= 2; ++q) m = max(m, __double_as_longlong(L.p[ol + q * st]));
      me = __longlong_as_double(m);
    }
    const long long ou = U.off(f.i, f.j, f.k), opf = PF.off(f.i, f.j, f.k);
    const DArr Fd = FR.f[f.d];
    const long long of = Fd.off(f.i, f.j, f.k);
    if (!REF_ORDER) {
#pragma unroll 1
      for (int n = 0; n < 5; ++n) {
        double u[6], p[6];
#pragma unroll
        for (int q = 0; q < 6; ++q) {
          u[q] = U.p[ou + (q - 3) * su + n * U.ns];
          p[q] = PF.p[opf + (q - 3) * su + n * PF.ns];
        }
        const double flx = weno5js_cd(fma(me, u[0], p[0]), fma(me, u[1], p[1]), fma(me, u[2], p[2]),
                                      fma(me, u[3], p[3]), fma(me, u[4], p[4])) +
                           weno5js_cd(fma(-me, u[5], p[5]), fma(-me, u[4], p[4]), fma(-me, u[3], p[3]),
                                      fma(-me, u[2], p[2]), fma(-me, u[1], p[1]));
        Fd.p[of + n * Fd.ns] = flx;
      }
    } else {
      // 0.5*(p + me*U) == fma(0.5, p, (0.5*me)*U): halving is exact, so the
      // split stencils round exactly as in the reference (normal range)
      const double hme = 0.5 * me;
      for (int n = 0; n < 5; ++n) {
        double h[6], p[6];
#pragma unroll
        for (int q = 0; q < 6; ++q) {
          h[q] = kmul<(AMRS_WENO_IMUL >> 8) & 1>(hme, U.p[ou + (q - 3) * su + n * U.ns]);
          p[q] = PF.p[opf + (q - 3) * su + n * PF.ns];
        }
        double flx = weno5js(fma(0.5, p[0], h[0]), fma(0.5, p[1], h[1]), fma(0.5, p[2], h[2]),
                             fma(0.5, p[3], h[3]), fma(0.5, p[4], h[4]));
        flx += weno5js(fma(0.5, p[5], -h[5]), fma(0.5, p[4], -h[4]), fma(0.5, p[3], -h[3]),
                       fma(0.5, p[2], -h[2]), fma(0.5, p[1], -h[1]));
        Fd.p[of + n * Fd.ns] = flx;
      }
    }
  }
}

// ----------------------------------------------------------- Riemann ----
// Square roots of the solver and the slopes, and the division of the
// WENO5-Riemann kernel's solver: integer-pipe (dsqrt_rn, ddiv_rn) or
// hardware, the same correctly rounded values; the defaults are the faster
// forms at 128^3 and 256^3.
#ifndef AMRS_RS_ISQRT
#define AMRS_RS_ISQRT 0
#endif
#ifndef AMRS_SLOPE_ISQRT
#define AMRS_SLOPE_ISQRT 1
#endif
#ifndef AMRS_WR_IDIV
#define AMRS_WR_IDIV 0
#endif
template <bool I>
__device__ __forceinline__ double sqrt_sel(double x) {
  return I ? dsqrt_rn(x) : sqrt(x);
}

__device__ __forceinline__ double mc_limiter(double dlft, double drgt) {
  // src/rhs/Riemann.h:9-17
  const double dcen = 0.5 * (dlft + drgt);
  const double dsgn = copysign(1.0, dcen);
  const double slop = 2.0 * rmin(fabs(dlft), fabs(drgt));
  const double dlim = (dlft * drgt >= 0.0) ? slop : 0.0;
  return dsgn * rmin(dlim, fabs(dcen));
}

// Characteristic slopes in direction d (src/rhs/Riemann.h:19-120).
__global__ void __launch_bounds__(256) slope_kernel(BoxTable tb, FaceTable ft, const long long* spre0,
                                                    const long long* spre1, const long long* spre2,
                                                    long long tot0, long long tot1, long long tot2) {
  if (list_idle(tb)) return;
  const long long total = tot0 + tot1 + tot2;
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < total;
       g += (long long)gridDim.x * blockDim.x) {
    int d;
    long long l;
    const long long* pre;
    if (g < tot0) { d = 0; l = g; pre = spre0; }
    else if (g < tot0 + tot1) { d = 1; l = g - tot0; pre = spre1; }
    else { d = 2; l = g - tot0 - tot1; pre = spre2; }
    const int b = find_box_ll(pre, tb.n, l);
    const BoxRec& R = tb.box[b];
    const int loc = (int)(l - pre[b]);
    const int nx = R.hi[0] - R.lo[0] + 1 + 2 * (d == 0), ny = R.hi[1] - R.lo[1] + 1 + 2 * (d == 1);
    const int i = loc % nx + R.lo[0] - (d == 0);
    const int t = loc / nx;
    const int j = t % ny + R.lo[1] - (d == 1);
    const int k = t / ny + R.lo[2] - (d == 2);
    const DArr q = R.q;
    const DClosures& cl = tb.cls[R.cl];
    const long long s = (d == 0) ? 1 : (d == 1 ? q.js : q.ks);
    const long long o = q.off(i, j, k);
    const int QN = QU + d, QT1 = (d == 0) ? QV : QU, QT2 = (d == 2) ? QV : QW;
    auto Q = [&](long long off, int n) { return q.p[off + n * q.ns]; };
    const double c0 = sqrt_sel<AMRS_SLOPE_ISQRT>(cl.gamma * cl.Rspec * Q(o, QT));
    const double cspeed = c0 + (d == 0 ? 2.e-40 : 1.e-40);
    double dlft = ddiv_rn(0.5 * (Q(o, QPRES) - Q(o - s, QPRES)), cspeed) - 0.5 * Q(o, QRHO) * (Q(o, QN) - Q(o - s, QN));
    double drgt = ddiv_rn(0.5 * (Q(o + s, QPRES) - Q(o, QPRES)), cspeed) - 0.5 * Q(o, QRHO) * (Q(o + s, QN) - Q(o, QN));
    const double d0 = mc_limiter(dlft, drgt);
    const double cs2 = cspeed * cspeed;
    dlft = (Q(o, QRHO) - Q(o - s, QRHO)) - ddiv_rn(Q(o, QPRES) - Q(o - s, QPRES), cs2);
    drgt = (Q(o + s, QRHO) - Q(o, QRHO)) - ddiv_rn(Q(o + s, QPRES) - Q(o, QPRES), cs2);
    const double d1 = mc_limiter(dlft, drgt);
    dlft = ddiv_rn(0.5 * (Q(o, QPRES) - Q(o - s, QPRES)), cspeed) + 0.5 * Q(o, QRHO) * (Q(o, QN) - Q(o - s, QN));
    drgt = ddiv_rn(0.5 * (Q(o + s, QPRES) - Q(o, QPRES)), cspeed) + 0.5 * Q(o, QRHO) * (Q(o + s, QN) - Q(o, QN));
    const double d2 = mc_limiter(dlft, drgt);
    const double d3 = mc_limiter(Q(o, QT1) - Q(o - s, QT1), Q(o + s, QT1) - Q(o, QT1));
    const double d4 = mc_limiter(Q(o, QT2) - Q(o - s, QT2), Q(o + s, QT2) - Q(o, QT2));
    // The terms of this cell's extrapolations to its two faces
    // (src/rhs/Riemann.h:251-337), formed once here instead of once per face
    // side: A = (d0+d2)/c + d1 (density), B = (d2-d0)/rho (normal velocity),
    // C = (d0+d2)*c (pressure), c the cell's sqrt(gamma R T) + 1e-40.
    const double csr = c0 + 1.e-40;
    const double s02 = d0 + d2;
    const DArr S = ft.fr[b].slope[d];
    const long long os = S.off(i, j, k);
    S.p[os + SL_A * S.ns] = ddiv_rn(s02, csr) + d1;
    S.p[os + SL_B * S.ns] = ddiv_rn(d2 - d0, Q(o, QRHO));
    S.p[os + SL_C * S.ns] = s02 * csr;
    S.p[os + SL_T1 * S.ns] = d3;
    S.p[os + SL_T2 * S.ns] = d4;
    if (d == 2 && k <= R.hi[2]) {
      // cns_riemann_z's left state takes its sound speed from q(i,j,k+1)
      // (src/rhs/Riemann.h:316): for the face above this cell, cell k + 2
      const double csl = sqrt_sel<AMRS_SLOPE_ISQRT>(cl.gamma * cl.Rspec * Q(o + 2 * s, QT)) + 1.e-40;
      S.p[os + SL_AL * S.ns] = ddiv_rn(s02, csl) + d1;
      S.p[os + SL_CL * S.ns] = s02 * csl;
    }
  }
}

// Division of the two-shock solver: IDIV picks the integer-pipe form
// (ddiv_rn) or the hardware one; both give the same correctly rounded bits.
template <bool IDIV>
__device__ __forceinline__ double rdiv(double a, double b) {
  return IDIV ? ddiv_rn(a, b) : a / b;
}

// Two-shock approximate Riemann solver (src/rhs/Riemann.h:123-249).  Its
// pressure iterations are one serial chain per face, so the choice of
// division is the caller's: the MUSCL face kernel runs faster with the
// integer-pipe division, the WENO5-Riemann kernel (whose reconstructions
// already load the integer pipe) with the hardware one; the square roots are
// the hardware's in both (AMRS_RS_ISQRT: their integer form lengthens the
// chain at the 128^3 and 256^3 sizes, though it shortens it at 64^3).
template <bool IDIV>
__device__ void riemann_prob(const double gamma, const double smallp, const double rl, const double ul,
                             const double pl, const double ut1l, const double ut2l, const double rr, const double ur,
                             const double pr, const double ut1r, const double ut2r, double& flxrho, double& flxu,
                             double& flxut, double& flxutt, double& flxe) {
  const double weakwv = 1.e-3;
  const double small = 1.e-6;
  const double clsql = gamma * pl * rl;
  const double clsqr = gamma * pr * rr;
  double wl = sqrt_sel<AMRS_RS_ISQRT>(clsql);
  double wr = sqrt_sel<AMRS_RS_ISQRT>(clsqr);
  const double cleft = rdiv<IDIV>(wl, rl);
  const double cright = rdiv<IDIV>(wr, rr);
  const double ccsmall = small * (cleft + cright);
  double pstar = rdiv<IDIV>(wl * pr + wr * pl - wr * wl * (ur - ul), wl + wr);
  pstar = rmax(pstar, smallp);
  double pstnm1 = pstar;
  double wlsq = (0.5 * (gamma - 1.) * (pstar + pl) + pstar) * rl;
  double wrsq = (0.5 * (gamma - 1.) * (pstar + pr) + pstar) * rr;
  wl = sqrt_sel<AMRS_RS_ISQRT>(wlsq);
  wr = sqrt_sel<AMRS_RS_ISQRT>(wrsq);
  double ustarp = ul - rdiv<IDIV>(pstar - pl, wl);
  double ustarm = ur + rdiv<IDIV>(pstar - pr, wr);
  pstar = rdiv<IDIV>(wl * pr + wr * pl - wr * wl * (ur - ul), wl + wr);
  pstar = rmax(pstar, smallp);
  double ustar = 0.0;
  for (int iter = 0; iter < 3; ++iter) {
    wlsq = (0.5 * (gamma - 1.) * (pstar + pl) + pstar) * rl;
    wrsq = (0.5 * (gamma - 1.) * (pstar + pr) + pstar) * rr;
    wl = rdiv<IDIV>(1., sqrt_sel<AMRS_RS_ISQRT>(wlsq));
    wr = rdiv<IDIV>(1., sqrt_sel<AMRS_RS_ISQRT>(wrsq));
    const double ustnm1 = ustarm;
    const double ustnp1 = ustarp;
    ustarm = ur - (pr - pstar) * wr;
    ustarp = ul + (pl - pstar) * wl;
    const double dpditer = fabs(pstnm1 - pstar);
    double zp = fabs(ustarp - ustnp1);
    if (zp - weakwv * cleft < 0.0) zp = dpditer * wl;
    double zm = fabs(ustarm - ustnm1);
    if (zm - weakwv * cright < 0.0) zm = dpditer * wr;
    const double zz = zp + zm;
    const double denom = rdiv<IDIV>(dpditer, rmax(zz, ccsmall));
    pstnm1 = pstar;
    pstar = pstar - denom * (ustarm - ustarp);
    pstar = rmax(pstar, smallp);
    ustar = 0.5 * (ustarm + ustarp);
  }
  double ro, uo, po, sgnm, utrans1, utrans2;
  if (ustar > 0.) {
    ro = rl; uo = ul; po = pl; sgnm = 1.; utrans1 = ut1l; utrans2 = ut2l;
  } else if (ustar < 0.) {
    ro = rr; uo = ur; po = pr; sgnm = -1.; utrans1 = ut1r; utrans2 = ut2r;
  } else {
    uo = 0.5 * (ur + ul);
    po = 0.5 * (pr + pl);
    ro = rdiv<IDIV>(2. * (rl * rr), rl + rr);
    sgnm = 1.;
    utrans1 = 0.5 * (ut1l + ut1r);
    utrans2 = 0.5 * (ut2l + ut2r);
  }
  const double wosq = (0.5 * (gamma - 1.) * (pstar + po) + pstar) * ro;
  const double dpjmp = pstar - po;
  const double suo = sgnm * uo;
  double rgdnv, ugdnv, pgdnv;
  // The reference evaluates every wave speed and the star density before it
  // selects the state; here each is evaluated on the branch that reads it
  // (same operations, same values, same selection, NaN included).
  auto mixed = [&](double spin, double spout, double rstar) {
    const double ss = rmax(spout - spin, spout + spin);
    const double frac = 0.5 * (1. + rdiv<IDIV>(spin + spout, rmax(ss, ccsmall)));
    rgdnv = frac * rstar + (1. - frac) * ro;
    ugdnv = frac * ustar + (1. - frac) * uo;
    pgdnv = frac * pstar + (1. - frac) * po;
  };
  if (pstar >= po) {
    // shock: spout == spin, so the side state or the star state
    const double spin = rdiv<IDIV>(sqrt_sel<AMRS_RS_ISQRT>(wosq), ro) - suo;
    if (spin < 0.) {
      rgdnv = ro; ugdnv = uo; pgdnv = po;
    } else if (spin >= 0.) {
      rgdnv = rdiv<IDIV>(ro, 1. - rdiv<IDIV>(ro * dpjmp, wosq)); ugdnv = ustar; pgdnv = pstar;
    } else {
      mixed(spin, spin, rdiv<IDIV>(ro, 1. - rdiv<IDIV>(ro * dpjmp, wosq)));
    }
  } else {
    const double rstar = rdiv<IDIV>(ro, 1. - rdiv<IDIV>(ro * dpjmp, wosq));
    const double spout = sqrt_sel<AMRS_RS_ISQRT>(rdiv<IDIV>(gamma * po, ro)) - suo;
    const double spin = sqrt_sel<AMRS_RS_ISQRT>(rdiv<IDIV>(gamma * pstar, rstar)) - suo;
    if (spout < 0.) {
      rgdnv = ro; ugdnv = uo; pgdnv = po;
    } else if (spin >= 0.) {
      rgdnv = rstar; ugdnv = ustar; pgdnv = pstar;
    } else {
      mixed(spin, spout, rstar);
    }
  }
  flxrho = rgdnv * ugdnv;
  flxu = rgdnv * ugdnv * ugdnv + pgdnv;
  flxut = rgdnv * ugdnv * utrans1;
  flxutt = rgdnv * ugdnv * utrans2;
  // (0.5*r)*k + x == fma(0.5, r*k, x): the halving is exact (normal range)
  flxe = ugdnv * (fma(0.5, rgdnv * (ugdnv * ugdnv + utrans1 * utrans1 + utrans2 * utrans2), rdiv<IDIV>(pgdnv, gamma - 1.)) +
                  pgdnv);
}

// MUSCL face states + Riemann flux (src/rhs/Riemann.h:251-337).
__global__ void __launch_bounds__(256) riemann_face_kernel(BoxTable tb, FaceTable ft, long long total) {
  if (list_idle(tb)) return;
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < total;
       g += (long long)gridDim.x * blockDim.x) {
    FaceIdx f;
    if (!decode_face(tb, ft, g, f)) continue;
    const BoxRec& R = tb.box[f.b];
    const int d = f.d;
    const DArr q = R.q;
    const DArr S = ft.fr[f.b].slope[d];
    const DClosures& cl = tb.cls[R.cl];
    const int QN = QU + d, QT1 = (d == 0) ? QV : QU, QT2 = (d == 2) ? QV : QW;
    const int UN = UMX + d, UT1 = (d == 0) ? UMY : UMX, UT2 = (d == 2) ? UMY : UMZ;
    const int im = f.i - (d == 0), jm = f.j - (d == 1), km = f.k - (d == 2);
    const long long oq = q.off(f.i, f.j, f.k), oqm = q.off(im, jm, km);
    const long long os = S.off(f.i, f.j, f.k), osm = S.off(im, jm, km);
    auto Q = [&](long long off, int n) { return q.p[off + n * q.ns]; };
    auto D = [&](long long off, int n) { return S.p[off + n * S.ns]; };
    const double gam = cl.gamma;
    // left state from cell i-1, right state from cell i, with the terms
    // slope_kernel formed (z: the left terms with the quirk's sound speed);
    // q + 0.5*t == fma(0.5, t, q): the halving is exact (normal range)
    const int cA = (d == 2) ? SL_AL : SL_A, cC = (d == 2) ? SL_CL : SL_C;
    const double rl = rmax(fma(0.5, D(osm, cA), Q(oqm, QRHO)), 1.0e-40);
    const double ul = fma(0.5, D(osm, SL_B), Q(oqm, QN));
    const double pl = rmax(fma(0.5, D(osm, cC), Q(oqm, QPRES)), 1.0e-40);
    const double ut1l = fma(0.5, D(osm, SL_T1), Q(oqm, QT1));
    const double ut2l = fma(0.5, D(osm, SL_T2), Q(oqm, QT2));
    const double rr = rmax(fma(-0.5, D(os, SL_A), Q(oq, QRHO)), 1.0e-40);
    const double ur = fma(-0.5, D(os, SL_B), Q(oq, QN));
    const double pr = rmax(fma(-0.5, D(os, SL_C), Q(oq, QPRES)), 1.0e-40);
    const double ut1r = fma(-0.5, D(os, SL_T1), Q(oq, QT1));
    const double ut2r = fma(-0.5, D(os, SL_T2), Q(oq, QT2));
    double frho, fu, fut, futt, fe;
    riemann_prob<true>(gam, 1.0e-40, rl, ul, pl, ut1l, ut2l, rr, ur, pr, ut1r, ut2r, frho, fu, fut, futt, fe);
    const DArr Fd = ft.fr[f.b].f[d];
    const long long of = Fd.off(f.i, f.j, f.k);
    Fd.p[of + URHO * Fd.ns] = frho;
    Fd.p[of + UN * Fd.ns] = fu;
    Fd.p[of + UT1 * Fd.ns] = fut;
    Fd.p[of + UT2 * Fd.ns] = futt;
    Fd.p[of + UET * Fd.ns] = fe;
  }
}

// WENO5-Riemann faces (riemann_weno = 1), an extension with no counterpart in
// the reference (which pairs WENO5 only with the Lax-Friedrichs split and
// the two-shock solver only with MUSCL): rho, u_n, p, u_t1, u_t2 are
// reconstructed to the face from each side with weno5js (left state: cells
// i-3..i+1; right state: the mirror i+2..i-2), rho and p floored at 1e-40
// as the MUSCL states are (src/rhs/Riemann.h:260-272), and riemann_prob
// gives the flux.  One thread per face.
__global__ void __launch_bounds__(256) weno_riemann_face_kernel(BoxTable tb, FaceTable ft, long long total) {
  if (list_idle(tb)) return;
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < total;
       g += (long long)gridDim.x * blockDim.x) {
    FaceIdx f;
    if (!decode_face(tb, ft, g, f)) continue;
    const BoxRec& R = tb.box[f.b];
    const int d = f.d;
    const DArr q = R.q;
    const DClosures& cl = tb.cls[R.cl];
    const int QN = QU + d, QT1 = (d == 0) ? QV : QU, QT2 = (d == 2) ? QV : QW;
    const int UN = UMX + d, UT1 = (d == 0) ? UMY : UMX, UT2 = (d == 2) ? UMY : UMZ;
    const long long sq = (d == 0) ? 1 : (d == 1 ? q.js : q.ks);
    const long long o = q.off(f.i, f.j, f.k);
    const int comp[5] = {QRHO, QN, QPRES, QT1, QT2};
    double lft[5], rgt[5];
#pragma unroll
    for (int m = 0; m < 5; ++m) {
      const double* p = q.p + o + comp[m] * q.ns;
      double v[6];
#pragma unroll
      for (int t = 0; t < 6; ++t) v[t] = p[(t - 3) * sq];
      lft[m] = weno5js<AMRS_WRREC_IMUL>(v[0], v[1], v[2], v[3], v[4]);
      rgt[m] = weno5js<AMRS_WRREC_IMUL>(v[5], v[4], v[3], v[2], v[1]);
    }
    double frho, fu, fut, futt, fe;
    riemann_prob<AMRS_WR_IDIV != 0>(cl.gamma, 1.0e-40, rmax(lft[0], 1.0e-40), lft[1], rmax(lft[2], 1.0e-40), lft[3], lft[4],
                        rmax(rgt[0], 1.0e-40), rgt[1], rmax(rgt[2], 1.0e-40), rgt[3], rgt[4], frho, fu, fut, futt, fe);
    const DArr Fd = ft.fr[f.b].f[d];
    const long long of = Fd.off(f.i, f.j, f.k);
    Fd.p[of + URHO * Fd.ns] = frho;
    Fd.p[of + UN * Fd.ns] = fu;
    Fd.p[of + UT1 * Fd.ns] = fut;
    Fd.p[of + UT2 * Fd.ns] = futt;
    Fd.p[of + UET * Fd.ns] = fe;
  }
}

// --------------------------------------------------------------- JST ----
__device__ __forceinline__ double discon_sensor(double pp, double pl, double pr) {
  // src/rhs/CNS_hydro_K.h:39-44
  const double pjst = pr + 2.0 * pp + pl;
  const double ptvd = fabs(pr - pp) + fabs(pp - pl);
  return fabs(ddiv_rn(2.0 * (pr - 2.0 * pp + pl), pjst + ptvd + 1.0e-40));
}

// Sensor and spectral radius on the valid box (src/rhs/CNS_hydro_K.h:46-75);
// the arrays are zeroed beforehand, as the reference zeroes its MultiFabs.
__global__ void __launch_bounds__(256) jst_sensor_kernel(BoxTable tb, FaceTable ft, long long total) {
  if (list_idle(tb)) return;
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < total;
       g += (long long)gridDim.x * blockDim.x) {
    const int b = find_box_ll(ft.vpre, tb.n, g);
    const BoxRec& R = tb.box[b];
    int i, j, k;
    decode_cell(R, (int)(g - ft.vpre[b]), 0, i, j, k);
    const DArr q = R.q;
    const long long o = q.off(i, j, k);
    auto P = [&](long long off) { return q.p[off + QPRES * q.ns]; };
    const double pp = P(o);
    const FaceRec& FR = ft.fr[b];
    const long long os = FR.sen.off(i, j, k);
    FR.sen.p[os] = discon_sensor(pp, P(o - 1), P(o + 1));
    FR.sen.p[os + FR.sen.ns] = discon_sensor(pp, P(o - q.js), P(o + q.js));
    FR.sen.p[os + 2 * FR.sen.ns] = discon_sensor(pp, P(o - q.ks), P(o + q.ks));
    const double ux = q.p[o + QU * q.ns], uy = q.p[o + QV * q.ns], uz = q.p[o + QW * q.ns];
    const double cs = dsqrt_rn(ddiv_rn(tb.cls[R.cl].gamma * pp, q.p[o + QRHO * q.ns]));
    FR.lam.p[os] = fabs(ux) + cs;
    FR.lam.p[os + FR.lam.ns] = fabs(uy) + cs;
    FR.lam.p[os + 2 * FR.lam.ns] = fabs(uz) + cs;
  }
}

// JST dissipation subtracted from face fluxes (src/rhs/CNS_hydro_K.h:78-104);
// y and z read component 0 of sensor and lambda, and the z fourth
// difference uses k-1 three times, as in the reference.
__global__ void __launch_bounds__(256) jst_face_kernel(BoxTable tb, FaceTable ft, int s_in, long long total) {
  if (list_idle(tb)) return;
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < total;
       g += (long long)gridDim.x * blockDim.x) {
    FaceIdx f;
    if (!decode_face(tb, ft, g, f)) continue;
    const BoxRec& R = tb.box[f.b];
    const FaceRec& FR = ft.fr[f.b];
    const DClosures& cl = tb.cls[R.cl];
    const DArr U = R.slot[s_in];
    const long long s = (f.d == 0) ? 1 : (f.d == 1 ? U.js : U.ks);
    const long long sl = (f.d == 0) ? 1 : (f.d == 1 ? FR.sen.js : FR.sen.ks);
    const long long ou = U.off(f.i, f.j, f.k), ol = FR.sen.off(f.i, f.j, f.k);
    const double sen = cl.Cshock * rmax(FR.sen.p[ol - sl], FR.sen.p[ol]);
    const double rr = rmax(FR.lam.p[ol - sl], FR.lam.p[ol]);
    const DArr Fd = FR.f[f.d];
    const long long of = Fd.off(f.i, f.j, f.k);
    for (int n = 0; n < 5; ++n) {
      const long long on = ou + n * U.ns;
      const double dw = (U.p[on] - U.p[on - s]);
      double fdamp;
      if (f.d < 2) fdamp = U.p[on + s] - 3.0 * U.p[on] + 3.0 * U.p[on - s] - U.p[on - 2 * s];
      else fdamp = U.p[on - s] - 3.0 * U.p[on] + 3.0 * U.p[on - s] - U.p[on - s];
      Fd.p[of + n * Fd.ns] -= (sen * dw - rmax(0.0, cl.Cdamp - sen) * fdamp) * rr;
    }
  }
}

// ---------------------------------------------- viscous face average ----
// src/rhs/CNS_hydro_K.h:254-261 (mass component adds zero and is skipped).
__global__ void __launch_bounds__(256) visc_face_add_kernel(BoxTable tb, FaceTable ft, long long total) {
  if (list_idle(tb)) return;
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < total;
       g += (long long)gridDim.x * blockDim.x) {
    FaceIdx f;
    if (!decode_face(tb, ft, g, f)) continue;
    const BoxRec& R = tb.box[f.b];
    const DArr V = R.vf;
    const long long s = (f.d == 0) ? 1 : (f.d == 1 ? V.js : V.ks);
    const long long ov = V.off(f.i, f.j, f.k);
    const DArr Fd = ft.fr[f.b].f[f.d];
    const long long of = Fd.off(f.i, f.j, f.k);
#pragma unroll
    for (int n = 0; n < 4; ++n) {
      const int c = 4 * f.d + n;
      Fd.p[of + (1 + n) * Fd.ns] = fma(0.5, V.p[ov - s + c * V.ns] + V.p[ov + c * V.ns], Fd.p[of + (1 + n) * Fd.ns]);
    }
  }
}

// --------------------------------------- divergence + stage program ----
// src/tim/CNS_advance.cpp:384-390, then the BLAS-1 program of the stage.
__global__ void __launch_bounds__(256) div_stage_kernel(BoxTable tb, FaceTable ft, int s_in, int s_s1, int s_out,
                                                        DProg prog_in, int rhs_only, long long total) {
  if (list_idle(tb)) return;
  const DProg prog = resolve_prog(prog_in);
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < total;
       g += (long long)gridDim.x * blockDim.x) {
    const int b = find_box_ll(ft.vpre, tb.n, g);
    const BoxRec& R = tb.box[b];
    int i, j, k;
    decode_cell(R, (int)(g - ft.vpre[b]), 0, i, j, k);
    const FaceRec& FR = ft.fr[b];
    const DArr Fx = FR.f[0], Fy = FR.f[1], Fz = FR.f[2];
    const long long ox = Fx.off(i, j, k), oy = Fy.off(i, j, k), oz = Fz.off(i, j, k);
    const DArr Uin = R.slot[s_in], U1 = R.slot[s_s1], Uo = R.slot[s_out];
    const DClosures& cl = tb.cls[R.cl];
    const long long oin = Uin.off(i, j, k);
    for (int n = 0; n < 5; ++n) {
      double ds = R.dxinv[0] * (Fx.p[ox + n * Fx.ns] - Fx.p[ox + 1 + n * Fx.ns]) +
                  R.dxinv[1] * (Fy.p[oy + n * Fy.ns] - Fy.p[oy + Fy.js + n * Fy.ns]) +
                  R.dxinv[2] * (Fz.p[oz + n * Fz.ns] - Fz.p[oz + Fz.ks + n * Fz.ns]);
      if (cl.source) ds = add_source(cl, Uin.p, oin, Uin.ns, n, ds);
      if (rhs_only) {
        Uo(i, j, k, n) = ds;
      } else {
        double reg[3] = {U1(i, j, k, n), Uin(i, j, k, n), ds};
        apply_prog(prog, reg);
        Uo(i, j, k, n) = reg[1];
      }
    }
  }
}

// ------------------------------------------------------------ launchers --
cudaError_t launch_keep_faces_plain(int order, const BoxTable& tb, const FaceTable& ft, long long nfaces[3], int nsm,
                                    cudaStream_t st) {
  const long long tot = nfaces[0] + nfaces[1] + nfaces[2];
  const int grid = grid_for(tot, nsm);
  if (order == 2) keep_faces_plain_kernel<2><<<grid, 256, 0, st>>>(tb, ft, tot);
  else if (order == 4) keep_faces_plain_kernel<4><<<grid, 256, 0, st>>>(tb, ft, tot);
  else keep_faces_plain_kernel<6><<<grid, 256, 0, st>>>(tb, ft, tot);
  return cudaGetLastError();
}

cudaError_t launch_weno_point(const BoxTable& tb, const FaceTable& ft, int s_in, long long ngcells, int nsm,
                              cudaStream_t st) {
  weno_flux_lambda_kernel<<<grid_for(ngcells, nsm), 256, 0, st>>>(tb, ft, s_in, ngcells);
  return cudaGetLastError();
}

cudaError_t launch_weno_faces(const BoxTable& tb, const FaceTable& ft, int s_in, long long nfaces[3], bool ref_order,
                              int nsm, cudaStream_t st) {
  const long long tot = nfaces[0] + nfaces[1] + nfaces[2];
  if (ref_order) weno_face_kernel<true><<<grid_for(tot, nsm), 256, 0, st>>>(tb, ft, s_in, tot);
  else weno_face_kernel<false><<<grid_for(tot, nsm), 256, 0, st>>>(tb, ft, s_in, tot);
  return cudaGetLastError();
}

cudaError_t launch_weno(const BoxTable& tb, const FaceTable& ft, int s_in, long long ngcells, long long nfaces[3],
                        bool ref_order, int nsm, cudaStream_t st) {
  weno_flux_lambda_kernel<<<grid_for(ngcells, nsm), 256, 0, st>>>(tb, ft, s_in, ngcells);
  launch_weno_faces(tb, ft, s_in, nfaces, ref_order, nsm, st);
  return cudaGetLastError();
}

cudaError_t launch_slopes(const BoxTable& tb, const FaceTable& ft, const long long* spre_d[3], long long nslope[3],
                          int nsm, cudaStream_t st) {
  const long long ts = nslope[0] + nslope[1] + nslope[2];
  slope_kernel<<<grid_for(ts, nsm), 256, 0, st>>>(tb, ft, spre_d[0], spre_d[1], spre_d[2], nslope[0], nslope[1],
                                                  nslope[2]);
  return cudaGetLastError();
}

cudaError_t launch_riemann(const BoxTable& tb, const FaceTable& ft, const long long* spre_d[3], long long nslope[3],
                           long long nfaces[3], int nsm, cudaStream_t st) {
  const long long ts = nslope[0] + nslope[1] + nslope[2];
  slope_kernel<<<grid_for(ts, nsm), 256, 0, st>>>(tb, ft, spre_d[0], spre_d[1], spre_d[2], nslope[0], nslope[1],
                                                  nslope[2]);
  const long long tot = nfaces[0] + nfaces[1] + nfaces[2];
  riemann_face_kernel<<<grid_for(tot, nsm), 256, 0, st>>>(tb, ft, tot);
  return cudaGetLastError();
}

cudaError_t launch_weno_riemann(const BoxTable& tb, const FaceTable& ft, long long nfaces[3], int nsm,
                                cudaStream_t st) {
  const long long tot = nfaces[0] + nfaces[1] + nfaces[2];
  weno_riemann_face_kernel<<<grid_for(tot, nsm), 256, 0, st>>>(tb, ft, tot);
  return cudaGetLastError();
}

cudaError_t launch_jst_sensor(const BoxTable& tb, const FaceTable& ft, long long nvalid, int nsm, cudaStream_t st) {
  jst_sensor_kernel<<<grid_for(nvalid, nsm), 256, 0, st>>>(tb, ft, nvalid);
  return cudaGetLastError();
}

cudaError_t launch_jst(const BoxTable& tb, const FaceTable& ft, int s_in, long long ngcells, long long nvalid,
                       long long nfaces[3], int nsm, cudaStream_t st) {
  (void)ngcells;
  jst_sensor_kernel<<<grid_for(nvalid, nsm), 256, 0, st>>>(tb, ft, nvalid);
  const long long tot = nfaces[0] + nfaces[1] + nfaces[2];
  jst_face_kernel<<<grid_for(tot, nsm), 256, 0, st>>>(tb, ft, s_in, tot);
  return cudaGetLastError();
}

cudaError_t launch_visc_face_add(const BoxTable& tb, const FaceTable& ft, long long nfaces[3], int nsm,
                                 cudaStream_t st) {
  const long long tot = nfaces[0] + nfaces[1] + nfaces[2];
  visc_face_add_kernel<<<grid_for(tot, nsm), 256, 0, st>>>(tb, ft, tot);
  return cudaGetLastError();
}

cudaError_t launch_div_stage(const BoxTable& tb, const FaceTable& ft, int s_in, int s_s1, int s_out,
                             const DProg& prog, int rhs_only, long long nvalid, int nsm, cudaStream_t st) {
  div_stage_kernel<<<grid_for(nvalid, nsm), 256, 0, st>>>(tb, ft, s_in, s_s1, s_out, prog, rhs_only, nvalid);
  return cudaGetLastError();
}

}  // namespace amrs
