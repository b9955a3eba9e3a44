// Pieces shared by the reverse-mode kernels.
#pragma once
#include "amrs_boxes.cuh"

namespace amrs {

constexpr int NQA = 6;  // primitive cotangents: rho, u, v, w, T, p (e = cv*T folded into T)

// Reverse of cons2prim (src/rhs/CNS_hydro_K.h:15-34) at cell (i,j,k) of box R:
// given the primitive cotangents qb (NQA order), the cotangents of the
// conserved state U = R.slot[0] there.  max(1e-40, rho) passes the density
// cotangent only where rho > 1e-40 (the forward's branch).
__device__ __forceinline__ void cons2prim_vjp(const BoxRec& R, const DClosures& cl, int i, int j, int k,
                                              const double qb[NQA], double ub5[5]) {
  const DArr Q = R.q;
  const long long oq = Q.off(i, j, k);
  const double rho = Q.p[oq + QRHO * Q.ns], u = Q.p[oq + QU * Q.ns], v = Q.p[oq + QV * Q.ns],
               w = Q.p[oq + QW * Q.ns], T = Q.p[oq + QT * Q.ns];
  double rb = qb[QRHO], ub = qb[QU], vb = qb[QV], wb = qb[QW];
  const double pb = qb[QPRES] + ddiv_rn(qb[QT], (rho * cl.Rspec));
  rb += ddiv_rn(-qb[QT] * T, rho);
  const double eib = (cl.gamma - 1.0) * pb;  // d/d rhoei
  const double keb = -eib;                   // d/d rhoke
  rb += 0.5 * (u * u + v * v + w * w) * keb;
  ub += rho * u * keb;
  vb += rho * v * keb;
  wb += rho * w * keb;
  const double rinv = ddiv_rn(1.0, rho);
  rb += -(ub * u + vb * v + wb * w) * rinv;
  const DArr U = R.slot[0];
  const double rho_raw = U(i, j, k, URHO);
  ub5[0] = (rho_raw > 1e-40) ? rb : 0.0;
  ub5[1] = ub * rinv;
  ub5[2] = vb * rinv;
  ub5[3] = wb * rinv;
  ub5[4] = eib;
}

// Gradient (and, through Wout, the value) of weno5js (src/rhs/High_resolution.h:124-159):
//   W = sum_k w_k v_k / 6,  w_k = a_k / A,  a_k = c_k / e_k^2,  e_k = beta_k + eps
//   dW/ds = sum_k (w_k/6) grad v_k + sum_k ebar_k grad beta_k,
//   ebar_k = -2 w_k (v_k/6 - W) / e_k.
// With q_k the product of the other two e's, P = e0 e1 e2 and
// D = sum_k c_k q_k^2: w_k = c_k q_k^2 / D and w_k / e_k = c_k q_k^3 / (D P),
// so one division 1/(D P) serves the weights and the e_k quotients (D P ~ e^7
// stays in range for e in [1e-40, 1e40]; outside it the four-division form).
// Standalone products (those no add consumes, so contraction leaves them as
// FP64 multiplies) may go to the integer pipe (kmul), by bit of
// AMRS_WGRAD_IMUL: 0 g^2 and the q_k, 1 the c_k q_k^2, 2 e0 q0, D P and r P,
// 3 the weights and w_k / e_k, 4 the v_k scalings, 5 the ebar_k, 6 the
// beta-gradient terms, 7 the w_k / 6.
#ifndef AMRS_WGRAD_IMUL
#define AMRS_WGRAD_IMUL 0xD0
#endif
template <int M = AMRS_WGRAD_IMUL>
__device__ __forceinline__ void weno5js_grad(const double s[5], double gr[5], double* Wout = nullptr) {
  constexpr bool M0 = M & 1, M1 = (M >> 1) & 1, M2 = (M >> 2) & 1, M3 = (M >> 3) & 1, M4 = (M >> 4) & 1,
                 M5 = (M >> 5) & 1, M6 = (M >> 6) & 1, M7 = (M >> 7) & 1;
  constexpr double eps = 1e-40;
  const double d1 = s[0] - 2.0 * s[1] + s[2], d2 = s[0] - 4.0 * s[1] + 3.0 * s[2];
  const double d3 = s[1] - 2.0 * s[2] + s[3], g = s[1] - s[3];
  const double d4 = s[2] - 2.0 * s[3] + s[4], d5 = 3.0 * s[2] - 4.0 * s[3] + s[4];
  const double g2 = kmul<M0>(g, g);
  const double b0 = (13.0 / 12.0) * d1 * d1 + 0.25 * d2 * d2;
  const double b1 = (13.0 / 12.0) * d3 * d3 + 0.25 * g2 * g2;
  const double b2 = (13.0 / 12.0) * d4 * d4 + 0.25 * d5 * d5;
  const double e0 = eps + b0, e1 = eps + b1, e2 = eps + b2;
  const double q0 = kmul<M0>(e1, e2), q1 = kmul<M0>(e0, e2), q2 = kmul<M0>(e0, e1);
  const double t0 = kmul<M1>(kmul<M1>(0.1, q0), q0), t1 = kmul<M1>(kmul<M1>(0.6, q1), q1),
               t2 = kmul<M1>(kmul<M1>(0.3, q2), q2);
  const double eq = kmul<M2>(e0, q0);
  const double DP = kmul<M2>(t0 + t1 + t2, eq);
  double w0, w1, w2, we0, we1, we2;  // w_k and w_k / e_k
  if (DP > 1e-300 && DP < 1e300) {
    const double r = ddiv_rn(1.0, DP), rP = kmul<M2>(r, eq);
    w0 = kmul<M3>(t0, rP); w1 = kmul<M3>(t1, rP); w2 = kmul<M3>(t2, rP);
    we0 = kmul<M3>(kmul<M3>(t0, q0), r); we1 = kmul<M3>(kmul<M3>(t1, q1), r); we2 = kmul<M3>(kmul<M3>(t2, q2), r);
  } else {
    const double ie0 = ddiv_rn(1.0, e0), ie1 = ddiv_rn(1.0, e1), ie2 = ddiv_rn(1.0, e2);
    const double a0 = 0.1 * ie0 * ie0, a1 = 0.6 * ie1 * ie1, a2 = 0.3 * ie2 * ie2;
    const double iA = ddiv_rn(1.0, (a0 + a1 + a2));
    w0 = a0 * iA; w1 = a1 * iA; w2 = a2 * iA;
    we0 = w0 * ie0; we1 = w1 * ie1; we2 = w2 * ie2;
  }
  const double v0 = kmul<M4>(2.0 * s[0] - 7.0 * s[1] + 11.0 * s[2], 1.0 / 6.0);
  const double v1 = kmul<M4>(-s[1] + 5.0 * s[2] + 2.0 * s[3], 1.0 / 6.0);
  const double v2 = kmul<M4>(2.0 * s[2] + 5.0 * s[3] - s[4], 1.0 / 6.0);
  const double W = w0 * v0 + w1 * v1 + w2 * v2;
  if (Wout) *Wout = W;
  const double eb0 = kmul<M5>(-2.0 * (v0 - W), we0);
  const double eb1 = kmul<M5>(-2.0 * (v1 - W), we1);
  const double eb2 = kmul<M5>(-2.0 * (v2 - W), we2);
  // grad beta_k scaled by ebar_k
  const double p1 = kmul<M6>(kmul<M6>(eb0, 13.0 / 6.0), d1), p2 = kmul<M6>(eb0 * 0.5, d2);
  const double p3 = kmul<M6>(kmul<M6>(eb1, 13.0 / 6.0), d3), p4 = kmul<M6>(kmul<M6>(eb1, g2), g);
  const double p5 = kmul<M6>(kmul<M6>(eb2, 13.0 / 6.0), d4), p6 = kmul<M6>(eb2 * 0.5, d5);
  const double x0 = kmul<M7>(w0, 1.0 / 6.0), x1 = kmul<M7>(w1, 1.0 / 6.0), x2 = kmul<M7>(w2, 1.0 / 6.0);
  gr[0] = 2.0 * x0 + p1 + p2;
  gr[1] = -7.0 * x0 - x1 - 2.0 * p1 - 4.0 * p2 + p3 + p4;
  gr[2] = 11.0 * x0 + 5.0 * x1 + 2.0 * x2 + p1 + 3.0 * p2 - 2.0 * p3 + p5 + 3.0 * p6;
  gr[3] = 2.0 * x1 + 5.0 * x2 + p3 - p4 - 2.0 * p5 - 4.0 * p6;
  gr[4] = -x2 + p5 + p6;
}

}  // namespace amrs
