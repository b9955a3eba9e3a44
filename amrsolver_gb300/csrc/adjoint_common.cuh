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
  const double pb = qb[QPRES] + qb[QT] / (rho * cl.Rspec);
  rb += -qb[QT] * T / rho;
  const double eib = (cl.gamma - 1.0) * pb;  // d/d rhoei
  const double keb = -eib;                   // d/d rhoke
  rb += 0.5 * (u * u + v * v + w * w) * keb;
  ub += rho * u * keb;
  vb += rho * v * keb;
  wb += rho * w * keb;
  const double rinv = 1.0 / rho;
  rb += -(ub * u + vb * v + wb * w) * rinv;
  const DArr U = R.slot[0];
  const double rho_raw = U(i, j, k, URHO);
  ub5[0] = (rho_raw > 1e-40) ? rb : 0.0;
  ub5[1] = ub * rinv;
  ub5[2] = vb * rinv;
  ub5[3] = wb * rinv;
  ub5[4] = eib;
}

}  // namespace amrs
