// Device-side types and point functions of the compressible RHS path.
//
// Every function keeps the floating-point operation order of the reference
// function it cites, and the forward translation units are compiled with
// -fmad=false, so results are bit-identical to the reference's CPU build
// (the reverse-mode units, which recompute linearisation points with these
// functions, allow contraction).
// Explicit fma() appears only where one multiplicand is a power of two
// (exact product), which rounds identically to the separate mul + add.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "ddiv.cuh"

namespace amrs {

constexpr int URHO = 0, UMX = 1, UMY = 2, UMZ = 3, UET = 4, NCONS = 5;
// primitive components; QE = cv*T, stored so KEEP reads it instead of recomputing
constexpr int QRHO = 0, QU = 1, QV = 2, QW = 3, QT = 4, QPRES = 5, QE = 6, NQ = 7;
constexpr int NGHOST = 3;
constexpr int NVF = 12;  // viscous cell fluxes: x,y,z directions x (UMX..UET)
// MUSCL face-state terms per cell and direction (see slope_kernel): the
// Riemann faces' L/R extrapolations read them instead of the raw slopes
constexpr int SL_A = 0, SL_B = 1, SL_C = 2, SL_T1 = 3, SL_T2 = 4, SL_AL = 5, SL_CL = 6, NSLOPE = 7;

// Array4-like view (amrex::Array4<Real>).
struct DArr {
  double* p;
  long long js, ks, ns;
  int b0, b1, b2;
  __host__ __device__ __forceinline__ double& operator()(int i, int j, int k, int n = 0) const {
    return p[(long long)(i - b0) + (long long)(j - b1) * js + (long long)(k - b2) * ks + (long long)n * ns];
  }
  __host__ __device__ __forceinline__ long long off(int i, int j, int k) const {
    return (long long)(i - b0) + (long long)(j - b1) * js + (long long)(k - b2) * ks;
  }
};

// Closures on the device (src/cls/Closures.h:72-182).
struct DClosures {
  double gamma, cv, cp, Rspec;
  int visc_law, cond_law;
  double visc_ref, Tvisc_ref, cond_ref, Tcond_ref;
  double Cshock, Cdamp;
  int source;       // cns.rhs_source with a body force
  double force[3];  // body force per unit mass
};

// compute_rhs's source step (src/tim/CNS_advance.cpp:396-407) with the
// channel problem's user_source (exm/Channel/prob.h:189-193: rhs(UMX) +=
// rho fx, rhs(UET) += m_x fx) for a body force f per unit mass: component n
// of the cell's RHS `ds` gets rho f_d (n = UMX+d) or the m_d f_d in x, y, z
// order (n = UET), for every d with f_d != 0.  U at offset o: the stage input.
__device__ __forceinline__ double add_source(const DClosures& c, const double* U, long long o, long long ns, int n,
                                             double ds) {
  if (n == UET) {
#pragma unroll
    for (int d = 0; d < 3; ++d)
      if (c.force[d] != 0.0) ds = ds + U[o + (UMX + d) * ns] * c.force[d];
  } else if (n != URHO) {
    const double f = c.force[n - UMX];
    if (f != 0.0) ds = ds + U[o + URHO * ns] * f;
  }
  return ds;
}

// visc_const_t::visc / visc_suth_t::visc (src/cls/Closures.h:103-120)
__device__ __forceinline__ double visc(const DClosures& c, double T) {
  if (c.visc_law == 0) return c.visc_ref;
  return ddiv_rn(c.visc_ref * T * dsqrt_rn(T), c.Tvisc_ref + T);
}
// cond_const_t::cond / cond_suth_t::cond (src/cls/Closures.h:130-166)
__device__ __forceinline__ double cond(const DClosures& c, double T) {
  if (c.cond_law == 0) return c.cond_ref;
  return ddiv_rn(c.cond_ref * T * dsqrt_rn(T), c.Tcond_ref + T);
}

// std::max / std::min semantics
__device__ __forceinline__ double rmax(double a, double b) { return (a < b) ? b : a; }
__device__ __forceinline__ double rmin(double a, double b) { return (b < a) ? b : a; }

// A product on the FP64 pipe (a * b) or, with I, the same correctly rounded
// product formed on the integer pipe (dmul_rn).  The kernels of this path
// are bound by the FP64 pipe while their integer pipe idles; the masks below
// (one per routine, chosen by measurement) move part of their products
// across without changing a bit of any result.
template <bool I>
__device__ __forceinline__ double kmul(double a, double b) {
  return I ? dmul_rn(a, b) : a * b;
}

// cons2prim products on the integer pipe: bit 0 the velocities, 1 their
// squares, 2 the kinetic-energy scalings, 3 pressure, rho R and e.
#ifndef AMRS_C2P_IMUL
#define AMRS_C2P_IMUL 0x02
#endif
// Viscous cell-flux products on the integer pipe (see viscous_cell_dy).
#ifndef AMRS_VISC_IMUL
#define AMRS_VISC_IMUL 0x17
#endif

// cons2prim (src/rhs/CNS_hydro_K.h:15-34) plus QE = cv*T.
__device__ __forceinline__ void cons2prim(const double u[5], double q[NQ], const DClosures& c) {
  double rho = rmax(1e-40, u[URHO]);
  constexpr int M = AMRS_C2P_IMUL;
  double rhoinv = ddiv_rn(1.0, rho);
  double ux = kmul<M & 1>(u[UMX], rhoinv);
  double uy = kmul<M & 1>(u[UMY], rhoinv);
  double uz = kmul<M & 1>(u[UMZ], rhoinv);
  double rhoke = kmul<(M >> 2) & 1>(kmul<(M >> 2) & 1>(0.5, rho),
                                    kmul<(M >> 1) & 1>(ux, ux) + kmul<(M >> 1) & 1>(uy, uy) +
                                        kmul<(M >> 1) & 1>(uz, uz));
  double rhoei = (u[UET] - rhoke);
  double p = kmul<(M >> 3) & 1>(c.gamma - 1.0, rhoei);
  q[QRHO] = rho;
  q[QU] = ux;
  q[QV] = uy;
  q[QW] = uz;
  q[QPRES] = p;
  q[QT] = ddiv_rn(p, kmul<(M >> 3) & 1>(rho, c.Rspec));
  q[QE] = kmul<(M >> 3) & 1>(c.cv, q[QT]);
}

// One KEEP pair term (src/rhs/CentralKEEP.h:19-36 helpers, :76-83 body),
// already multiplied by its coefficient: the contribution of pair
// (point 1 = larger index, point 2 = smaller index) to the face flux in
// direction d.  q1/q2 give rho,u,v,w,T,p,e.
//
// IM selects, bit by bit, the products formed on the integer pipe
// (dmul_rn, the same correctly rounded product): 0 P, 1-3 the three
// products of s3, 4-7 the momentum and energy cubic products, 8-9 the two
// products of pu, 10-14 the coefficient scalings of the five components,
// 15 P s3.  The FP64 pipe is the bound of the kernels calling this, and the
// integer pipe is otherwise idle in them, so moving part of the products
// there shortens the FP64 stream without changing a bit of the result.
#ifndef AMRS_KEEP_IMUL
#define AMRS_KEEP_IMUL 0x7C00
#endif
template <int D, int IM = AMRS_KEEP_IMUL>
__device__ __forceinline__ void keep_pair(const double* q1, const double* q2, double coef, double T[5]) {
  constexpr int QN = QU + D;
  const double rhoS = q1[QRHO] + q2[QRHO];
  const double unS = q1[QN] + q2[QN];
  // Binary scalings commute with rounding (normal range), so every power of
  // two in the reference's expressions moves into the pair's constant
  // coefficient, to the bit:
  //   fghCubic: 0.125*rhoS*unS*h == 0.125*(P*h), P = rhoS*unS;
  //   fgQuad massflx 0.25*rhoS*unS == 0.25*P, and massflx*ke with
  //   ke = 0.5*(u1u2+v1v2+w1w2) == 0.125*(P*s3);
  //   fDiv 0.5*(p1+p2) and fgDiv 0.5*(p1*un2+p2*un1) added to an eighth:
  //   x/8 + s/2 == (x + 4s)/8 == fma(4, s, x)/8.
  // So coef*(...) == (coef/8)*(...) with the eighths taken out, and no
  // FP64 instruction is spent on a power-of-two scaling.
  const double c8 = 0.125 * coef, c4 = 0.25 * coef;
  const double P = kmul<(IM >> 0) & 1>(rhoS, unS);
  const double s3 = kmul<(IM >> 1) & 1>(q1[QU], q2[QU]) + kmul<(IM >> 2) & 1>(q1[QV], q2[QV]) +
                    kmul<(IM >> 3) & 1>(q1[QW], q2[QW]);
  const double cx = kmul<(IM >> 4) & 1>(P, q1[QU] + q2[QU]);
  const double cy = kmul<(IM >> 5) & 1>(P, q1[QV] + q2[QV]);
  const double cz = kmul<(IM >> 6) & 1>(P, q1[QW] + q2[QW]);
  const double ce = kmul<(IM >> 7) & 1>(P, q1[QE] + q2[QE]);
  const double psum = q1[QPRES] + q2[QPRES];
  const double pu = kmul<(IM >> 8) & 1>(q1[QPRES], q2[QN]) + kmul<(IM >> 9) & 1>(q2[QPRES], q1[QN]);
  T[URHO] = kmul<(IM >> 10) & 1>(c4, P);
  T[UMX] = kmul<(IM >> 11) & 1>(c8, D == 0 ? fma(4.0, psum, cx) : cx);
  T[UMY] = kmul<(IM >> 12) & 1>(c8, D == 1 ? fma(4.0, psum, cy) : cy);
  T[UMZ] = kmul<(IM >> 13) & 1>(c8, D == 2 ? fma(4.0, psum, cz) : cz);
  T[UET] = kmul<(IM >> 14) & 1>(c8, fma(4.0, pu, kmul<(IM >> 15) & 1>(P, s3) + ce));
}

// Cell-centred viscous fluxes (src/rhs/CNS_hydro_K.h:108-172) from the
// primitive values at the cell and its six neighbours.  Output: x, y, z
// blocks of (UMX..UET); the mass entries are zero in the reference.
// `qc` centre, `qxm/qxp`, `qym/qyp`, `qzm/qzp` neighbours (u,v,w,T read).
// The same with the four y derivatives (u, v, w, T) given: the body shared
// by the interior form and the wall rows' one-sided form.
__device__ __forceinline__ void viscous_cell_dy(const double* qc, const double* qxm, const double* qxp,
                                                const double dy[4], const double* qzm, const double* qzp,
                                                const double dxinv[3], const DClosures& c, double f[NVF]) {
  // (a-b)*0.5*dxinv == (a-b)*(0.5*dxinv) exactly: the 0.5 scalings are exact.
  // Products on the integer pipe (AMRS_VISC_IMUL): bit 0 the x derivative
  // scalings, 1 the y ones (formed by viscous_cell), 2 the z ones, 3 the
  // r1_3*div terms, 4 the stress scalings by mu, 5 the energy-flux products.
  constexpr int M = AMRS_VISC_IMUL;
  const double hx = 0.5 * dxinv[0], hz = 0.5 * dxinv[2];
  const double ux = qc[QU];
  const double dudx = kmul<M & 1>(qxp[QU] - qxm[QU], hx);
  const double dvdx = kmul<M & 1>(qxp[QV] - qxm[QV], hx);
  const double dwdx = kmul<M & 1>(qxp[QW] - qxm[QW], hx);
  const double dTdx = kmul<M & 1>(qxp[QT] - qxm[QT], hx);
  const double uy = qc[QV];
  const double dudy = dy[0], dvdy = dy[1], dwdy = dy[2], dTdy = dy[3];
  const double uz = qc[QW];
  const double dudz = kmul<(M >> 2) & 1>(qzp[QU] - qzm[QU], hz);
  const double dvdz = kmul<(M >> 2) & 1>(qzp[QV] - qzm[QV], hz);
  const double dwdz = kmul<(M >> 2) & 1>(qzp[QW] - qzm[QW], hz);
  const double dTdz = kmul<(M >> 2) & 1>(qzp[QT] - qzm[QT], hz);
  const double div = dudx + dvdy + dwdz;
  const double mu = visc(c, qc[QT]);
  const double lambda = cond(c, qc[QT]);
  const double r1_3 = 1.0 / 3.0;
  // The fluxes are stored negated (-tau, -lambda dT - tau.u).  Negation is
  // exact, so (-2mu)*d == -(2mu*d) and a + (-t)*u == a - t*u to the bit:
  // the negated stresses n.. are formed directly and the sums add them,
  // with no separate negations.
  constexpr bool MD = (M >> 3) & 1, MS = (M >> 4) & 1, ME = (M >> 5) & 1;
  const double nmu = -mu, nmu2 = -2.0 * mu, nlam = -lambda;
  const double nxx = kmul<MS>(nmu2, dudx - kmul<MD>(r1_3, div));
  const double nxy = kmul<MS>(nmu, dudy + dvdx);
  const double nxz = kmul<MS>(nmu, dudz + dwdx);
  const double nyy = kmul<MS>(nmu2, dvdy - kmul<MD>(r1_3, div));
  const double nyz = kmul<MS>(nmu, dvdz + dwdy);
  const double nzz = kmul<MS>(nmu2, dwdz - kmul<MD>(r1_3, div));
  f[0] = nxx;
  f[1] = nxy;
  f[2] = nxz;
  f[3] = kmul<ME>(nlam, dTdx) + kmul<ME>(nxx, ux) + kmul<ME>(nxy, uy) + kmul<ME>(nxz, uz);
  f[4] = nxy;
  f[5] = nyy;
  f[6] = nyz;
  f[7] = kmul<ME>(nlam, dTdy) + kmul<ME>(nxy, ux) + kmul<ME>(nyy, uy) + kmul<ME>(nyz, uz);
  f[8] = nxz;
  f[9] = nyz;
  f[10] = nzz;
  f[11] = kmul<ME>(nlam, dTdz) + kmul<ME>(nxz, ux) + kmul<ME>(nyz, uy) + kmul<ME>(nzz, uz);
}

__device__ __forceinline__ void viscous_cell(const double* qc, const double* qxm, const double* qxp,
                                             const double* qym, const double* qyp, const double* qzm,
                                             const double* qzp, const double dxinv[3], const DClosures& c,
                                             double f[NVF]) {
  constexpr bool MY = (AMRS_VISC_IMUL >> 1) & 1;
  const double hy = 0.5 * dxinv[1];
  const double dy[4] = {kmul<MY>(qyp[QU] - qym[QU], hy), kmul<MY>(qyp[QV] - qym[QV], hy),
                        kmul<MY>(qyp[QW] - qym[QW], hy), kmul<MY>(qyp[QT] - qym[QT], hy)};
  viscous_cell_dy(qc, qxm, qxp, dy, qzm, qzp, dxinv, c, f);
}

// ViscousWallFluxes (src/rhs/CNS_hydro_K.h:177-251): the cell viscous fluxes
// of the ghost row next to a y wall with second-order one-sided y
// derivatives; loc 0 (lower wall) reads rows j, j+1, j+2 as (q0, q1, q2),
// loc 1 (upper wall) rows j, j-1, j-2.  -a + 4b and 3c - 4b are single fmas
// (the factor 4 is exact).
__device__ __forceinline__ void viscous_wall_cell(int loc, const double* qc, const double* qxm, const double* qxp,
                                                  const double* q1, const double* q2, const double* qzm,
                                                  const double* qzp, const double dxinv[3], const DClosures& c,
                                                  double f[NVF]) {
  const double hy = 0.5 * dxinv[1];
  double dy[4];
#pragma unroll
  for (int n = 0; n < 4; ++n) {
    const int m = QU + n;
    dy[n] = (loc == 0) ? (fma(4.0, q1[m], -q2[m]) - 3.0 * qc[m]) * hy
                       : (fma(-4.0, q1[m], 3.0 * qc[m]) + q2[m]) * hy;
  }
  viscous_cell_dy(qc, qxm, qxp, dy, qzm, qzp, dxinv, c, f);
}

// RK stage program (AMReX BLAS-1 semantics), registers S1, S2, dS.
// fa/fb: 0 the coefficient is a / b; 1 it is dt * a / dt * b; 2 it is
// dt / a / dt / b, with dt read from device memory (dtp) when the kernel
// starts: the device-resident time loop changes dt without new launches.
struct DOp {
  int kind, dst, x, y;
  double a, b;
  int fa, fb;
};
struct DProg {
  int nops;
  DOp ops[3];
  const double* dtp;
};

__device__ __forceinline__ double dt_coef(int form, double c, double dt) {
  return form == 1 ? dt * c : (form == 2 ? dt / c : c);
}
// The program with its dt-dependent coefficients evaluated (dt * c and
// dt / c round exactly as the host's CNS::advance arithmetic).
__device__ __forceinline__ DProg resolve_prog(DProg p) {
  if (p.dtp) {
    const double dt = *p.dtp;
#pragma unroll
    for (int o = 0; o < 3; ++o) {
      p.ops[o].a = dt_coef(p.ops[o].fa, p.ops[o].a, dt);
      p.ops[o].b = dt_coef(p.ops[o].fb, p.ops[o].b, dt);
    }
  }
  return p;
}

__device__ __forceinline__ void apply_prog(const DProg& p, double reg[3]) {
#pragma unroll
  for (int o = 0; o < 3; ++o) {
    if (o >= p.nops) break;
    const DOp& q = p.ops[o];
    if (q.kind == 0) reg[q.dst] = q.a * reg[q.x] + q.b * reg[q.y];
    else if (q.kind == 1) reg[q.dst] = reg[q.dst] + q.a * reg[q.x];
    else if (q.kind == 2) reg[q.dst] = reg[q.x] + q.a * reg[q.dst];
    else reg[q.dst] = reg[q.x];
  }
}

}  // namespace amrs
