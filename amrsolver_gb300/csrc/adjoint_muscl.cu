// Hand-written adjoint (vector-Jacobian product) of the MUSCL + two-shock
// Riemann Euler flux (src/rhs/Riemann.h:9-408) for one box.
//
// Forward, per direction d (slope_kernel / riemann_face_kernel):
//   per cell c of grow(box,1) along d: characteristic differences of the
//     primitives at c-1, c, c+1, MC-limited to d0..d4, and the face-state
//     terms A = (d0+d2)/cs + d1, B = (d2-d0)/rho, C = (d0+d2)*cs with
//     cs = sqrt(gamma R T(c)) + 1e-40 (z: the left-state terms A_L, C_L use
//     the sound speed of cell c+2, cns_riemann_z's quirk);
//   per face f: left state from cell f-1 (q + terms/2), right state from
//     cell f (q - terms/2), rho and p floored at 1e-40, riemann_prob.
//
// Reverse, one direction at a time (every output element written by one
// thread, fixed summation order: deterministic):
//   muscl_vjp_face_kernel : Fbar = dxinv_d (vbar(f) - vbar(f-1)); the
//       riemann_prob reverse gives the cotangents of the ten state inputs,
//       then of both cells' primitives and face-state terms (20 slots).
//   muscl_vjp_slope_kernel: per cell, the term cotangents of its two faces
//       through A, B, C, the MC limiters and the characteristic differences
//       to primitive cotangents at c-1, c, c+1 (and T at c+2 for z), plus the
//       faces' direct primitive cotangents (19 slots).
// Then muscl_vjp_gather_kernel sums, per cell of grow(box,2), the slots that
// reach it from all three directions and adds the cons2prim reverse of that
// sum to Ubar.  Non-smooth points follow the forward's branch (max, |.|,
// the limiter's cases, the solver's state selection); the iteration's
// branch tests (weak-wave switch) carry no derivative.
#include "adjoint_common.cuh"
#include "amrs_kernels.h"
#include "riemann_vjp.cuh"

namespace amrs {

namespace {

using rpvjp::riemann_prob_vjp;
using rpvjp::sgn1;

constexpr int FSLOT = 20;  // per face: left prims (5), left terms (5), right prims (5), right terms (5)
constexpr int SSLOT = 19;  // per cell: Qbar at c-1 (6), c (6), c+1 (6), T at c+2 (1, z only)

__device__ __forceinline__ double vget0(const DArr& v, const BoxRec& R, int i, int j, int k, int n) {
  if (i < R.lo[0] || i > R.hi[0] || j < R.lo[1] || j > R.hi[1] || k < R.lo[2] || k > R.hi[2]) return 0.0;
  return v(i, j, k, n);
}
// Faces nodal in d over the box: index = (i-lo0) + nx*((j-lo1) + ny*(k-lo2)).
struct FBuf {
  double* p;
  long long nf;
  int nx, ny;
};
// Cells of grow(box,1) along d only: index = (i-lo0+e0) + mx*((j-lo1+e1) + my*(k-lo2+e2)).
struct SBuf {
  double* p;
  long long nc;
  int mx, my;
};

// Resident CTAs per SM asked of the slope and gather reverse kernels.
#ifndef AMRS_MVJP_CTAS
#define AMRS_MVJP_CTAS 4
#endif

// Two CTAs per SM (128 registers): the reverse solver is a long dependent
// chain per face, and 16 warps hide its latency better than 8 with all the
// registers it would otherwise take (measured: 7.97 against 8.97 ms per
// SSPRK3 step VJP at 64^3).
__global__ void __launch_bounds__(256, 2) muscl_vjp_face_kernel(BoxTable tb, FaceRec fr, DArr vbar, FBuf fs, int d,
                                                             long long total) {
  const BoxRec& R = tb.box[0];
  const DArr q = R.q;
  const DArr S = fr.slope[d];
  const DClosures& cl = tb.cls[R.cl];
  const int di = d == 0, dj = d == 1, dk = d == 2;
  const int QN = QU + d, QT1 = (d == 0) ? QV : QU, QT2 = (d == 2) ? QV : QW;
  const int UN = UMX + d, UT1 = (d == 0) ? UMY : UMX, UT2 = (d == 2) ? UMY : UMZ;
  const int cA = (d == 2) ? SL_AL : SL_A, cC = (d == 2) ? SL_CL : SL_C;
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < total;
       g += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(g % fs.nx) + R.lo[0];
    const long long t = g / fs.nx;
    const int j = (int)(t % fs.ny) + R.lo[1], k = (int)(t / fs.ny) + R.lo[2];
    const int im = i - di, jm = j - dj, km = k - dk;
    const long long oq = q.off(i, j, k), oqm = q.off(im, jm, km);
    const long long os = S.off(i, j, k), osm = S.off(im, jm, km);
    auto Q = [&](long long o, int n) { return q.p[o + n * q.ns]; };
    auto D = [&](long long o, int n) { return S.p[o + n * S.ns]; };
    const double xrl = Q(oqm, QRHO) + 0.5 * D(osm, cA), xpl = Q(oqm, QPRES) + 0.5 * D(osm, cC);
    const double xrr = Q(oq, QRHO) - 0.5 * D(os, SL_A), xpr = Q(oq, QPRES) - 0.5 * D(os, SL_C);
    double in[10];
    in[0] = (xrl < 1.0e-40) ? 1.0e-40 : xrl;
    in[1] = Q(oqm, QN) + 0.5 * D(osm, SL_B);
    in[2] = (xpl < 1.0e-40) ? 1.0e-40 : xpl;
    in[3] = Q(oqm, QT1) + 0.5 * D(osm, SL_T1);
    in[4] = Q(oqm, QT2) + 0.5 * D(osm, SL_T2);
    in[5] = (xrr < 1.0e-40) ? 1.0e-40 : xrr;
    in[6] = Q(oq, QN) - 0.5 * D(os, SL_B);
    in[7] = (xpr < 1.0e-40) ? 1.0e-40 : xpr;
    in[8] = Q(oq, QT1) - 0.5 * D(os, SL_T1);
    in[9] = Q(oq, QT2) - 0.5 * D(os, SL_T2);
    const double h = R.dxinv[d];
    double fb[5];
    const int cmp[5] = {URHO, UN, UT1, UT2, UET};
#pragma unroll
    for (int n = 0; n < 5; ++n)
      fb[n] = h * (vget0(vbar, R, i, j, k, cmp[n]) - vget0(vbar, R, im, jm, km, cmp[n]));
    double ib[10];
    riemann_prob_vjp(cl.gamma, 1.0e-40, in, fb, ib);
    const double rlb = (xrl < 1.0e-40) ? 0.0 : ib[0], plb = (xpl < 1.0e-40) ? 0.0 : ib[2];
    const double rrb = (xrr < 1.0e-40) ? 0.0 : ib[5], prb = (xpr < 1.0e-40) ? 0.0 : ib[7];
    double* o = fs.p + g;
    const long long s = fs.nf;
    // left cell: prims (rho, u_n, p, u_t1, u_t2), terms (A, B, C, d3, d4)
    o[0 * s] = rlb; o[1 * s] = ib[1]; o[2 * s] = plb; o[3 * s] = ib[3]; o[4 * s] = ib[4];
    o[5 * s] = 0.5 * rlb; o[6 * s] = 0.5 * ib[1]; o[7 * s] = 0.5 * plb; o[8 * s] = 0.5 * ib[3]; o[9 * s] = 0.5 * ib[4];
    // right cell
    o[10 * s] = rrb; o[11 * s] = ib[6]; o[12 * s] = prb; o[13 * s] = ib[8]; o[14 * s] = ib[9];
    o[15 * s] = -0.5 * rrb; o[16 * s] = -0.5 * ib[6]; o[17 * s] = -0.5 * prb; o[18 * s] = -0.5 * ib[8];
    o[19 * s] = -0.5 * ib[9];
  }
}

// MC limiter (src/rhs/Riemann.h:9-17) and its reverse along the taken case.
__device__ __forceinline__ void mc_vjp(double l, double r, double db, double& lb, double& rb) {
  const double dcen = 0.5 * (l + r);
  const double dsgn = copysign(1.0, dcen);
  const double al = fabs(l), ar = fabs(r);
  const bool rsmall = ar < al;                 // rmin(|l|, |r|) takes |r|
  const double slop = 2.0 * (rsmall ? ar : al);
  const bool same = l * r >= 0.0;
  const double dlim = same ? slop : 0.0;
  const double ac = fabs(dcen);
  const bool take_c = ac < dlim;               // rmin(dlim, |dcen|) takes |dcen|
  if (take_c) {
    // dsgn * |dcen| = dcen
    lb += 0.5 * db;
    rb += 0.5 * db;
  } else if (same) {
    // dsgn * 2 min(|l|, |r|)
    const double sb = dsgn * 2.0 * db;
    if (rsmall) rb += sb * sgn1(r);
    else lb += sb * sgn1(l);
  }
}

__global__ void __launch_bounds__(256, AMRS_MVJP_CTAS) muscl_vjp_slope_kernel(BoxTable tb, FaceRec fr, FBuf fs, SBuf ss, int d,
                                                              long long total) {
  const BoxRec& R = tb.box[0];
  const DArr q = R.q;
  const DClosures& cl = tb.cls[R.cl];
  const int di = d == 0, dj = d == 1, dk = d == 2;
  const int QN = QU + d, QT1 = (d == 0) ? QV : QU, QT2 = (d == 2) ? QV : QW;
  const long long s = (d == 0) ? 1 : (d == 1 ? q.js : q.ks);
  const double gR = cl.gamma * cl.Rspec;
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < total;
       g += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(g % ss.mx) + R.lo[0] - di;
    const long long t = g / ss.mx;
    const int j = (int)(t % ss.my) + R.lo[1] - dj, k = (int)(t / ss.my) + R.lo[2] - dk;
    const int c = (d == 0) ? i : (d == 1 ? j : k);
    const long long o = q.off(i, j, k);
    auto Q = [&](long long off, int n) { return q.p[off + n * q.ns]; };
    // forward recompute (slope_kernel)
    const double c0 = sqrt(gR * Q(o, QT));
    const double cs = c0 + (d == 0 ? 2.e-40 : 1.e-40);
    const double csr = c0 + 1.e-40;
    const double rc = Q(o, QRHO);
    const double dpl = Q(o, QPRES) - Q(o - s, QPRES), dpr = Q(o + s, QPRES) - Q(o, QPRES);
    const double dul = Q(o, QN) - Q(o - s, QN), dur = Q(o + s, QN) - Q(o, QN);
    const double drl = Q(o, QRHO) - Q(o - s, QRHO), drr = Q(o + s, QRHO) - Q(o, QRHO);
    const double d1l = Q(o, QT1) - Q(o - s, QT1), d1r = Q(o + s, QT1) - Q(o, QT1);
    const double d2l = Q(o, QT2) - Q(o - s, QT2), d2r = Q(o + s, QT2) - Q(o, QT2);
    const double cs2 = cs * cs;
    const double l0 = ddiv_rn(0.5 * dpl, cs) - 0.5 * rc * dul, r0 = ddiv_rn(0.5 * dpr, cs) - 0.5 * rc * dur;
    const double l1 = drl - ddiv_rn(dpl, cs2), r1 = drr - ddiv_rn(dpr, cs2);
    const double l2 = ddiv_rn(0.5 * dpl, cs) + 0.5 * rc * dul, r2 = ddiv_rn(0.5 * dpr, cs) + 0.5 * rc * dur;
    auto mc = [](double a, double b) {
      const double dcen = 0.5 * (a + b);
      const double dsgn = copysign(1.0, dcen);
      const double aa = fabs(a), ab = fabs(b);
      const double slop = 2.0 * ((ab < aa) ? ab : aa);
      const double dlim = (a * b >= 0.0) ? slop : 0.0;
      const double ac = fabs(dcen);
      return dsgn * ((ac < dlim) ? ac : dlim);
    };
    const double d0 = mc(l0, r0), d2 = mc(l2, r2);
    const double s02 = d0 + d2;
    // term cotangents from the two faces of this cell
    double Ab = 0.0, Bb = 0.0, Cb = 0.0, d3b = 0.0, d4b = 0.0, ALb = 0.0, CLb = 0.0;
    double qb0[NQA] = {0, 0, 0, 0, 0, 0};  // direct prim cotangents at c
    auto fidx = [&](int fi, int fj, int fk) {
      return (long long)(fi - R.lo[0]) + (long long)fs.nx * ((fj - R.lo[1]) + (long long)fs.ny * (fk - R.lo[2]));
    };
    if (c >= R.lo[d]) {  // right role at face c
      const double* f = fs.p + fidx(i, j, k);
      const long long n = fs.nf;
      qb0[QRHO] += f[10 * n]; qb0[QN] += f[11 * n]; qb0[QPRES] += f[12 * n]; qb0[QT1] += f[13 * n];
      qb0[QT2] += f[14 * n];
      Ab += f[15 * n]; Bb += f[16 * n]; Cb += f[17 * n]; d3b += f[18 * n]; d4b += f[19 * n];
    }
    if (c <= R.hi[d]) {  // left role at face c+1
      const double* f = fs.p + fidx(i + di, j + dj, k + dk);
      const long long n = fs.nf;
      qb0[QRHO] += f[0 * n]; qb0[QN] += f[1 * n]; qb0[QPRES] += f[2 * n]; qb0[QT1] += f[3 * n];
      qb0[QT2] += f[4 * n];
      if (d == 2) { ALb += f[5 * n]; CLb += f[7 * n]; }
      else { Ab += f[5 * n]; Cb += f[7 * n]; }
      Bb += f[6 * n]; d3b += f[8 * n]; d4b += f[9 * n];
    }
    // A = s02/csr + d1, B = (d2 - d0)/rho, C = s02*csr (z: A_L, C_L with csl).
    // The cotangents use reciprocals: the reverse pass has no bit-exact
    // counterpart (its bar is agreement with forward-mode derivatives), and
    // four divisions serve the sixteen quotients below.
    const double icsr = ddiv_rn(1.0, csr), irc = ddiv_rn(1.0, rc), ics = ddiv_rn(1.0, cs);
    const double ics2 = ics * ics;
    double s02b = Ab * icsr + Cb * csr;
    double csrb = -Ab * (s02 * icsr) * icsr + Cb * s02;
    double d1b = Ab + ALb;
    double d0b = -Bb * irc, d2b = Bb * irc;
    double rcb = -Bb * ((d2 - d0) * irc) * irc;
    double csl = 0.0, c0l = 0.0, cslb = 0.0;
    if (d == 2 && c <= R.hi[2]) {
      c0l = sqrt(gR * Q(o + 2 * s, QT));
      csl = c0l + 1.e-40;
      const double icsl = ddiv_rn(1.0, csl);
      s02b += ALb * icsl + CLb * csl;
      cslb = -ALb * (s02 * icsl) * icsl + CLb * s02;
    }
    d0b += s02b;
    d2b += s02b;
    // limiters
    double l0b = 0.0, r0b = 0.0, l1b = 0.0, r1b = 0.0, l2b = 0.0, r2b = 0.0, l3b = 0.0, r3b = 0.0, l4b = 0.0,
           r4b = 0.0;
    mc_vjp(l0, r0, d0b, l0b, r0b);
    mc_vjp(l1, r1, d1b, l1b, r1b);
    mc_vjp(l2, r2, d2b, l2b, r2b);
    mc_vjp(d1l, d1r, d3b, l3b, r3b);
    mc_vjp(d2l, d2r, d4b, l4b, r4b);
    // characteristic differences
    double csb = 0.0;
    double dplb = 0.5 * (l0b + l2b) * ics - l1b * ics2, dprb = 0.5 * (r0b + r2b) * ics - r1b * ics2;
    csb += (-0.5 * (l0b + l2b) * dpl - 0.5 * (r0b + r2b) * dpr) * ics2;
    csb += 2.0 * (l1b * dpl + r1b * dpr) * (ics2 * ics);
    const double dulb = 0.5 * rc * (l2b - l0b), durb = 0.5 * rc * (r2b - r0b);
    rcb += 0.5 * ((l2b - l0b) * dul + (r2b - r0b) * dur);
    const double drlb = l1b, drrb = r1b;
    // c0 = sqrt(gamma R T)
    const double c0b = csb + csrb;
    double Tb = (c0 > 0.0) ? ddiv_rn(c0b * gR, (2.0 * c0)) : 0.0;
    // Qbar at c-1 (m), c (z), c+1 (p), NQA order (rho, u, v, w, T, p)
    double qm[NQA] = {0, 0, 0, 0, 0, 0}, qz[NQA], qp[NQA] = {0, 0, 0, 0, 0, 0};
#pragma unroll
    for (int n = 0; n < NQA; ++n) qz[n] = qb0[n];
    qz[QPRES] += dplb - dprb; qm[QPRES] -= dplb; qp[QPRES] += dprb;
    qz[QN] += dulb - durb; qm[QN] -= dulb; qp[QN] += durb;
    qz[QRHO] += drlb - drrb + rcb; qm[QRHO] -= drlb; qp[QRHO] += drrb;
    qz[QT1] += l3b - r3b; qm[QT1] -= l3b; qp[QT1] += r3b;
    qz[QT2] += l4b - r4b; qm[QT2] -= l4b; qp[QT2] += r4b;
    qz[QT] += Tb;
    double* w = ss.p + g;
    const long long n = ss.nc;
#pragma unroll
    for (int m = 0; m < NQA; ++m) {
      w[m * n] = qm[m];
      w[(NQA + m) * n] = qz[m];
      w[(2 * NQA + m) * n] = qp[m];
    }
    w[(3 * NQA) * n] = (d == 2 && c <= R.hi[2] && c0l > 0.0) ? ddiv_rn(cslb * gR, (2.0 * c0l)) : 0.0;
  }
}

__global__ void __launch_bounds__(256, AMRS_MVJP_CTAS) muscl_vjp_gather_kernel(BoxTable tb, DArr ubar, SBuf s0, SBuf s1, SBuf s2,
                                                               long long total) {
  const BoxRec& R = tb.box[0];
  const DClosures& cl = tb.cls[R.cl];
  const int nx = R.hi[0] - R.lo[0] + 5, ny = R.hi[1] - R.lo[1] + 5;
  const SBuf sb[3] = {s0, s1, s2};
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < total;
       g += (long long)gridDim.x * blockDim.x) {
    const int c[3] = {(int)(g % nx) + R.lo[0] - 2, (int)((g / nx) % ny) + R.lo[1] - 2,
                      (int)(g / ((long long)nx * ny)) + R.lo[2] - 2};
    double qb[NQA] = {0, 0, 0, 0, 0, 0};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const SBuf& S = sb[d];
      // the slope cell x reaches this cell with offset (c - x) along d
      auto in_region = [&](const int x[3]) {
        for (int a = 0; a < 3; ++a) {
          const int lo = R.lo[a] - (a == d), hi = R.hi[a] + (a == d);
          if (x[a] < lo || x[a] > hi) return false;
        }
        return true;
      };
      auto sidx = [&](const int x[3]) {
        return (long long)(x[0] - R.lo[0] + (d == 0)) +
               (long long)S.mx * ((x[1] - R.lo[1] + (d == 1)) + (long long)S.my * (x[2] - R.lo[2] + (d == 2)));
      };
#pragma unroll
      for (int off = -1; off <= 1; ++off) {
        int x[3] = {c[0], c[1], c[2]};
        x[d] -= off;  // this cell is x + off
        if (!in_region(x)) continue;
        const double* p = S.p + sidx(x);
        const int base = (off + 1) * NQA;
#pragma unroll
        for (int n = 0; n < NQA; ++n) qb[n] += p[(base + n) * S.nc];
      }
      if (d == 2) {
        int x[3] = {c[0], c[1], c[2] - 2};
        if (in_region(x)) qb[QT] += S.p[sidx(x) + (3 * NQA) * S.nc];
      }
    }
    double ub[5];
    cons2prim_vjp(R, cl, c[0], c[1], c[2], qb, ub);
    const long long ou = ubar.off(c[0], c[1], c[2]);
#pragma unroll
    for (int n = 0; n < 5; ++n) ubar.p[ou + n * ubar.ns] += ub[n];
  }
}

int grid_m(long long n, int nsm) {
  long long b = (n + 255) / 256;
  const long long cap = (long long)nsm * 8;
  return (int)(b < 1 ? 1 : (b < cap ? b : cap));
}

long long slope_cells(const int n[3], int d) {
  return (long long)(n[0] + 2 * (d == 0)) * (n[1] + 2 * (d == 1)) * (n[2] + 2 * (d == 2));
}
long long face_count(const int n[3], int d) {
  return (long long)(n[0] + (d == 0)) * (n[1] + (d == 1)) * (n[2] + (d == 2));
}

}  // namespace

size_t muscl_vjp_buffer_bytes(const int n[3]) {
  long long mf = 0, sc = 0;
  for (int d = 0; d < 3; ++d) {
    mf = face_count(n, d) > mf ? face_count(n, d) : mf;
    sc += slope_cells(n, d);
  }
  return (size_t)(mf * FSLOT + sc * SSLOT) * sizeof(double);
}

// Adds the MUSCL-Riemann Euler part of the RHS VJP to ubar (which the
// viscous / cons2prim reverse pass has already written).  Q and the slope
// terms of the state must be current (launch_prims, launch_slopes).
cudaError_t launch_muscl_vjp(const BoxTable& tb, const FaceRec& fr, const DArr& vbar, const DArr& ubar, double* buf,
                             const int n[3], int nsm, cudaStream_t st) {
  long long mf = 0;
  for (int d = 0; d < 3; ++d) mf = face_count(n, d) > mf ? face_count(n, d) : mf;
  double* fsp = buf;
  double* sp = buf + mf * FSLOT;
  SBuf sb[3];
  for (int d = 0; d < 3; ++d) {
    sb[d].p = sp;
    sb[d].nc = slope_cells(n, d);
    sb[d].mx = n[0] + 2 * (d == 0);
    sb[d].my = n[1] + 2 * (d == 1);
    sp += sb[d].nc * SSLOT;
    FBuf fb;
    fb.p = fsp;
    fb.nf = face_count(n, d);
    fb.nx = n[0] + (d == 0);
    fb.ny = n[1] + (d == 1);
    muscl_vjp_face_kernel<<<grid_m(fb.nf, nsm), 256, 0, st>>>(tb, fr, vbar, fb, d, fb.nf);
    muscl_vjp_slope_kernel<<<grid_m(sb[d].nc, nsm), 256, 0, st>>>(tb, fr, fb, sb[d], d, sb[d].nc);
  }
  const long long tot = (long long)(n[0] + 4) * (n[1] + 4) * (n[2] + 4);
  muscl_vjp_gather_kernel<<<grid_m(tot, nsm), 256, 0, st>>>(tb, ubar, sb[0], sb[1], sb[2], tot);
  return cudaGetLastError();
}

}  // namespace amrs
