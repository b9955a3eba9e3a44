// Hand-written adjoint (vector-Jacobian product) of the WENO5-JS LLF
// Euler flux (src/rhs/High_resolution.h:83-319) for one box.
//
// Forward, per face f of direction d (cells f-3 .. f+2 along d):
//   alpha   = max lambda_d over the six cells
//   s+_q    = (pf_q + alpha U_q) / 2,  q = 0..4   (cells f-3 .. f+1)
//   s-_r    = (pf_{5-r} - alpha U_{5-r}) / 2, r = 0..4  (cells f+2 .. f-2)
//   F_n     = W(s+) + W(s-)   per conserved component n
// with W = weno5js and (pf_d, lambda_d) = cons2eulerflux_lambda(U) per cell.
//
// Reverse, one direction at a time (all sums in a fixed order, every output
// element written by one thread, so results are deterministic):
//   weno_vjp_face_kernel  : Fbar_n = dxinv_d (vbar(c) - vbar(c - e_d)); the
//       gradient of W at s+ and s- gives, per stencil cell q, the cotangents
//       of pf_d (5 comps), of U through alpha U (5 comps) and of lambda_d
//       (the first cell attaining the maximum takes alpha's cotangent);
//       they go to a per-face buffer of 6 x 11 values.
//   weno_vjp_gather_kernel: every cell sums the slots of the six faces whose
//       stencils hold it, applies the VJP of cons2eulerflux_lambda for
//       direction d and adds the result to Ubar.
// Non-smooth points follow the branch the forward pass takes (max, |.|).
#include "adjoint_common.cuh"
#include "amrs_kernels.h"

namespace amrs {

namespace {

constexpr int WSLOT = 11;            // pf (5), U (5), lambda (1) per stencil cell
constexpr int WCOMP = 6 * WSLOT;     // six stencil cells per face

// Faces nodal in d over the box: index = (i-lo0) + nx*((j-lo1) + ny*(k-lo2)).
struct FaceBuf {
  double* p;
  long long nf;  // component stride (number of faces)
  int nx, ny;
};

__device__ __forceinline__ double vget0(const DArr& v, const BoxRec& R, int i, int j, int k, int n) {
  if (i < R.lo[0] || i > R.hi[0] || j < R.lo[1] || j > R.hi[1] || k < R.lo[2] || k > R.hi[2]) return 0.0;
  return v(i, j, k, n);
}

// One thread per face of direction d.
__global__ void __launch_bounds__(256) weno_vjp_face_kernel(BoxTable tb, FaceRec fr, DArr vbar, FaceBuf fb, int d,
                                                            long long total) {
  const BoxRec& R = tb.box[0];
  const int di = d == 0, dj = d == 1, dk = d == 2;
  const DArr U = R.slot[0];
  const DArr PF = fr.pf[d];
  const DArr L = fr.lam;
  const long long su = (d == 0) ? 1 : (d == 1 ? U.js : U.ks);
  const long long sp = (d == 0) ? 1 : (d == 1 ? PF.js : PF.ks);
  const long long sl = (d == 0) ? 1 : (d == 1 ? L.js : L.ks);
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < total;
       g += (long long)gridDim.x * blockDim.x) {
    const int li = (int)(g % fb.nx);
    const long long t = g / fb.nx;
    const int i = li + R.lo[0], j = (int)(t % fb.ny) + R.lo[1], k = (int)(t / fb.ny) + R.lo[2];
    // alpha and the first cell attaining it (the forward's rmax chain)
    const long long ol = L.off(i, j, k) + d * L.ns;
    double me = L.p[ol - 3 * sl];
    int qs = 0;
#pragma unroll
    for (int q = 1; q < 6; ++q) {
      const double x = L.p[ol + (q - 3) * sl];
      if (me < x) { me = x; qs = q; }
    }
    const long long ou = U.off(i, j, k), op = PF.off(i, j, k);
    double abar = 0.0;
#pragma unroll 1
    for (int n = 0; n < NCONS; ++n) {
      const double fbn = R.dxinv[d] * (vget0(vbar, R, i, j, k, n) - vget0(vbar, R, i - di, j - dj, k - dk, n));
      double u[6], p[6];
#pragma unroll
      for (int q = 0; q < 6; ++q) {
        u[q] = U.p[ou + (q - 3) * su + n * U.ns];
        p[q] = PF.p[op + (q - 3) * sp + n * PF.ns];
      }
      double sp5[5], sm5[5], gp[5], gm[5];
#pragma unroll
      for (int q = 0; q < 5; ++q) {
        sp5[q] = 0.5 * (p[q] + me * u[q]);
        sm5[q] = 0.5 * (p[5 - q] - me * u[5 - q]);
      }
      weno5js_grad(sp5, gp);
      weno5js_grad(sm5, gm);
#pragma unroll
      for (int q = 0; q < 6; ++q) {
        const double a = (q < 5) ? kmul<(AMRS_WGRAD_IMUL >> 8) & 1>(fbn, gp[q]) : 0.0;      // cotangent of s+_q
        const double b = (q > 0) ? kmul<(AMRS_WGRAD_IMUL >> 8) & 1>(fbn, gm[5 - q]) : 0.0;  // cotangent of s-_{5-q}
        const double dlt = a - b;
        fb.p[g + (q * WSLOT + n) * fb.nf] = 0.5 * (a + b);
        fb.p[g + (q * WSLOT + 5 + n) * fb.nf] = 0.5 * me * dlt;
        abar += 0.5 * u[q] * dlt;
      }
    }
#pragma unroll
    for (int q = 0; q < 6; ++q) fb.p[g + (q * WSLOT + 10) * fb.nf] = (q == qs) ? abar : 0.0;
  }
}

// Gather + VJP of cons2eulerflux_lambda (src/rhs/High_resolution.h:83-121)
// for direction d, over cells [lo-3, hi+3] along d and the valid range across.
__global__ void __launch_bounds__(256) weno_vjp_gather_kernel(BoxTable tb, DArr ubar, FaceBuf fb, int d, int m0,
                                                              int m1, long long total) {
  const BoxRec& R = tb.box[0];
  const DClosures& cl = tb.cls[R.cl];
  const DArr U = R.slot[0];
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < total;
       g += (long long)gridDim.x * blockDim.x) {
    // region dims: along d (n_d + 6), the others valid
    const int ax = (int)(g % m0);
    const long long t = g / m0;
    const int ay = (int)(t % m1), az = (int)(t / m1);
    int c[3];
    c[0] = ax + R.lo[0] - (d == 0 ? 3 : 0);
    c[1] = ay + R.lo[1] - (d == 1 ? 3 : 0);
    c[2] = az + R.lo[2] - (d == 2 ? 3 : 0);
    double pb[5] = {0, 0, 0, 0, 0}, ub[5] = {0, 0, 0, 0, 0}, lb = 0.0;
#pragma unroll
    for (int q = 0; q < 6; ++q) {
      // the face whose stencil cell q is this cell: f = c + 3 - q along d
      int f[3] = {c[0], c[1], c[2]};
      f[d] += 3 - q;
      if (f[d] < R.lo[d] || f[d] > R.hi[d] + 1) continue;
      const long long fi = (long long)(f[0] - R.lo[0]) + (long long)fb.nx * ((f[1] - R.lo[1]) + (long long)fb.ny * (f[2] - R.lo[2]));
#pragma unroll
      for (int n = 0; n < 5; ++n) {
        pb[n] += fb.p[fi + (q * WSLOT + n) * fb.nf];
        ub[n] += fb.p[fi + (q * WSLOT + 5 + n) * fb.nf];
      }
      lb += fb.p[fi + (q * WSLOT + 10) * fb.nf];
    }
    // forward recompute at the cell
    const long long o = U.off(c[0], c[1], c[2]);
    const double gam = cl.gamma;
    const double rho = U.p[o];
    const double m[3] = {U.p[o + U.ns], U.p[o + 2 * U.ns], U.p[o + 3 * U.ns]};
    const double rhoet = U.p[o + 4 * U.ns];
    const double rhoinv = 1.0 / rho;
    const double uu[3] = {m[0] * rhoinv, m[1] * rhoinv, m[2] * rhoinv};
    const double rhoekin = 0.5 * rhoinv * (m[0] * m[0] + m[1] * m[1] + m[2] * m[2]);
    const double P = (gam - 1.0) * (rhoet - rhoekin);
    const double cs = sqrt(gam * P * rhoinv);
    const double ud = uu[d];
    // lambda_d = |rmax(rmax(ud + cs, ud - cs), ud)|: derivative along the taken branch
    const double ca = ud + cs, cb = ud - cs;
    double mx = ca, dcs = 1.0;
    if (mx < cb) { mx = cb; dcs = -1.0; }
    if (mx < ud) { mx = ud; dcs = 0.0; }
    const double sg = (mx > 0.0) ? 1.0 : (mx < 0.0 ? -1.0 : 0.0);
    // cotangents of the intermediates
    double mb[3] = {0, 0, 0}, ubv[3] = {0, 0, 0};
    double Pb = 0.0, Eb = 0.0, rinvb = 0.0;
    // physical flux f_d: (m_d, m_x u_d (+P), m_y u_d (+P), m_z u_d (+P), (E+P) u_d)
    mb[d] += pb[0];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      mb[a] += pb[1 + a] * ud;
      ubv[d] += pb[1 + a] * m[a];
    }
    Pb += pb[1 + d];
    Eb += pb[4] * ud;
    Pb += pb[4] * ud;
    ubv[d] += pb[4] * (rhoet + P);
    // lambda_d
    const double mxb = lb * sg;
    ubv[d] += mxb;
    const double csb = mxb * dcs;
    if (cs > 0.0) {
      const double h = csb * gam / (2.0 * cs);
      Pb += h * rhoinv;
      rinvb += h * P;
    }
    // u_a = m_a * rhoinv
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      mb[a] += ubv[a] * rhoinv;
      rinvb += ubv[a] * m[a];
    }
    // P = (gam-1) (E - rhoekin), rhoekin = rhoinv (m.m) / 2
    Eb += (gam - 1.0) * Pb;
    const double kb = -(gam - 1.0) * Pb;
    rinvb += 0.5 * (m[0] * m[0] + m[1] * m[1] + m[2] * m[2]) * kb;
#pragma unroll
    for (int a = 0; a < 3; ++a) mb[a] += rhoinv * m[a] * kb;
    const double rb = -rhoinv * rhoinv * rinvb;
    // direct U cotangents through alpha*U
    const long long ob = ubar.off(c[0], c[1], c[2]);
    ubar.p[ob] += rb + ub[0];
    ubar.p[ob + ubar.ns] += mb[0] + ub[1];
    ubar.p[ob + 2 * ubar.ns] += mb[1] + ub[2];
    ubar.p[ob + 3 * ubar.ns] += mb[2] + ub[3];
    ubar.p[ob + 4 * ubar.ns] += Eb + ub[4];
  }
}

int grid_n(long long n, int nsm) {
  long long b = (n + 255) / 256;
  const long long cap = (long long)nsm * 8;
  return (int)(b < 1 ? 1 : (b < cap ? b : cap));
}

}  // namespace

size_t weno_vjp_buffer_bytes(const int n[3]) {
  long long mx = 0;
  for (int d = 0; d < 3; ++d) {
    const long long nf = (long long)(n[0] + (d == 0)) * (n[1] + (d == 1)) * (n[2] + (d == 2));
    if (nf > mx) mx = nf;
  }
  return (size_t)mx * WCOMP * sizeof(double);
}

// Adds the WENO5 Euler part of the RHS VJP to ubar (which the viscous /
// cons2prim reverse pass has already written).  pf and lambda of the state
// must be current (launch_weno_point).
cudaError_t launch_weno_vjp(const BoxTable& tb, const FaceRec& fr, const DArr& vbar, const DArr& ubar, double* buf,
                            const int n[3], int nsm, cudaStream_t st) {
  for (int d = 0; d < 3; ++d) {
    FaceBuf fb;
    fb.p = buf;
    fb.nx = n[0] + (d == 0);
    fb.ny = n[1] + (d == 1);
    fb.nf = (long long)fb.nx * fb.ny * (n[2] + (d == 2));
    weno_vjp_face_kernel<<<grid_n(fb.nf, nsm), 256, 0, st>>>(tb, fr, vbar, fb, d, fb.nf);
    const int m0 = n[0] + (d == 0 ? 6 : 0), m1 = n[1] + (d == 1 ? 6 : 0), m2 = n[2] + (d == 2 ? 6 : 0);
    const long long tot = (long long)m0 * m1 * m2;
    weno_vjp_gather_kernel<<<grid_n(tot, nsm), 256, 0, st>>>(tb, ubar, fb, d, m0, m1, tot);
  }
  return cudaGetLastError();
}

}  // namespace amrs
