// Hand-written adjoint (vector-Jacobian product) of the WENO5-Riemann Euler
// flux (the riemann_weno extension: weno_riemann_face_kernel) for one box.
//
// Forward, per face f of direction d: rho, u_n, p, u_t1, u_t2 reconstructed
// from each side with weno5js over the cells f-3 .. f+2 (left state: f-3 ..
// f+1; right state: the mirror f+2 .. f-2), rho and p floored at 1e-40, the
// two-shock solver riemann_prob.
//
// Reverse, one direction at a time (deterministic, no atomics):
//   wr_vjp_face_kernel  : Fbar = dxinv_d (vbar(f) - vbar(f-1)); the solver's
//       reverse (riemann_vjp.cuh) gives the cotangents of the ten states, the
//       gradients of weno5js take them to the six stencil cells' primitives
//       (6 x 5 slots per face).
//   wr_vjp_gather_kernel: every cell sums the slots of the six faces whose
//       stencils hold it and adds the cons2prim reverse of that sum to Ubar.
#include "adjoint_common.cuh"
#include "amrs_kernels.h"
#include "riemann_vjp.cuh"

// Integer-pipe products of the WENO5 gradients here (see weno5js_grad).
#ifndef AMRS_WRGRAD_IMUL
#define AMRS_WRGRAD_IMUL 0x40
#endif

namespace amrs {

namespace {

constexpr int RSLOT = 30;  // six stencil cells x (rho, u_n, p, u_t1, u_t2)

struct RBuf {
  double* p;
  long long nf;
  int nx, ny;
};

__device__ __forceinline__ double vget_r(const DArr& v, const BoxRec& R, int i, int j, int k, int n) {
  if (i < R.lo[0] || i > R.hi[0] || j < R.lo[1] || j > R.hi[1] || k < R.lo[2] || k > R.hi[2]) return 0.0;
  return v(i, j, k, n);
}

// Three CTAs per SM (85 registers, the rest spilled): 24 warps hide the
// latency of the reverse solver's chain (measured: 11.96 against 13.96 ms
// per SSPRK3 step VJP at 64^3 with the unconstrained 255 registers).
__global__ void __launch_bounds__(256, 3) wr_vjp_face_kernel(BoxTable tb, DArr vbar, RBuf rb, int d, long long total) {
  const BoxRec& R = tb.box[0];
  const DArr q = R.q;
  const DClosures& cl = tb.cls[R.cl];
  const int di = d == 0, dj = d == 1, dk = d == 2;
  const int UN = UMX + d, UT1 = (d == 0) ? UMY : UMX, UT2 = (d == 2) ? UMY : UMZ;
  const int comp[5] = {QRHO, QU + d, QPRES, (d == 0) ? QV : QU, (d == 2) ? QV : QW};
  const long long sq = (d == 0) ? 1 : (d == 1 ? q.js : q.ks);
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < total;
       g += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(g % rb.nx) + R.lo[0];
    const long long t = g / rb.nx;
    const int j = (int)(t % rb.ny) + R.lo[1], k = (int)(t / rb.ny) + R.lo[2];
    const long long o = q.off(i, j, k);
    double gl[5][5], gr[5][5], in[10];
    double lraw[5], rraw[5];
#pragma unroll
    for (int m = 0; m < 5; ++m) {
      double v[6];
#pragma unroll
      for (int s = 0; s < 6; ++s) v[s] = q.p[o + (s - 3) * sq + comp[m] * q.ns];
      const double sl[5] = {v[0], v[1], v[2], v[3], v[4]};
      const double sr[5] = {v[5], v[4], v[3], v[2], v[1]};
      weno5js_grad<AMRS_WRGRAD_IMUL>(sl, gl[m], &lraw[m]);
      weno5js_grad<AMRS_WRGRAD_IMUL>(sr, gr[m], &rraw[m]);
    }
    in[0] = (lraw[0] < 1.0e-40) ? 1.0e-40 : lraw[0];
    in[1] = lraw[1];
    in[2] = (lraw[2] < 1.0e-40) ? 1.0e-40 : lraw[2];
    in[3] = lraw[3];
    in[4] = lraw[4];
    in[5] = (rraw[0] < 1.0e-40) ? 1.0e-40 : rraw[0];
    in[6] = rraw[1];
    in[7] = (rraw[2] < 1.0e-40) ? 1.0e-40 : rraw[2];
    in[8] = rraw[3];
    in[9] = rraw[4];
    const double h = R.dxinv[d];
    const int cmp[5] = {URHO, UN, UT1, UT2, UET};
    double fb[5];
#pragma unroll
    for (int n = 0; n < 5; ++n)
      fb[n] = h * (vget_r(vbar, R, i, j, k, cmp[n]) - vget_r(vbar, R, i - di, j - dj, k - dk, cmp[n]));
    double ib[10];
    rpvjp::riemann_prob_vjp(cl.gamma, 1.0e-40, in, fb, ib);
    const double lb[5] = {(lraw[0] < 1.0e-40) ? 0.0 : ib[0], ib[1], (lraw[2] < 1.0e-40) ? 0.0 : ib[2], ib[3], ib[4]};
    const double rbv[5] = {(rraw[0] < 1.0e-40) ? 0.0 : ib[5], ib[6], (rraw[2] < 1.0e-40) ? 0.0 : ib[7], ib[8],
                           ib[9]};
#pragma unroll
    for (int s = 0; s < 6; ++s)
#pragma unroll
      for (int m = 0; m < 5; ++m) {
        double a = 0.0;
        if (s < 5) a += lb[m] * gl[m][s];
        if (s > 0) a += rbv[m] * gr[m][5 - s];
        rb.p[g + (s * 5 + m) * rb.nf] = a;
      }
  }
}

// Cells lo-3 .. hi+3 along d (the stencils of faces lo .. hi+1), the valid
// range across.
__global__ void __launch_bounds__(256) wr_vjp_gather_kernel(BoxTable tb, DArr ubar, RBuf rb, int d, int m0, int m1,
                                                            long long total) {
  const BoxRec& R = tb.box[0];
  const DClosures& cl = tb.cls[R.cl];
  const int comp[5] = {QRHO, QU + d, QPRES, (d == 0) ? QV : QU, (d == 2) ? QV : QW};
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < total;
       g += (long long)gridDim.x * blockDim.x) {
    const int ax = (int)(g % m0);
    const long long t = g / m0;
    const int ay = (int)(t % m1), az = (int)(t / m1);
    int c[3];
    c[0] = ax + R.lo[0] - (d == 0 ? 3 : 0);
    c[1] = ay + R.lo[1] - (d == 1 ? 3 : 0);
    c[2] = az + R.lo[2] - (d == 2 ? 3 : 0);
    double qb[NQA] = {0, 0, 0, 0, 0, 0};
#pragma unroll
    for (int s = 0; s < 6; ++s) {
      // the face whose stencil cell s is this cell: f = c + 3 - s along d
      int f[3] = {c[0], c[1], c[2]};
      f[d] += 3 - s;
      if (f[d] < R.lo[d] || f[d] > R.hi[d] + 1) continue;
      const long long fi =
          (long long)(f[0] - R.lo[0]) + (long long)rb.nx * ((f[1] - R.lo[1]) + (long long)rb.ny * (f[2] - R.lo[2]));
#pragma unroll
      for (int m = 0; m < 5; ++m) qb[comp[m]] += rb.p[fi + (s * 5 + m) * rb.nf];
    }
    double ub[5];
    cons2prim_vjp(R, cl, c[0], c[1], c[2], qb, ub);
    const long long ou = ubar.off(c[0], c[1], c[2]);
#pragma unroll
    for (int n = 0; n < 5; ++n) ubar.p[ou + n * ubar.ns] += ub[n];
  }
}

int grid_r(long long n, int nsm) {
  long long b = (n + 255) / 256;
  const long long cap = (long long)nsm * 8;
  return (int)(b < 1 ? 1 : (b < cap ? b : cap));
}

}  // namespace

size_t weno_riemann_vjp_buffer_bytes(const int n[3]) {
  long long mx = 0;
  for (int d = 0; d < 3; ++d) {
    const long long nf = (long long)(n[0] + (d == 0)) * (n[1] + (d == 1)) * (n[2] + (d == 2));
    if (nf > mx) mx = nf;
  }
  return (size_t)mx * RSLOT * sizeof(double);
}

// Adds the WENO5-Riemann Euler part of the RHS VJP to ubar (which the
// viscous / cons2prim reverse pass has already written); Q must be current.
cudaError_t launch_weno_riemann_vjp(const BoxTable& tb, const DArr& vbar, const DArr& ubar, double* buf,
                                    const int n[3], int nsm, cudaStream_t st) {
  for (int d = 0; d < 3; ++d) {
    RBuf rb;
    rb.p = buf;
    rb.nx = n[0] + (d == 0);
    rb.ny = n[1] + (d == 1);
    rb.nf = (long long)rb.nx * rb.ny * (n[2] + (d == 2));
    wr_vjp_face_kernel<<<grid_r(rb.nf, nsm), 256, 0, st>>>(tb, vbar, rb, d, rb.nf);
    const int m0 = n[0] + (d == 0 ? 6 : 0), m1 = n[1] + (d == 1 ? 6 : 0), m2 = n[2] + (d == 2 ? 6 : 0);
    const long long tot = (long long)m0 * m1 * m2;
    wr_vjp_gather_kernel<<<grid_r(tot, nsm), 256, 0, st>>>(tb, ubar, rb, d, m0, m1, tot);
  }
  return cudaGetLastError();
}

}  // namespace amrs
