// Hand-written adjoint (vector-Jacobian product) of the JST artificial
// dissipation (src/rhs/CNS_hydro_K.h:38-104, applied by compute_rhs at
// src/tim/CNS_advance.cpp:235-265) for one box.
//
// Forward, per face f of direction d and conserved component n:
//   F_n -= (s dw - max(0, Cdamp - s) fd) rr,
//   s  = Cshock max(S(f-1), S(f)),  rr = max(L(f-1), L(f)),
//   dw = U(f) - U(f-1),  fd = U(f+1) - 3U(f) + 3U(f-1) - U(f-2)
//   (z: U(f-1) - 3U(f) + 3U(f-1) - U(f-1), the reference's k-1 quirk),
// with S = the pressure sensor along x and L = |u_x| + c (component 0 of
// both arrays for every direction, as in the reference), computed on the
// valid cells and zero on ghost cells.
//
// Reverse (deterministic, no atomics):
//   jst_vjp_face_kernel  : per face, the cotangents of U at f-2 .. f+1
//       (direct, 20 slots) and of S and L at f-1, f (4 slots);
//   jst_vjp_sensor_kernel: per valid cell, S and L cotangents gathered from
//       its six faces, through the sensor and the spectral radius to the
//       primitive cotangents (rho, u_x, p at the cell, p at its x neighbours);
//   jst_vjp_gather_kernel: per cell of grow(box,2), the direct U cotangents
//       of the faces that reach it plus the cons2prim reverse of the
//       primitive cotangents, added to Ubar.
// Non-smooth points follow the forward's branch (max, |.|).
#include "adjoint_common.cuh"
#include "amrs_kernels.h"

namespace amrs {

namespace {

constexpr int JSLOT = 24;  // U at f-2, f-1, f, f+1 (5 each); S(f-1), S(f), L(f-1), L(f)
constexpr int CSLOT = 5;   // rho, u_x, p at the cell; p at c-x, c+x

struct JBuf {
  double* p;
  long long nf;
  int nx, ny;
};

__device__ __forceinline__ double sgnj(double x) { return x < 0.0 ? -1.0 : 1.0; }  // fabs's branch

__device__ __forceinline__ bool valid_cell(const BoxRec& R, int i, int j, int k) {
  return i >= R.lo[0] && i <= R.hi[0] && j >= R.lo[1] && j <= R.hi[1] && k >= R.lo[2] && k <= R.hi[2];
}

__global__ void __launch_bounds__(256) jst_vjp_face_kernel(BoxTable tb, FaceRec fr, DArr vbar, JBuf jb, int d,
                                                           long long total) {
  const BoxRec& R = tb.box[0];
  const DClosures& cl = tb.cls[R.cl];
  const DArr U = R.slot[0];
  const DArr S = fr.sen, L = fr.lam;
  const int di = d == 0, dj = d == 1, dk = d == 2;
  const long long su = (d == 0) ? 1 : (d == 1 ? U.js : U.ks);
  const long long ss = (d == 0) ? 1 : (d == 1 ? S.js : S.ks);
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < total;
       g += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(g % jb.nx) + R.lo[0];
    const long long t = g / jb.nx;
    const int j = (int)(t % jb.ny) + R.lo[1], k = (int)(t / jb.ny) + R.lo[2];
    const long long os = S.off(i, j, k);
    const double sm = S.p[os - ss], sp = S.p[os];
    const double lm = L.p[os - ss], lp = L.p[os];
    const bool s_takes_f = sm < sp, l_takes_f = lm < lp;
    const double s = cl.Cshock * (s_takes_f ? sp : sm);
    const double rr = l_takes_f ? lp : lm;
    const double x = cl.Cdamp - s;
    const bool mpos = 0.0 < x;
    const double mx = mpos ? x : 0.0;
    const long long ou = U.off(i, j, k);
    double sb = 0.0, rrb = 0.0, mxb = 0.0;
    double* o = jb.p + g;
    const long long nf = jb.nf;
    for (int n = 0; n < 5; ++n) {
      const long long on = ou + n * U.ns;
      const double dw = U.p[on] - U.p[on - su];
      const double fd = (d < 2) ? (U.p[on + su] - 3.0 * U.p[on] + 3.0 * U.p[on - su] - U.p[on - 2 * su])
                                : (U.p[on - su] - 3.0 * U.p[on] + 3.0 * U.p[on - su] - U.p[on - su]);
      const double Fb = R.dxinv[d] * ((valid_cell(R, i, j, k) ? vbar(i, j, k, n) : 0.0) -
                                      (valid_cell(R, i - di, j - dj, k - dk) ? vbar(i - di, j - dj, k - dk, n) : 0.0));
      const double tn = s * dw - mx * fd;
      const double tb_ = -Fb * rr;
      rrb += -Fb * tn;
      sb += tb_ * dw;
      mxb += -tb_ * fd;
      const double dwb = tb_ * s, fdb = -tb_ * mx;
      // offsets f-2, f-1, f, f+1 -> slots 0..3
      double u2, u1, u0, up;
      if (d < 2) { u2 = -fdb; u1 = -dwb + 3.0 * fdb; u0 = dwb - 3.0 * fdb; up = fdb; }
      else { u2 = 0.0; u1 = -dwb + 3.0 * fdb; u0 = dwb - 3.0 * fdb; up = 0.0; }
      o[(0 * 5 + n) * nf] = u2;
      o[(1 * 5 + n) * nf] = u1;
      o[(2 * 5 + n) * nf] = u0;
      o[(3 * 5 + n) * nf] = up;
    }
    if (mpos) sb -= mxb;
    const double Sb = cl.Cshock * sb;
    o[20 * nf] = s_takes_f ? 0.0 : Sb;
    o[21 * nf] = s_takes_f ? Sb : 0.0;
    o[22 * nf] = l_takes_f ? 0.0 : rrb;
    o[23 * nf] = l_takes_f ? rrb : 0.0;
  }
}

__global__ void __launch_bounds__(256) jst_vjp_sensor_kernel(BoxTable tb, JBuf j0, JBuf j1, JBuf j2, double* cs_buf,
                                                             long long total) {
  const BoxRec& R = tb.box[0];
  const DClosures& cl = tb.cls[R.cl];
  const DArr q = R.q;
  const int nx = R.hi[0] - R.lo[0] + 1, ny = R.hi[1] - R.lo[1] + 1;
  const JBuf jb[3] = {j0, j1, j2};
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < total;
       g += (long long)gridDim.x * blockDim.x) {
    const int c[3] = {(int)(g % nx) + R.lo[0], (int)((g / nx) % ny) + R.lo[1],
                      (int)(g / ((long long)nx * ny)) + R.lo[2]};
    double Sb = 0.0, Lb = 0.0;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const JBuf& J = jb[d];
      auto fidx = [&](int a0, int a1, int a2) {
        return (long long)(a0 - R.lo[0]) + (long long)J.nx * ((a1 - R.lo[1]) + (long long)J.ny * (a2 - R.lo[2]));
      };
      // face c (this cell is its f) and face c + e_d (this cell is its f-1)
      const long long f0 = fidx(c[0], c[1], c[2]);
      const long long f1 = fidx(c[0] + (d == 0), c[1] + (d == 1), c[2] + (d == 2));
      Sb += J.p[f0 + 21 * J.nf] + J.p[f1 + 20 * J.nf];
      Lb += J.p[f0 + 23 * J.nf] + J.p[f1 + 22 * J.nf];
    }
    const long long o = q.off(c[0], c[1], c[2]);
    const double pp = q.p[o + QPRES * q.ns], pl = q.p[o - 1 + QPRES * q.ns], pr = q.p[o + 1 + QPRES * q.ns];
    const double rho = q.p[o + QRHO * q.ns], ux = q.p[o + QU * q.ns];
    // L = |u_x| + sqrt(gamma p / rho)
    double uxb = Lb * sgnj(ux), rhob = 0.0, ppb = 0.0, plb = 0.0, prb = 0.0;
    const double cs = sqrt(cl.gamma * pp / rho);
    if (cs > 0.0) {
      const double xb = Lb / (2.0 * cs);
      ppb += xb * cl.gamma / rho;
      rhob += -xb * cl.gamma * pp / (rho * rho);
    }
    // S = |2 (pr - 2 pp + pl) / (pr + 2 pp + pl + |pr - pp| + |pp - pl| + 1e-40)|
    const double num = pr - 2.0 * pp + pl;
    const double a = pr - pp, b = pp - pl;
    const double den = pr + 2.0 * pp + pl + (fabs(a) + fabs(b)) + 1.0e-40;
    const double z = 2.0 * num / den;
    const double zb = Sb * sgnj(z);
    const double numb = 2.0 * zb / den, denb = -zb * z / den;
    const double ab = denb * sgnj(a), bb = denb * sgnj(b);
    prb += numb + denb + ab;
    ppb += -2.0 * numb + 2.0 * denb - ab + bb;
    plb += numb + denb - bb;
    double* w = cs_buf + g;
    w[0 * total] = rhob;
    w[1 * total] = uxb;
    w[2 * total] = ppb;
    w[3 * total] = plb;
    w[4 * total] = prb;
  }
}

__global__ void __launch_bounds__(256) jst_vjp_gather_kernel(BoxTable tb, DArr ubar, JBuf j0, JBuf j1, JBuf j2,
                                                             const double* cs_buf, long long nvalid, long long total) {
  const BoxRec& R = tb.box[0];
  const DClosures& cl = tb.cls[R.cl];
  const int mx = R.hi[0] - R.lo[0] + 5, my = R.hi[1] - R.lo[1] + 5;
  const int vx = R.hi[0] - R.lo[0] + 1, vy = R.hi[1] - R.lo[1] + 1;
  const JBuf jb[3] = {j0, j1, j2};
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < total;
       g += (long long)gridDim.x * blockDim.x) {
    const int c[3] = {(int)(g % mx) + R.lo[0] - 2, (int)((g / mx) % my) + R.lo[1] - 2,
                      (int)(g / ((long long)mx * my)) + R.lo[2] - 2};
    double ub[5] = {0, 0, 0, 0, 0};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const JBuf& J = jb[d];
#pragma unroll
      for (int sl = 0; sl < 4; ++sl) {
        // slot sl holds offset sl-2 from face f: this cell is f + sl - 2
        int f[3] = {c[0], c[1], c[2]};
        f[d] -= sl - 2;
        bool ok = true;
        for (int a = 0; a < 3; ++a) {
          const int hi = R.hi[a] + (a == d);
          if (f[a] < R.lo[a] || f[a] > hi) ok = false;
        }
        if (!ok) continue;
        const long long fi =
            (long long)(f[0] - R.lo[0]) + (long long)J.nx * ((f[1] - R.lo[1]) + (long long)J.ny * (f[2] - R.lo[2]));
#pragma unroll
        for (int n = 0; n < 5; ++n) ub[n] += J.p[fi + (sl * 5 + n) * J.nf];
      }
    }
    // primitive cotangents: own slots and the x neighbours' pressure slots
    double qb[NQA] = {0, 0, 0, 0, 0, 0};
    bool any = false;
    auto vidx = [&](int a0, int a1, int a2) {
      return (long long)(a0 - R.lo[0]) + (long long)vx * ((a1 - R.lo[1]) + (long long)vy * (a2 - R.lo[2]));
    };
    if (valid_cell(R, c[0], c[1], c[2])) {
      const long long v = vidx(c[0], c[1], c[2]);
      qb[QRHO] += cs_buf[v];
      qb[QU] += cs_buf[v + nvalid];
      qb[QPRES] += cs_buf[v + 2 * nvalid];
      any = true;
    }
    if (valid_cell(R, c[0] + 1, c[1], c[2])) {  // this cell is its c - x
      qb[QPRES] += cs_buf[vidx(c[0] + 1, c[1], c[2]) + 3 * nvalid];
      any = true;
    }
    if (valid_cell(R, c[0] - 1, c[1], c[2])) {  // this cell is its c + x
      qb[QPRES] += cs_buf[vidx(c[0] - 1, c[1], c[2]) + 4 * nvalid];
      any = true;
    }
    if (any) {
      double pb[5];
      cons2prim_vjp(R, cl, c[0], c[1], c[2], qb, pb);
#pragma unroll
      for (int n = 0; n < 5; ++n) ub[n] += pb[n];
    }
    const long long ou = ubar.off(c[0], c[1], c[2]);
#pragma unroll
    for (int n = 0; n < 5; ++n) ubar.p[ou + n * ubar.ns] += ub[n];
  }
}

int grid_j(long long n, int nsm) {
  long long b = (n + 255) / 256;
  const long long cap = (long long)nsm * 8;
  return (int)(b < 1 ? 1 : (b < cap ? b : cap));
}

long long jfaces(const int n[3], int d) {
  return (long long)(n[0] + (d == 0)) * (n[1] + (d == 1)) * (n[2] + (d == 2));
}

}  // namespace

size_t jst_vjp_buffer_bytes(const int n[3]) {
  long long t = 0;
  for (int d = 0; d < 3; ++d) t += jfaces(n, d) * JSLOT;
  t += (long long)n[0] * n[1] * n[2] * CSLOT;
  return (size_t)t * sizeof(double);
}

// Adds the JST part of the RHS VJP to ubar.  The sensor and spectral-radius
// arrays of the state must be current (launch_jst_sensor after zeroing).
cudaError_t launch_jst_vjp(const BoxTable& tb, const FaceRec& fr, const DArr& vbar, const DArr& ubar, double* buf,
                           const int n[3], int nsm, cudaStream_t st) {
  JBuf jb[3];
  double* p = buf;
  for (int d = 0; d < 3; ++d) {
    jb[d].p = p;
    jb[d].nf = jfaces(n, d);
    jb[d].nx = n[0] + (d == 0);
    jb[d].ny = n[1] + (d == 1);
    p += jb[d].nf * JSLOT;
    jst_vjp_face_kernel<<<grid_j(jb[d].nf, nsm), 256, 0, st>>>(tb, fr, vbar, jb[d], d, jb[d].nf);
  }
  const long long nvalid = (long long)n[0] * n[1] * n[2];
  jst_vjp_sensor_kernel<<<grid_j(nvalid, nsm), 256, 0, st>>>(tb, jb[0], jb[1], jb[2], p, nvalid);
  const long long tot = (long long)(n[0] + 4) * (n[1] + 4) * (n[2] + 4);
  jst_vjp_gather_kernel<<<grid_j(tot, nsm), 256, 0, st>>>(tb, ubar, jb[0], jb[1], jb[2], p, nvalid, tot);
  return cudaGetLastError();
}

}  // namespace amrs
