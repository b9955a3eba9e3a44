// Hand-written adjoint (vector-Jacobian product) of the KEEP + viscous RHS
// and of one RK stage.
//
// Forward map of one RHS (src/tim/CNS_advance.cpp:186-391):
//   U --cons2prim--> Q --KEEP pairs, viscous cell fluxes--> face fluxes F
//     --divergence--> dSdt.
// Reverse, given a cotangent vbar on the valid cells of dSdt:
//   Fbar_d(face f) = dxinv_d (vbar(f) - vbar(f-1))            (divergence^T)
//   adj_pair_kernel : every KEEP pair (a, a+l) once: Tbar = sum of Fbar over
//                     the l faces it feeds; pair VJP -> Qbar contributions of
//                     both ends into per-(direction, separation) buffers
//   adj_visc_kernel : every cell of grow(box,1): Vbar = average of Fbar over
//                     its two faces per direction; VJP of the cell viscous
//                     flux -> Qbar at the centre and gradient cotangents
//   adj_gather_kernel: Qbar(c) = sum of the buffers + gradient cotangents of
//                     the six neighbours; then the cons2prim VJP -> Ubar(c)
// Non-smooth points follow the branch the forward pass takes (max(1e-40,rho)
// passes the derivative only when rho > 1e-40).  Sums are deterministic:
// every output element is written by exactly one thread.
#include "adjoint_common.cuh"
#include "amrs_kernels.h"

namespace amrs {

struct AdjRec {
  DArr vbar;    // cotangent of dSdt, valid cells
  DArr ubar;    // output cotangent of the state, grow(box,3)
  DArr pair[3][3];  // [d][l-1]: NQA comps lo-end (0..5) + hi-end (6..11) over grow(box,3)
  DArr vg;      // viscous cotangents over grow(box,1): centre u,v,w,T (0..3), gradients (4..15)
  int visc;     // vg holds data (the viscous reverse pass ran)
  double* part; // per-block partial sums of d/d(visc_ref), d/d(cond_ref): 2 per block of adj_visc_kernel
};

__device__ __forceinline__ double vget(const DArr& v, const BoxRec& R, int i, int j, int k, int n) {
  if (i < R.lo[0] || i > R.hi[0] || j < R.lo[1] || j > R.hi[1] || k < R.lo[2] || k > R.hi[2]) return 0.0;
  return v(i, j, k, n);
}

// Fbar of the d-face below cell (i,j,k), component n.
__device__ __forceinline__ double fbar(const DArr& v, const BoxRec& R, int d, int i, int j, int k, int n) {
  const int di = d == 0, dj = d == 1, dk = d == 2;
  return R.dxinv[d] * (vget(v, R, i, j, k, n) - vget(v, R, i - di, j - dj, k - dk, n));
}

// VJP of one KEEP pair term (keep_pair in amrs_device.cuh) given its
// cotangent a[5] (already times the coefficient): contributions to the
// primitive cotangents of point 1 (larger index) and point 2.  With
// P = R N, the mass flux m = P/4 and the cubic factor t8 = P/8, so the
// cotangents of R and N share one factor s = mb/4 + t8b/8 (exact scalings;
// the reverse pass has no bit-exact counterpart).  Standalone products may
// go to the integer pipe (kmul, AMRS_PVJP_IMUL): bit 0 the cotangents of
// the velocity sums and of E, bit 1 those of R and N, bit 2 cv Eb.
#ifndef AMRS_PVJP_IMUL
#define AMRS_PVJP_IMUL 0x3
#endif
template <int D>
__device__ __forceinline__ void keep_pair_vjp(const double* q1, const double* q2, const double a[5], double cv,
                                              double b1[NQA], double b2[NQA]) {
  constexpr int QN = QU + D;
  constexpr bool M0 = AMRS_PVJP_IMUL & 1, M1 = (AMRS_PVJP_IMUL >> 1) & 1, M2 = (AMRS_PVJP_IMUL >> 2) & 1;
  const double R = q1[QRHO] + q2[QRHO];
  const double N = q1[QN] + q2[QN];
  const double Ux = q1[QU] + q2[QU], Uy = q1[QV] + q2[QV], Uz = q1[QW] + q2[QW];
  const double E = q1[QE] + q2[QE];
  const double P = R * N;
  const double ke = 0.5 * (q1[QU] * q2[QU] + q1[QV] * q2[QV] + q1[QW] * q2[QW]);
  const double t8 = 0.125 * P;
  const double mb = a[0] + a[4] * ke;
  const double keb = 0.25 * (a[4] * P);
  const double t8b = a[1] * Ux + a[2] * Uy + a[3] * Uz + a[4] * E;
  const double Uxb = kmul<M0>(a[1], t8), Uyb = kmul<M0>(a[2], t8), Uzb = kmul<M0>(a[3], t8),
               Eb = kmul<M0>(a[4], t8);
  const double fdivb = a[1 + D];
  const double fgb = a[4];
  const double sb = 0.25 * mb + 0.125 * t8b;
  const double Rb = kmul<M1>(N, sb);
  const double Nb = kmul<M1>(R, sb);
  const double Pb = 0.5 * fdivb;
  const double Ub[3] = {Uxb, Uyb, Uzb};
  const double hk = 0.5 * keb, hg = 0.5 * fgb;
  const double cvE = kmul<M2>(cv, Eb);
#pragma unroll
  for (int s = 0; s < 2; ++s) {
    const double* qo = s ? q1 : q2;
    double* b = s ? b2 : b1;
    b[0] = Rb;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      double t = Ub[c] + hk * qo[QU + c];
      if (c == D) t += Nb + hg * qo[QPRES];
      b[1 + c] = t;
    }
    b[4] = cvE;
    b[5] = Pb + hg * qo[QN];
  }
}

// One thread per (direction, separation, pair): pairs (a, a+l) along d
// with a in [lo-l, hi] and transverse indices in the valid box.
template <int ORDER>
__global__ void __launch_bounds__(256) adj_pair_kernel(BoxTable tb, AdjRec ar, long long total) {
  constexpr int H = ORDER / 2;
  double coef[3];
  if (ORDER == 6) { coef[0] = 6.0 / 4; coef[1] = -6.0 / 20; coef[2] = 2.0 / 60; }
  else if (ORDER == 4) { coef[0] = 4.0 / 3; coef[1] = -2.0 / 12; coef[2] = 0.0; }
  else { coef[0] = 1.0; coef[1] = 0.0; coef[2] = 0.0; }
  const BoxRec& R = tb.box[0];
  const DClosures& cl = tb.cls[R.cl];
  const int n0 = R.hi[0] - R.lo[0] + 1, n1 = R.hi[1] - R.lo[1] + 1, n2 = R.hi[2] - R.lo[2] + 1;
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < total;
       g += (long long)gridDim.x * blockDim.x) {
    // decode (d, l, i, j, k): per (d,l) block, extent n_d + l in d
    long long r = g;
    int d = 0, l = 1;
    bool found = false;
    for (int dd = 0; dd < 3 && !found; ++dd)
      for (int ll = 1; ll <= H && !found; ++ll) {
        const long long cnt = (long long)(n0 + (dd == 0) * ll) * (n1 + (dd == 1) * ll) * (n2 + (dd == 2) * ll);
        if (r < cnt) { d = dd; l = ll; found = true; }
        else r -= cnt;
      }
    if (!found) continue;
    const int e0 = n0 + (d == 0) * l, e1 = n1 + (d == 1) * l;
    const int ii = (int)(r % e0);
    const long long t = r / e0;
    const int jj = (int)(t % e1), kk = (int)(t / e1);
    const int i = R.lo[0] + ii - (d == 0) * l, j = R.lo[1] + jj - (d == 1) * l, k = R.lo[2] + kk - (d == 2) * l;
    const int di = d == 0, dj = d == 1, dk = d == 2;
    // pair (a = (i,j,k), a + l e_d); faces a+1 .. a+l.  Next to a code-6 y
    // wall the reduced y faces take only the l = 1 pair, with coefficient 1
    // (Flux_2nd_Order_KEEP, src/rhs/CentralKEEP.h:232-287).
    double a[5] = {0, 0, 0, 0, 0};
    if (d == 1 && R.walls) {
      for (int m = 1; m <= l; ++m) {
        double w = coef[l - 1];
        const int jf = j + m;
        if (jf <= R.red_lo || (jf >= R.red_hi && jf <= R.hi[1])) w = (l == 1) ? 1.0 : 0.0;
        if (w == 0.0) continue;
#pragma unroll
        for (int n = 0; n < 5; ++n) a[n] += w * fbar(ar.vbar, R, d, i + m * di, j + m * dj, k + m * dk, n);
      }
    } else {
      // one coefficient for all l faces: sum_m Fbar(a + m) telescopes to
      // dxinv_d (vbar(a + l) - vbar(a))
      const double wd = coef[l - 1] * R.dxinv[d];
#pragma unroll
      for (int n = 0; n < 5; ++n)
        a[n] = wd * (vget(ar.vbar, R, i + l * di, j + l * dj, k + l * dk, n) - vget(ar.vbar, R, i, j, k, n));
    }
    double q1[NQ], q2[NQ], b1[NQA], b2[NQA];
    const long long o2 = R.q.off(i, j, k), o1 = R.q.off(i + l * di, j + l * dj, k + l * dk);
#pragma unroll
    for (int n = 0; n < NQ; ++n) { q1[n] = R.q.p[o1 + n * R.q.ns]; q2[n] = R.q.p[o2 + n * R.q.ns]; }
    if (d == 0) keep_pair_vjp<0>(q1, q2, a, cl.cv, b1, b2);
    else if (d == 1) keep_pair_vjp<1>(q1, q2, a, cl.cv, b1, b2);
    else keep_pair_vjp<2>(q1, q2, a, cl.cv, b1, b2);
    const DArr P = ar.pair[d][l - 1];
    const long long olo = P.off(i, j, k), ohi = P.off(i + l * di, j + l * dj, k + l * dk);
#pragma unroll
    for (int n = 0; n < NQA; ++n) {
      P.p[olo + n * P.ns] = b2[n];
      P.p[ohi + (NQA + n) * P.ns] = b1[n];
    }
  }
}

// VJP of the cell viscous fluxes (viscous_cell in amrs_device.cuh) for every
// cell of grow(box,1).  With `pbar`, each block also sums d/d(visc_ref) and
// d/d(cond_ref) over its cells in a fixed order (grid-stride, then warp
// shuffles, then the warps in order) into ar.part; adj_param_sum_kernel adds
// the blocks' sums in block order.  No atomics: the result is the same bits
// on every run.
__global__ void __launch_bounds__(256) adj_visc_kernel(BoxTable tb, AdjRec ar, long long total, double* pbar) {
  const BoxRec& R = tb.box[0];
  const DClosures& cl = tb.cls[R.cl];
  const int nx = R.hi[0] - R.lo[0] + 3, ny = R.hi[1] - R.lo[1] + 3;
  double mu_acc = 0.0, la_acc = 0.0;
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < total;
       g += (long long)gridDim.x * blockDim.x) {
    const int l = (int)g;
    const int i = l % nx + R.lo[0] - 1;
    const int t = l / nx;
    const int j = t % ny + R.lo[1] - 1;
    const int k = t / ny + R.lo[2] - 1;
    const double hx = 0.5 * R.dxinv[0], hy = 0.5 * R.dxinv[1], hz = 0.5 * R.dxinv[2];
    // Vbar: each cell flux enters the faces below and above it with 0.5, and
    // Fbar(c) + Fbar(c + e_d) = dxinv_d (vbar(c + e_d) - vbar(c - e_d))
    double fb[NVF];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const int di = d == 0, dj = d == 1, dk = d == 2;
      const double h = d == 0 ? hx : (d == 1 ? hy : hz);
#pragma unroll
      for (int n = 0; n < 4; ++n)
        fb[4 * d + n] = h * (vget(ar.vbar, R, i + di, j + dj, k + dk, 1 + n) -
                             vget(ar.vbar, R, i - di, j - dj, k - dk, 1 + n));
    }
    const DArr Q = R.q;
    const long long o = Q.off(i, j, k);
    auto q = [&](long long off, int n) { return Q.p[off + n * Q.ns]; };
    const long long sx = 1, sy = Q.js, sz = Q.ks;
    const double u = q(o, QU), v = q(o, QV), w = q(o, QW), T = q(o, QT);
    const double dudx = (q(o + sx, QU) - q(o - sx, QU)) * hx, dvdx = (q(o + sx, QV) - q(o - sx, QV)) * hx;
    const double dwdx = (q(o + sx, QW) - q(o - sx, QW)) * hx, dTdx = (q(o + sx, QT) - q(o - sx, QT)) * hx;
    // y derivatives: central, or one-sided on the ghost row beyond a code-6
    // wall (ViscousWallFluxes, src/rhs/CNS_hydro_K.h:177-251)
    auto ddy = [&](int n) {
      if (R.walls && j == R.wrow_lo) return (4.0 * q(o + sy, n) - q(o + 2 * sy, n) - 3.0 * q(o, n)) * hy;
      if (R.walls && j == R.wrow_hi) return (-4.0 * q(o - sy, n) + 3.0 * q(o, n) + q(o - 2 * sy, n)) * hy;
      return (q(o + sy, n) - q(o - sy, n)) * hy;
    };
    const double dudy = ddy(QU), dvdy = ddy(QV), dwdy = ddy(QW), dTdy = ddy(QT);
    const double dudz = (q(o + sz, QU) - q(o - sz, QU)) * hz, dvdz = (q(o + sz, QV) - q(o - sz, QV)) * hz;
    const double dwdz = (q(o + sz, QW) - q(o - sz, QW)) * hz, dTdz = (q(o + sz, QT) - q(o - sz, QT)) * hz;
    const double div = dudx + dvdy + dwdz;
    const double mu = visc(cl, T), lam = cond(cl, T);
    const double r13 = 1.0 / 3.0;
    const double txx = 2.0 * mu * (dudx - r13 * div), tyy = 2.0 * mu * (dvdy - r13 * div);
    const double tzz = 2.0 * mu * (dwdz - r13 * div);
    const double txy = mu * (dudy + dvdx), txz = mu * (dudz + dwdx), tyz = mu * (dvdz + dwdy);
    const double txxb = -fb[0] - fb[3] * u;
    const double txyb = -fb[1] - fb[3] * v - fb[4] - fb[7] * u;
    const double txzb = -fb[2] - fb[3] * w - fb[8] - fb[11] * u;
    const double tyyb = -fb[5] - fb[7] * v;
    const double tyzb = -fb[6] - fb[7] * w - fb[9] - fb[11] * v;
    const double tzzb = -fb[10] - fb[11] * w;
    const double ub = -(fb[3] * txx + fb[7] * txy + fb[11] * txz);
    const double vb = -(fb[3] * txy + fb[7] * tyy + fb[11] * tyz);
    const double wb = -(fb[3] * txz + fb[7] * tyz + fb[11] * tzz);
    const double lamb = -(fb[3] * dTdx + fb[7] * dTdy + fb[11] * dTdz);
    const double mub = txxb * 2.0 * (dudx - r13 * div) + tyyb * 2.0 * (dvdy - r13 * div) +
                       tzzb * 2.0 * (dwdz - r13 * div) + txyb * (dudy + dvdx) + txzb * (dudz + dwdx) +
                       tyzb * (dvdz + dwdy);
    const double divb = -(2.0 / 3.0) * mu * (txxb + tyyb + tzzb);
    double gb[12];
    const double gxy = mu * txyb, gxz = mu * txzb, gyz = mu * tyzb;
    gb[0] = 2.0 * mu * txxb + divb;  // dudx
    gb[1] = gxy;                     // dvdx
    gb[2] = gxz;                     // dwdx
    gb[3] = -lam * fb[3];            // dTdx
    gb[4] = gxy;                     // dudy
    gb[5] = 2.0 * mu * tyyb + divb;  // dvdy
    gb[6] = gyz;                     // dwdy
    gb[7] = -lam * fb[7];            // dTdy
    gb[8] = gxz;                     // dudz
    gb[9] = gyz;                     // dvdz
    gb[10] = 2.0 * mu * tzzb + divb; // dwdz
    gb[11] = -lam * fb[11];          // dTdz
    double Tb = 0.0;
    if (cl.visc_law == 1) Tb += mub * mu * (1.5 / T - 1.0 / (cl.Tvisc_ref + T));
    else mu_acc += mub;
    if (cl.cond_law == 1) Tb += lamb * lam * (1.5 / T - 1.0 / (cl.Tcond_ref + T));
    else la_acc += lamb;
    const DArr G = ar.vg;
    const long long og = G.off(i, j, k);
    G.p[og] = ub;
    G.p[og + G.ns] = vb;
    G.p[og + 2 * G.ns] = wb;
    G.p[og + 3 * G.ns] = Tb;
#pragma unroll
    for (int n = 0; n < 12; ++n) G.p[og + (4 + n) * G.ns] = gb[n];
  }
  if (pbar) {
    __shared__ double wsum[2][8];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      mu_acc += __shfl_down_sync(0xffffffffu, mu_acc, off);
      la_acc += __shfl_down_sync(0xffffffffu, la_acc, off);
    }
    if ((threadIdx.x & 31) == 0) {
      wsum[0][threadIdx.x >> 5] = mu_acc;
      wsum[1][threadIdx.x >> 5] = la_acc;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      double m = 0.0, a = 0.0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
        m += wsum[0][w];
        a += wsum[1][w];
      }
      ar.part[2 * blockIdx.x] = m;
      ar.part[2 * blockIdx.x + 1] = a;
    }
  }
}

// pbar += the per-block sums of adj_visc_kernel, in block order.
__global__ void adj_param_sum_kernel(const double* part, int nblocks, double* pbar) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double m = 0.0, a = 0.0;
  for (int b = 0; b < nblocks; ++b) {
    m += part[2 * b];
    a += part[2 * b + 1];
  }
  pbar[0] += m;
  pbar[1] += a;
}

// Qbar gather + cons2prim VJP for every cell of grow(box,3).
template <int ORDER>
__global__ void __launch_bounds__(256) adj_gather_kernel(BoxTable tb, AdjRec ar, long long total, int gpair) {
  constexpr int H = ORDER / 2;
  const BoxRec& R = tb.box[0];
  const DClosures& cl = tb.cls[R.cl];
  const int g3 = NGHOST;
  const int nx = R.hi[0] - R.lo[0] + 1 + 2 * g3, ny = R.hi[1] - R.lo[1] + 1 + 2 * g3;
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < total;
       g += (long long)gridDim.x * blockDim.x) {
    const int l0 = (int)g;
    const int i = l0 % nx + R.lo[0] - g3;
    const int t = l0 / nx;
    const int j = t % ny + R.lo[1] - g3;
    const int k = t / ny + R.lo[2] - g3;
    const DArr Ub = ar.ubar;
    const long long ou = Ub.off(i, j, k);
    // cells any cotangent of this pass reaches (viscous stencils: 2 ghosts);
    // beyond them Q is not computed and ubar is zero
    const int gvisc = ar.visc ? 2 : 0;
    const int gact = gpair > gvisc ? gpair : gvisc;
    if (i < R.lo[0] - gact || i > R.hi[0] + gact || j < R.lo[1] - gact || j > R.hi[1] + gact ||
        k < R.lo[2] - gact || k > R.hi[2] + gact) {
#pragma unroll
      for (int n = 0; n < 5; ++n) Ub.p[ou + n * Ub.ns] = 0.0;
      continue;
    }
    double qb[NQA] = {0, 0, 0, 0, 0, 0};
    const bool in_pair = i >= R.lo[0] - gpair && i <= R.hi[0] + gpair && j >= R.lo[1] - gpair &&
                         j <= R.hi[1] + gpair && k >= R.lo[2] - gpair && k <= R.hi[2] + gpair;
    if (in_pair) {
#pragma unroll
      for (int d = 0; d < 3; ++d)
#pragma unroll
        for (int l = 1; l <= H; ++l) {
          const DArr P = ar.pair[d][l - 1];
          const long long o = P.off(i, j, k);
#pragma unroll
          for (int n = 0; n < NQA; ++n) qb[n] += P.p[o + n * P.ns] + P.p[o + (NQA + n) * P.ns];
        }
    }
    const DArr G = ar.vg;
    auto inside1 = [&](int a, int b, int c) {
      return ar.visc && a >= R.lo[0] - 1 && a <= R.hi[0] + 1 && b >= R.lo[1] - 1 && b <= R.hi[1] + 1 &&
             c >= R.lo[2] - 1 && c <= R.hi[2] + 1;
    };
    if (inside1(i, j, k)) {
      const long long o = G.off(i, j, k);
      qb[QU] += G.p[o];
      qb[QV] += G.p[o + G.ns];
      qb[QW] += G.p[o + 2 * G.ns];
      qb[QT] += G.p[o + 3 * G.ns];
    }
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const int di = d == 0, dj = d == 1, dk = d == 2;
      const double h = 0.5 * R.dxinv[d];
      // the gradient at e = c + s e_d reads q(c) with weight wt: central
      // differences give +h at s = -1 and -h at s = +1; the one-sided y
      // derivative of a wall's ghost row e reads e, e+1, e+2 (lower wall)
      // with -3h, 4h, -h, or e, e-1, e-2 (upper wall) with 3h, -4h, h
#pragma unroll
      for (int s = -2; s <= 2; ++s) {
        const int a = i + s * di, b = j + s * dj, c = k + s * dk;
        if (!inside1(a, b, c)) continue;
        double wt = 0.0;
        if (d == 1 && R.walls && b == R.wrow_lo) wt = (s == 0) ? -3.0 * h : (s == -1 ? 4.0 * h : (s == -2 ? -h : 0.0));
        else if (d == 1 && R.walls && b == R.wrow_hi) wt = (s == 0) ? 3.0 * h : (s == 1 ? -4.0 * h : (s == 2 ? h : 0.0));
        else wt = (s == -1) ? h : (s == 1 ? -h : 0.0);
        if (wt == 0.0) continue;
        const long long o = G.off(a, b, c);
#pragma unroll
        for (int n = 0; n < 4; ++n) qb[QU + n] += wt * G.p[o + (4 + 4 * d + n) * G.ns];
      }
    }
    // cons2prim VJP (src/rhs/CNS_hydro_K.h:15-34)
    double ub5[5];
    cons2prim_vjp(R, cl, i, j, k, qb, ub5);
#pragma unroll
    for (int n = 0; n < 5; ++n) Ub.p[ou + n * Ub.ns] = ub5[n];
  }
}

// Reverse of one stage's BLAS-1 program per valid cell: given the cotangent
// of the stage result (register S2), produce the cotangents of S1, of the
// stage input's valid values (register S2 before the program) and of dSdt.
__global__ void __launch_bounds__(256) adj_prog_kernel(BoxRec R, DProg prog, DArr wbar, DArr s1bar, DArr inbar,
                                                       DArr vbar, long long total, int accumulate) {
  const int nx = R.hi[0] - R.lo[0] + 1, ny = R.hi[1] - R.lo[1] + 1;
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < total;
       g += (long long)gridDim.x * blockDim.x) {
    const int l = (int)g;
    const int i = l % nx + R.lo[0];
    const int t = l / nx;
    const int j = t % ny + R.lo[1];
    const int k = t / ny + R.lo[2];
    for (int n = 0; n < 5; ++n) {
      double b[3] = {0.0, wbar(i, j, k, n), 0.0};
      for (int o = prog.nops - 1; o >= 0; --o) {
        const DOp& q = prog.ops[o];
        if (q.kind == 0) {
          const double gg = b[q.dst];
          b[q.dst] = 0.0;
          b[q.x] += q.a * gg;
          b[q.y] += q.b * gg;
        } else if (q.kind == 1) {
          b[q.x] += q.a * b[q.dst];
        } else if (q.kind == 2) {
          const double gg = b[q.dst];
          b[q.dst] = q.a * gg;
          b[q.x] += gg;
        } else {
          const double gg = b[q.dst];
          b[q.dst] = 0.0;
          b[q.x] += gg;
        }
      }
      if (accumulate) {
        s1bar(i, j, k, n) += b[0];
        inbar(i, j, k, n) += b[1];
      } else {
        s1bar(i, j, k, n) = b[0];
        inbar(i, j, k, n) = b[1];
      }
      vbar(i, j, k, n) = b[2];
    }
  }
}

// Ghost fold: the adjoint of amrs_fill_halo_box.  Every valid cell adds the
// cotangents of the ghost cells filled from it (with the reflect_odd sign).
__device__ __forceinline__ int images(int c, int lo, int hi, int bcl, int bch, int comp, int dir, int* out,
                                      int* sgn) {
  int nimg = 0;
  out[nimg] = c; sgn[nimg] = 1; ++nimg;
  const int n = hi - lo + 1;
  const bool vel = comp >= UMX && comp <= UMZ, normal = comp == UMX + dir;
  for (int side = 0; side < 2; ++side) {
    const int phys = side ? bch : bcl;
    for (int gidx = 1; gidx <= NGHOST; ++gidx) {
      const int gc = side ? hi + gidx : lo - gidx;  // ghost coordinate
      int src;
      int s = 1;
      if (phys == -1) {
        int r = (gc - lo) % n;
        if (r < 0) r += n;
        src = lo + r;
      } else if (phys == 2) {
        src = side ? hi : lo;
      } else if (phys == 3 || phys == 4 || phys == 5) {
        src = side ? 2 * hi - gc + 1 : 2 * lo - gc - 1;
        const bool odd = (phys == 5) ? vel : (vel && normal);
        if (odd) s = -1;
      } else {
        continue;
      }
      if (src == c) { out[nimg] = gc; sgn[nimg] = s; ++nimg; }
    }
  }
  return nimg;
}

__global__ void __launch_bounds__(256) adj_halo_kernel(HaloBox hb, long long total) {
  const int nx = hb.hi[0] - hb.lo[0] + 1, ny = hb.hi[1] - hb.lo[1] + 1;
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < total;
       g += (long long)gridDim.x * blockDim.x) {
    const int l = (int)g;
    const int i = l % nx + hb.lo[0];
    const int t = l / nx;
    const int j = t % ny + hb.lo[1];
    const int k = t / ny + hb.lo[2];
    for (int n = 0; n < hb.ncomp; ++n) {
      int xi[8], xs[8], yi[8], ys[8], zi[8], zs[8];
      const int nxi = images(i, hb.lo[0], hb.hi[0], hb.bc_lo[0], hb.bc_hi[0], n, 0, xi, xs);
      const int nyi = images(j, hb.lo[1], hb.hi[1], hb.bc_lo[1], hb.bc_hi[1], n, 1, yi, ys);
      const int nzi = images(k, hb.lo[2], hb.hi[2], hb.bc_lo[2], hb.bc_hi[2], n, 2, zi, zs);
      double s = 0.0;
      for (int a = 0; a < nzi; ++a)
        for (int b = 0; b < nyi; ++b)
          for (int c = 0; c < nxi; ++c) s += (double)(xs[c] * ys[b] * zs[a]) * hb.u(xi[c], yi[b], zi[a], n);
      hb.u(i, j, k, n) = s;
    }
  }
}

// Reverse of the body-force source (add_source) on the valid cells:
// ubar(URHO) += vbar(UMX+d) f_d and ubar(UMX+d) += vbar(UET) f_d.
__global__ void __launch_bounds__(256) adj_source_kernel(BoxRec R, double f0, double f1, double f2, DArr vbar,
                                                         DArr ubar, long long total) {
  const int nx = R.hi[0] - R.lo[0] + 1, ny = R.hi[1] - R.lo[1] + 1;
  const double f[3] = {f0, f1, f2};
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < total;
       g += (long long)gridDim.x * blockDim.x) {
    const int l = (int)g;
    const int i = l % nx + R.lo[0];
    const int t = l / nx;
    const int j = t % ny + R.lo[1];
    const int k = t / ny + R.lo[2];
    const double ve = vbar(i, j, k, UET);
    double rb = 0.0;
    for (int d = 0; d < 3; ++d) {
      if (f[d] == 0.0) continue;
      rb += vbar(i, j, k, UMX + d) * f[d];
      ubar(i, j, k, UMX + d) += ve * f[d];
    }
    ubar(i, j, k, URHO) += rb;
  }
}

// ------------------------------------------------------------ launchers --
static int grid256(long long n, int nsm) {
  long long b = (n + 255) / 256;
  const long long cap = (long long)nsm * 8;
  return (int)(b < 1 ? 1 : (b < cap ? b : cap));
}

cudaError_t launch_rhs_vjp(int order, const BoxTable& tb, const AdjRecHost& ah, double* pbar, int nsm,
                           cudaStream_t st) {
  AdjRec ar;
  ar.vbar = ah.vbar;
  ar.ubar = ah.ubar;
  for (int d = 0; d < 3; ++d)
    for (int l = 0; l < 3; ++l) ar.pair[d][l] = ah.pair[d][l];
  ar.vg = ah.vg;
  ar.visc = ah.visc;
  ar.part = ah.part;
  if (pbar && !ah.part) return cudaErrorInvalidValue;
  const int H = order / 2;
  const long long n0 = ah.n[0], n1 = ah.n[1], n2 = ah.n[2];
  long long npair = 0;
  for (int d = 0; d < 3; ++d)
    for (int l = 1; l <= H; ++l) npair += (n0 + (d == 0) * l) * (n1 + (d == 1) * l) * (n2 + (d == 2) * l);
  // order 0: no KEEP pairs (the viscous part of another scheme's RHS)
  if (order == 2) adj_pair_kernel<2><<<grid256(npair, nsm), 256, 0, st>>>(tb, ar, npair);
  else if (order == 4) adj_pair_kernel<4><<<grid256(npair, nsm), 256, 0, st>>>(tb, ar, npair);
  else if (order == 6) adj_pair_kernel<6><<<grid256(npair, nsm), 256, 0, st>>>(tb, ar, npair);
  const long long nv = (n0 + 2) * (n1 + 2) * (n2 + 2);
  if (ah.visc) {
    const int nbv = grid256(nv, nsm);  // at most 8 blocks per SM: ah.part holds 2 x 8 x nsm doubles
    adj_visc_kernel<<<nbv, 256, 0, st>>>(tb, ar, nv, pbar);
    if (pbar) adj_param_sum_kernel<<<1, 32, 0, st>>>(ah.part, nbv, pbar);
  }
  const long long ng = (n0 + 6) * (n1 + 6) * (n2 + 6);
  if (order == 0) adj_gather_kernel<0><<<grid256(ng, nsm), 256, 0, st>>>(tb, ar, ng, 0);
  else if (order == 2) adj_gather_kernel<2><<<grid256(ng, nsm), 256, 0, st>>>(tb, ar, ng, H);
  else if (order == 4) adj_gather_kernel<4><<<grid256(ng, nsm), 256, 0, st>>>(tb, ar, ng, H);
  else adj_gather_kernel<6><<<grid256(ng, nsm), 256, 0, st>>>(tb, ar, ng, H);
  return cudaGetLastError();
}

cudaError_t launch_adj_prog(const BoxRec& R, const DProg& prog, const DArr& wbar, const DArr& s1bar, const DArr& inbar,
                            const DArr& vbar, int accumulate, int nsm, cudaStream_t st) {
  const long long n = (long long)(R.hi[0] - R.lo[0] + 1) * (R.hi[1] - R.lo[1] + 1) * (R.hi[2] - R.lo[2] + 1);
  adj_prog_kernel<<<grid256(n, nsm), 256, 0, st>>>(R, prog, wbar, s1bar, inbar, vbar, n, accumulate);
  return cudaGetLastError();
}

cudaError_t launch_source_vjp(const BoxRec& R, const double force[3], const DArr& vbar, const DArr& ubar, int nsm,
                              cudaStream_t st) {
  const long long n = (long long)(R.hi[0] - R.lo[0] + 1) * (R.hi[1] - R.lo[1] + 1) * (R.hi[2] - R.lo[2] + 1);
  adj_source_kernel<<<grid256(n, nsm), 256, 0, st>>>(R, force[0], force[1], force[2], vbar, ubar, n);
  return cudaGetLastError();
}

cudaError_t launch_adj_halo(const HaloBox& hb, int nsm, cudaStream_t st) {
  const long long n = (long long)(hb.hi[0] - hb.lo[0] + 1) * (hb.hi[1] - hb.lo[1] + 1) * (hb.hi[2] - hb.lo[2] + 1);
  adj_halo_kernel<<<grid256(n, nsm), 256, 0, st>>>(hb, n);
  return cudaGetLastError();
}

}  // namespace amrs
