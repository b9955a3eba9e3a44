// KEEP split-form + viscous RHS and the fused RK-stage epilogue.
//
// Three kernels per stage (all flattened over a box list):
//   prims_kernel     cons2prim over grow(box, gq)            (src/rhs/CNS_hydro_K.h:15-34)
//   visc_cell_kernel cell-centred viscous fluxes, grow(box,1) (src/rhs/CNS_hydro_K.h:108-172)
//   keep_face_kernel KEEP face fluxes (src/rhs/CentralKEEP.h:40-145), viscous face
//                    averages (src/rhs/CNS_hydro_K.h:254-261), flux divergence
//                    (src/tim/CNS_advance.cpp:384-390) and the stage's BLAS-1
//                    program (src/tim/CNS_advance.cpp:51-166), fused.
//
// GB300's FP64 pipe (about 1 TFLOP/s) is ~60x slower than its HBM relative
// to this kernel's 9 flop/byte, so primitives and viscous cell fluxes are
// produced once per cell into HBM scratch instead of being recomputed for
// every tile halo.  The face kernel streams z-planes through shared memory
// (2-deep ring, filled by TMA when the layout allows) and evaluates every
// KEEP pair term once: a pair (a+l, a) feeds l faces, so it is stored in
// shared memory (x, y) or carried in registers (z) and reused.
#include <atomic>
#include "amrs_boxes.cuh"
#include "amrs_kernels.h"
#include "tma.cuh"

namespace amrs {

// ------------------------------------------------------------- prims ----
__global__ void __launch_bounds__(256) prims_kernel(BoxTable tb, int s_in) {
  if (list_idle(tb)) return;
  const long long total = tb.pcell[tb.n];
  const int g = tb.gq;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < total;
       c += (long long)gridDim.x * blockDim.x) {
    const int b = find_box_ll(tb.pcell, tb.n, c);
    const BoxRec& R = tb.box[b];
    const int l = (int)(c - tb.pcell[b]);
    const int nx = R.hi[0] - R.lo[0] + 1 + 2 * g, ny = R.hi[1] - R.lo[1] + 1 + 2 * g;
    const int i = l % nx + R.lo[0] - g;
    const int t = l / nx;
    const int j = t % ny + R.lo[1] - g;
    const int k = t / ny + R.lo[2] - g;
    const DArr U = R.slot[s_in];
    const long long o = U.off(i, j, k);
    double u[5];
#pragma unroll
    for (int n = 0; n < 5; ++n) u[n] = U.p[o + n * U.ns];
    double q[NQ];
    cons2prim(u, q, tb.cls[R.cl]);
    const long long oq = R.q.off(i, j, k);
#pragma unroll
    for (int n = 0; n < NQ; ++n) R.q.p[oq + n * R.q.ns] = q[n];
  }
}

// ------------------------------------------------- viscous cell fluxes ----
__global__ void __launch_bounds__(256) visc_cell_kernel(BoxTable tb) {
  if (list_idle(tb)) return;
  const long long total = tb.vcell[tb.n];
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < total;
       c += (long long)gridDim.x * blockDim.x) {
    const int b = find_box_ll(tb.vcell, tb.n, c);
    const BoxRec& R = tb.box[b];
    const int l = (int)(c - tb.vcell[b]);
    const int nx = R.hi[0] - R.lo[0] + 3, ny = R.hi[1] - R.lo[1] + 3;
    const int i = l % nx + R.lo[0] - 1;
    const int t = l / nx;
    const int j = t % ny + R.lo[1] - 1;
    const int k = t / ny + R.lo[2] - 1;
    const DArr Q = R.q;
    const long long o = Q.off(i, j, k);
    const long long sx = 1, sy = Q.js, sz = Q.ks, sn = Q.ns;
    double qc[NQ], qxm[NQ], qxp[NQ], qym[NQ], qyp[NQ], qzm[NQ], qzp[NQ];
#pragma unroll
    for (int n = QU; n <= QT; ++n) {
      qc[n] = Q.p[o + n * sn];
      qxm[n] = Q.p[o - sx + n * sn];
      qxp[n] = Q.p[o + sx + n * sn];
      qym[n] = Q.p[o - sy + n * sn];
      qyp[n] = Q.p[o + sy + n * sn];
      qzm[n] = Q.p[o - sz + n * sn];
      qzp[n] = Q.p[o + sz + n * sn];
    }
    double f[NVF];
    if (R.walls && (j == R.wrow_lo || j == R.wrow_hi)) {
      // ghost row of a code-6 y wall: one-sided y derivatives into the box
      const int loc = (j == R.wrow_lo) ? 0 : 1;
      const long long s1 = loc == 0 ? sy : -sy;
      double q1[NQ], q2[NQ];
#pragma unroll
      for (int n = QU; n <= QT; ++n) {
        q1[n] = Q.p[o + s1 + n * sn];
        q2[n] = Q.p[o + 2 * s1 + n * sn];
      }
      viscous_wall_cell(loc, qc, qxm, qxp, q1, q2, qzm, qzp, R.dxinv, tb.cls[R.cl], f);
    } else {
      viscous_cell(qc, qxm, qxp, qym, qyp, qzm, qzp, R.dxinv, tb.cls[R.cl], f);
    }
    const long long ov = R.vf.off(i, j, k);
#pragma unroll
    for (int n = 0; n < NVF; ++n) R.vf.p[ov + n * R.vf.ns] = f[n];
  }
}

// ------------------------------------------------ fused face kernel -----
// Products of the divergence epilogue on the integer pipe, one bit per
// direction (see kmul).
#ifndef AMRS_DIV_IMUL
#define AMRS_DIV_IMUL 0x4
#endif

template <int ORDER> struct KeepCfg {
  static constexpr int H = ORDER / 2;
  static constexpr int QS_CAP = (ORDER == 6) ? 544 : 480;  // (tx+6)*(ty+2H) capacity
  static constexpr int T_CAP = 352;                         // pair-term tile capacity per level
  static constexpr int F_CAP = 288;                         // face-flux tile capacity
  static constexpr int NLEV = (H > 1) ? H - 1 : 1;          // stored separations l = 2..H
  static constexpr int SMEM_DOUBLES = 2 * NQ * QS_CAP + 2 * NLEV * 5 * T_CAP + 2 * 5 * F_CAP;
};

template <int ORDER> int keep_smem_bytes() { return KeepCfg<ORDER>::SMEM_DOUBLES * 8 + 256; }

__device__ __forceinline__ void keep_coeffs(int order, double c[3]) {
  // CPU-branch coefficients of the reference (src/CNS.cpp:241-252)
  if (order == 6) { c[0] = 6.0 / 4; c[1] = -6.0 / 20; c[2] = 2.0 / 60; }
  else if (order == 4) { c[0] = 4.0 / 3; c[1] = -2.0 / 12; c[2] = 0.0; }
  else { c[0] = 1.0; c[1] = 0.0; c[2] = 0.0; }
}

__device__ __forceinline__ void ld_q(const DArr& Q, int i, int j, int k, double* q) {
  const long long o = Q.off(i, j, k);
#pragma unroll
  for (int n = 0; n < NQ; ++n) q[n] = Q.p[o + n * Q.ns];
}
__device__ __forceinline__ void ld_qs(const double* buf, int idx, int QS, double* q) {
#pragma unroll
  for (int n = 0; n < NQ; ++n) q[n] = buf[n * QS + idx];
}

// One work item = one (tx x ty) column tile of one box over a chunk of z.
template <int ORDER, bool VISC, bool SRC>
__global__ void __launch_bounds__(F_THREADS, (ORDER == 6) ? 1 : 2)
keep_face_kernel(BoxTable tb, int s_in, int s_s1, int s_out, DProg prog_in, int rhs_only, TmaDesc tma,
                 int* err) {
  using C = KeepCfg<ORDER>;
  constexpr int H = C::H;
  if (list_idle(tb)) return;  // uniform over the CTA: before any barrier
  const DProg prog = resolve_prog(prog_in);
  extern __shared__ __align__(128) unsigned char smem_raw[];
  double* smem = reinterpret_cast<double*>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127));
  double* qsbuf = smem;                                   // [2][NQ][QS_CAP]
  double* tsx = qsbuf + 2 * NQ * C::QS_CAP;               // [NLEV][5][T_CAP]
  double* tsy = tsx + C::NLEV * 5 * C::T_CAP;             // [NLEV][5][T_CAP]
  double* fsx = tsy + C::NLEV * 5 * C::T_CAP;             // [5][F_CAP]
  double* fsy = fsx + 5 * C::F_CAP;                       // [5][F_CAP]
  __shared__ __align__(8) unsigned long long mbar[2];

  const int tid = threadIdx.x;
  double coef[3];
  keep_coeffs(ORDER, coef);
  unsigned int phase_bits = 0u;
  const bool use_tma = tma.enabled != 0;
  if (use_tma) {
    if (tid == 0) { mbar_init(&mbar[0], 1); mbar_init(&mbar[1], 1); fence_mbar_init(); }
    __syncthreads();
  }

  // balanced static schedule: this CTA's segments cover an equal share of
  // the (tile column x plane) work of the whole list
  const int sbeg = tb.cta_seg[blockIdx.x], send = tb.cta_seg[blockIdx.x + 1];
  for (int sgi = sbeg; sgi < send; ++sgi) {
    const int4 sg = tb.seg[sgi];
    const int b = sg.x;
    const BoxRec& R = tb.box[b];
    const int tyi = sg.y / R.ntx, txi = sg.y - (sg.y / R.ntx) * R.ntx;
    const int TX = R.tx, TY = R.ty;
    const int x0 = R.lo[0] + txi * TX, y0 = R.lo[1] + tyi * TY;
    const int txw = min(TX, R.hi[0] + 1 - x0), tyw = min(TY, R.hi[1] + 1 - y0);
    const int k0 = sg.z;
    const int k1 = sg.w;
    const int QP = TX + 6, QR = TY + 2 * H, QS = QP * QR;
    const int TXP = TX + H;  // row pitch of x pair terms
    const DArr Q = R.q, VF = R.vf;
    const DArr Uin = R.slot[s_in], U1 = R.slot[s_s1], Uo = R.slot[s_out];
    const double dxi0 = R.dxinv[0], dxi1 = R.dxinv[1], dxi2 = R.dxinv[2];
    const bool src = SRC && tb.cls[R.cl].source != 0;  // SRC: a list with a source term
    // allocation bounds of Q (grow(box,3))
    const int qlo0 = R.lo[0] - NGHOST, qhi0 = R.hi[0] + NGHOST;
    const int qlo1 = R.lo[1] - NGHOST, qhi1 = R.hi[1] + NGHOST;

    // own column (one per thread while tid < txw*tyw)
    const bool has_col = tid < txw * tyw;
    const int ca = has_col ? tid % txw : 0;
    const int cb = has_col ? tid / txw : 0;
    const int ci = x0 + ca, cj = y0 + cb;

    // z carries: Tz[l][m] = T_l(k+1-l+m) for m=0..l-2 (l>=2); ring of Q(k+1..k+H-1)
    double tz[3][2][5];
    double ring[3][NQ];
    double fzprev[5];
    double fzk[4];
    if (has_col) {
      // prologue: F_z at face k0 (between k0-1 and k0) and carries
      double qcol[2 * 3][NQ];  // planes k0-H .. k0+H-1
#pragma unroll
      for (int p = 0; p < 2 * H; ++p) ld_q(Q, ci, cj, k0 - H + p, qcol[p]);
      double F[5];
      // l = 1: T_1(k0-1) = pair (k0, k0-1)
      keep_pair<2>(qcol[H], qcol[H - 1], coef[0], F);
#pragma unroll
      for (int l = 2; l <= H; ++l) {
#pragma unroll
        for (int m = 0; m < l; ++m) {
          const int a = -l + m;  // T_l(k0+a), pair (k0+a+l, k0+a)
          double T[5];
          keep_pair<2>(qcol[H + a + l], qcol[H + a], coef[l - 1], T);
#pragma unroll
          for (int n = 0; n < 5; ++n) F[n] = F[n] + T[n];
          if (m >= 1) {
#pragma unroll
            for (int n = 0; n < 5; ++n) tz[l - 1][m - 1][n] = T[n];
          }
        }
      }
      if (VISC) {
        const long long om = VF.off(ci, cj, k0 - 1), o0 = VF.off(ci, cj, k0);
#pragma unroll
        for (int n = 0; n < 4; ++n) {
          const double a = VF.p[om + (8 + n) * VF.ns], c0 = VF.p[o0 + (8 + n) * VF.ns];
          F[1 + n] = fma(0.5, a + c0, F[1 + n]);
          fzk[n] = c0;
        }
      }
#pragma unroll
      for (int n = 0; n < 5; ++n) fzprev[n] = F[n];
#pragma unroll
      for (int p = 0; p < H - 1; ++p)
#pragma unroll
        for (int n = 0; n < NQ; ++n) ring[p][n] = qcol[H + 1 + p][n];
    }

    // first plane into the ring
    int buf = 0;
    if (use_tma) {
      if (tid == 0) tma_load_plane(tma, b, &mbar[0], qsbuf, x0 - 3 - qlo0, y0 - H - qlo1, k0 - (R.lo[2] - NGHOST), QS * NQ * 8);
    }

    // Per plane k two barriers: A publishes plane k (and closes the faces
    // of plane k-1), B closes the pair terms of plane k.  Between A and B:
    // the divergence of plane k-1 (phase 3) and the pair terms of plane k
    // (phase 1); after B: the faces of plane k (phase 2).  One extra
    // iteration k = k1 runs the last plane's phase 3.
    double fznew[5];
    for (int k = k0; k <= k1; ++k) {
      const bool plane = k < k1;
      double* qs = qsbuf + buf * NQ * C::QS_CAP;
      // ---- phase 0: plane k of Q into shared memory
      if (plane) {
        if (use_tma) {
          if (!mbar_wait(&mbar[buf], (phase_bits >> buf) & 1u)) { if (tid == 0) atomicExch(err, 1); }
          phase_bits ^= (1u << buf);
        } else {
          // buffer buf held plane k-2, whose readers finished before the last barrier A
          const int nel = NQ * QS;
          for (int e = tid; e < nel; e += F_THREADS) {
            const int n = e / QS;
            const int r = e - n * QS;
            const int yy = r / QP, xx = r - (r / QP) * QP;
            const int gi = x0 - 3 + xx, gj = y0 - H + yy;
            double v = 0.0;
            if (gi >= qlo0 && gi <= qhi0 && gj >= qlo1 && gj <= qhi1) v = Q(gi, gj, k, n);
            qs[e] = v;
          }
        }
      }
      __syncthreads();  // A
      // the next plane into the other buffer: its plane k-1 was last read
      // by the faces of plane k-1, which every thread finished before A
      if (plane && use_tma && tid == 0 && k + 1 < k1) {
        fence_proxy_async();
        tma_load_plane(tma, b, &mbar[buf ^ 1], qsbuf + (buf ^ 1) * NQ * C::QS_CAP, x0 - 3 - qlo0, y0 - H - qlo1,
                       k + 1 - (R.lo[2] - NGHOST), QS * NQ * 8);
      }

      // ---- phase 3 of plane k-1: divergence + stage program for the own cell
      if (k > k0 && has_col) {
        const int kc = k - 1;
        const long long oin = Uin.off(ci, cj, kc), o1 = U1.off(ci, cj, kc), oo = Uo.off(ci, cj, kc);
#pragma unroll
        for (int n = 0; n < 5; ++n) {
          const double* fx = fsx + n * C::F_CAP + cb * (TX + 1) + ca;
          const double* fy = fsy + n * C::F_CAP + cb * TX + ca;
          double ds = kmul<AMRS_DIV_IMUL & 1>(dxi0, fx[0] - fx[1]) + kmul<(AMRS_DIV_IMUL >> 1) & 1>(dxi1, fy[0] - fy[TX]) +
                      kmul<(AMRS_DIV_IMUL >> 2) & 1>(dxi2, fzprev[n] - fznew[n]);
          if (src) ds = add_source(tb.cls[R.cl], Uin.p, oin, Uin.ns, n, ds);
          if (rhs_only) {
            Uo.p[oo + n * Uo.ns] = ds;
          } else {
            double reg[3];
            reg[0] = U1.p[o1 + n * U1.ns];
            reg[1] = Uin.p[oin + n * Uin.ns];
            reg[2] = ds;
            apply_prog(prog, reg);
            Uo.p[oo + n * Uo.ns] = reg[1];
          }
          fzprev[n] = fznew[n];
        }
      }
      if (!plane) break;

      // ---- phase 1: stored pair terms (x, y) and the z face above plane k
      if (has_col) {
        double qk[NQ], qtop[NQ];
        ld_qs(qs, (cb + H) * QP + (ca + 3), QS, qk);
        ld_q(Q, ci, cj, k + H, qtop);
        // T_l(k) = pair (k+l, k), l = 1..H
        double T1[5];
        keep_pair<2>(H == 1 ? qtop : ring[0], qk, coef[0], T1);
#pragma unroll
        for (int n = 0; n < 5; ++n) fznew[n] = T1[n];
#pragma unroll
        for (int l = 2; l <= H; ++l) {
          double Tn[5];
          keep_pair<2>(l == H ? qtop : ring[l - 1], qk, coef[l - 1], Tn);
          // F += T_l(k+1-l+m), m = 0..l-1 (m = l-1 is the new term)
#pragma unroll
          for (int m = 0; m < l - 1; ++m)
#pragma unroll
            for (int n = 0; n < 5; ++n) fznew[n] = fznew[n] + tz[l - 1][m][n];
#pragma unroll
          for (int n = 0; n < 5; ++n) fznew[n] = fznew[n] + Tn[n];
          // shift carries: drop T_l(k+1-l), append T_l(k)
#pragma unroll
          for (int m = 0; m < l - 2; ++m)
#pragma unroll
            for (int n = 0; n < 5; ++n) tz[l - 1][m][n] = tz[l - 1][m + 1][n];
#pragma unroll
          for (int n = 0; n < 5; ++n) tz[l - 1][l - 2][n] = Tn[n];
        }
        if (VISC) {
          const long long o1 = VF.off(ci, cj, k + 1);
#pragma unroll
          for (int n = 0; n < 4; ++n) {
            const double c1 = VF.p[o1 + (8 + n) * VF.ns];
            fznew[1 + n] = fma(0.5, fzk[n] + c1, fznew[1 + n]);
            fzk[n] = c1;
          }
        }
        // ring shift: Q(k+2..k+H) become Q(k+1..k+H-1) of the next plane
#pragma unroll
        for (int p = 0; p < H - 2; ++p)
#pragma unroll
          for (int n = 0; n < NQ; ++n) ring[p][n] = ring[p + 1][n];
        if (H >= 2) {
#pragma unroll
          for (int n = 0; n < NQ; ++n) ring[H - 2][n] = qtop[n];
        }
      }
      if (H >= 2) {
        // x: T_l(a, row) for a in [-l, txw-1]; y: T_l(col, b) for b in [-l, tyw-1]
        int nxit = 0, nyit = 0;
#pragma unroll
        for (int l = 2; l <= H; ++l) { nxit += (txw + l) * tyw; nyit += txw * (tyw + l); }
        for (int e = tid; e < nxit + nyit; e += F_THREADS) {
          double q1[NQ], q2[NQ], T[5];
          if (e < nxit) {
            int r = e, l = 2;
#pragma unroll
            for (int ll = 2; ll < H; ++ll) {
              if (r >= (txw + ll) * tyw) { r -= (txw + ll) * tyw; l = ll + 1; }
            }
            const int w2 = txw + l;
            const int row = r / w2, a = r - row * w2 - l;
            const int base = (row + H) * QP + 3;
            ld_qs(qs, base + a + l, QS, q1);
            ld_qs(qs, base + a, QS, q2);
            keep_pair<0>(q1, q2, coef[l - 1], T);
            double* dst = tsx + (l - 2) * 5 * C::T_CAP + row * TXP + (a + l);
#pragma unroll
            for (int n = 0; n < 5; ++n) dst[n * C::T_CAP] = T[n];
          } else {
            int r = e - nxit, l = 2;
#pragma unroll
            for (int ll = 2; ll < H; ++ll) {
              if (r >= txw * (tyw + ll)) { r -= txw * (tyw + ll); l = ll + 1; }
            }
            const int bb = r / txw - l, col = r - (r / txw) * txw;
            ld_qs(qs, (bb + l + H) * QP + col + 3, QS, q1);
            ld_qs(qs, (bb + H) * QP + col + 3, QS, q2);
            keep_pair<1>(q1, q2, coef[l - 1], T);
            double* dst = tsy + (l - 2) * 5 * C::T_CAP + (bb + l) * TX + col;
#pragma unroll
            for (int n = 0; n < 5; ++n) dst[n * C::T_CAP] = T[n];
          }
        }
      }
      __syncthreads();

      // ---- phase 2: x faces f in [0, txw] and y faces f in [0, tyw]
      {
        const int nxf = (txw + 1) * tyw, nyf = txw * (tyw + 1);
        // items in reverse thread order: the last, partial round of faces
        // falls on the last warps, while the partial round of pair terms
        // before the barrier fell on the first ones (measured 0.2% faster)
        for (int e = F_THREADS - 1 - tid; e < nxf + nyf; e += F_THREADS) {
          double F[5], q1[NQ], q2[NQ];
          if (e < nxf) {
            const int row = e / (txw + 1), f = e - row * (txw + 1);
            const int base = (row + H) * QP + 3;
            ld_qs(qs, base + f, QS, q1);
            ld_qs(qs, base + f - 1, QS, q2);
            keep_pair<0>(q1, q2, coef[0], F);
#pragma unroll
            for (int l = 2; l <= H; ++l)
#pragma unroll
              for (int m = 0; m < l; ++m) {
                const double* src = tsx + (l - 2) * 5 * C::T_CAP + row * TXP + (f - l + m + l);
#pragma unroll
                for (int n = 0; n < 5; ++n) F[n] = F[n] + src[n * C::T_CAP];
              }
            if (VISC) {
              const long long oR = VF.off(x0 + f, y0 + row, k);
#pragma unroll
              for (int n = 0; n < 4; ++n) F[1 + n] = fma(0.5, VF.p[oR - 1 + n * VF.ns] + VF.p[oR + n * VF.ns], F[1 + n]);
            }
            double* dst = fsx + row * (TX + 1) + f;
#pragma unroll
            for (int n = 0; n < 5; ++n) dst[n * C::F_CAP] = F[n];
          } else {
            const int r = e - nxf;
            const int f = r / txw, col = r - (r / txw) * txw;
            ld_qs(qs, (f + H) * QP + col + 3, QS, q1);
            ld_qs(qs, (f - 1 + H) * QP + col + 3, QS, q2);
            const int jf = y0 + f;
            if (R.walls && (jf <= R.red_lo || (jf >= R.red_hi && jf <= R.hi[1]))) {
              // next to a code-6 y wall: second-order KEEP (halfsten 1, coefficient 1)
              keep_pair<1>(q1, q2, 1.0, F);
            } else {
              keep_pair<1>(q1, q2, coef[0], F);
#pragma unroll
              for (int l = 2; l <= H; ++l)
#pragma unroll
                for (int m = 0; m < l; ++m) {
                  const double* src = tsy + (l - 2) * 5 * C::T_CAP + (f - l + m + l) * TX + col;
#pragma unroll
                  for (int n = 0; n < 5; ++n) F[n] = F[n] + src[n * C::T_CAP];
                }
            }
            if (VISC) {
              const long long oR = VF.off(x0 + col, y0 + f, k);
#pragma unroll
              for (int n = 0; n < 4; ++n)
                F[1 + n] = fma(0.5, VF.p[oR - VF.js + (4 + n) * VF.ns] + VF.p[oR + (4 + n) * VF.ns], F[1 + n]);
            }
            double* dst = fsy + f * TX + col;
#pragma unroll
            for (int n = 0; n < 5; ++n) dst[n * C::F_CAP] = F[n];
          }
        }
      }
      // phase 3 of this plane (its divergence) runs in the next iteration,
      // after the barrier that also publishes the next plane
      buf ^= 1;
    }
    // the TMA ring is drained at the last plane; nothing is in flight here
  }
}

// explicit instantiations + launchers
template <int ORDER, bool VISC, bool SRC>
static cudaError_t launch_face_t(const BoxTable& tb, int s_in, int s_s1, int s_out, const DProg& prog, int rhs_only,
                                 const TmaDesc& tma, int* err, int grid, cudaStream_t st) {
  const int smem = keep_smem_bytes<ORDER>();
  // the shared-memory opt-in is a per-device function attribute: set it once
  // for each device this process launches on (devices 0..63 tracked)
  static std::atomic<unsigned long long> attr_set{0ull};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const unsigned long long bit = 1ull << (dev & 63);
  if (dev >= 64 || !(attr_set.load() & bit)) {
    e = cudaFuncSetAttribute(keep_face_kernel<ORDER, VISC, SRC>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    attr_set.fetch_or(bit);
  }
  keep_face_kernel<ORDER, VISC, SRC><<<grid, F_THREADS, smem, st>>>(tb, s_in, s_s1, s_out, prog, rhs_only, tma, err);
  return cudaGetLastError();
}

cudaError_t launch_prims(const BoxTable& tb, int s_in, long long ncells, int nsm, cudaStream_t st) {
  if (ncells <= 0) return cudaSuccess;
  long long blocks = (ncells + 255) / 256;
  const long long cap = (long long)nsm * 8;
  if (blocks > cap) blocks = cap;
  prims_kernel<<<(int)blocks, 256, 0, st>>>(tb, s_in);
  return cudaGetLastError();
}

cudaError_t launch_visc(const BoxTable& tb, long long ncells, int nsm, cudaStream_t st) {
  if (ncells <= 0) return cudaSuccess;
  long long blocks = (ncells + 255) / 256;
  const long long cap = (long long)nsm * 8;
  if (blocks > cap) blocks = cap;
  visc_cell_kernel<<<(int)blocks, 256, 0, st>>>(tb);
  return cudaGetLastError();
}

cudaError_t launch_keep_face(int order, bool visc, bool src, const BoxTable& tb, int s_in, int s_s1, int s_out,
                             const DProg& prog, int rhs_only, const TmaDesc& tma, int* err, int grid, int nsm,
                             cudaStream_t st) {
  (void)nsm;
  if (grid <= 0) return cudaSuccess;
#define AMRS_FACE(O, V, S) launch_face_t<O, V, S>(tb, s_in, s_s1, s_out, prog, rhs_only, tma, err, grid, st)
#define AMRS_FACE_VS(O) \
  (visc ? (src ? AMRS_FACE(O, true, true) : AMRS_FACE(O, true, false)) \
        : (src ? AMRS_FACE(O, false, true) : AMRS_FACE(O, false, false)))
  if (order == 2) return AMRS_FACE_VS(2);
  if (order == 4) return AMRS_FACE_VS(4);
  return AMRS_FACE_VS(6);
#undef AMRS_FACE_VS
#undef AMRS_FACE
}

int keep_ctas_per_sm(int order) { return order == 6 ? 1 : 2; }

bool keep_tile_fits(int order, int tx, int ty) {
  if (tx < 8 || ty < 1 || (tx % 2) || tx * ty > F_THREADS) return false;
  const int H = order / 2;
  int qcap = order == 6 ? KeepCfg<6>::QS_CAP : KeepCfg<4>::QS_CAP;
  if ((tx + 6) * (ty + 2 * H) > qcap) return false;
  if ((tx + H) * ty > KeepCfg<4>::T_CAP || tx * (ty + H) > KeepCfg<4>::T_CAP) return false;
  if ((tx + 1) * ty > KeepCfg<4>::F_CAP || tx * (ty + 1) > KeepCfg<4>::F_CAP) return false;
  return true;
}

}  // namespace amrs
