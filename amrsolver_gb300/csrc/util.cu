// Ghost fill and time-step reduction kernels.
#include "amrs_kernels.h"
#include "ddiv.cuh"
#include "tma.cuh"

namespace amrs {

// ---------------------------------------------------------------- halo ----
// Single-level FillPatch for a box that is the whole domain.  Each ghost
// cell takes the value of the valid cell obtained by mapping every
// out-of-range coordinate independently (periodic wrap, foextrap clamp,
// reflection), with a sign flip for every reflect_odd mapping; this equals
// AMReX's sequential fill (periodic images, then physical BCs direction by
// direction).  BC types per component: src/set/CNS_setup.cpp:18-31.
__device__ __forceinline__ int map_coord(int c, int lo, int hi, int bcl, int bch, int comp, int dir, bool& flip) {
  if (c >= lo && c <= hi) return c;
  const int n = hi - lo + 1;
  const bool low = c < lo;
  const int phys = low ? bcl : bch;
  if (phys == -1) {  // periodic
    int r = (c - lo) % n;
    if (r < 0) r += n;
    return lo + r;
  }
  if (phys == 2) return low ? lo : hi;  // foextrap
  const bool vel = comp >= UMX && comp <= UMZ;
  const bool normal = comp == UMX + dir;
  bool odd = false;
  if (phys == 3 || phys == 4) odd = vel && normal;
  else if (phys == 5) odd = vel;
  if (odd) flip = !flip;
  return low ? 2 * lo - c - 1 : 2 * hi - c + 1;
}

// A ghost coordinate beyond an ext_dir side (codes 1 inflow and 6
// user-defined: the problem's bcnormal fills those cells, src/set/bcs.cpp):
// the library leaves such cells, corners included, as the caller stored them.
__device__ __forceinline__ bool ext_dir_ghost(int c, int lo, int hi, int bcl, int bch) {
  return (c < lo && (bcl == 1 || bcl == 6)) || (c > hi && (bch == 1 || bch == 6));
}

__global__ void __launch_bounds__(256) halo_kernel(HaloBox hb) {
  const int g = NGHOST;
  const int nx = hb.hi[0] - hb.lo[0] + 1 + 2 * g, ny = hb.hi[1] - hb.lo[1] + 1 + 2 * g,
            nz = hb.hi[2] - hb.lo[2] + 1 + 2 * g;
  const long long total = (long long)nx * ny * nz;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < total;
       c += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(c % nx) + hb.lo[0] - g;
    const long long t = c / nx;
    const int j = (int)(t % ny) + hb.lo[1] - g;
    const int k = (int)(t / ny) + hb.lo[2] - g;
    const bool inside = i >= hb.lo[0] && i <= hb.hi[0] && j >= hb.lo[1] && j <= hb.hi[1] && k >= hb.lo[2] &&
                        k <= hb.hi[2];
    if (inside) continue;
    if (ext_dir_ghost(i, hb.lo[0], hb.hi[0], hb.bc_lo[0], hb.bc_hi[0]) ||
        ext_dir_ghost(j, hb.lo[1], hb.hi[1], hb.bc_lo[1], hb.bc_hi[1]) ||
        ext_dir_ghost(k, hb.lo[2], hb.hi[2], hb.bc_lo[2], hb.bc_hi[2]))
      continue;
    for (int n = 0; n < hb.ncomp; ++n) {
      bool flip = false;
      const int si = map_coord(i, hb.lo[0], hb.hi[0], hb.bc_lo[0], hb.bc_hi[0], n, 0, flip);
      const int sj = map_coord(j, hb.lo[1], hb.hi[1], hb.bc_lo[1], hb.bc_hi[1], n, 1, flip);
      const int sk = map_coord(k, hb.lo[2], hb.hi[2], hb.bc_lo[2], hb.bc_hi[2], n, 2, flip);
      const double v = hb.u(si, sj, sk, n);
      hb.u(i, j, k, n) = flip ? -v : v;
    }
  }
}

// Ghost fill of every box of a list, each box being its own domain (an
// ensemble member or an isolated box), one launch for all boxes.
__global__ void __launch_bounds__(256) halo_list_kernel(BoxTable tb, const long long* gpre, int slot, int bl0, int bl1,
                                                        int bl2, int bh0, int bh1, int bh2) {
  if (list_idle(tb)) return;
  const long long total = gpre[tb.n];
  const int g = NGHOST;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < total;
       c += (long long)gridDim.x * blockDim.x) {
    const int b = find_box_ll(gpre, tb.n, c);
    const BoxRec& R = tb.box[b];
    const int l = (int)(c - gpre[b]);
    const int nx = R.hi[0] - R.lo[0] + 1 + 2 * g, ny = R.hi[1] - R.lo[1] + 1 + 2 * g;
    const int i = l % nx + R.lo[0] - g;
    const int t = l / nx;
    const int j = t % ny + R.lo[1] - g;
    const int k = t / ny + R.lo[2] - g;
    const bool inside = i >= R.lo[0] && i <= R.hi[0] && j >= R.lo[1] && j <= R.hi[1] && k >= R.lo[2] &&
                        k <= R.hi[2];
    if (inside) continue;
    if (ext_dir_ghost(i, R.lo[0], R.hi[0], bl0, bh0) || ext_dir_ghost(j, R.lo[1], R.hi[1], bl1, bh1) ||
        ext_dir_ghost(k, R.lo[2], R.hi[2], bl2, bh2))
      continue;
    const DArr U = R.slot[slot];
    for (int n = 0; n < NCONS; ++n) {
      bool flip = false;
      const int si = map_coord(i, R.lo[0], R.hi[0], bl0, bh0, n, 0, flip);
      const int sj = map_coord(j, R.lo[1], R.hi[1], bl1, bh1, n, 1, flip);
      const int sk = map_coord(k, R.lo[2], R.hi[2], bl2, bh2, n, 2, flip);
      const double v = U(si, sj, sk, n);
      U(i, j, k, n) = flip ? -v : v;
    }
  }
}

// Single-level FillPatch of a level whose boxes tile the domain: a ghost
// cell of box b maps to a cell of the domain exactly as in halo_kernel
// (periodic images, physical BCs) and takes that cell's value from the box
// that owns it (owner table built on the host, one entry per cell of every
// grow(box,3), in the gpre order).  Sources are valid cells only, so the
// fill has no order dependence between boxes and is bit-identical to the
// fill of one box covering the domain.
__global__ void __launch_bounds__(256) halo_level_kernel(BoxTable tb, const long long* gpre, const int* owner,
                                                         int slot, LevelDomain dom) {
  if (list_idle(tb)) return;
  const long long total = gpre[tb.n];
  const int g = NGHOST;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < total;
       c += (long long)gridDim.x * blockDim.x) {
    const int src = owner[c];
    if (src < 0) continue;  // a valid cell
    const int b = find_box_ll(gpre, tb.n, c);
    const BoxRec& R = tb.box[b];
    const int l = (int)(c - gpre[b]);
    const int nx = R.hi[0] - R.lo[0] + 1 + 2 * g, ny = R.hi[1] - R.lo[1] + 1 + 2 * g;
    const int i = l % nx + R.lo[0] - g;
    const int t = l / nx;
    const int j = t % ny + R.lo[1] - g;
    const int k = t / ny + R.lo[2] - g;
    const DArr U = R.slot[slot];
    const DArr S = tb.box[src].slot[slot];
    for (int n = 0; n < NCONS; ++n) {
      bool flip = false;
      const int si = map_coord(i, dom.lo[0], dom.hi[0], dom.bc_lo[0], dom.bc_hi[0], n, 0, flip);
      const int sj = map_coord(j, dom.lo[1], dom.hi[1], dom.bc_lo[1], dom.bc_hi[1], n, 1, flip);
      const int sk = map_coord(k, dom.lo[2], dom.hi[2], dom.bc_lo[2], dom.bc_hi[2], n, 2, flip);
      const double v = S(si, sj, sk, n);
      U(i, j, k, n) = flip ? -v : v;
    }
  }
}

cudaError_t launch_halo_level(const BoxTable& tb, const long long* gpre, const int* owner, long long total, int slot,
                              const LevelDomain& dom, int nsm, cudaStream_t st) {
  long long blocks = (total + 255) / 256;
  if (blocks > (long long)nsm * 8) blocks = (long long)nsm * 8;
  if (blocks < 1) blocks = 1;
  halo_level_kernel<<<(int)blocks, 256, 0, st>>>(tb, gpre, owner, slot, dom);
  return cudaGetLastError();
}

cudaError_t launch_halo_list(const BoxTable& tb, const long long* gpre, long long total, int slot, const int bc_lo[3],
                             const int bc_hi[3], int nsm, cudaStream_t st) {
  long long blocks = (total + 255) / 256;
  if (blocks > (long long)nsm * 8) blocks = (long long)nsm * 8;
  if (blocks < 1) blocks = 1;
  halo_list_kernel<<<(int)blocks, 256, 0, st>>>(tb, gpre, slot, bc_lo[0], bc_lo[1], bc_lo[2], bc_hi[0], bc_hi[1],
                                                bc_hi[2]);
  return cudaGetLastError();
}

cudaError_t launch_halo(const HaloBox& hb, cudaStream_t st) {
  const long long total = (long long)(hb.hi[0] - hb.lo[0] + 7) * (hb.hi[1] - hb.lo[1] + 7) * (hb.hi[2] - hb.lo[2] + 7);
  long long blocks = (total + 255) / 256;
  if (blocks > 4096) blocks = 4096;
  halo_kernel<<<(int)blocks, 256, 0, st>>>(hb);
  return cudaGetLastError();
}

// ------------------------------------------------------ device bcnormal --
// The ghost cell (i, j, k) beyond a code-6 y side (side 0: below the domain,
// 1: above) from the first interior row jf, as cns_bcfill
// (src/set/bcs.cpp:40-100) calls the channel problem's bcnormal
// (exm/Channel/prob.h:158-186): x = prob_lo + (j + 0.5) dx of the ghost,
// dratio = de/di (ghost-to-wall over first-cell-to-wall distance), no-slip
// velocity (the interior velocity negated), the interior pressure, the wall
// temperature extrapolated, T = max(Tw + dratio (Tw - T_int), Tmin), and
// rho = p / (R T), written back as conserved variables.
__device__ void bcnormal_isothermal_cell(const DArr& U, int i, int j, int k, int jf, int side,
                                         const DClosures& c, const DBcNormal& bn) {
  const double rho = U(i, jf, k, URHO), mx = U(i, jf, k, UMX), my = U(i, jf, k, UMY), mz = U(i, jf, k, UMZ);
  const double et = U(i, jf, k, UET);
  const double ue = -mx / rho, ve = -my / rho, we = -mz / rho;
  const double eint = (et - 0.5 * (mx * mx + my * my + mz * mz) / rho) / rho;
  const double p = (c.gamma - 1.0) * rho * eint;
  const double Tint = p / (c.Rspec * rho);
  const double x = bn.prob_lo[1] + (double)(j + 0.5) * bn.dx[1];
  double di, de;
  if (side == 0) {
    di = (double)(jf + 0.5) * bn.dx[1] - bn.prob_lo[1];
    de = bn.prob_lo[1] - x;
  } else {
    di = bn.prob_hi[1] - (double)(jf + 0.5) * bn.dx[1];
    de = x - bn.prob_hi[1];
  }
  const double dratio = de / di;
  const double Te = rmax(bn.Tw + dratio * (bn.Tw - Tint), bn.Tmin);
  const double re = p / (c.Rspec * Te);
  const double ekin = 0.5 * (ue * ue + ve * ve + we * we);
  const double eint_e = p / (re * (c.gamma - 1.0));
  U(i, j, k, URHO) = re;
  U(i, j, k, UMX) = re * ue;
  U(i, j, k, UMY) = re * ve;
  U(i, j, k, UMZ) = re * we;
  U(i, j, k, UET) = re * (eint_e + ekin);
}

// One box that is the domain: every ghost row beyond a code-6 y side, over
// the whole grown x/z extent (the x/z ghost columns of the first interior
// row were filled by the library's fill before).
__global__ void __launch_bounds__(256) bcnormal_box_kernel(DArr U, int lo0, int lo1, int lo2, int hi0, int hi1,
                                                           int hi2, int wlo, int whi, DClosures c, DBcNormal bn) {
  const int g = NGHOST;
  const int nx = hi0 - lo0 + 1 + 2 * g, nz = hi2 - lo2 + 1 + 2 * g;
  const long long total = (long long)nx * nz * 2 * g;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(t % nx) + lo0 - g;
    const long long r = t / nx;
    const int k = (int)(r % nz) + lo2 - g;
    const int row = (int)(r / nz);  // 0..g-1 below, g..2g-1 above
    const int side = row >= g;
    if (side ? !whi : !wlo) continue;
    const int gi = side ? row - g + 1 : row + 1;  // ghost distance 1..g
    const int j = side ? hi1 + gi : lo1 - gi;
    bcnormal_isothermal_cell(U, i, j, k, side ? hi1 : lo1, side, c, bn);
  }
}

// Every box of a level whose y extent touches a code-6 side of the domain:
// the box's own ghost rows beyond that side (its first interior row and the
// ghost columns of it were filled by halo_level_kernel).
__global__ void __launch_bounds__(256) bcnormal_list_kernel(BoxTable tb, int slot, LevelDomain dom, DBcNormal bn) {
  if (list_idle(tb)) return;
  const int g = NGHOST;
  for (int b = blockIdx.y; b < tb.n; b += gridDim.y) {
    const BoxRec& R = tb.box[b];
    const bool wlo = dom.bc_lo[1] == 6 && R.lo[1] == dom.lo[1];
    const bool whi = dom.bc_hi[1] == 6 && R.hi[1] == dom.hi[1];
    if (!wlo && !whi) continue;
    const int nx = R.hi[0] - R.lo[0] + 1 + 2 * g, nz = R.hi[2] - R.lo[2] + 1 + 2 * g;
    const long long total = (long long)nx * nz * 2 * g;
    const DArr U = R.slot[slot];
    const DClosures& c = tb.cls[R.cl];
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
      const int i = (int)(t % nx) + R.lo[0] - g;
      const long long r = t / nx;
      const int k = (int)(r % nz) + R.lo[2] - g;
      const int row = (int)(r / nz);
      const int side = row >= g;
      if (side ? !whi : !wlo) continue;
      const int gi = side ? row - g + 1 : row + 1;
      const int j = side ? R.hi[1] + gi : R.lo[1] - gi;
      bcnormal_isothermal_cell(U, i, j, k, side ? R.hi[1] : R.lo[1], side, c, bn);
    }
  }
}

cudaError_t launch_bcnormal_box(const DArr& u, const int lo[3], const int hi[3], const int bc_lo[3],
                                const int bc_hi[3], const DClosures& cl, const DBcNormal& bn, cudaStream_t st) {
  const int wlo = bc_lo[1] == 6, whi = bc_hi[1] == 6;
  if (bn.kind != 1 || (!wlo && !whi)) return cudaSuccess;
  const long long total = (long long)(hi[0] - lo[0] + 7) * (hi[2] - lo[2] + 7) * 2 * NGHOST;
  long long blocks = (total + 255) / 256;
  if (blocks > 4096) blocks = 4096;
  bcnormal_box_kernel<<<(int)blocks, 256, 0, st>>>(u, lo[0], lo[1], lo[2], hi[0], hi[1], hi[2], wlo, whi, cl, bn);
  return cudaGetLastError();
}

cudaError_t launch_bcnormal_list(const BoxTable& tb, int slot, const LevelDomain& dom, const DBcNormal& bn, int nsm,
                                 cudaStream_t st) {
  if (bn.kind != 1 || (dom.bc_lo[1] != 6 && dom.bc_hi[1] != 6)) return cudaSuccess;
  const int gy = tb.n < nsm * 4 ? tb.n : nsm * 4;
  dim3 grid(8, (unsigned)(gy < 1 ? 1 : gy));
  bcnormal_list_kernel<<<grid, 256, 0, st>>>(tb, slot, dom, bn);
  return cudaGetLastError();
}

// ----------------------------------------------------------- time step ----
// cns_estdt (src/cls/CNS_K.h:12-47, z-velocity from UMY as there) reduced
// with min over cells.  Positive doubles order like their bit patterns, so
// the block minima meet in one unsigned 64-bit atomicMin; the result is the
// exact minimum whatever the order.
__global__ void __launch_bounds__(256) estdt_kernel(BoxTable tb, int s_in, long long total,
                                                     unsigned long long* bits) {
  if (list_idle(tb)) return;  // uniform over the grid
  unsigned long long best = ~0ull;
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < total;
       g += (long long)gridDim.x * blockDim.x) {
    int b = 0;
    {
      // valid-cell prefix = pcell when gq == 0; recompute from box sizes
      long long acc = 0;
      for (b = 0; b < tb.n; ++b) {
        const BoxRec& R = tb.box[b];
        const long long nc = (long long)(R.hi[0] - R.lo[0] + 1) * (R.hi[1] - R.lo[1] + 1) * (R.hi[2] - R.lo[2] + 1);
        if (g < acc + nc) { g -= acc; break; }
        acc += nc;
      }
      if (b == tb.n) break;
      const BoxRec& R = tb.box[b];
      const int nx = R.hi[0] - R.lo[0] + 1, ny = R.hi[1] - R.lo[1] + 1;
      const int l = (int)g;
      g += acc;
      const int i = l % nx + R.lo[0];
      const int t = l / nx;
      const int j = t % ny + R.lo[1];
      const int k = t / ny + R.lo[2];
      const DArr S = R.slot[s_in];
      const DClosures& cl = tb.cls[R.cl];
      const long long o = S.off(i, j, k);
      const double rho = S.p[o], mx = S.p[o + S.ns], my = S.p[o + 2 * S.ns], mz = S.p[o + 2 * S.ns];
      const double rhoinv = ddiv_rn(1.0, rmax(rho, 1.0e-40));
      const double vx = mx * rhoinv, vy = my * rhoinv, vz = mz * rhoinv;
      const double ke = 0.5 * rho * (vx * vx + vy * vy + vz * vz);
      const double rhoei = (S.p[o + 4 * S.ns] - ke);
      const double p = (cl.gamma - 1.0) * rhoei;
      const double cs = dsqrt_rn(cl.gamma * p * rhoinv);
      const double dtx = ddiv_rn(R.dx[0], fabs(vx) + cs);
      const double dty = ddiv_rn(R.dx[1], fabs(vy) + cs);
      const double dtz = ddiv_rn(R.dx[2], fabs(vz) + cs);
      const double dt = rmin(dtx, rmin(dty, dtz));
      const unsigned long long bb = (unsigned long long)__double_as_longlong(dt);
      if (dt >= 0.0 && bb < best) best = bb;
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long v = __shfl_down_sync(0xffffffffu, best, o);
    best = v < best ? v : best;
  }
  __shared__ unsigned long long sm[8];
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = best;
  __syncthreads();
  if (threadIdx.x < 8) {
    unsigned long long v = sm[threadIdx.x];
#pragma unroll
    for (int o = 4; o > 0; o >>= 1) {
      const unsigned long long w = __shfl_down_sync(0xffu, v, o);
      v = w < v ? w : v;
    }
    if (threadIdx.x == 0 && v != ~0ull) atomicMin(bits, v);
  }
}

__global__ void estdt_init(unsigned long long* bits) { *bits = ~0ull; }

__global__ void estdt_final(const unsigned long long* bits, double cfl, double* out) {
  const unsigned long long b = *bits;
  const double dt = (b == ~0ull) ? 1.7976931348623157e308 : __longlong_as_double((long long)b);
  *out = dt * cfl;
}

cudaError_t launch_estdt(const BoxTable& tb, int s_in, long long nvalid, double cfl, unsigned long long* bits,
                         double* dt_out, int nsm, cudaStream_t st) {
  estdt_init<<<1, 1, 0, st>>>(bits);
  long long blocks = (nvalid + 255) / 256;
  if (blocks > (long long)nsm * 4) blocks = (long long)nsm * 4;
  if (blocks < 1) blocks = 1;
  estdt_kernel<<<(int)blocks, 256, 0, st>>>(tb, s_in, nvalid, bits);
  estdt_final<<<1, 1, 0, st>>>(bits, cfl, dt_out);
  return cudaGetLastError();
}

// ------------------------------------------------- device time loop ----
// One launch of a captured step graph inside a conditional WHILE node runs
// CNS::advance steps with the reference's single-level dt control
// (computeInitialDt / computeNewDt, src/CNS.cpp:282-377) without host syncs.
__global__ void run_estdt_reset(RunCtl* c) {
  if (c->active) c->bits = ~0ull;
}

// After a step: time += dt, step += 1, the next dt (CFL: min(cfl * min
// dx/(|u|+c), change_max * dt), the last step clamped to stop_time with
// eps = 0.001 dt as the reference does), then whether to go on.
__global__ void run_step_done(RunCtl* c, cudaGraphConditionalHandle cond) {
  if (c->active) {
    c->time = c->time + c->dt;
    c->step += 1;
    if (c->use_cfl) {
      const unsigned long long b = c->bits;
      const double est = ((b == ~0ull) ? 1.7976931348623157e308 : __longlong_as_double((long long)b)) * c->cfl;
      const double grow = c->change_max * c->dt;
      double dt0 = (grow < est) ? grow : est;  // std::min(est, grow)
      const double eps = 0.001 * dt0;
      if (c->stop >= 0.0 && c->time + dt0 > c->stop - eps) dt0 = c->stop - c->time;
      c->dt = dt0;
    }
    c->active = (c->step < c->max_steps && c->time < c->stop) ? 1 : 0;
  }
  cudaGraphSetConditional(cond, c->active ? 1u : 0u);
}

// Initial dt (computeInitialDt: cfl * min dx/(|u|+c)) and whether to start.
__global__ void run_begin(RunCtl* c) {
  if (c->use_cfl) {
    const unsigned long long b = c->bits;
    c->dt = ((b == ~0ull) ? 1.7976931348623157e308 : __longlong_as_double((long long)b)) * c->cfl;
  }
  c->active = (c->step < c->max_steps && c->time < c->stop) ? 1 : 0;
}

// Valid cells of slot `from` into slot `to` for every box (the step's result
// back into the S1 slot the next step reads).
__global__ void __launch_bounds__(256) copy_slot_kernel(BoxTable tb, int from, int to, long long total) {
  if (list_idle(tb)) return;
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < total;
       g += (long long)gridDim.x * blockDim.x) {
    long long acc = 0;
    int b = 0;
    for (; b < tb.n; ++b) {
      const BoxRec& R = tb.box[b];
      const long long nc = (long long)(R.hi[0] - R.lo[0] + 1) * (R.hi[1] - R.lo[1] + 1) * (R.hi[2] - R.lo[2] + 1);
      if (g < acc + nc) break;
      acc += nc;
    }
    if (b == tb.n) break;
    const BoxRec& R = tb.box[b];
    const int nx = R.hi[0] - R.lo[0] + 1, ny = R.hi[1] - R.lo[1] + 1;
    const int l = (int)(g - acc);
    const int i = l % nx + R.lo[0];
    const int t = l / nx;
    const int j = t % ny + R.lo[1];
    const int k = t / ny + R.lo[2];
    const DArr A = R.slot[from], B = R.slot[to];
    const long long oa = A.off(i, j, k), ob = B.off(i, j, k);
#pragma unroll
    for (int n = 0; n < NCONS; ++n) B.p[ob + n * B.ns] = A.p[oa + n * A.ns];
  }
}

// Non-finite check of slot `slot` over the valid cells of every box: raises
// *flag when any component is a NaN or an infinity (exponent bits all ones,
// tested on the integer bits, so the FP64 pipe is not used).  One extra
// read of the slot (40 B per cell); run only when the caller opted in.
__global__ void __launch_bounds__(256) nonfinite_check_kernel(BoxTable tb, const long long* vpre, int slot,
                                                              long long total, int* flag) {
  if (list_idle(tb)) return;
  int bad = 0;
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < total;
       g += (long long)gridDim.x * blockDim.x) {
    const int b = find_box_ll(vpre, tb.n, g);
    const BoxRec& R = tb.box[b];
    const int nx = R.hi[0] - R.lo[0] + 1, ny = R.hi[1] - R.lo[1] + 1;
    const long long l = g - vpre[b];
    const int i = (int)(l % nx) + R.lo[0];
    const long long t = l / nx;
    const int j = (int)(t % ny) + R.lo[1], k = (int)(t / ny) + R.lo[2];
    const DArr A = R.slot[slot];
    const long long o = A.off(i, j, k);
#pragma unroll
    for (int n = 0; n < NCONS; ++n) {
      const unsigned long long bits = (unsigned long long)__double_as_longlong(A.p[o + n * A.ns]);
      bad |= (bits & 0x7ff0000000000000ull) == 0x7ff0000000000000ull;
    }
  }
  if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(flag, 1);
}

cudaError_t launch_nonfinite_check(const BoxTable& tb, const long long* vpre, int slot, long long nvalid, int* flag,
                                   int nsm, cudaStream_t st) {
  long long blocks = (nvalid + 255) / 256;
  if (blocks > (long long)nsm * 4) blocks = (long long)nsm * 4;
  if (blocks < 1) blocks = 1;
  nonfinite_check_kernel<<<(int)blocks, 256, 0, st>>>(tb, vpre, slot, nvalid, flag);
  return cudaGetLastError();
}

// ---------------------------------------------------- printTotal stats ----
// CNS::printTotal's primitive extrema and convective CFL table
// (src/CNS.cpp:532-611; pointCFL, src/cls/CNS_K.h:49-59) over the valid
// cells of every box.  Extrema do not depend on the order they are taken
// in, so each warp reduces with shuffles and lane 0 folds its values into
// order-preserving integer encodings with atomicMin/atomicMax: race-free,
// and the same bits on every run.  The CFL entry of direction d is
// max(|u_d + c|, |u_d - c|) * dt / dx_d per cell, maximised: rounding is
// monotonic, so this equals the reference's max(A0, A1) * dt / dx_d of the
// global maxima A0, A1.
__device__ __forceinline__ unsigned long long ord_enc(double x) {
  if (x == 0.0) x = 0.0;  // -0 counts as +0
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double ord_dec(unsigned long long e) {
  const unsigned long long b = (e >> 63) ? (e & 0x7fffffffffffffffull) : ~e;
  return __longlong_as_double((long long)b);
}

constexpr int NSTAT = 21;  // min[6], max[6], table[3][3]

__global__ void prim_stats_init(unsigned long long* cells) {
  const int t = threadIdx.x;
  if (t < NSTAT) cells[t] = t < 6 ? ~0ull : 0ull;
}

__global__ void __launch_bounds__(256) prim_stats_kernel(BoxTable tb, const long long* vpre, int slot, double dt,
                                                         double dx0, double dx1, double dx2, long long total,
                                                         unsigned long long* cells) {
  double mn[6], mx[6], t[9];
#pragma unroll
  for (int n = 0; n < 6; ++n) { mn[n] = __longlong_as_double(0x7ff0000000000000ll); mx[n] = -mn[n]; }
#pragma unroll
  for (int n = 0; n < 9; ++n) t[n] = 0.0;
  const double dxs[3] = {dx0, dx1, dx2};
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < total;
       g += (long long)gridDim.x * blockDim.x) {
    const int b = find_box_ll(vpre, tb.n, g);
    const BoxRec& R = tb.box[b];
    const DClosures& cl = tb.cls[R.cl];
    const int nx = R.hi[0] - R.lo[0] + 1, ny = R.hi[1] - R.lo[1] + 1;
    const long long l = g - vpre[b];
    const int i = (int)(l % nx) + R.lo[0];
    const long long tt = l / nx;
    const int j = (int)(tt % ny) + R.lo[1], k = (int)(tt / ny) + R.lo[2];
    double q[NQ];
    if (slot >= 0) {
      const DArr A = R.slot[slot];
      const long long o = A.off(i, j, k);
      double u[NCONS];
#pragma unroll
      for (int n = 0; n < NCONS; ++n) u[n] = A.p[o + n * A.ns];
      cons2prim(u, q, cl);
    } else {
      const DArr Q = R.q;
      const long long o = Q.off(i, j, k);
#pragma unroll
      for (int n = 0; n < 6; ++n) q[n] = Q.p[o + n * Q.ns];
    }
#pragma unroll
    for (int n = 0; n < 6; ++n) {
      mn[n] = fmin(mn[n], q[n]);
      mx[n] = fmax(mx[n], q[n]);
    }
    const double sos = dsqrt_rn(cl.gamma * cl.Rspec * q[QT]);
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const double a0 = fabs(q[QU + d] + sos), a1 = fabs(q[QU + d] - sos);
      t[3 * d] = fmax(t[3 * d], a0);
      t[3 * d + 1] = fmax(t[3 * d + 1], a1);
      t[3 * d + 2] = fmax(t[3 * d + 2], ddiv_rn(fmax(a0, a1) * dt, dxs[d]));
    }
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
#pragma unroll
    for (int n = 0; n < 6; ++n) {
      mn[n] = fmin(mn[n], __shfl_down_sync(0xffffffffu, mn[n], off));
      mx[n] = fmax(mx[n], __shfl_down_sync(0xffffffffu, mx[n], off));
    }
#pragma unroll
    for (int n = 0; n < 9; ++n) t[n] = fmax(t[n], __shfl_down_sync(0xffffffffu, t[n], off));
  }
  if ((threadIdx.x & 31) == 0) {
#pragma unroll
    for (int n = 0; n < 6; ++n) {
      if (mn[n] <= mx[n]) {  // this warp saw a cell
        atomicMin(&cells[n], ord_enc(mn[n]));
        atomicMax(&cells[6 + n], ord_enc(mx[n]));
      }
    }
#pragma unroll
    for (int n = 0; n < 9; ++n) atomicMax(&cells[12 + n], ord_enc(t[n]));
  }
}

__global__ void prim_stats_final(const unsigned long long* cells, double* out) {
  const int t = threadIdx.x;
  if (t < NSTAT) out[t] = ord_dec(cells[t]);
}

cudaError_t launch_prim_stats(const BoxTable& tb, const long long* vpre, int slot, double dt, const double dx[3],
                              long long nvalid, unsigned long long* cells, double* out, int nsm, cudaStream_t st) {
  prim_stats_init<<<1, 32, 0, st>>>(cells);
  long long blocks = (nvalid + 255) / 256;
  if (blocks > (long long)nsm * 4) blocks = (long long)nsm * 4;
  if (blocks < 1) blocks = 1;
  prim_stats_kernel<<<(int)blocks, 256, 0, st>>>(tb, vpre, slot, dt, dx[0], dx[1], dx[2], nvalid, cells);
  prim_stats_final<<<1, 32, 0, st>>>(cells, out);
  return cudaGetLastError();
}

// Conserved totals of slot `slot` over the valid cells of every box:
// per-block sums in a fixed order, then one block sums the partials in
// block order (deterministic; not the serial sum's rounding).
__global__ void __launch_bounds__(256) totals_partial_kernel(BoxTable tb, int slot, long long total, double* part) {
  double acc[NCONS] = {0, 0, 0, 0, 0};
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < total;
       g += (long long)gridDim.x * blockDim.x) {
    long long base = 0;
    int b = 0;
    for (; b < tb.n; ++b) {
      const BoxRec& R = tb.box[b];
      const long long nc = (long long)(R.hi[0] - R.lo[0] + 1) * (R.hi[1] - R.lo[1] + 1) * (R.hi[2] - R.lo[2] + 1);
      if (g < base + nc) break;
      base += nc;
    }
    if (b == tb.n) break;
    const BoxRec& R = tb.box[b];
    const int nx = R.hi[0] - R.lo[0] + 1, ny = R.hi[1] - R.lo[1] + 1;
    const int l = (int)(g - base);
    const DArr S = R.slot[slot];
    const long long o = S.off(l % nx + R.lo[0], (l / nx) % ny + R.lo[1], l / nx / ny + R.lo[2]);
#pragma unroll
    for (int n = 0; n < NCONS; ++n) acc[n] += S.p[o + n * S.ns];
  }
  __shared__ double sm[NCONS][256];
#pragma unroll
  for (int n = 0; n < NCONS; ++n) sm[n][threadIdx.x] = acc[n];
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w)
#pragma unroll
      for (int n = 0; n < NCONS; ++n) sm[n][threadIdx.x] += sm[n][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x < NCONS) part[(long long)blockIdx.x * NCONS + threadIdx.x] = sm[threadIdx.x][0];
}

__global__ void totals_final_kernel(const double* part, int nblocks, double scale, double* out) {
  if (threadIdx.x < NCONS) {
    double s = 0.0;
    for (int b = 0; b < nblocks; ++b) s += part[(long long)b * NCONS + threadIdx.x];
    out[threadIdx.x] = s * scale;
  }
}

cudaError_t launch_run_estdt(const BoxTable& tb, int s_in, long long nvalid, RunCtl* c, int nsm, cudaStream_t st) {
  run_estdt_reset<<<1, 1, 0, st>>>(c);
  long long blocks = (nvalid + 255) / 256;
  if (blocks > (long long)nsm * 4) blocks = (long long)nsm * 4;
  if (blocks < 1) blocks = 1;
  estdt_kernel<<<(int)blocks, 256, 0, st>>>(tb, s_in, nvalid, &c->bits);
  return cudaGetLastError();
}

cudaError_t launch_run_step_done(RunCtl* c, cudaGraphConditionalHandle cond, cudaStream_t st) {
  run_step_done<<<1, 1, 0, st>>>(c, cond);
  return cudaGetLastError();
}

cudaError_t launch_run_begin(RunCtl* c, cudaStream_t st) {
  run_begin<<<1, 1, 0, st>>>(c);
  return cudaGetLastError();
}

cudaError_t launch_copy_slot(const BoxTable& tb, int from, int to, long long nvalid, int nsm, cudaStream_t st) {
  long long blocks = (nvalid + 255) / 256;
  if (blocks > (long long)nsm * 8) blocks = (long long)nsm * 8;
  if (blocks < 1) blocks = 1;
  copy_slot_kernel<<<(int)blocks, 256, 0, st>>>(tb, from, to, nvalid);
  return cudaGetLastError();
}

int totals_blocks(long long nvalid, int nsm) {
  long long blocks = (nvalid + 255) / 256;
  if (blocks > (long long)nsm * 2) blocks = (long long)nsm * 2;
  return (int)(blocks < 1 ? 1 : blocks);
}

cudaError_t launch_totals(const BoxTable& tb, int slot, long long nvalid, double scale, double* part, double* out,
                          int nsm, cudaStream_t st) {
  const int nb = totals_blocks(nvalid, nsm);
  totals_partial_kernel<<<nb, 256, 0, st>>>(tb, slot, nvalid, part);
  totals_final_kernel<<<1, 32, 0, st>>>(part, nb, scale, out);
  return cudaGetLastError();
}

// ------------------------------------------------------- FP64 probe ----
// Eight independent DFMA chains per thread: the FP64 pipe's issue rate, the
// denominator of this path's roofline (the path is FP64-bound on GB300).
// FP64 peak probe: sixteen independent DFMA chains per thread (latency
// hidden many times over at 32 warps per SM), nothing else in the loop body
// but the chains, so the FP64 pipe is the only unit the loop can saturate.
__global__ void __launch_bounds__(256) fp64_probe_kernel(double* out, int iters, double s) {
  double a[16];
#pragma unroll
  for (int c = 0; c < 16; ++c) a[c] = threadIdx.x * 1e-3 + 1.0 + 0.05 * c;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int c = 0; c < 16; ++c) a[c] = fma(a[c], s, 0.5);
  }
  double r = 0.0;
#pragma unroll
  for (int c = 0; c < 16; ++c) r += a[c];
  out[blockIdx.x * blockDim.x + threadIdx.x] = r;
}

cudaError_t launch_fp64_probe(double* out, int blocks, int iters, cudaStream_t st) {
  fp64_probe_kernel<<<blocks, 256, 0, st>>>(out, iters, 0.999);
  return cudaGetLastError();
}

// Overlap probe of the integer-pipe product: sixteen DFMA chains per thread
// (the FP64 pipe saturated at 16 warps per SM) plus, per iteration, four
// further chains of products: none (MODE 0), hardware products (MODE 1) or
// dmul_rn (MODE 2).  The time over MODE 0's is what the four products cost a
// kernel whose FP64 pipe is already full.
template <int MODE>
__global__ void __launch_bounds__(256, 2) intpipe_probe_kernel(double* out, int iters, double m, double a) {
  double f[16], g[4];
#pragma unroll
  for (int c = 0; c < 16; ++c) f[c] = 1.0 + threadIdx.x * 1e-9 + c * 1e-3;
#pragma unroll
  for (int c = 0; c < 4; ++c) g[c] = 1.0 + threadIdx.x * 1e-9 + c * 1e-3;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int c = 0; c < 16; ++c) f[c] = fma(f[c], m, a);
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      if (MODE == 1) g[c] = __dmul_rn(g[c], m);
      if (MODE == 2) g[c] = dmul_rn(g[c], m);
    }
  }
  double r = 0.0;
#pragma unroll
  for (int c = 0; c < 16; ++c) r += f[c];
#pragma unroll
  for (int c = 0; c < 4; ++c) r += g[c];
  out[blockIdx.x * blockDim.x + threadIdx.x] = r;
}

cudaError_t launch_intpipe_probe(int mode, double* out, int blocks, int iters, cudaStream_t st) {
  const double m = 0.9999999, a = 1e-7;
  if (mode == 0) intpipe_probe_kernel<0><<<blocks, 256, 0, st>>>(out, iters, m, a);
  else if (mode == 1) intpipe_probe_kernel<1><<<blocks, 256, 0, st>>>(out, iters, m, a);
  else intpipe_probe_kernel<2><<<blocks, 256, 0, st>>>(out, iters, m, a);
  return cudaGetLastError();
}

// ------------------------------------------------------ division check ----
// ddiv_rn against the hardware division over generated operands: index i
// of the launch draws (a, b) from one of four families (WENO weights
// c_k / (eps + beta)^2, 1 / sum, arbitrary bit patterns, random significands
// at moderate exponents) with a counter-based generator; mismatching bit
// patterns are counted and the first one is recorded.
__device__ __forceinline__ unsigned long long splitmix(unsigned long long x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

__global__ void __launch_bounds__(256) ddiv_check_kernel(unsigned long long seed, long long count,
                                                         unsigned long long* bad, double* first) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count;
       i += (long long)gridDim.x * blockDim.x) {
    const unsigned long long r1 = splitmix(seed ^ (2 * (unsigned long long)i)),
                             r2 = splitmix(seed ^ (2 * (unsigned long long)i + 1));
    double a, b;
    switch ((int)(i & 3)) {
      case 0: {  // c_k / (1e-40 + beta)^2, beta = 2^[-200, 200) x random significand
        const double beta = __longlong_as_double((long long)((r2 & 0xFFFFFFFFFFFFFull) | ((823ull + (r2 >> 55)) << 52)));
        const double e = 1e-40 + beta;
        const double c[4] = {0.1, 0.6, 0.3, 1.0};
        a = c[r1 & 3];
        b = e * e;
        break;
      }
      case 1:  // 1 / sum of weights: sums over 2^[-140, 300)
        a = 1.0;
        b = __longlong_as_double((long long)((r2 & 0xFFFFFFFFFFFFFull) | ((883ull + (r2 >> 55) % 440ull) << 52)));
        break;
      case 2:  // arbitrary bit patterns (also the fallback domain)
        a = __longlong_as_double((long long)r1);
        b = __longlong_as_double((long long)r2);
        break;
      default:  // random significands and signs, exponents within +-128; one in 32 numerators +-0
        a = __longlong_as_double((long long)((r1 & 0x800FFFFFFFFFFFFFull) | ((960ull + (r1 >> 56) % 128ull) << 52)));
        b = __longlong_as_double((long long)((r2 & 0x800FFFFFFFFFFFFFull) | ((960ull + (r2 >> 56) % 128ull) << 52)));
        if (((r1 >> 51) & 31ull) == 0ull) a = __longlong_as_double((long long)(r1 & 0x8000000000000000ull));
        // one in 4 divisors with a significand near 2 (the reciprocal seed
        // then sits at the edge of its binade)
        if (((r2 >> 40) & 3ull) == 0ull)
          b = __longlong_as_double(__double_as_longlong(b) | 0x000FFFFFFF000000ll);
    }
    const double ref = a / b, got = ddiv_rn(a, b);
    const bool nan2 = ref != ref && got != got;
    if (__double_as_longlong(ref) != __double_as_longlong(got) && !nan2) {
      if (atomicAdd(bad, 1ull) == 0ull) {
        first[0] = a; first[1] = b; first[2] = ref; first[3] = got;
      }
    }
  }
}

// dsqrt_rn against the hardware square root: arbitrary bit patterns,
// positive doubles over the whole exponent range, squares of random doubles
// and their neighbours.
__global__ void __launch_bounds__(256) dsqrt_check_kernel(unsigned long long seed, long long count,
                                                          unsigned long long* bad, double* first) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count;
       i += (long long)gridDim.x * blockDim.x) {
    const unsigned long long r1 = splitmix(seed ^ (2 * (unsigned long long)i)),
                             r2 = splitmix(seed ^ (2 * (unsigned long long)i + 1));
    double x;
    switch ((int)(i % 4)) {
      case 0: x = __longlong_as_double((long long)r1); break;
      case 1: x = __longlong_as_double((long long)(r1 & 0x7FFFFFFFFFFFFFFFull)); break;
      case 2:  // significands near 1 and near 2, both exponent parities
        x = __longlong_as_double((long long)((((r1 & 1ull) ? (0xFFFFFFFFFFFFFull - (r2 & 0xFFFFFFull)) : (r2 & 0xFFFFFFull))) |
                                             ((1ull + r1 % 2046ull) << 52)));
        break;
      default: {
        const double r = __longlong_as_double((long long)((r1 & 0xFFFFFFFFFFFFFull) | ((600ull + r2 % 800ull) << 52)));
        x = __longlong_as_double(__double_as_longlong(r * r) + (long long)((r2 >> 32) % 5ull) - 2);
      }
    }
    const double ref = sqrt(x), got = dsqrt_rn(x);
    const bool nan2 = ref != ref && got != got;
    if (__double_as_longlong(ref) != __double_as_longlong(got) && !nan2) {
      if (atomicAdd(bad, 1ull) == 0ull) {
        first[0] = x; first[1] = 0.0; first[2] = ref; first[3] = got;
      }
    }
  }
}

// dmul_rn against the hardware product: arbitrary bit patterns, random
// significands and signs at moderate exponents, short significands whose
// products fall on rounding ties, exponent sums at the edges of the integer
// path's domain (underflow, overflow), zeros, subnormals and specials, and
// the kernels' constant factors (1/6, -1/48, 1/3, 13/12, 3, 5, 7, 11) against
// random values.
__global__ void __launch_bounds__(256) dmul_check_kernel(unsigned long long seed, long long count,
                                                         unsigned long long* bad, double* first) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count;
       i += (long long)gridDim.x * blockDim.x) {
    const unsigned long long r1 = splitmix(seed ^ (2 * (unsigned long long)i)),
                             r2 = splitmix(seed ^ (2 * (unsigned long long)i + 1));
    const unsigned long long SGN = 1ull << 63, FR = 0xFFFFFFFFFFFFFull;
    double a, b;
    switch ((int)(i % 6)) {
      case 0:
        a = __longlong_as_double((long long)r1);
        b = __longlong_as_double((long long)r2);
        break;
      case 1:
        a = __longlong_as_double((long long)((r1 & (SGN | FR)) | ((900ull + (r1 >> 52) % 250ull) << 52)));
        b = __longlong_as_double((long long)((r2 & (SGN | FR)) | ((900ull + (r2 >> 52) % 250ull) << 52)));
        break;
      case 2: {  // 20..33-bit significands whose products need 53 or 54 bits
        const int wa = 20 + (int)(r1 % 14ull), wb = 54 - wa + (int)((r2 >> 60) % 3ull) - 1;
        const unsigned long long sa = ((r1 >> 8) & ((1ull << (wa - 1)) - 1)) | (1ull << (wa - 1));
        const unsigned long long sb = ((r2 >> 8) & ((1ull << (wb - 1)) - 1)) | (1ull << (wb - 1));
        a = __longlong_as_double((long long)((r1 & SGN) | ((sa << (53 - wa)) & FR) | ((1000ull + (r2 & 31ull)) << 52)));
        b = __longlong_as_double((long long)((r2 & SGN) | ((sb << (53 - wb)) & FR) | ((1000ull + ((r1 >> 3) & 31ull)) << 52)));
        break;
      }
      case 3: {  // exponent sums next to underflow and overflow
        const int ea = 1 + (int)(r1 % 2046ull);
        const int target = (r2 & 1ull) ? (int)((r2 >> 1) % 6ull) - 3 : 2043 + (int)((r2 >> 1) % 6ull);
        int eb = target - ea + 1023;
        eb = eb < 0 ? 0 : (eb > 2046 ? 2046 : eb);
        a = __longlong_as_double((long long)((r1 & (SGN | FR)) | ((unsigned long long)ea << 52)));
        b = __longlong_as_double((long long)((r2 & (SGN | FR)) | ((unsigned long long)eb << 52)));
        break;
      }
      case 4: {  // zeros, subnormals, infinities and NaNs against random values
        const unsigned long long sp[6] = {0ull, SGN, 0x7FF0000000000000ull, 0x7FF8000000000000ull, r1 & FR,
                                          r1 & (SGN | FR)};
        a = __longlong_as_double((long long)sp[(r1 >> 58) % 6ull]);
        b = __longlong_as_double((long long)((r2 & (SGN | FR)) | (((r2 >> 52) % 2048ull) << 52)));
        if (r2 & 1ull) { const double t = a; a = b; b = t; }
        break;
      }
      default: {  // the kernels' constant factors
        const double cst[8] = {0.125 * (4.0 / 3.0), 0.125 * (-2.0 / 12.0), 1.0 / 3.0, 13.0 / 12.0, 3.0, 5.0, 7.0, 11.0};
        a = cst[r1 & 7ull];
        b = __longlong_as_double((long long)((r2 & (SGN | FR)) | ((700ull + (r2 >> 52) % 650ull) << 52)));
      }
    }
    const double ref = __dmul_rn(a, b), got = dmul_rn(a, b);
    const bool nan2 = ref != ref && got != got;
    if (__double_as_longlong(ref) != __double_as_longlong(got) && !nan2) {
      if (atomicAdd(bad, 1ull) == 0ull) {
        first[0] = a; first[1] = b; first[2] = ref; first[3] = got;
      }
    }
  }
}

cudaError_t launch_dmul_check(unsigned long long seed, long long count, unsigned long long* bad, double* first,
                              int nsm, cudaStream_t st) {
  dmul_check_kernel<<<nsm * 8, 256, 0, st>>>(seed, count, bad, first);
  return cudaGetLastError();
}

cudaError_t launch_ddiv_check(unsigned long long seed, long long count, unsigned long long* bad, double* first,
                              int nsm, cudaStream_t st) {
  ddiv_check_kernel<<<nsm * 8, 256, 0, st>>>(seed, count, bad, first);
  return cudaGetLastError();
}

cudaError_t launch_dsqrt_check(unsigned long long seed, long long count, unsigned long long* bad, double* first,
                               int nsm, cudaStream_t st) {
  dsqrt_check_kernel<<<nsm * 8, 256, 0, st>>>(seed, count, bad, first);
  return cudaGetLastError();
}

// ------------------------------------------------------- plot fields ----
// The derived plot variables of CNS (src/set/CNS_setup.cpp:153-176) over the
// valid cells of one box, in the operation order of their derive functions
// (src/cls/CNS_K.h:76-129): pressure (derpres), temperature (dertemp, from
// the internal energy and cv, not from p / (rho R)) and the three
// velocities (dervel: momentum / density).  out: 5 components in that order.
__global__ void __launch_bounds__(256) plot_derive_kernel(DArr U, DArr O, int lo0, int lo1, int lo2, int nx,
                                                          int ny, long long total, double gamma, double cv) {
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < total;
       g += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(g % nx) + lo0;
    const long long t = g / nx;
    const int j = (int)(t % ny) + lo1, k = (int)(t / ny) + lo2;
    const double rho = U(i, j, k, URHO), mx = U(i, j, k, UMX), my = U(i, j, k, UMY), mz = U(i, j, k, UMZ);
    const double rhoinv = ddiv_rn(1.0, rho);
    const double rhoeint = U(i, j, k, UET) - 0.5 * rhoinv * (mx * mx + my * my + mz * mz);
    O(i, j, k, 0) = (gamma - 1.0) * rhoeint;
    O(i, j, k, 1) = ddiv_rn(rhoeint * rhoinv, cv);
    O(i, j, k, 2) = ddiv_rn(mx, rho);
    O(i, j, k, 3) = ddiv_rn(my, rho);
    O(i, j, k, 4) = ddiv_rn(mz, rho);
  }
}

cudaError_t launch_plot_derive(const DArr& U, const DArr& O, const int lo[3], const int n[3], double gamma, double cv,
                               int nsm, cudaStream_t st) {
  const long long total = (long long)n[0] * n[1] * n[2];
  long long blocks = (total + 255) / 256;
  if (blocks > (long long)nsm * 8) blocks = (long long)nsm * 8;
  if (blocks < 1) blocks = 1;
  plot_derive_kernel<<<(int)blocks, 256, 0, st>>>(U, O, lo[0], lo[1], lo[2], n[0], n[1], total, gamma, cv);
  return cudaGetLastError();
}

// ------------------------------------------------------ average_down ----
// amrex::average_down of cell-centred data on a Cartesian grid (called by
// CNS::avgDown, src/CNS.cpp:513-530): each coarse cell of the box becomes
// the mean of its rx*ry*rz fine cells, summed from zero with the fine k
// offset outermost and i innermost and scaled by 1/(rx*ry*rz), the order of
// AMReX's amrex_avgdown.  One thread per coarse cell, all components.
__global__ void __launch_bounds__(256) avgdown_kernel(DArr fine, DArr crse, int lo0, int lo1, int lo2, int nx,
                                                      int ny, long long total, int rx, int ry, int rz, int scomp,
                                                      int ncomp, double volfrac) {
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < total;
       g += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(g % nx) + lo0;
    const long long t = g / nx;
    const int j = (int)(t % ny) + lo1, k = (int)(t / ny) + lo2;
    for (int n = scomp; n < scomp + ncomp; ++n) {
      double c = 0.0;
      for (int kr = 0; kr < rz; ++kr)
        for (int jr = 0; jr < ry; ++jr)
          for (int ir = 0; ir < rx; ++ir) c += fine(i * rx + ir, j * ry + jr, k * rz + kr, n);
      crse(i, j, k, n) = volfrac * c;
    }
  }
}

cudaError_t launch_avgdown(const DArr& fine, const DArr& crse, const int lo[3], const int n[3], const int r[3],
                           int scomp, int ncomp, double volfrac, int nsm, cudaStream_t st) {
  const long long total = (long long)n[0] * n[1] * n[2];
  if (total <= 0) return cudaSuccess;
  long long blocks = (total + 255) / 256;
  if (blocks > 8LL * nsm) blocks = 8LL * nsm;
  avgdown_kernel<<<(int)blocks, 256, 0, st>>>(fine, crse, lo[0], lo[1], lo[2], n[0], n[1], total, r[0], r[1], r[2],
                                               scomp, ncomp, volfrac);
  return cudaGetLastError();
}

// ----------------------------------------------------- timeout probe ----
// The error path of the bounded waits, without a hang: one thread waits on
// an mbarrier that nothing arrives at, with the same bounded wait the face
// kernel uses (at most `polls` polls), gives up, raises the error flag and
// returns.
__global__ void wait_timeout_probe_kernel(int* err, long long polls) {
  __shared__ unsigned long long bar;
  mbar_init(&bar, 1);
  fence_mbar_init();
  if (!mbar_wait(&bar, 0u, polls)) atomicExch(err, 1);
}

cudaError_t launch_wait_timeout_probe(int* err, long long polls, cudaStream_t st) {
  wait_timeout_probe_kernel<<<1, 1, 0, st>>>(err, polls);
  return cudaGetLastError();
}

}  // namespace amrs
