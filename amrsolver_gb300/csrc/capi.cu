// C ABI of the GB300 RHS + SSP-RK path (include/amrs_gb300.h).
//
// Host-side orchestration mirrors CNS::compute_rhs and CNS::advance
// (src/tim/CNS_advance.cpp:14-427): for every stage, the scheme's kernel
// sequence runs over a device box table, then the stage's BLAS-1 program is
// applied in the last kernel's epilogue.  Nothing here synchronises the host
// except where the header says so.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "../../include/amrs_gb300.h"
#include "amrs_kernels.h"

using namespace amrs;

namespace {

thread_local std::string g_cuda_err;

amrs_status cuda_fail(cudaError_t e, const char* where) {
  g_cuda_err = std::string(where) + ": " + cudaGetErrorString(e);
  return AMRS_ERR_CUDA;
}
#define CK(call)                                         \
  do {                                                   \
    cudaError_t e_ = (call);                             \
    if (e_ != cudaSuccess) return cuda_fail(e_, #call);  \
  } while (0)

DClosures to_dev(const amrs_closures& c) {
  DClosures d;
  d.gamma = c.gamma; d.cv = c.cv; d.cp = c.cp; d.Rspec = c.Rspec;
  d.visc_law = c.visc_law; d.cond_law = c.cond_law;
  d.visc_ref = c.visc_ref; d.Tvisc_ref = c.Tvisc_ref;
  d.cond_ref = c.cond_ref; d.Tcond_ref = c.Tcond_ref;
  d.Cshock = c.Cshock; d.Cdamp = c.Cdamp;
  d.source = 0;
  d.force[0] = d.force[1] = d.force[2] = 0.0;
  return d;
}

amrs_status check_bcnormal(const amrs_bcnormal& b) {
  if (b.kind < 0 || b.kind > 1) return AMRS_ERR_BC;
  if (b.kind == 1) {
    if (!(b.Tw > 0.0) || !std::isfinite(b.Tw) || !std::isfinite(b.Tmin)) return AMRS_ERR_BC;
    if (!(b.dx[1] > 0.0) || !(b.prob_hi[1] > b.prob_lo[1])) return AMRS_ERR_BC;
  }
  return AMRS_OK;
}

DBcNormal to_dbcn(const amrs_bcnormal& b) {
  DBcNormal d{};
  d.kind = b.kind;
  d.Tw = b.Tw;
  d.Tmin = b.Tmin;
  for (int k = 0; k < 3; ++k) { d.prob_lo[k] = b.prob_lo[k]; d.prob_hi[k] = b.prob_hi[k]; d.dx[k] = b.dx[k]; }
  return d;
}

DArr to_darr(const amrs_array4& a) {
  DArr d;
  d.p = a.p; d.js = a.jstride; d.ks = a.kstride; d.ns = a.nstride;
  d.b0 = a.begin[0]; d.b1 = a.begin[1]; d.b2 = a.begin[2];
  return d;
}

// array covers box grown by g with ncomp components?
bool covers(const amrs_array4& a, const amrs_box& b, int g, int ncomp) {
  if (!a.p || a.ncomp < ncomp) return false;
  for (int d = 0; d < 3; ++d)
    if (a.begin[d] > b.lo[d] - g || a.end[d] < b.hi[d] + g + 1) return false;
  const long long nx = a.end[0] - a.begin[0], ny = a.end[1] - a.begin[1], nz = a.end[2] - a.begin[2];
  if (a.jstride < nx || a.kstride < a.jstride * ny || a.nstride < a.kstride * nz) return false;
  return true;
}

int bn(const amrs_box& b, int d) { return b.hi[d] - b.lo[d] + 1; }
long long grown_cells(const amrs_box& b, int g) {
  return (long long)(bn(b, 0) + 2 * g) * (bn(b, 1) + 2 * g) * (bn(b, 2) + 2 * g);
}
// Non-empty, and small enough that a box's cells with 3 ghosts fit the
// kernels' 32-bit per-box cell index (about 1290^3 cells, ~86 GB per state).
bool box_ok(const amrs_box& b) {
  for (int d = 0; d < 3; ++d)
    if (b.hi[d] < b.lo[d] || (long long)b.hi[d] - b.lo[d] >= (1 << 20)) return false;
  return grown_cells(b, NGHOST) < (1LL << 31);
}

// The library's internal Euler-flux code: 1 KEEP, 2 WENO5 LLF, 0 MUSCL +
// Riemann, 3 WENO5-Riemann.  The public flux_euler sends every value other
// than 1 and 2 to the Riemann path, as the reference's compute_rhs does;
// riemann_weno picks the states there.
amrs_scheme canonical_scheme(amrs_scheme s) {
  if (s.flux_euler != 1 && s.flux_euler != 2) s.flux_euler = s.riemann_weno ? 3 : 0;
  return s;
}

amrs_status check_scheme(const amrs_scheme& s) {
  if (s.riemann_weno != 0 && s.riemann_weno != 1) return AMRS_ERR_SCHEME;
  if (s.flux_euler == 1 && !(s.order_keep == 2 || s.order_keep == 4 || s.order_keep == 6)) return AMRS_ERR_SCHEME;
  if (s.art_diss != 0 && s.art_diss != 1) return AMRS_ERR_SCHEME;
  if (s.weno_fast != 0 && s.weno_fast != 1) return AMRS_ERR_SCHEME;
  return AMRS_OK;
}

// ghost depth of the primitive region each scheme reads
int prim_ghost(const amrs_scheme& s) {
  int g = 0;
  if (s.rhs_euler) {
    if (s.flux_euler == 1) g = std::max(g, s.order_keep / 2);
    else if (s.flux_euler == 0) g = std::max(g, 2);  // slopes on grow(bx,1) read +-1
    else if (s.flux_euler == 3) g = std::max(g, 3);  // five-point stencils of the faces
    if (s.art_diss) g = std::max(g, 1);
  }
  if (s.rhs_visc) g = std::max(g, 2);
  return g;
}

bool fused_path(const amrs_scheme& s) { return s.rhs_euler && s.flux_euler == 1 && !s.art_diss; }

// Tile choice for one box (the autotuner can override per box size).
void default_tile(const amrs_box& b, int order, int& tx, int& ty, int& kc, int nsm) {
  const int nx = bn(b, 0), ny = bn(b, 1), nz = bn(b, 2);
  static const int cand[][2] = {{32, 8}, {16, 16}, {24, 10}, {8, 30}, {16, 8}, {8, 16}, {8, 8}};
  double best = 1e300;
  tx = 16; ty = 8;
  for (auto& c : cand) {
    if (!keep_tile_fits(order, c[0], c[1])) continue;
    const long long ntx = (nx + c[0] - 1) / c[0], nty = (ny + c[1] - 1) / c[1];
    // cost: lanes issued per useful cell, plus the x/y halo pair overheads
    const double lanes = (double)ntx * nty * F_THREADS;
    const double useful = (double)nx * ny;
    const double halo = 1.0 + (double)(order / 2) / c[0] + (double)(order / 2) / c[1];
    const double cost = lanes / useful * halo;
    if (cost < best) { best = cost; tx = c[0]; ty = c[1]; }
  }
  const long long ncol = (long long)((nx + tx - 1) / tx) * ((ny + ty - 1) / ty);
  // enough z chunks to give every SM two tiles, but at least 8 planes each
  long long want = (2LL * nsm + ncol - 1) / ncol;
  kc = (int)std::max<long long>(8, (nz + want - 1) / std::max<long long>(want, 1));
  kc = std::min(kc, nz);
}

// Time a CTA of the fused face kernel spends on one plane of a txw x tyw
// tile column, in units of one KEEP pair evaluation by one thread.  The
// kernel's phases are separated by barriers and deal their items
// round-robin over F_THREADS threads, so a phase costs its rounds: phase 1
// the H z pairs of a column plus the x/y stored pairs of separation >= 2,
// phase 2 the x and y faces (~1.5 pairs each with their sums and viscous
// averages), phase 3 the divergence (~0.5), plus a fixed ~1 per plane
// (barriers, the wait for the plane's load).  A thin partial tile thus
// costs about half a full one per plane, not its share of cells.
double face_plane_cost(int H, int txw, int tyw) {
  int nxy = 0;
  for (int l = 2; l <= H; ++l) nxy += (txw + l) * tyw + txw * (tyw + l);
  const int nf = (txw + 1) * tyw + txw * (tyw + 1);
  auto rounds = [](int items) { return (double)((items + F_THREADS - 1) / F_THREADS); };
  return 1.0 + H + rounds(nxy) + 1.5 * rounds(nf) + 0.5;
}

// Stage programs of CNS::advance (src/tim/CNS_advance.cpp:51-166) for
// (order_rk, stages_rk): numeric coefficients for `dt` into `st`, and, when
// `forms` is given, the same programs with every dt-dependent coefficient
// kept as its form (dt * c or dt / c, exactly as the reference writes it)
// for kernels that read dt from device memory.
struct Cf {
  int f;     // 0 constant c, 1 dt * c, 2 dt / c
  double c;
};
double cf_val(Cf x, double dt) { return x.f == 1 ? dt * x.c : (x.f == 2 ? dt / x.c : x.c); }

amrs_status rk_build(int order_rk, int stages_rk, double dt, amrs_stage_prog* st, int cap, int32_t* nstages,
                     DProg* forms) {
  const Cf K0{0, 0.0}, DT{1, 1.0};
  auto K = [](double v) { return Cf{0, v}; };
  const int S1 = 0, S2 = 1, DS = 2;
  int n = -1;
  if (order_rk == -2) n = 2;
  else if (order_rk == 0 || order_rk == 1) n = 1;
  else if (order_rk == 2) n = (stages_rk >= 2) ? stages_rk : -1;
  else if (order_rk == 3 && (stages_rk == 3 || stages_rk == 4)) n = stages_rk;
  if (n < 0) return AMRS_ERR_RK;
  if (n > cap) return AMRS_ERR_SIZE;
  std::memset(st, 0, sizeof(amrs_stage_prog) * n);
  if (forms) std::memset(forms, 0, sizeof(DProg) * n);
  auto op = [&](int i, int j, int kind, int dst, int x, int y, Cf a, Cf b) {
    amrs_rk_op& o = st[i].ops[j];
    o.kind = kind; o.dst = dst; o.x = x; o.y = y; o.a = cf_val(a, dt); o.b = cf_val(b, dt);
    if (forms) {
      DOp& d = forms[i].ops[j];
      d.kind = kind; d.dst = dst; d.x = x; d.y = y; d.a = a.c; d.b = b.c; d.fa = a.f; d.fb = b.f;
    }
  };
  auto set = [&](int i, int src, int nops) {
    st[i].src_state = src; st[i].nops = nops;
    if (forms) forms[i].nops = nops;
  };
  if (order_rk == -2) {  // src/tim/CNS_advance.cpp:51-70
    set(0, 0, 1); op(0, 0, 0, S2, S1, DS, K(1.0), DT);
    set(1, 1, 2); op(1, 0, 0, S2, S2, S1, K(0.5), K(0.5)); op(1, 1, 1, S2, DS, 0, Cf{1, 0.5}, K0);
  } else if (order_rk == 0) {  // :71-75
    set(0, 0, 1); op(0, 0, 3, S2, DS, 0, K0, K0);
  } else if (order_rk == 1) {  // :76-80
    set(0, 0, 1); op(0, 0, 0, S2, S1, DS, K(1.0), DT);
  } else if (order_rk == 2) {  // :81-114
    const int m = stages_rk;
    for (int i = 1; i <= m - 1; ++i) { set(i - 1, i == 1 ? 0 : 1, 1); op(i - 1, 0, 1, S2, DS, 0, Cf{2, double(m - 1)}, K0); }
    set(m - 1, 1, 2);
    op(m - 1, 0, 0, S2, S2, DS, K(double(m - 1)), DT);
    op(m - 1, 1, 0, S2, S1, S2, K(1.0 / m), K(1.0 / m));
  } else if (stages_rk == 3) {  // :118-139
    set(0, 0, 1); op(0, 0, 0, S2, S1, DS, K(1.0), DT);
    set(1, 1, 2); op(1, 0, 2, DS, S2, 0, DT, K0); op(1, 1, 0, S2, S1, DS, K(3.0 / 4), K(1.0 / 4));
    set(2, 1, 2); op(2, 0, 2, DS, S2, 0, DT, K0); op(2, 1, 0, S2, S1, DS, K(1.0 / 3), K(2.0 / 3));
  } else {  // :141-166
    set(0, 0, 1); op(0, 0, 0, S2, S1, DS, K(1.0), Cf{2, 2.0});
    set(1, 1, 1); op(1, 0, 1, S2, DS, 0, Cf{2, 2.0}, K0);
    set(2, 1, 2); op(2, 0, 0, S2, S1, S2, K(2.0 / 3), K(1.0 / 3)); op(2, 1, 1, S2, DS, 0, Cf{2, 6.0}, K0);
    set(3, 1, 1); op(3, 0, 1, S2, DS, 0, Cf{2, 2.0}, K0);
  }
  *nstages = n;
  return AMRS_OK;
}

// y sides of the domain with boundary code 6 (user-defined walls) and the
// domain's y extent: the reference's wall treatment in compute_rhs
// (src/tim/CNS_advance.cpp:226-229, :300-333) for boxes that touch them.
struct WallCfg {
  int lo = 0, hi = 0;
  int dom_lo = 0, dom_hi = 0;
};

void set_walls(BoxRec& R, const WallCfg& w, const amrs_scheme& sc) {
  const bool tl = w.lo && R.lo[1] == w.dom_lo, th = w.hi && R.hi[1] == w.dom_hi;
  const bool reduce = sc.rhs_euler && sc.flux_euler == 1 && sc.order_keep != 2;
  const int H = sc.order_keep / 2;
  const int none = -(1 << 29);
  R.walls = (tl || th) ? 1 : 0;
  R.wrow_lo = tl ? R.lo[1] - 1 : none;
  R.wrow_hi = th ? R.hi[1] + 1 : none;
  R.red_lo = (tl && reduce) ? R.lo[1] + H - 1 : none;
  R.red_hi = (th && reduce) ? R.hi[1] - H + 1 : (1 << 29);
}

// -------------------------------------------------------------- list ----
// Host + device state of one box list (a level, or one box for the per-box
// entry points).
struct List {
  int n = 0, nslots = 0;
  amrs_scheme sc{};
  int gq = 2;
  bool fused = true;
  std::vector<amrs_box> boxes;
  std::vector<BoxRec> hbox;
  std::vector<FaceRec> hface;
  std::vector<long long> pcell, vcell, gcell, valid, fpre[3], spre[3];
  std::vector<int> fwork;
  std::vector<DClosures> cls;
  bool source = false;    // some closures carry a source term
  // device
  void* dtab = nullptr;   // all tables in one allocation
  size_t dtab_bytes = 0;
  void* dscr = nullptr;   // scratch fields in one allocation
  size_t dscr_bytes = 0;
  CUtensorMap* dmaps = nullptr;
  BoxTable tb{};
  FaceTable ft{};
  TmaDesc tma{};
  const long long* d_spre[3] = {nullptr, nullptr, nullptr};
  long long tot_p = 0, tot_v = 0, tot_g = 0, tot_valid = 0, tot_f[3] = {0, 0, 0}, tot_s[3] = {0, 0, 0};
  int tot_work = 0;
  int face_grid = 0;  // CTAs of the balanced face-kernel schedule
  int waves = 1;      // shares of the schedule per resident CTA (amrs_boxlist_set_schedule)
  cudaGraphExec_t graph = nullptr;
  int graph_key[6] = {0, 0, 0, 0, 0, 0};
  double graph_dt = 0.0;
  int graph_result = -1;
  // ghost fill of each stage input: 0 none (ghosts frozen), 1 every box its
  // own domain (amrs_boxlist_set_bc), 2 the boxes tile one domain
  // (amrs_boxlist_set_domain: neighbour copies, periodic images, physical BCs)
  int has_bc = 0;
  int bc_lo[3] = {-1, -1, -1}, bc_hi[3] = {-1, -1, -1};
  LevelDomain dom{};
  DBcNormal bcn{};         // device bcnormal of the code-6 y sides (kind 0: none)
  int* d_owner = nullptr;  // has_bc == 2: owning box of every grown cell's source (-1: valid cell)
  WallCfg wall{};          // code-6 y walls of the list's domain (amrs_boxlist_set_domain)
  // device-resident time loop (amrs_rk_run_boxlist)
  RunCtl* d_run = nullptr;
  RunCtl h_run{};
  cudaGraphExec_t run_graph = nullptr;
  int run_key[6] = {0, 0, 0, 0, 0, 0};
  double* d_tot = nullptr;  // per-block partial sums of amrs_boxlist_totals
  size_t d_tot_n = 0;
  double* d_step_dt = nullptr;  // dt the step graph's stage programs read
  double h_step_dt = 0.0;
  unsigned long long* d_stats = nullptr;  // reduction cells of the printTotal statistics
  ~List() {
    if (d_stats) cudaFree(d_stats);
    if (d_step_dt) cudaFree(d_step_dt);
    if (run_graph) cudaGraphExecDestroy(run_graph);
    if (d_run) cudaFree(d_run);
    if (d_tot) cudaFree(d_tot);
    if (graph) cudaGraphExecDestroy(graph);
    if (dtab) cudaFree(dtab);
    if (dscr) cudaFree(dscr);
    if (d_owner) cudaFree(d_owner);
  }
};

}  // namespace

struct amrs_handle {
  int device = 0;
  int nsm = 0;
  amrs_scheme sc{};
  amrs_closures cl{};
  int* derr = nullptr;               // device flags: [0] bounded waits timed out, [1] non-finite result
  int check_nonfinite = 0;           // amrs_set_check_nonfinite
  unsigned long long* dred = nullptr;  // reduction cell
  bool tma_ok = true;
  void* encode_fn = nullptr;
  List* one = nullptr;               // reusable single-box list for per-box calls
  WallCfg wall{};                    // code-6 y walls of the per-box calls' domain (amrs_set_domain)
  int source = 0;                    // rhs_source with a body force (amrs_set_source)
  double force[3] = {0.0, 0.0, 0.0};
  void* adj = nullptr;               // adjoint scratch (pair and viscous cotangents), grow-only
  size_t adj_bytes = 0;
  BoxRec* dring = nullptr;           // per-call box records of per-box calls (device ring)
  BoxRec* hring = nullptr;           // pinned staging of the ring
  cudaEvent_t ring_ev[64];
  int ring_used[64] = {0};
  int ring_pos = 0, ring_cur = -1;
  std::mutex mu;
};

struct amrs_boxlist {
  amrs_handle* h;
  int device = 0;  // the handle's device, kept so that destroying the list never reads the handle
  List L;
};

namespace {

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// Tensor map of one box's primitive scratch: dims (x, y, z, comp) over
// grow(box,3), box {tx+6, ty+2H, 1, NQ}.  Returns false when the layout
// cannot be described (row pitch not a multiple of 16 bytes, etc.).
bool make_qmap(amrs_handle* h, const BoxRec& R, int order, CUtensorMap* out) {
  if (!h->encode_fn || !h->tma_ok) return false;
  const int H = order / 2;
  const cuuint64_t dims[4] = {(cuuint64_t)(R.hi[0] - R.lo[0] + 1 + 6), (cuuint64_t)(R.hi[1] - R.lo[1] + 1 + 6),
                              (cuuint64_t)(R.hi[2] - R.lo[2] + 1 + 6), (cuuint64_t)NQ};
  const cuuint64_t strides[3] = {(cuuint64_t)R.q.js * 8, (cuuint64_t)R.q.ks * 8, (cuuint64_t)R.q.ns * 8};
  for (int i = 0; i < 3; ++i)
    if (strides[i] % 16) return false;
  if (((uintptr_t)R.q.p) % 16) return false;
  const cuuint32_t box[4] = {(cuuint32_t)(R.tx + 6), (cuuint32_t)(R.ty + 2 * H), 1u, (cuuint32_t)NQ};
  if ((box[0] * 8) % 16 || box[0] > 256 || box[1] > 256) return false;
  const cuuint32_t es[4] = {1, 1, 1, 1};
  CUresult r = reinterpret_cast<EncodeTiledFn>(h->encode_fn)(
      out, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 4, R.q.p, dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
      CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// Build host tables and allocate/upload device tables + scratch.
amrs_status list_build(amrs_handle* h, List& L, int n, const amrs_box* boxes, const double* dxinv3, int nslots,
                       const amrs_array4* states, const int32_t* cidx, int ncl, const amrs_closures* cls,
                       const int* tiles /* per box tx,ty,kc or null */) {
  L.n = n;
  L.nslots = nslots;
  L.sc = h->sc;
  L.gq = prim_ghost(h->sc);
  L.fused = fused_path(h->sc);
  L.boxes.assign(boxes, boxes + n);
  L.hbox.assign(n, BoxRec{});
  L.cls.resize(std::max(ncl, 1));
  if (ncl > 0) for (int c = 0; c < ncl; ++c) L.cls[c] = to_dev(cls[c]);
  else L.cls[0] = to_dev(h->cl);
  for (DClosures& c : L.cls) {
    c.source = h->source;
    for (int d = 0; d < 3; ++d) c.force[d] = h->force[d];
  }
  L.source = h->source != 0;
  const int order = h->sc.order_keep;
  const bool need_faces = !L.fused;
  const bool need_visc = h->sc.rhs_visc != 0;
  const bool need_weno = h->sc.rhs_euler && h->sc.flux_euler == 2;
  const bool need_slope = h->sc.rhs_euler && h->sc.flux_euler == 0;
  const bool need_jst = h->sc.rhs_euler && h->sc.art_diss == 1;
  L.pcell.assign(n + 1, 0); L.vcell.assign(n + 1, 0); L.gcell.assign(n + 1, 0); L.valid.assign(n + 1, 0);
  L.fwork.assign(n + 1, 0);
  for (int d = 0; d < 3; ++d) { L.fpre[d].assign(n + 1, 0); L.spre[d].assign(n + 1, 0); }
  // scratch layout: per box, Q [NQ x grow3], VF [NVF x grow1], faces, pf, lam, sen, slopes
  size_t off = 0;
  std::vector<size_t> q_off(n), vf_off(n), f_off(n * 3), pf_off(n), lam_off(n), sen_off(n), sl_off(n * 3);
  for (int b = 0; b < n; ++b) {
    const amrs_box& B = boxes[b];
    if (!box_ok(B)) return AMRS_ERR_BOX;
    q_off[b] = off; off = align_up(off + grown_cells(B, 3) * NQ * 8, 256);
    if (need_visc) { vf_off[b] = off; off = align_up(off + grown_cells(B, 1) * NVF * 8, 256); }
    if (need_faces)
      for (int d = 0; d < 3; ++d) {
        const long long nf = (long long)(bn(B, 0) + (d == 0)) * (bn(B, 1) + (d == 1)) * (bn(B, 2) + (d == 2));
        f_off[b * 3 + d] = off; off = align_up(off + nf * NCONS * 8, 256);
      }
    if (need_weno) {
      pf_off[b] = off; off = align_up(off + grown_cells(B, 3) * 3 * NCONS * 8, 256);
    }
    if (need_weno || need_jst) { lam_off[b] = off; off = align_up(off + grown_cells(B, 3) * 3 * 8, 256); }
    if (need_jst) { sen_off[b] = off; off = align_up(off + grown_cells(B, 3) * 3 * 8, 256); }
    if (need_slope)
      for (int d = 0; d < 3; ++d) { sl_off[b * 3 + d] = off; off = align_up(off + grown_cells(B, 1) * NSLOPE * 8, 256); }
  }
  if (off > L.dscr_bytes) {
    if (L.dscr) { cudaFree(L.dscr); L.dscr = nullptr; L.dscr_bytes = 0; }
    CK(cudaMalloc(&L.dscr, off));
    L.dscr_bytes = off;
  }
  char* S = static_cast<char*>(L.dscr);
  L.hface.assign(need_faces ? n : 0, FaceRec{});
  for (int b = 0; b < n; ++b) {
    const amrs_box& B = boxes[b];
    BoxRec& R = L.hbox[b];
    for (int d = 0; d < 3; ++d) {
      R.lo[d] = B.lo[d]; R.hi[d] = B.hi[d];
      R.dxinv[d] = dxinv3[3 * b + d];
      R.dx[d] = 1.0 / dxinv3[3 * b + d];
    }
    for (int s = 0; s < nslots && s < MAX_SLOTS; ++s) R.slot[s] = to_darr(states[b * nslots + s]);
    set_walls(R, L.wall, h->sc);
    auto mk = [&](size_t o, int g, int nodal_d, int ncomp_unused) {
      (void)ncomp_unused;
      DArr a;
      a.p = reinterpret_cast<double*>(S + o);
      const int nx = bn(B, 0) + 2 * g + (nodal_d == 0), ny = bn(B, 1) + 2 * g + (nodal_d == 1),
                nz = bn(B, 2) + 2 * g + (nodal_d == 2);
      a.js = nx; a.ks = (long long)nx * ny; a.ns = (long long)nx * ny * nz;
      a.b0 = B.lo[0] - g; a.b1 = B.lo[1] - g; a.b2 = B.lo[2] - g;
      return a;
    };
    R.q = mk(q_off[b], 3, -1, NQ);
    if (need_visc) R.vf = mk(vf_off[b], 1, -1, NVF);
    R.cl = cidx ? cidx[b] : 0;
    int tx, ty, kc;
    if (tiles) { tx = tiles[3 * b]; ty = tiles[3 * b + 1]; kc = tiles[3 * b + 2]; }
    else default_tile(B, order, tx, ty, kc, h->nsm);
    R.tx = tx; R.ty = ty; R.kc = kc;
    R.ntx = (bn(B, 0) + tx - 1) / tx; R.nty = (bn(B, 1) + ty - 1) / ty; R.nkz = (bn(B, 2) + kc - 1) / kc;
    if (need_faces) {
      FaceRec& F = L.hface[b];
      for (int d = 0; d < 3; ++d) F.f[d] = mk(f_off[b * 3 + d], 0, d, NCONS);
      if (need_weno) {
        DArr pf = mk(pf_off[b], 3, -1, 3 * NCONS);
        for (int d = 0; d < 3; ++d) { F.pf[d] = pf; F.pf[d].p = pf.p + d * NCONS * pf.ns; }
      }
      if (need_weno || need_jst) F.lam = mk(lam_off[b], 3, -1, 3);
      if (need_jst) F.sen = mk(sen_off[b], 3, -1, 3);
      if (need_slope) for (int d = 0; d < 3; ++d) F.slope[d] = mk(sl_off[b * 3 + d], 1, -1, NSLOPE);
    }
    const int g = L.gq;
    L.pcell[b + 1] = L.pcell[b] + grown_cells(B, g);
    L.vcell[b + 1] = L.vcell[b] + (need_visc ? grown_cells(B, 1) : 0);
    L.gcell[b + 1] = L.gcell[b] + grown_cells(B, 3);
    L.valid[b + 1] = L.valid[b] + grown_cells(B, 0);
    L.fwork[b + 1] = L.fwork[b] + R.ntx * R.nty * R.nkz;
    for (int d = 0; d < 3; ++d) {
      const long long nf = (long long)(bn(B, 0) + (d == 0)) * (bn(B, 1) + (d == 1)) * (bn(B, 2) + (d == 2));
      L.fpre[d][b + 1] = L.fpre[d][b] + nf;
      const long long ns = (long long)(bn(B, 0) + 2 * (d == 0)) * (bn(B, 1) + 2 * (d == 1)) * (bn(B, 2) + 2 * (d == 2));
      L.spre[d][b + 1] = L.spre[d][b] + ns;
    }
  }
  L.tot_p = L.pcell[n]; L.tot_v = L.vcell[n]; L.tot_g = L.gcell[n]; L.tot_valid = L.valid[n];
  L.tot_work = L.fwork[n];
  for (int d = 0; d < 3; ++d) { L.tot_f[d] = L.fpre[d][n]; L.tot_s[d] = L.spre[d][n]; }

  // Balanced static schedule of the fused face kernel: the (tile column x
  // plane) work of all boxes, weighted by the time a CTA spends on one plane
  // of that column (face_plane_cost), is cut into G equal shares (G =
  // resident CTAs); a share is a run of segments (box, column, k0, k1),
  // each segment costing one z-prologue.
  std::vector<int4> segs;
  std::vector<int> cta_seg;
  L.face_grid = 0;
  if (L.fused) {
    double total = 0.0;
    long long colplanes = 0;
    for (int b = 0; b < n; ++b) {
      const BoxRec& R = L.hbox[b];
      for (int c = 0; c < R.ntx * R.nty; ++c) {
        const int txi = c % R.ntx, tyi = c / R.ntx;
        const int txw = std::min(R.tx, R.hi[0] + 1 - (R.lo[0] + txi * R.tx));
        const int tyw = std::min(R.ty, R.hi[1] + 1 - (R.lo[1] + tyi * R.ty));
        total += face_plane_cost(order / 2, txw, tyw) * bn(boxes[b], 2);
        colplanes += bn(boxes[b], 2);
      }
    }
    const long long G = std::min<long long>((long long)L.waves * keep_ctas_per_sm(order) * h->nsm, colplanes);
    const double per = total / (double)G;
    int cta = 0;
    double acc = 0.0;
    cta_seg.push_back(0);
    for (int b = 0; b < n; ++b) {
      const BoxRec& R = L.hbox[b];
      for (int c = 0; c < R.ntx * R.nty; ++c) {
        const int txi = c % R.ntx, tyi = c / R.ntx;
        const int txw = std::min(R.tx, R.hi[0] + 1 - (R.lo[0] + txi * R.tx));
        const int tyw = std::min(R.ty, R.hi[1] + 1 - (R.lo[1] + tyi * R.ty));
        const double w = face_plane_cost(order / 2, txw, tyw);
        int k = R.lo[2];
        while (k <= R.hi[2]) {
          const double boundary = (cta + 1) * per;
          long long fit = (long long)((boundary - acc) / w + 0.5);
          if (fit < 1) fit = 1;
          const int kend = (int)std::min<long long>(R.hi[2] + 1, k + fit);
          segs.push_back(make_int4(b, c, k, kend));
          acc += (kend - k) * w;
          k = kend;
          if (acc >= boundary - 0.5 * w && cta < G - 1) {
            ++cta;
            cta_seg.push_back((int)segs.size());
          }
        }
      }
    }
    while ((long long)cta_seg.size() < G + 1) cta_seg.push_back((int)segs.size());
    cta_seg[G] = (int)segs.size();
    L.face_grid = (int)G;
  }

  // tensor maps (fused path only)
  std::vector<CUtensorMap> maps;
  bool tma_all = L.fused && h->tma_ok && h->encode_fn;
  if (tma_all) {
    maps.resize(n);
    for (int b = 0; b < n && tma_all; ++b) tma_all = make_qmap(h, L.hbox[b], order, &maps[b]);
  }

  // device tables in one allocation
  size_t t = 0;
  const size_t o_box = t; t = align_up(t + sizeof(BoxRec) * n, 128);
  const size_t o_face = t; t = align_up(t + sizeof(FaceRec) * L.hface.size(), 128);
  const size_t o_cls = t; t = align_up(t + sizeof(DClosures) * L.cls.size(), 128);
  const size_t o_maps = t; t = align_up(t + sizeof(CUtensorMap) * (tma_all ? n : 0), 128);
  const size_t o_p = t; t = align_up(t + 8 * (n + 1), 128);
  const size_t o_v = t; t = align_up(t + 8 * (n + 1), 128);
  const size_t o_g = t; t = align_up(t + 8 * (n + 1), 128);
  const size_t o_va = t; t = align_up(t + 8 * (n + 1), 128);
  size_t o_f[3], o_s[3];
  for (int d = 0; d < 3; ++d) { o_f[d] = t; t = align_up(t + 8 * (n + 1), 128); }
  for (int d = 0; d < 3; ++d) { o_s[d] = t; t = align_up(t + 8 * (n + 1), 128); }
  const size_t o_w = t; t = align_up(t + 4 * (n + 1), 128);
  const size_t o_seg = t; t = align_up(t + sizeof(int4) * segs.size(), 128);
  const size_t o_cs = t; t = align_up(t + 4 * cta_seg.size(), 128);
  if (t > L.dtab_bytes) {
    if (L.dtab) { cudaFree(L.dtab); L.dtab = nullptr; L.dtab_bytes = 0; }
    CK(cudaMalloc(&L.dtab, t));
    L.dtab_bytes = t;
  }
  std::vector<char> host(t, 0);
  std::memcpy(&host[o_box], L.hbox.data(), sizeof(BoxRec) * n);
  if (!L.hface.empty()) std::memcpy(&host[o_face], L.hface.data(), sizeof(FaceRec) * L.hface.size());
  std::memcpy(&host[o_cls], L.cls.data(), sizeof(DClosures) * L.cls.size());
  if (tma_all) std::memcpy(&host[o_maps], maps.data(), sizeof(CUtensorMap) * n);
  std::memcpy(&host[o_p], L.pcell.data(), 8 * (n + 1));
  std::memcpy(&host[o_v], L.vcell.data(), 8 * (n + 1));
  std::memcpy(&host[o_g], L.gcell.data(), 8 * (n + 1));
  std::memcpy(&host[o_va], L.valid.data(), 8 * (n + 1));
  for (int d = 0; d < 3; ++d) {
    std::memcpy(&host[o_f[d]], L.fpre[d].data(), 8 * (n + 1));
    std::memcpy(&host[o_s[d]], L.spre[d].data(), 8 * (n + 1));
  }
  std::memcpy(&host[o_w], L.fwork.data(), 4 * (n + 1));
  if (!segs.empty()) std::memcpy(&host[o_seg], segs.data(), sizeof(int4) * segs.size());
  if (!cta_seg.empty()) std::memcpy(&host[o_cs], cta_seg.data(), 4 * cta_seg.size());
  CK(cudaMemcpy(L.dtab, host.data(), t, cudaMemcpyHostToDevice));
  char* D = static_cast<char*>(L.dtab);
  L.tb.box = reinterpret_cast<const BoxRec*>(D + o_box);
  L.tb.pcell = reinterpret_cast<const long long*>(D + o_p);
  L.tb.vcell = reinterpret_cast<const long long*>(D + o_v);
  L.tb.fwork = reinterpret_cast<const int*>(D + o_w);
  L.tb.seg = reinterpret_cast<const int4*>(D + o_seg);
  L.tb.cta_seg = reinterpret_cast<const int*>(D + o_cs);
  L.tb.cls = reinterpret_cast<const DClosures*>(D + o_cls);
  L.tb.n = n;
  L.tb.gq = L.gq;
  L.ft.fr = reinterpret_cast<const FaceRec*>(D + o_face);
  for (int d = 0; d < 3; ++d) {
    L.ft.fpre[d] = reinterpret_cast<const long long*>(D + o_f[d]);
    L.d_spre[d] = reinterpret_cast<const long long*>(D + o_s[d]);
  }
  L.ft.gpre = reinterpret_cast<const long long*>(D + o_g);
  L.ft.vpre = reinterpret_cast<const long long*>(D + o_va);
  L.tma.maps = tma_all ? reinterpret_cast<const CUtensorMap*>(D + o_maps) : nullptr;
  L.tma.enabled = tma_all ? 1 : 0;
  return AMRS_OK;
}

DProg to_dprog(const amrs_stage_prog* p) {
  DProg d{};
  d.nops = p ? p->nops : 0;
  for (int i = 0; i < 3; ++i) {
    if (p && i < p->nops) {
      d.ops[i].kind = p->ops[i].kind; d.ops[i].dst = p->ops[i].dst; d.ops[i].x = p->ops[i].x;
      d.ops[i].y = p->ops[i].y; d.ops[i].a = p->ops[i].a; d.ops[i].b = p->ops[i].b;
    }
  }
  return d;
}

// One RHS evaluation (+ stage program) over the list: the kernel sequence of
// CNS::compute_rhs (src/tim/CNS_advance.cpp:186-391).
amrs_status list_stage(amrs_handle* h, List& L, const DProg& prog, int s_in, int s_s1, int s_out, int rhs_only,
                       cudaStream_t st) {
  const amrs_scheme& sc = L.sc;
  const int nsm = h->nsm;
  // 1. primitives over the grown boxes
  if (L.gq > 0 || sc.rhs_visc) CK(launch_prims(L.tb, s_in, L.tot_p, nsm, st));
  // 2. viscous cell fluxes
  if (sc.rhs_visc) CK(launch_visc(L.tb, L.tot_v, nsm, st));
  if (L.fused) {
    // 3. fused KEEP faces + viscous averages + divergence + stage program
    CK(launch_keep_face(sc.order_keep, sc.rhs_visc != 0, L.source, L.tb, s_in, s_s1, s_out, prog, rhs_only, L.tma,
                        h->derr, L.face_grid, nsm, st));
    if (h->check_nonfinite) CK(launch_nonfinite_check(L.tb, L.ft.vpre, s_out, L.tot_valid, h->derr + 1, nsm, st));
    return AMRS_OK;
  }
  long long nf[3] = {L.tot_f[0], L.tot_f[1], L.tot_f[2]};
  // face arrays start from zero (pure viscous runs add to them)
  for (int b = 0; b < L.n; ++b)
    for (int d = 0; d < 3; ++d) {
      const FaceRec& F = L.hface[b];
      CK(cudaMemsetAsync(F.f[d].p, 0, (size_t)F.f[d].ns * NCONS * 8, st));
    }
  if (sc.rhs_euler) {
    if (sc.flux_euler == 1) CK(launch_keep_faces_plain(sc.order_keep, L.tb, L.ft, nf, nsm, st));
    else if (sc.flux_euler == 2) CK(launch_weno(L.tb, L.ft, s_in, L.tot_g, nf, sc.weno_fast == 0, nsm, st));
    else if (sc.flux_euler == 3) CK(launch_weno_riemann(L.tb, L.ft, nf, nsm, st));
    else {
      long long ns[3] = {L.tot_s[0], L.tot_s[1], L.tot_s[2]};
      CK(launch_riemann(L.tb, L.ft, L.d_spre, ns, nf, nsm, st));
    }
    if (sc.art_diss == 1) {
      for (int b = 0; b < L.n; ++b) {
        const FaceRec& F = L.hface[b];
        CK(cudaMemsetAsync(F.sen.p, 0, (size_t)F.sen.ns * 3 * 8, st));
        CK(cudaMemsetAsync(F.lam.p, 0, (size_t)F.lam.ns * 3 * 8, st));
      }
      CK(launch_jst(L.tb, L.ft, s_in, L.tot_g, L.tot_valid, nf, nsm, st));
    }
  }
  if (sc.rhs_visc) CK(launch_visc_face_add(L.tb, L.ft, nf, nsm, st));
  CK(launch_div_stage(L.tb, L.ft, s_in, s_s1, s_out, prog, rhs_only, L.tot_valid, nsm, st));
  if (h->check_nonfinite) CK(launch_nonfinite_check(L.tb, L.ft.vpre, s_out, L.tot_valid, h->derr + 1, nsm, st));
  return AMRS_OK;
}

bool same_box(const amrs_box& a, const amrs_box& b) {
  for (int d = 0; d < 3; ++d)
    if (a.lo[d] != b.lo[d] || a.hi[d] != b.hi[d]) return false;
  return true;
}

// Per-box calls reuse one single-box list; its tables are rebuilt only when
// the box or the arrays change.
// Per-box calls: the geometry tables (prefixes, schedule, scratch, tensor
// maps) of the single-box list are rebuilt only when the box or its cell
// size changes; the per-call box record (state pointers) goes through a ring
// of device records filled from pinned staging by an async copy on the
// call's stream.  A ring entry is reused only after the event recorded
// behind the kernels of its previous call has completed.
constexpr int RING = 64;

amrs_status one_box(amrs_handle* h, const amrs_box* bx, const double dxinv[3], const amrs_array4* slots, int nslots,
                    cudaStream_t st, const double* dx_override = nullptr) {
  List*& L = h->one;
  bool same = L && L->n == 1 && same_box(L->boxes[0], *bx) && L->nslots == nslots;
  if (same) {
    const BoxRec& R = L->hbox[0];
    for (int d = 0; d < 3 && same; ++d) same = R.dxinv[d] == dxinv[d];
  }
  if (!same) {
    if (!L) L = new (std::nothrow) List();
    if (!L) return AMRS_ERR_ALLOC;
    if (L->graph) { cudaGraphExecDestroy(L->graph); L->graph = nullptr; }
    // the previous tables may still be read by queued kernels
    CK(cudaDeviceSynchronize());
    if (amrs_status s = list_build(h, *L, 1, bx, dxinv, nslots, slots, nullptr, 0, nullptr, nullptr)) return s;
  }
  if (!h->dring) {
    CK(cudaMalloc(&h->dring, sizeof(BoxRec) * RING));
    CK(cudaMallocHost(&h->hring, sizeof(BoxRec) * RING));
    for (int i = 0; i < RING; ++i) {
      CK(cudaEventCreateWithFlags(&h->ring_ev[i], cudaEventDisableTiming));
      h->ring_used[i] = 0;
    }
  }
  const int i = h->ring_pos;
  h->ring_pos = (i + 1) % RING;
  if (h->ring_used[i]) CK(cudaEventSynchronize(h->ring_ev[i]));
  BoxRec R = L->hbox[0];
  for (int s = 0; s < nslots; ++s) R.slot[s] = to_darr(slots[s]);
  set_walls(R, h->wall, h->sc);
  if (dx_override)
    for (int d = 0; d < 3; ++d) R.dx[d] = dx_override[d];
  h->hring[i] = R;
  CK(cudaMemcpyAsync(&h->dring[i], &h->hring[i], sizeof(BoxRec), cudaMemcpyHostToDevice, st));
  L->tb.box = &h->dring[i];
  h->ring_cur = i;
  return AMRS_OK;
}

// Mark the current ring entry as in use by the work queued on `st`.
void ring_release(amrs_handle* h, cudaStream_t st) {
  const int i = h->ring_cur;
  if (i >= 0 && cudaEventRecord(h->ring_ev[i], st) == cudaSuccess) h->ring_used[i] = 1;
}

}  // namespace

// ===================================================================== API ==
extern "C" {

int32_t amrs_version(void) { return 100; }
int32_t amrs_cuda_arch(void) { return 1030; }

const char* amrs_last_cuda_error(void) { return g_cuda_err.c_str(); }

const char* amrs_status_string(amrs_status s) {
  switch (s) {
    case AMRS_OK: return "ok";
    case AMRS_ERR_NULL: return "null pointer";
    case AMRS_ERR_BOX: return "bad box";
    case AMRS_ERR_BC: return "unsupported boundary condition";
    case AMRS_ERR_SCHEME: return "unsupported scheme";
    case AMRS_ERR_RK: return "unsupported RK order/stages";
    case AMRS_ERR_CUDA: return "CUDA error";
    case AMRS_ERR_ALLOC: return "allocation failed";
    case AMRS_ERR_LAYOUT: return "array layout does not cover the box";
    case AMRS_ERR_SIZE: return "size beyond limit";
    case AMRS_ERR_NONFINITE: return "non-finite value";
    case AMRS_ERR_TIMEOUT: return "device wait timed out";
    case AMRS_ERR_STATE: return "invalid call sequence";
  }
  return "unknown status";
}

amrs_status amrs_create(amrs_handle** out, const amrs_scheme* scheme, const amrs_closures* closures, int device) {
  if (!out || !scheme || !closures) return AMRS_ERR_NULL;
  *out = nullptr;
  if (amrs_status s = check_scheme(*scheme)) return s;
  amrs_handle* h = new (std::nothrow) amrs_handle();
  if (!h) return AMRS_ERR_ALLOC;
  h->device = device;
  h->sc = canonical_scheme(*scheme);
  h->cl = *closures;
  cudaError_t e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&h->nsm, cudaDevAttrMultiProcessorCount, device);
  if (e == cudaSuccess) e = cudaMalloc(&h->derr, 64);
  if (e == cudaSuccess) e = cudaMemset(h->derr, 0, 64);
  if (e == cudaSuccess) e = cudaMalloc(&h->dred, 64);
  if (e != cudaSuccess) {
    amrs_status s = cuda_fail(e, "amrs_create");
    amrs_destroy(h);
    return s;
  }
  const char* tma_env = std::getenv("AMRS_TMA");
  h->tma_ok = !(tma_env && tma_env[0] == '0');
  cudaDriverEntryPointQueryResult q;
  void* fn = nullptr;
  if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) == cudaSuccess &&
      q == cudaDriverEntryPointSuccess)
    h->encode_fn = fn;
  *out = h;
  return AMRS_OK;
}

amrs_status amrs_destroy(amrs_handle* h) {
  if (!h) return AMRS_ERR_NULL;
  cudaSetDevice(h->device);
  delete h->one;
  if (h->adj) cudaFree(h->adj);
  if (h->dring) {
    cudaFree(h->dring);
    cudaFreeHost(h->hring);
    for (int i = 0; i < 64; ++i) cudaEventDestroy(h->ring_ev[i]);
  }
  if (h->derr) cudaFree(h->derr);
  if (h->dred) cudaFree(h->dred);
  delete h;
  return AMRS_OK;
}

amrs_status amrs_set_closures(amrs_handle* h, const amrs_closures* closures) {
  if (!h || !closures) return AMRS_ERR_NULL;
  std::lock_guard<std::mutex> lk(h->mu);
  h->cl = *closures;
  if (h->one) { CK(cudaDeviceSynchronize()); delete h->one; h->one = nullptr; }
  return AMRS_OK;
}

amrs_status amrs_set_source(amrs_handle* h, int32_t rhs_source, const double force[3]) {
  if (!h) return AMRS_ERR_NULL;
  if (rhs_source && !force) return AMRS_ERR_NULL;
  std::lock_guard<std::mutex> lk(h->mu);
  const bool on = rhs_source && (force[0] != 0.0 || force[1] != 0.0 || force[2] != 0.0);
  for (int d = 0; d < 3; ++d) {
    if (on && !std::isfinite(force[d])) return AMRS_ERR_SCHEME;
    h->force[d] = on ? force[d] : 0.0;
  }
  h->source = on ? 1 : 0;
  // the per-box list caches its closures table
  if (h->one) { CK(cudaDeviceSynchronize()); delete h->one; h->one = nullptr; }
  return AMRS_OK;
}

amrs_status amrs_set_domain(amrs_handle* h, const amrs_box* domain, const int32_t bc_lo[3], const int32_t bc_hi[3]) {
  if (!h) return AMRS_ERR_NULL;
  std::lock_guard<std::mutex> lk(h->mu);
  if (!domain || !bc_lo || !bc_hi) {
    h->wall = WallCfg{};
    return AMRS_OK;
  }
  if (!box_ok(*domain)) return AMRS_ERR_BOX;
  for (int d = 0; d < 3; ++d) {
    if ((bc_lo[d] == -1) != (bc_hi[d] == -1)) return AMRS_ERR_BC;
    if (bc_lo[d] < -1 || bc_lo[d] > 6 || bc_hi[d] < -1 || bc_hi[d] > 6) return AMRS_ERR_BC;
  }
  WallCfg w;
  w.lo = bc_lo[1] == 6; w.hi = bc_hi[1] == 6; w.dom_lo = domain->lo[1]; w.dom_hi = domain->hi[1];
  h->wall = w;
  return AMRS_OK;
}

amrs_status amrs_rk_program(int32_t order_rk, int32_t stages_rk, double dt, amrs_stage_prog* st, int32_t cap,
                            int32_t* nstages) {
  if (!st || !nstages) return AMRS_ERR_NULL;
  return rk_build(order_rk, stages_rk, dt, st, cap, nstages, nullptr);
}

amrs_status amrs_rhs_box(amrs_handle* h, const amrs_box* bx, const double dxinv[3], amrs_array4 state,
                         amrs_array4 dsdt, void* stream) {
  if (!h || !bx || !dxinv) return AMRS_ERR_NULL;
  if (!box_ok(*bx)) return AMRS_ERR_BOX;
  if (!covers(state, *bx, NGHOST, NCONS) || !covers(dsdt, *bx, 0, NCONS)) return AMRS_ERR_LAYOUT;
  std::lock_guard<std::mutex> lk(h->mu);
  CK(cudaSetDevice(h->device));
  amrs_array4 slots[3] = {state, state, dsdt};
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (amrs_status s = one_box(h, bx, dxinv, slots, 3, st)) return s;
  DProg p{};
  amrs_status rs = list_stage(h, *h->one, p, 0, 1, 2, 1, st);
  ring_release(h, st);
  return rs;
}

amrs_status amrs_rk_stage_box(amrs_handle* h, const amrs_box* bx, const double dxinv[3], const amrs_stage_prog* prog,
                              double dt, amrs_array4 stage_in, amrs_array4 s1, amrs_array4 out, void* stream) {
  (void)dt;
  if (!h || !bx || !dxinv || !prog) return AMRS_ERR_NULL;
  if (!box_ok(*bx)) return AMRS_ERR_BOX;
  if (prog->nops < 0 || prog->nops > 3) return AMRS_ERR_RK;
  if (!covers(stage_in, *bx, NGHOST, NCONS) || !covers(s1, *bx, 0, NCONS) || !covers(out, *bx, 0, NCONS))
    return AMRS_ERR_LAYOUT;
  if (out.p == stage_in.p) return AMRS_ERR_LAYOUT;
  std::lock_guard<std::mutex> lk(h->mu);
  CK(cudaSetDevice(h->device));
  amrs_array4 slots[3] = {stage_in, s1, out};
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (amrs_status s = one_box(h, bx, dxinv, slots, 3, st)) return s;
  amrs_status rs = list_stage(h, *h->one, to_dprog(prog), 0, 1, 2, 0, st);
  ring_release(h, st);
  return rs;
}

amrs_status amrs_fill_halo_box(const amrs_box* domain, const int32_t bc_lo[3], const int32_t bc_hi[3],
                               amrs_array4 state, void* stream) {
  if (!domain || !bc_lo || !bc_hi) return AMRS_ERR_NULL;
  if (!box_ok(*domain)) return AMRS_ERR_BOX;
  if (!covers(state, *domain, NGHOST, 1)) return AMRS_ERR_LAYOUT;
  HaloBox hb;
  hb.u = to_darr(state);
  hb.ncomp = state.ncomp;
  for (int d = 0; d < 3; ++d) {
    if ((bc_lo[d] == -1) != (bc_hi[d] == -1)) return AMRS_ERR_BC;
    for (int s = 0; s < 2; ++s) {
      const int p = s ? bc_hi[d] : bc_lo[d];
      if (p < -1 || p > 6) return AMRS_ERR_BC;  // 1, 6: ext_dir, caller-filled
    }
    if (bn(*domain, d) < NGHOST && bc_lo[d] != -1 && bc_lo[d] != 2) return AMRS_ERR_BOX;
    hb.lo[d] = domain->lo[d]; hb.hi[d] = domain->hi[d]; hb.bc_lo[d] = bc_lo[d]; hb.bc_hi[d] = bc_hi[d];
  }
  CK(launch_halo(hb, static_cast<cudaStream_t>(stream)));
  return AMRS_OK;
}

amrs_status amrs_fill_halo_box_bcnormal(const amrs_box* domain, const int32_t bc_lo[3], const int32_t bc_hi[3],
                                        const amrs_closures* closures, const amrs_bcnormal* bnp, amrs_array4 state,
                                        void* stream) {
  if (!closures || !bnp) return AMRS_ERR_NULL;
  if (amrs_status s = check_bcnormal(*bnp)) return s;
  if (state.ncomp < NCONS) return AMRS_ERR_LAYOUT;
  if (amrs_status s = amrs_fill_halo_box(domain, bc_lo, bc_hi, state, stream)) return s;
  const int lo[3] = {domain->lo[0], domain->lo[1], domain->lo[2]};
  const int hi[3] = {domain->hi[0], domain->hi[1], domain->hi[2]};
  const int bl[3] = {bc_lo[0], bc_lo[1], bc_lo[2]}, bh[3] = {bc_hi[0], bc_hi[1], bc_hi[2]};
  CK(launch_bcnormal_box(to_darr(state), lo, hi, bl, bh, to_dev(*closures), to_dbcn(*bnp),
                         static_cast<cudaStream_t>(stream)));
  return AMRS_OK;
}

amrs_status amrs_average_down(const amrs_box* crse_box, const int32_t ratio[3], amrs_array4 fine, amrs_array4 crse,
                               int32_t scomp, int32_t ncomp, void* stream) {
  if (!crse_box || !ratio) return AMRS_ERR_NULL;
  if (!box_ok(*crse_box)) return AMRS_ERR_BOX;
  if (scomp < 0 || ncomp < 1) return AMRS_ERR_LAYOUT;
  amrs_box fb;
  int r[3], lo[3], n[3];
  for (int d = 0; d < 3; ++d) {
    if (ratio[d] < 1 || ratio[d] > 16) return AMRS_ERR_SIZE;
    r[d] = ratio[d];
    lo[d] = crse_box->lo[d];
    n[d] = bn(*crse_box, d);
    fb.lo[d] = crse_box->lo[d] * ratio[d];
    fb.hi[d] = (crse_box->hi[d] + 1) * ratio[d] - 1;
  }
  if (!box_ok(fb)) return AMRS_ERR_BOX;
  if (!covers(fine, fb, 0, scomp + ncomp) || !covers(crse, *crse_box, 0, scomp + ncomp)) return AMRS_ERR_LAYOUT;
  if (fine.p == crse.p) return AMRS_ERR_LAYOUT;
  int dev = 0, nsm = 1;
  CK(cudaGetDevice(&dev));
  CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  CK(launch_avgdown(to_darr(fine), to_darr(crse), lo, n, r, scomp, ncomp, 1.0 / (double)(r[0] * r[1] * r[2]), nsm,
                    static_cast<cudaStream_t>(stream)));
  return AMRS_OK;
}

amrs_status amrs_plot_derive_box(const amrs_closures* closures, const amrs_box* bx, amrs_array4 state, amrs_array4 out,
                                 void* stream) {
  if (!closures || !bx) return AMRS_ERR_NULL;
  if (!box_ok(*bx)) return AMRS_ERR_BOX;
  if (!covers(state, *bx, 0, NCONS) || !covers(out, *bx, 0, 5)) return AMRS_ERR_LAYOUT;
  if (!(closures->cv > 0.0)) return AMRS_ERR_SCHEME;
  int dev = 0, nsm = 0;
  CK(cudaGetDevice(&dev));
  CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  const int lo[3] = {bx->lo[0], bx->lo[1], bx->lo[2]};
  const int n[3] = {bn(*bx, 0), bn(*bx, 1), bn(*bx, 2)};
  CK(launch_plot_derive(to_darr(state), to_darr(out), lo, n, closures->gamma, closures->cv, nsm,
                        static_cast<cudaStream_t>(stream)));
  return AMRS_OK;
}

amrs_status amrs_est_timestep_box(amrs_handle* h, const amrs_box* bx, const double dx[3], double cfl,
                                  amrs_array4 state, double* dt_device, void* stream) {
  if (!h || !bx || !dx || !dt_device) return AMRS_ERR_NULL;
  if (!box_ok(*bx)) return AMRS_ERR_BOX;
  if (!covers(state, *bx, 0, NCONS)) return AMRS_ERR_LAYOUT;
  std::lock_guard<std::mutex> lk(h->mu);
  CK(cudaSetDevice(h->device));
  amrs_array4 slots[3] = {state, state, state};
  const double dxinv[3] = {1.0 / dx[0], 1.0 / dx[1], 1.0 / dx[2]};
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  // cns_estdt divides dx by the wave speed: the record carries dx exactly as given
  if (amrs_status s = one_box(h, bx, dxinv, slots, 3, st, dx)) return s;
  List& L = *h->one;
  cudaError_t e = launch_estdt(L.tb, 0, L.tot_valid, cfl, h->dred, dt_device, h->nsm, st);
  ring_release(h, st);
  if (e != cudaSuccess) return cuda_fail(e, "launch_estdt");
  return AMRS_OK;
}

amrs_status amrs_prim_stats_box(amrs_handle* h, const amrs_box* bx, const double dx[3], amrs_array4 state, double dt,
                                double* out, void* stream) {
  if (!h || !bx || !dx || !out) return AMRS_ERR_NULL;
  if (!box_ok(*bx)) return AMRS_ERR_BOX;
  if (!covers(state, *bx, 0, NCONS)) return AMRS_ERR_LAYOUT;
  double dxinv[3];
  for (int d = 0; d < 3; ++d) {
    if (!(dx[d] > 0.0)) return AMRS_ERR_BOX;
    dxinv[d] = 1.0 / dx[d];
  }
  std::lock_guard<std::mutex> lk(h->mu);
  CK(cudaSetDevice(h->device));
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  amrs_array4 slots[3] = {state, state, state};
  if (amrs_status s = one_box(h, bx, dxinv, slots, 3, st)) return s;
  List& L = *h->one;
  cudaError_t e = cudaSuccess;
  if (!L.d_stats) e = cudaMalloc(&L.d_stats, 32 * sizeof(unsigned long long));
  if (e == cudaSuccess) e = launch_prim_stats(L.tb, L.ft.vpre, 0, dt, dx, L.tot_valid, L.d_stats, out, h->nsm, st);
  ring_release(h, st);
  if (e != cudaSuccess) return cuda_fail(e, "amrs_prim_stats_box");
  return AMRS_OK;
}

amrs_status amrs_boxlist_create(amrs_handle* h, int32_t nboxes, const amrs_box* boxes, const double* dxinv3,
                                int32_t nslots, const amrs_array4* states, const int32_t* closure_index,
                                int32_t nclosures, const amrs_closures* closures, amrs_boxlist** out) {
  if (!h || !boxes || !dxinv3 || !states || !out) return AMRS_ERR_NULL;
  *out = nullptr;
  if (nboxes <= 0 || nslots < 1 || nslots > MAX_SLOTS) return AMRS_ERR_SIZE;
  if (closure_index && (nclosures <= 0 || !closures)) return AMRS_ERR_NULL;
  for (int b = 0; b < nboxes; ++b) {
    if (!box_ok(boxes[b])) return AMRS_ERR_BOX;
    for (int s = 0; s < nslots; ++s)
      if (!covers(states[b * nslots + s], boxes[b], NGHOST, NCONS)) return AMRS_ERR_LAYOUT;
    if (closure_index && (closure_index[b] < 0 || closure_index[b] >= nclosures)) return AMRS_ERR_SIZE;
  }
  std::lock_guard<std::mutex> lk(h->mu);
  CK(cudaSetDevice(h->device));
  amrs_boxlist* bl = new (std::nothrow) amrs_boxlist();
  if (!bl) return AMRS_ERR_ALLOC;
  bl->h = h;
  bl->device = h->device;
  amrs_status s = list_build(h, bl->L, nboxes, boxes, dxinv3, nslots, states, closure_index,
                             closure_index ? nclosures : 0, closures, nullptr);
  if (s) { delete bl; return s; }
  *out = bl;
  return AMRS_OK;
}

amrs_status amrs_boxlist_destroy(amrs_boxlist* bl) {
  if (!bl) return AMRS_ERR_NULL;
  cudaError_t e = cudaSetDevice(bl->device);
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  delete bl;
  if (e != cudaSuccess) return cuda_fail(e, "amrs_boxlist_destroy");
  return AMRS_OK;
}

}  // extern "C"

namespace {

// Rebuild a list's tables with per-box tiles (tiles[3*b] = tx, ty, kchunk).
amrs_status relist_with_tiles(amrs_boxlist* bl, const std::vector<int>& tiles) {
  List& L = bl->L;
  std::vector<amrs_array4> states(L.n * L.nslots);
  std::vector<double> dxinv(3 * L.n);
  std::vector<int32_t> cidx(L.n);
  std::vector<amrs_closures> cls(L.cls.size());
  for (int b = 0; b < L.n; ++b) {
    const BoxRec& R = L.hbox[b];
    for (int d = 0; d < 3; ++d) dxinv[3 * b + d] = R.dxinv[d];
    cidx[b] = R.cl;
    for (int s = 0; s < L.nslots; ++s) {
      amrs_array4 a{};
      a.p = R.slot[s].p; a.jstride = R.slot[s].js; a.kstride = R.slot[s].ks; a.nstride = R.slot[s].ns;
      a.begin[0] = R.slot[s].b0; a.begin[1] = R.slot[s].b1; a.begin[2] = R.slot[s].b2;
      const amrs_box& B = L.boxes[b];
      for (int d = 0; d < 3; ++d) a.end[d] = B.hi[d] + NGHOST + 1;
      a.ncomp = NCONS;
      states[b * L.nslots + s] = a;
    }
  }
  for (size_t c = 0; c < L.cls.size(); ++c) {
    const DClosures& d = L.cls[c];
    amrs_closures& o = cls[c];
    o.gamma = d.gamma; o.cv = d.cv; o.cp = d.cp; o.Rspec = d.Rspec; o.visc_law = d.visc_law; o.cond_law = d.cond_law;
    o.visc_ref = d.visc_ref; o.Tvisc_ref = d.Tvisc_ref; o.cond_ref = d.cond_ref; o.Tcond_ref = d.Tcond_ref;
    o.Cshock = d.Cshock; o.Cdamp = d.Cdamp;
  }
  std::vector<amrs_box> boxes = L.boxes;
  // recorded graphs hold the old tables' addresses
  if (L.graph) { cudaGraphExecDestroy(L.graph); L.graph = nullptr; }
  if (L.run_graph) { cudaGraphExecDestroy(L.run_graph); L.run_graph = nullptr; }
  return list_build(bl->h, L, L.n, boxes.data(), dxinv.data(), L.nslots, states.data(), cidx.data(),
                    (int)cls.size(), cls.data(), tiles.data());
}

// Host mirror of the device map_coord (coordinates only): the domain cell a
// ghost coordinate reads under periodic / foextrap / reflecting boundaries.
int map_coord_host(int c, int lo, int hi, int bcl, int bch) {
  if (c >= lo && c <= hi) return c;
  const int n = hi - lo + 1;
  const bool low = c < lo;
  const int phys = low ? bcl : bch;
  if (phys == -1) {
    int r = (c - lo) % n;
    if (r < 0) r += n;
    return lo + r;
  }
  if (phys == 2) return low ? lo : hi;
  return low ? 2 * lo - c - 1 : 2 * hi - c + 1;
}

bool box_has(const amrs_box& b, int i, int j, int k) {
  return i >= b.lo[0] && i <= b.hi[0] && j >= b.lo[1] && j <= b.hi[1] && k >= b.lo[2] && k <= b.hi[2];
}

bool boxes_meet(const amrs_box& a, const amrs_box& b) {
  for (int d = 0; d < 3; ++d)
    if (a.hi[d] < b.lo[d] || b.hi[d] < a.lo[d]) return false;
  return true;
}

// Owner table of a level tiling `dom`: for every cell of every grow(box,3)
// (in the order of the flattened ghost-fill launch) the box whose valid
// cell the ghost reads, -1 for valid cells.  Boxes must be disjoint and
// every source cell covered (AMRS_ERR_BOX otherwise).
amrs_status level_owner_table(const List& L, const LevelDomain& dom, std::vector<int>& owner) {
  constexpr int BS = 8;  // bins of 8^3 domain cells listing the boxes that meet them
  int nb[3];
  for (int d = 0; d < 3; ++d) nb[d] = (dom.hi[d] - dom.lo[d] + BS) / BS;
  std::vector<std::vector<int>> bins((size_t)nb[0] * nb[1] * nb[2]);
  auto bin_of = [&](int i, int j, int k) {
    return ((size_t)((k - dom.lo[2]) / BS) * nb[1] + (size_t)((j - dom.lo[1]) / BS)) * nb[0] +
           (size_t)((i - dom.lo[0]) / BS);
  };
  for (int b = 0; b < L.n; ++b) {
    const amrs_box& B = L.boxes[b];
    int b0[3], b1[3];
    for (int d = 0; d < 3; ++d) { b0[d] = (B.lo[d] - dom.lo[d]) / BS; b1[d] = (B.hi[d] - dom.lo[d]) / BS; }
    for (int z = b0[2]; z <= b1[2]; ++z)
      for (int y = b0[1]; y <= b1[1]; ++y)
        for (int x = b0[0]; x <= b1[0]; ++x) {
          auto& v = bins[((size_t)z * nb[1] + y) * nb[0] + x];
          for (int o : v)
            if (boxes_meet(L.boxes[o], B)) return AMRS_ERR_BOX;  // overlapping boxes
          v.push_back(b);
        }
  }
  owner.assign((size_t)L.gcell[L.n], -1);
  const int g = NGHOST;
  for (int b = 0; b < L.n; ++b) {
    const amrs_box& B = L.boxes[b];
    size_t idx = (size_t)L.gcell[b];
    for (int k = B.lo[2] - g; k <= B.hi[2] + g; ++k)
      for (int j = B.lo[1] - g; j <= B.hi[1] + g; ++j)
        for (int i = B.lo[0] - g; i <= B.hi[0] + g; ++i, ++idx) {
          if (box_has(B, i, j, k)) continue;
          // beyond an ext_dir side (codes 1, 6) the caller's values stay
          bool ext = false;
          const int cc[3] = {i, j, k};
          for (int d = 0; d < 3; ++d) {
            const int p = cc[d] < dom.lo[d] ? dom.bc_lo[d] : (cc[d] > dom.hi[d] ? dom.bc_hi[d] : 0);
            if (p == 1 || p == 6) ext = true;
          }
          if (ext) continue;
          const int si = map_coord_host(i, dom.lo[0], dom.hi[0], dom.bc_lo[0], dom.bc_hi[0]);
          const int sj = map_coord_host(j, dom.lo[1], dom.hi[1], dom.bc_lo[1], dom.bc_hi[1]);
          const int sk = map_coord_host(k, dom.lo[2], dom.hi[2], dom.bc_lo[2], dom.bc_hi[2]);
          int src = -1;
          for (int o : bins[bin_of(si, sj, sk)])
            if (box_has(L.boxes[o], si, sj, sk)) { src = o; break; }
          if (src < 0) return AMRS_ERR_BOX;  // the level does not cover this source cell
          owner[idx] = src;
        }
  }
  return AMRS_OK;
}

// Ghost fill of one state slot of every box of a list (before a stage).
cudaError_t list_fill(amrs_handle* h, List& L, int slot, cudaStream_t st) {
  if (L.has_bc == 2) {
    cudaError_t e = launch_halo_level(L.tb, L.ft.gpre, L.d_owner, L.tot_g, slot, L.dom, h->nsm, st);
    // then the problem's bcnormal beyond code-6 y sides (it reads the
    // first interior row, ghost columns included, that the fill wrote)
    if (e == cudaSuccess && L.bcn.kind) e = launch_bcnormal_list(L.tb, slot, L.dom, L.bcn, h->nsm, st);
    return e;
  }
  return launch_halo_list(L.tb, L.ft.gpre, L.tot_g, slot, L.bc_lo, L.bc_hi, h->nsm, st);
}

}  // namespace

extern "C" {

amrs_status amrs_boxlist_set_tile(amrs_boxlist* bl, int32_t nx, int32_t ny, int32_t nz, int32_t tx, int32_t ty,
                                  int32_t kchunk) {
  if (!bl) return AMRS_ERR_NULL;
  List& L = bl->L;
  if (!keep_tile_fits(L.sc.order_keep, tx, ty) || kchunk < 1) return AMRS_ERR_SIZE;
  std::lock_guard<std::mutex> lk(bl->h->mu);
  CK(cudaSetDevice(bl->h->device));
  CK(cudaDeviceSynchronize());
  std::vector<int> tiles(3 * L.n);
  for (int b = 0; b < L.n; ++b) {
    const BoxRec& R = L.hbox[b];
    const bool match = (nx == 0 && ny == 0 && nz == 0) ||
                       (bn(L.boxes[b], 0) == nx && bn(L.boxes[b], 1) == ny && bn(L.boxes[b], 2) == nz);
    tiles[3 * b] = match ? tx : R.tx;
    tiles[3 * b + 1] = match ? ty : R.ty;
    tiles[3 * b + 2] = match ? std::min<int>(kchunk, bn(L.boxes[b], 2)) : R.kc;
  }
  return relist_with_tiles(bl, tiles);
}

amrs_status amrs_boxlist_set_tiles(amrs_boxlist* bl, const int32_t* tiles) {
  if (!bl || !tiles) return AMRS_ERR_NULL;
  List& L = bl->L;
  std::vector<int> t(3 * L.n);
  for (int b = 0; b < L.n; ++b) {
    if (!keep_tile_fits(L.sc.order_keep, tiles[3 * b], tiles[3 * b + 1]) || tiles[3 * b + 2] < 1)
      return AMRS_ERR_SIZE;
    t[3 * b] = tiles[3 * b];
    t[3 * b + 1] = tiles[3 * b + 1];
    t[3 * b + 2] = std::min<int>(tiles[3 * b + 2], bn(L.boxes[b], 2));
  }
  std::lock_guard<std::mutex> lk(bl->h->mu);
  CK(cudaSetDevice(bl->h->device));
  CK(cudaDeviceSynchronize());
  return relist_with_tiles(bl, t);
}

amrs_status amrs_boxlist_set_schedule(amrs_boxlist* bl, int32_t waves) {
  if (!bl) return AMRS_ERR_NULL;
  if (waves < 1 || waves > 8) return AMRS_ERR_SIZE;
  List& L = bl->L;
  std::lock_guard<std::mutex> lk(bl->h->mu);
  CK(cudaSetDevice(bl->h->device));
  CK(cudaDeviceSynchronize());
  L.waves = waves;
  std::vector<int> t(3 * L.n);
  for (int b = 0; b < L.n; ++b) {
    t[3 * b] = L.hbox[b].tx;
    t[3 * b + 1] = L.hbox[b].ty;
    t[3 * b + 2] = L.hbox[b].kc;
  }
  return relist_with_tiles(bl, t);
}

int32_t amrs_boxlist_face_grid(amrs_boxlist* bl) { return bl ? bl->L.face_grid : -1; }

amrs_status amrs_boxlist_get_tiles(amrs_boxlist* bl, int32_t* tiles) {
  if (!bl || !tiles) return AMRS_ERR_NULL;
  const List& L = bl->L;
  for (int b = 0; b < L.n; ++b) {
    tiles[3 * b] = L.hbox[b].tx;
    tiles[3 * b + 1] = L.hbox[b].ty;
    tiles[3 * b + 2] = L.hbox[b].kc;
  }
  return AMRS_OK;
}

amrs_status amrs_boxlist_set_bc(amrs_boxlist* bl, const int32_t bc_lo[3], const int32_t bc_hi[3]) {
  if (!bl) return AMRS_ERR_NULL;
  List& L = bl->L;
  if (!bc_lo || !bc_hi) {
    L.has_bc = 0;
  } else {
    for (int d = 0; d < 3; ++d) {
      if ((bc_lo[d] == -1) != (bc_hi[d] == -1)) return AMRS_ERR_BC;
      for (int s = 0; s < 2; ++s) {
        const int p = s ? bc_hi[d] : bc_lo[d];
        if (p < -1 || p > 6) return AMRS_ERR_BC;  // 1, 6: ext_dir, caller-filled
      }
      for (int b = 0; b < L.n; ++b)
        if (bn(L.boxes[b], d) < NGHOST && bc_lo[d] != -1 && bc_lo[d] != 2) return AMRS_ERR_BOX;
      L.bc_lo[d] = bc_lo[d];
      L.bc_hi[d] = bc_hi[d];
    }
    L.has_bc = 1;
  }
  if (L.graph) { cudaGraphExecDestroy(L.graph); L.graph = nullptr; }
  return AMRS_OK;
}

amrs_status amrs_boxlist_set_domain(amrs_boxlist* bl, const amrs_box* domain, const int32_t bc_lo[3],
                                    const int32_t bc_hi[3]) {
  if (!bl || !domain || !bc_lo || !bc_hi) return AMRS_ERR_NULL;
  List& L = bl->L;
  if (!box_ok(*domain)) return AMRS_ERR_BOX;
  LevelDomain dom{};
  for (int d = 0; d < 3; ++d) {
    if ((bc_lo[d] == -1) != (bc_hi[d] == -1)) return AMRS_ERR_BC;
    for (int s = 0; s < 2; ++s) {
      const int p = s ? bc_hi[d] : bc_lo[d];
      if (p < -1 || p > 6) return AMRS_ERR_BC;  // 1, 6: ext_dir, caller-filled
    }
    // reflections and periodic images stay inside a domain of >= 3 cells
    if (bn(*domain, d) < NGHOST) return AMRS_ERR_BOX;
    dom.lo[d] = domain->lo[d]; dom.hi[d] = domain->hi[d];
    dom.bc_lo[d] = bc_lo[d]; dom.bc_hi[d] = bc_hi[d];
  }
  for (int b = 0; b < L.n; ++b)
    for (int d = 0; d < 3; ++d)
      if (L.boxes[b].lo[d] < dom.lo[d] || L.boxes[b].hi[d] > dom.hi[d]) return AMRS_ERR_BOX;
  WallCfg w;
  w.lo = bc_lo[1] == 6; w.hi = bc_hi[1] == 6; w.dom_lo = dom.lo[1]; w.dom_hi = dom.hi[1];
  if (w.lo != L.wall.lo || w.hi != L.wall.hi || w.dom_lo != L.wall.dom_lo || w.dom_hi != L.wall.dom_hi) {
    // the box records carry the wall rows: rebuild the tables with the current tiles
    L.wall = w;
    std::vector<int> tiles(3 * L.n);
    for (int b = 0; b < L.n; ++b) {
      tiles[3 * b] = L.hbox[b].tx; tiles[3 * b + 1] = L.hbox[b].ty; tiles[3 * b + 2] = L.hbox[b].kc;
    }
    std::lock_guard<std::mutex> lk(bl->h->mu);
    CK(cudaSetDevice(bl->h->device));
    CK(cudaDeviceSynchronize());
    if (amrs_status s = relist_with_tiles(bl, tiles)) return s;
  }
  std::vector<int> owner;
  if (amrs_status s = level_owner_table(L, dom, owner)) return s;
  CK(cudaSetDevice(bl->h->device));
  if (L.d_owner) { CK(cudaDeviceSynchronize()); cudaFree(L.d_owner); L.d_owner = nullptr; }
  CK(cudaMalloc(&L.d_owner, owner.size() * sizeof(int)));
  CK(cudaMemcpy(L.d_owner, owner.data(), owner.size() * sizeof(int), cudaMemcpyHostToDevice));
  L.dom = dom;
  L.has_bc = 2;
  if (L.graph) { cudaGraphExecDestroy(L.graph); L.graph = nullptr; }
  if (L.run_graph) { cudaGraphExecDestroy(L.run_graph); L.run_graph = nullptr; }
  return AMRS_OK;
}

amrs_status amrs_boxlist_set_bcnormal(amrs_boxlist* bl, const amrs_bcnormal* bnp) {
  if (!bl) return AMRS_ERR_NULL;
  DBcNormal d{};
  if (bnp) {
    if (amrs_status s = check_bcnormal(*bnp)) return s;
    d = to_dbcn(*bnp);
  }
  List& L = bl->L;
  CK(cudaSetDevice(bl->h->device));
  CK(cudaDeviceSynchronize());  // queued fills may read the old setting
  L.bcn = d;
  if (L.graph) { cudaGraphExecDestroy(L.graph); L.graph = nullptr; }
  if (L.run_graph) { cudaGraphExecDestroy(L.run_graph); L.run_graph = nullptr; }
  return AMRS_OK;
}

amrs_status amrs_boxlist_fill_halo(amrs_boxlist* bl, int32_t slot, void* stream) {
  if (!bl) return AMRS_ERR_NULL;
  List& L = bl->L;
  if (!L.has_bc) return AMRS_ERR_STATE;
  if (slot < 0 || slot >= L.nslots) return AMRS_ERR_SIZE;
  CK(cudaSetDevice(bl->h->device));
  CK(list_fill(bl->h, L, slot, static_cast<cudaStream_t>(stream)));
  return AMRS_OK;
}

amrs_status amrs_rk_stage_boxlist(amrs_boxlist* bl, const amrs_stage_prog* prog, int32_t in, int32_t s1, int32_t out,
                                  void* stream) {
  if (!bl || !prog) return AMRS_ERR_NULL;
  List& L = bl->L;
  if (in < 0 || s1 < 0 || out < 0 || in >= L.nslots || s1 >= L.nslots || out >= L.nslots || in == out)
    return AMRS_ERR_SIZE;
  CK(cudaSetDevice(bl->h->device));
  return list_stage(bl->h, L, to_dprog(prog), in, s1, out, 0, static_cast<cudaStream_t>(stream));
}

amrs_status amrs_rk_step_boxlist(amrs_boxlist* bl, int32_t order_rk, int32_t stages_rk, double dt, int32_t s1,
                                 int32_t w1, int32_t w2, int32_t use_graph, void* stream, int32_t* result_slot) {
  if (!bl || !result_slot) return AMRS_ERR_NULL;
  List& L = bl->L;
  if (s1 < 0 || w1 < 0 || w2 < 0 || s1 >= L.nslots || w1 >= L.nslots || w2 >= L.nslots || s1 == w1 || s1 == w2 ||
      w1 == w2)
    return AMRS_ERR_SIZE;
  amrs_stage_prog progs[16];
  DProg forms[16];
  int32_t ns = 0;
  if (amrs_status s = rk_build(order_rk, stages_rk, dt, progs, 16, &ns, forms)) return s;
  CK(cudaSetDevice(bl->h->device));
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  // slot rotation: stage input is S1 for src_state 0, else the last output;
  // outputs alternate between the two work slots.  In a graph the stage
  // programs read dt from device memory, so one graph serves every dt.
  auto record = [&](cudaStream_t s, int* res, bool device_dt) -> amrs_status {
    int cur = s1;  // holds S2 values (stage input)
    int outs[2] = {w1, w2};
    int which = 0;
    for (int i = 0; i < ns; ++i) {
      const int in = (progs[i].src_state == 0) ? s1 : cur;
      int out = outs[which];
      if (out == in) { which ^= 1; out = outs[which]; }
      if (L.has_bc) CK(list_fill(bl->h, L, in, s));
      DProg p = to_dprog(&progs[i]);
      if (device_dt) { p = forms[i]; p.dtp = L.d_step_dt; }
      if (amrs_status e = list_stage(bl->h, L, p, in, s1, out, 0, s)) return e;
      cur = out;
      which ^= 1;
    }
    *res = cur;
    return AMRS_OK;
  };
  if (!use_graph) return record(st, result_slot, false);
  if (!L.d_step_dt) CK(cudaMalloc(&L.d_step_dt, sizeof(double)));
  L.h_step_dt = dt;
  CK(cudaMemcpyAsync(L.d_step_dt, &L.h_step_dt, sizeof(double), cudaMemcpyHostToDevice, st));
  const int key[6] = {order_rk, stages_rk, s1, w1, w2, 1 + 2 * bl->h->check_nonfinite};
  if (!L.graph || std::memcmp(key, L.graph_key, sizeof(key)) != 0) {
    if (L.graph) { cudaGraphExecDestroy(L.graph); L.graph = nullptr; }
    cudaStream_t cs;
    CK(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    cudaGraph_t g;
    cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) { cudaStreamDestroy(cs); return cuda_fail(e, "cudaStreamBeginCapture"); }
    int res = -1;
    amrs_status rs = record(cs, &res, true);
    e = cudaStreamEndCapture(cs, &g);
    cudaStreamDestroy(cs);
    if (rs) { if (e == cudaSuccess) cudaGraphDestroy(g); return rs; }
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
    e = cudaGraphInstantiate(&L.graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
    std::memcpy(L.graph_key, key, sizeof(key));
    L.graph_dt = dt;
    L.graph_result = res;
  }
  CK(cudaGraphLaunch(L.graph, st));
  *result_slot = L.graph_result;
  return AMRS_OK;
}

amrs_status amrs_rk_run_boxlist(amrs_boxlist* bl, int32_t order_rk, int32_t stages_rk, double cfl, double dt,
                                double time, double stop_time, int32_t max_steps, int32_t s1, int32_t w1, int32_t w2,
                                void* stream) {
  if (!bl) return AMRS_ERR_NULL;
  List& L = bl->L;
  amrs_handle* h = bl->h;
  if (s1 < 0 || w1 < 0 || w2 < 0 || s1 >= L.nslots || w1 >= L.nslots || w2 >= L.nslots || s1 == w1 || s1 == w2 ||
      w1 == w2 || max_steps < 0)
    return AMRS_ERR_SIZE;
  const int use_cfl = cfl > 0.0 ? 1 : 0;
  if (!use_cfl && !(dt > 0.0)) return AMRS_ERR_SIZE;
  amrs_stage_prog st16[16];
  DProg forms[16];
  int32_t ns = 0;
  if (amrs_status s = rk_build(order_rk, stages_rk, 1.0, st16, 16, &ns, forms)) return s;
  CK(cudaSetDevice(h->device));
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (!L.d_run) CK(cudaMalloc(&L.d_run, sizeof(RunCtl)));
  const int key[6] = {order_rk, stages_rk, s1, w1, w2, use_cfl + 2 * h->check_nonfinite};
  if (!L.run_graph || std::memcmp(key, L.run_key, sizeof(key)) != 0) {
    if (L.run_graph) { CK(cudaStreamSynchronize(st)); cudaGraphExecDestroy(L.run_graph); L.run_graph = nullptr; }
    // outer graph: one conditional WHILE node whose body is one step
    cudaGraph_t g = nullptr;
    CK(cudaGraphCreate(&g, 0));
    cudaGraphConditionalHandle cond;
    cudaError_t e = cudaGraphConditionalHandleCreate(&cond, g, 1, cudaGraphCondAssignDefault);
    cudaGraphNodeParams np{};
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = cond;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    cudaGraphNode_t node;
    if (e == cudaSuccess) e = cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &np);
    cudaStream_t cs = nullptr;
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
    if (e == cudaSuccess)
      e = cudaStreamBeginCaptureToGraph(cs, np.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                        cudaStreamCaptureModeThreadLocal);
    amrs_status rs = AMRS_OK;
    if (e == cudaSuccess) {
      // every kernel of the body returns at once while the loop is inactive
      const BoxTable saved = L.tb;
      L.tb.active = &L.d_run->active;
      int cur = s1;
      const int outs[2] = {w1, w2};
      int which = 0;
      for (int i = 0; i < ns && rs == AMRS_OK && e == cudaSuccess; ++i) {
        const int in = (st16[i].src_state == 0) ? s1 : cur;
        int out = outs[which];
        if (out == in) { which ^= 1; out = outs[which]; }
        if (L.has_bc) e = list_fill(h, L, in, cs);
        DProg pr = forms[i];
        pr.dtp = &L.d_run->dt;
        if (e == cudaSuccess) rs = list_stage(h, L, pr, in, s1, out, 0, cs);
        cur = out;
        which ^= 1;
      }
      if (e == cudaSuccess && rs == AMRS_OK && cur != s1) e = launch_copy_slot(L.tb, cur, s1, L.tot_valid, h->nsm, cs);
      if (e == cudaSuccess && rs == AMRS_OK && use_cfl) e = launch_run_estdt(L.tb, s1, L.tot_valid, L.d_run, h->nsm, cs);
      if (e == cudaSuccess && rs == AMRS_OK) e = launch_run_step_done(L.d_run, cond, cs);
      L.tb = saved;
      cudaGraph_t body = nullptr;
      const cudaError_t e2 = cudaStreamEndCapture(cs, &body);
      if (e == cudaSuccess) e = e2;
    }
    if (cs) cudaStreamDestroy(cs);
    if (e == cudaSuccess && rs == AMRS_OK) e = cudaGraphInstantiate(&L.run_graph, g, 0);
    cudaGraphDestroy(g);
    if (rs) return rs;
    if (e != cudaSuccess) return cuda_fail(e, "amrs_rk_run_boxlist graph");
    std::memcpy(L.run_key, key, sizeof(key));
  }
  // loop state, initial dt, then the whole run as one launch
  RunCtl& c = L.h_run;
  c.time = time; c.dt = use_cfl ? 0.0 : dt; c.stop = stop_time; c.cfl = cfl; c.change_max = 1.1;
  c.step = 0; c.max_steps = max_steps; c.use_cfl = use_cfl; c.active = 0; c.bits = ~0ull;
  CK(cudaMemcpyAsync(L.d_run, &c, sizeof(RunCtl), cudaMemcpyHostToDevice, st));
  if (use_cfl) {
    // computeInitialDt on the initial state (the list's kernels unguarded here)
    CK(launch_run_estdt(L.tb, s1, L.tot_valid, L.d_run, h->nsm, st));
  }
  CK(launch_run_begin(L.d_run, st));
  CK(cudaGraphLaunch(L.run_graph, st));
  return AMRS_OK;
}

amrs_status amrs_boxlist_run_state(amrs_boxlist* bl, double* time, double* dt, int32_t* steps, void* stream) {
  if (!bl || !time || !dt || !steps) return AMRS_ERR_NULL;
  List& L = bl->L;
  if (!L.d_run) return AMRS_ERR_STATE;
  CK(cudaSetDevice(bl->h->device));
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  RunCtl c{};
  CK(cudaMemcpyAsync(&c, L.d_run, sizeof(RunCtl), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  *time = c.time;
  *dt = c.dt;
  *steps = c.step;
  return AMRS_OK;
}

amrs_status amrs_boxlist_prim_stats(amrs_boxlist* bl, int32_t slot, const double dx[3], double dt, double* out,
                                    void* stream) {
  if (!bl || !dx || !out) return AMRS_ERR_NULL;
  List& L = bl->L;
  if (slot < -1 || slot >= L.nslots) return AMRS_ERR_SIZE;
  for (int d = 0; d < 3; ++d)
    if (!(dx[d] > 0.0)) return AMRS_ERR_BOX;
  CK(cudaSetDevice(bl->h->device));
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (!L.d_stats) CK(cudaMalloc(&L.d_stats, 32 * sizeof(unsigned long long)));
  CK(launch_prim_stats(L.tb, L.ft.vpre, slot, dt, dx, L.tot_valid, L.d_stats, out, bl->h->nsm, st));
  return AMRS_OK;
}

amrs_status amrs_boxlist_totals(amrs_boxlist* bl, int32_t slot, double scale, double* totals, void* stream) {
  if (!bl || !totals) return AMRS_ERR_NULL;
  List& L = bl->L;
  if (slot < 0 || slot >= L.nslots) return AMRS_ERR_SIZE;
  CK(cudaSetDevice(bl->h->device));
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const size_t need = (size_t)totals_blocks(L.tot_valid, bl->h->nsm) * NCONS;
  if (need > L.d_tot_n) {
    if (L.d_tot) { CK(cudaStreamSynchronize(st)); cudaFree(L.d_tot); L.d_tot = nullptr; L.d_tot_n = 0; }
    CK(cudaMalloc(&L.d_tot, need * sizeof(double)));
    L.d_tot_n = need;
  }
  CK(launch_totals(L.tb, slot, L.tot_valid, scale, L.d_tot, totals, bl->h->nsm, st));
  return AMRS_OK;
}

}  // extern "C"

namespace {

// Adjoint scratch of one box: per (direction, separation) pair cotangents
// (12 comps over grow(box,3)), viscous cotangents (16 comps over
// grow(box,1)), a valid-cell dSdt cotangent and a ghosted state cotangent.
struct AdjScratch {
  AdjRecHost ah{};
  DArr vbar_tmp, ubar_tmp;
  double* wbuf = nullptr;  // WENO / MUSCL per-face and per-cell cotangent slots
  double* jbuf = nullptr;  // JST per-face and per-cell cotangent slots
  int order = 0;           // KEEP order of the pair pass (0: none)
};

// Schemes with a reverse pass: KEEP, WENO5 LLF, MUSCL-Riemann, WENO5-Riemann
// (each with or without JST and viscous fluxes), viscous only.  (Internal
// flux codes: 0 MUSCL, 3 WENO5-Riemann.)
bool vjp_scheme(const amrs_scheme& s) {
  if (!s.rhs_euler) return s.rhs_visc != 0;
  return s.flux_euler >= 0 && s.flux_euler <= 3;
}
bool jst_scheme(const amrs_scheme& s) { return s.rhs_euler && s.art_diss == 1; }
bool weno_scheme(const amrs_scheme& s) { return s.rhs_euler && s.flux_euler == 2; }
bool muscl_scheme(const amrs_scheme& s) { return s.rhs_euler && s.flux_euler == 0; }
bool weno_riemann_scheme(const amrs_scheme& s) { return s.rhs_euler && s.flux_euler == 3; }

amrs_status adj_prepare(amrs_handle* h, const amrs_box& B, AdjScratch& S, cudaStream_t st) {
  // the KEEP pair pass runs whether the forward used the fused kernel or
  // (with JST) the face-array path: both compute the same fluxes
  S.order = (h->sc.rhs_euler && h->sc.flux_euler == 1) ? h->sc.order_keep : 0;
  const int H = S.order / 2;
  const int nb[3] = {bn(B, 0), bn(B, 1), bn(B, 2)};
  auto cells = [&](int g) { return (size_t)grown_cells(B, g); };
  size_t off = 0;
  const size_t o_pair = off; off = align_up(off + cells(3) * 12 * 8 * 3 * H, 256);
  const size_t o_vg = off; off = align_up(off + cells(1) * 16 * 8, 256);
  const size_t o_v = off; off = align_up(off + cells(0) * 5 * 8, 256);
  const size_t o_u = off; off = align_up(off + cells(3) * 5 * 8, 256);
  const size_t euler_bytes = weno_scheme(h->sc)         ? weno_vjp_buffer_bytes(nb)
                            : muscl_scheme(h->sc)        ? muscl_vjp_buffer_bytes(nb)
                            : weno_riemann_scheme(h->sc) ? weno_riemann_vjp_buffer_bytes(nb)
                                                         : 0;
  const size_t o_w = off; off = align_up(off + euler_bytes, 256);
  const size_t o_j = off; off = align_up(off + (jst_scheme(h->sc) ? jst_vjp_buffer_bytes(nb) : 0), 256);
  const size_t o_part = off; off = align_up(off + sizeof(double) * 2 * 8 * (size_t)h->nsm, 256);
  if (off > h->adj_bytes) {
    if (h->adj) { CK(cudaStreamSynchronize(st)); cudaFree(h->adj); h->adj = nullptr; h->adj_bytes = 0; }
    CK(cudaMalloc(&h->adj, off));
    h->adj_bytes = off;
  }
  char* P = static_cast<char*>(h->adj);
  auto mk = [&](size_t o, int g) {
    DArr a;
    a.p = reinterpret_cast<double*>(P + o);
    const int nx = bn(B, 0) + 2 * g, ny = bn(B, 1) + 2 * g, nz = bn(B, 2) + 2 * g;
    a.js = nx; a.ks = (long long)nx * ny; a.ns = (long long)nx * ny * nz;
    a.b0 = B.lo[0] - g; a.b1 = B.lo[1] - g; a.b2 = B.lo[2] - g;
    return a;
  };
  for (int d = 0; d < 3; ++d)
    for (int l = 0; l < 3; ++l) S.ah.pair[d][l] = mk(o_pair + (l < H ? (size_t)(d * H + l) * cells(3) * 12 * 8 : 0), 3);
  S.ah.vg = mk(o_vg, 1);
  S.vbar_tmp = mk(o_v, 0);
  S.ubar_tmp = mk(o_u, 3);
  for (int d = 0; d < 3; ++d) S.ah.n[d] = bn(B, d);
  S.ah.visc = h->sc.rhs_visc != 0;
  S.wbuf = reinterpret_cast<double*>(P + o_w);
  S.jbuf = reinterpret_cast<double*>(P + o_j);  // WENO or MUSCL per-face / per-cell slots
  S.ah.part = reinterpret_cast<double*>(P + o_part);
  if (H > 0) CK(cudaMemsetAsync(P + o_pair, 0, cells(3) * 12 * 8 * 3 * H, st));
  return AMRS_OK;
}

// Reverse pass of one RHS of the list's single box (state in slot 0):
// primitives, then the KEEP-pair / viscous / cons2prim reverse kernels,
// then the WENO5, MUSCL-Riemann or WENO5-Riemann Euler part.
cudaError_t rhs_vjp_launch(amrs_handle* h, List& L, const amrs_box& B, AdjScratch& S, double* param_bar,
                           cudaStream_t st) {
  cudaError_t e = launch_prims(L.tb, 0, L.tot_p, h->nsm, st);
  if (e == cudaSuccess) e = launch_rhs_vjp(S.order, L.tb, S.ah, param_bar, h->nsm, st);
  if (e == cudaSuccess && weno_scheme(h->sc)) {
    const int nb[3] = {bn(B, 0), bn(B, 1), bn(B, 2)};
    e = launch_weno_point(L.tb, L.ft, 0, L.tot_g, h->nsm, st);
    if (e == cudaSuccess) e = launch_weno_vjp(L.tb, L.hface[0], S.ah.vbar, S.ah.ubar, S.wbuf, nb, h->nsm, st);
  }
  if (e == cudaSuccess && muscl_scheme(h->sc)) {
    const int nb[3] = {bn(B, 0), bn(B, 1), bn(B, 2)};
    long long ns[3] = {L.tot_s[0], L.tot_s[1], L.tot_s[2]};
    e = launch_slopes(L.tb, L.ft, L.d_spre, ns, h->nsm, st);
    if (e == cudaSuccess) e = launch_muscl_vjp(L.tb, L.hface[0], S.ah.vbar, S.ah.ubar, S.wbuf, nb, h->nsm, st);
  }
  if (e == cudaSuccess && weno_riemann_scheme(h->sc)) {
    const int nb[3] = {bn(B, 0), bn(B, 1), bn(B, 2)};
    e = launch_weno_riemann_vjp(L.tb, S.ah.vbar, S.ah.ubar, S.wbuf, nb, h->nsm, st);
  }
  if (e == cudaSuccess && h->source) {
    const BoxRec& R = L.hbox[0];
    e = launch_source_vjp(R, h->force, S.ah.vbar, S.ah.ubar, h->nsm, st);
  }
  if (e == cudaSuccess && jst_scheme(h->sc)) {
    // after the Euler part: the WENO5 pass reads lambda from the array the
    // JST sensor pass overwrites
    const int nb[3] = {bn(B, 0), bn(B, 1), bn(B, 2)};
    const FaceRec& F = L.hface[0];
    e = cudaMemsetAsync(F.sen.p, 0, (size_t)F.sen.ns * 3 * 8, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(F.lam.p, 0, (size_t)F.lam.ns * 3 * 8, st);
    if (e == cudaSuccess) e = launch_jst_sensor(L.tb, L.ft, L.tot_valid, h->nsm, st);
    if (e == cudaSuccess) e = launch_jst_vjp(L.tb, F, S.ah.vbar, S.ah.ubar, S.jbuf, nb, h->nsm, st);
  }
  return e;
}

}  // namespace

extern "C" {

amrs_status amrs_rhs_vjp_box(amrs_handle* h, const amrs_box* bx, const double dxinv[3], amrs_array4 state,
                             amrs_array4 vbar, amrs_array4 ubar, double* param_bar, void* stream) {
  if (!h || !bx || !dxinv) return AMRS_ERR_NULL;
  if (!box_ok(*bx)) return AMRS_ERR_BOX;
  if (!vjp_scheme(h->sc)) return AMRS_ERR_SCHEME;
  if (!covers(state, *bx, NGHOST, NCONS) || !covers(vbar, *bx, 0, NCONS) || !covers(ubar, *bx, NGHOST, NCONS))
    return AMRS_ERR_LAYOUT;
  std::lock_guard<std::mutex> lk(h->mu);
  CK(cudaSetDevice(h->device));
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  amrs_array4 slots[3] = {state, state, state};
  if (amrs_status s = one_box(h, bx, dxinv, slots, 3, st)) return s;
  List& L = *h->one;
  AdjScratch S;
  if (amrs_status s = adj_prepare(h, *bx, S, st)) { ring_release(h, st); return s; }
  S.ah.vbar = to_darr(vbar);
  S.ah.ubar = to_darr(ubar);
  cudaError_t e = rhs_vjp_launch(h, L, *bx, S, param_bar, st);
  ring_release(h, st);
  if (e != cudaSuccess) return cuda_fail(e, "amrs_rhs_vjp_box");
  return AMRS_OK;
}

amrs_status amrs_fill_halo_box_adjoint(const amrs_box* domain, const int32_t bc_lo[3], const int32_t bc_hi[3],
                                       amrs_array4 ubar, void* stream) {
  if (!domain || !bc_lo || !bc_hi) return AMRS_ERR_NULL;
  if (!box_ok(*domain)) return AMRS_ERR_BOX;
  if (!covers(ubar, *domain, NGHOST, 1)) return AMRS_ERR_LAYOUT;
  HaloBox hb;
  hb.u = to_darr(ubar);
  hb.ncomp = ubar.ncomp;
  for (int d = 0; d < 3; ++d) {
    if ((bc_lo[d] == -1) != (bc_hi[d] == -1)) return AMRS_ERR_BC;
    for (int s = 0; s < 2; ++s) {
      const int p = s ? bc_hi[d] : bc_lo[d];
      if (p < -1 || p > 6) return AMRS_ERR_BC;  // 1, 6: ext_dir, left in place
    }
    if (bn(*domain, d) < NGHOST && bc_lo[d] != -1 && bc_lo[d] != 2) return AMRS_ERR_BOX;
    hb.lo[d] = domain->lo[d]; hb.hi[d] = domain->hi[d]; hb.bc_lo[d] = bc_lo[d]; hb.bc_hi[d] = bc_hi[d];
  }
  int nsm = 0;
  int dev = 0;
  CK(cudaGetDevice(&dev));
  CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  CK(launch_adj_halo(hb, nsm, static_cast<cudaStream_t>(stream)));
  return AMRS_OK;
}

amrs_status amrs_rk_stage_vjp_box(amrs_handle* h, const amrs_box* bx, const double dxinv[3],
                                  const amrs_stage_prog* prog, const int32_t bc_lo[3], const int32_t bc_hi[3],
                                  amrs_array4 stage_in, amrs_array4 wbar, amrs_array4 s1bar, amrs_array4 inbar,
                                  double* param_bar, void* stream) {
  if (!h || !bx || !dxinv || !prog || !bc_lo || !bc_hi) return AMRS_ERR_NULL;
  if (!box_ok(*bx)) return AMRS_ERR_BOX;
  if (!vjp_scheme(h->sc) || h->wall.lo || h->wall.hi) return AMRS_ERR_SCHEME;
  // the fold's BC checks up front, so that nothing is queued for a call
  // that fails; ghosts beyond ext_dir sides come from the caller's
  // bcnormal: their cotangents cannot be folded here
  // (amrs_rk_stage_vjp_box_ghosted)
  for (int d = 0; d < 3; ++d) {
    if ((bc_lo[d] == -1) != (bc_hi[d] == -1)) return AMRS_ERR_BC;
    for (int sd = 0; sd < 2; ++sd) {
      const int p = sd ? bc_hi[d] : bc_lo[d];
      if (p < -1 || p > 6 || p == 1 || p == 6) return AMRS_ERR_BC;
    }
    if (bn(*bx, d) < NGHOST && bc_lo[d] != -1 && bc_lo[d] != 2) return AMRS_ERR_BOX;
  }
  if (!covers(stage_in, *bx, NGHOST, NCONS) || !covers(wbar, *bx, 0, NCONS) || !covers(s1bar, *bx, 0, NCONS) ||
      !covers(inbar, *bx, 0, NCONS))
    return AMRS_ERR_LAYOUT;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  // the handle's scratch (ubar_tmp) is used until the last launch: hold the
  // handle for the whole call
  std::lock_guard<std::mutex> lk(h->mu);
  CK(cudaSetDevice(h->device));
  amrs_array4 slots[3] = {stage_in, stage_in, stage_in};
  if (amrs_status s = one_box(h, bx, dxinv, slots, 3, st)) return s;
  AdjScratch S;
  if (amrs_status s = adj_prepare(h, *bx, S, st)) { ring_release(h, st); return s; }
  const BoxRec R = h->one->hbox[0];
  // 1. reverse of the BLAS-1 program: cotangents of S1, of the stage input
  //    (register S2) and of dSdt
  cudaError_t e = launch_adj_prog(R, to_dprog(prog), to_darr(wbar), to_darr(s1bar), to_darr(inbar), S.vbar_tmp, 1,
                                  h->nsm, st);
  // 2. RHS VJP of the ghost-filled stage input
  if (e == cudaSuccess) {
    S.ah.vbar = S.vbar_tmp;
    S.ah.ubar = S.ubar_tmp;
    e = rhs_vjp_launch(h, *h->one, *bx, S, param_bar, st);
  }
  // 3. ghost fold (adjoint of FillPatch), then inbar += valid(ubar): the
  //    reverse kernel with an empty program routes its input cotangent into
  //    the stage-input cotangent (vbar_tmp is free here)
  if (e == cudaSuccess) {
    HaloBox hb;
    hb.u = S.ubar_tmp;
    hb.ncomp = NCONS;
    for (int d = 0; d < 3; ++d) {
      hb.lo[d] = bx->lo[d]; hb.hi[d] = bx->hi[d]; hb.bc_lo[d] = bc_lo[d]; hb.bc_hi[d] = bc_hi[d];
    }
    e = launch_adj_halo(hb, h->nsm, st);
  }
  if (e == cudaSuccess) {
    amrs_stage_prog ident{};
    ident.nops = 0;
    e = launch_adj_prog(R, to_dprog(&ident), S.ubar_tmp, S.vbar_tmp, to_darr(inbar), S.vbar_tmp, 1, h->nsm, st);
  }
  ring_release(h, st);
  if (e != cudaSuccess) return cuda_fail(e, "amrs_rk_stage_vjp_box");
  return AMRS_OK;
}

amrs_status amrs_rk_stage_vjp_box_ghosted(amrs_handle* h, const amrs_box* bx, const double dxinv[3],
                                          const amrs_stage_prog* prog, amrs_array4 stage_in, amrs_array4 wbar,
                                          amrs_array4 s1bar, amrs_array4 ubar, double* param_bar, void* stream) {
  if (!h || !bx || !dxinv || !prog) return AMRS_ERR_NULL;
  if (!box_ok(*bx)) return AMRS_ERR_BOX;
  if (!vjp_scheme(h->sc)) return AMRS_ERR_SCHEME;
  if (!covers(stage_in, *bx, NGHOST, NCONS) || !covers(wbar, *bx, 0, NCONS) || !covers(s1bar, *bx, 0, NCONS) ||
      !covers(ubar, *bx, NGHOST, NCONS))
    return AMRS_ERR_LAYOUT;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  std::lock_guard<std::mutex> lk(h->mu);
  CK(cudaSetDevice(h->device));
  amrs_array4 slots[3] = {stage_in, stage_in, stage_in};
  if (amrs_status s = one_box(h, bx, dxinv, slots, 3, st)) return s;
  AdjScratch S;
  if (amrs_status s = adj_prepare(h, *bx, S, st)) { ring_release(h, st); return s; }
  const BoxRec R = h->one->hbox[0];
  cudaError_t e = cudaMemsetAsync(S.ubar_tmp.p, 0, (size_t)S.ubar_tmp.ns * NCONS * sizeof(double), st);
  // 1. reverse of the BLAS-1 program: S1 cotangent added to s1bar, the stage
  //    input's direct cotangent parked in ubar_tmp, dSdt's in vbar_tmp
  if (e == cudaSuccess)
    e = launch_adj_prog(R, to_dprog(prog), to_darr(wbar), to_darr(s1bar), S.ubar_tmp, S.vbar_tmp, 1, h->nsm, st);
  // 2. RHS VJP of the ghost-filled stage input, written into the caller's ubar
  if (e == cudaSuccess) {
    S.ah.vbar = S.vbar_tmp;
    S.ah.ubar = to_darr(ubar);
    e = rhs_vjp_launch(h, *h->one, *bx, S, param_bar, st);
  }
  // 3. ubar(valid) += the parked direct cotangent (the empty program routes
  //    its input into the stage-input slot; vbar_tmp takes the zeros)
  if (e == cudaSuccess) {
    amrs_stage_prog ident{};
    ident.nops = 0;
    e = launch_adj_prog(R, to_dprog(&ident), S.ubar_tmp, S.vbar_tmp, to_darr(ubar), S.vbar_tmp, 1, h->nsm, st);
  }
  ring_release(h, st);
  if (e != cudaSuccess) return cuda_fail(e, "amrs_rk_stage_vjp_box_ghosted");
  return AMRS_OK;
}

// Synchronise `stream`, then report (and clear) one raised device flag: a
// bounded wait that timed out first, else a non-finite result seen by the
// opt-in check.  Host-synchronising.
amrs_status amrs_sync_check(amrs_handle* h, void* stream) {
  if (!h) return AMRS_ERR_NULL;
  CK(cudaSetDevice(h->device));
  CK(cudaStreamSynchronize(static_cast<cudaStream_t>(stream)));
  int flag[2] = {0, 0};
  CK(cudaMemcpy(flag, h->derr, sizeof(flag), cudaMemcpyDeviceToHost));
  if (flag[0]) {
    CK(cudaMemset(h->derr, 0, sizeof(int)));
    return AMRS_ERR_TIMEOUT;
  }
  if (flag[1]) {
    CK(cudaMemset(h->derr + 1, 0, sizeof(int)));
    return AMRS_ERR_NONFINITE;
  }
  return AMRS_OK;
}

// Opt-in detection of non-finite results (see the header).
amrs_status amrs_set_check_nonfinite(amrs_handle* h, int32_t on) {
  if (!h) return AMRS_ERR_NULL;
  if (on != 0 && on != 1) return AMRS_ERR_SIZE;
  std::lock_guard<std::mutex> lk(h->mu);
  h->check_nonfinite = on;
  return AMRS_OK;
}

// Exercises the timeout path of the bounded device waits (see the header).
amrs_status amrs_debug_wait_timeout(amrs_handle* h, int32_t polls, void* stream) {
  if (!h) return AMRS_ERR_NULL;
  if (polls < 1 || polls > (1 << 20)) return AMRS_ERR_SIZE;
  CK(cudaSetDevice(h->device));
  CK(launch_wait_timeout_probe(h->derr, polls, static_cast<cudaStream_t>(stream)));
  return AMRS_OK;
}

// Measured FP64 FMA throughput of the handle's device in TFLOP/s (an FMA
// counts 2 flops): 4 CTAs of 256 threads per SM, sixteen DFMA chains per
// thread.  A short launch calibrates the loop count so that the timed launch
// runs for about `seconds` (clamped to [0.01, 10]); it is timed with CUDA
// events after the calibration launch.  *ms receives its duration (callers
// sample the SM clock over it).  Host-synchronising.
amrs_status amrs_probe_fp64_tflops_timed(amrs_handle* h, double seconds, double* tflops, double* ms_out) {
  if (!h || !tflops) return AMRS_ERR_NULL;
  if (!(seconds >= 0.01 && seconds <= 10.0)) return AMRS_ERR_SIZE;
  CK(cudaSetDevice(h->device));
  const int blocks = 4 * h->nsm, threads = 256, chains = 16;
  double* buf = nullptr;
  CK(cudaMalloc(&buf, sizeof(double) * blocks * threads));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  auto timed = [&](int iters, float* ms) {
    cudaError_t e = cudaEventRecord(e0, 0);
    if (e == cudaSuccess) e = launch_fp64_probe(buf, blocks, iters, 0);
    if (e == cudaSuccess) e = cudaEventRecord(e1, 0);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    if (e == cudaSuccess) e = cudaEventElapsedTime(ms, e0, e1);
    return e;
  };
  float ms = 0.f;
  int iters = 4096;
  cudaError_t e = timed(iters, &ms);  // calibration (also the warm-up)
  if (e == cudaSuccess && ms > 0.f) {
    const double want = seconds * 1e3 / ms * iters;
    iters = (int)std::min(std::max(want, 4096.0), (double)(1 << 30));
    e = timed(iters, &ms);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(buf);
  if (e != cudaSuccess) return cuda_fail(e, "amrs_probe_fp64_tflops_timed");
  *tflops = 2.0 * chains * (double)blocks * threads * iters / (ms * 1e-3) / 1e12;
  if (ms_out) *ms_out = ms;
  return AMRS_OK;
}

amrs_status amrs_probe_intpipe(amrs_handle* h, int32_t mode, double* ms_out) {
  if (!h || !ms_out) return AMRS_ERR_NULL;
  if (mode < 0 || mode > 2) return AMRS_ERR_SIZE;
  CK(cudaSetDevice(h->device));
  const int blocks = 2 * h->nsm, iters = 8000;
  double* buf = nullptr;
  CK(cudaMalloc(&buf, sizeof(double) * blocks * 256));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaError_t e = launch_intpipe_probe(mode, buf, blocks, iters, 0);  // warm-up
  if (e == cudaSuccess) e = cudaEventRecord(e0, 0);
  for (int r = 0; r < 3 && e == cudaSuccess; ++r) e = launch_intpipe_probe(mode, buf, blocks, iters, 0);
  if (e == cudaSuccess) e = cudaEventRecord(e1, 0);
  if (e == cudaSuccess) e = cudaEventSynchronize(e1);
  float ms = 0.f;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(buf);
  if (e != cudaSuccess) return cuda_fail(e, "amrs_probe_intpipe");
  *ms_out = ms / 3.0;
  return AMRS_OK;
}

// The integer-pipe division (what = 0), square root (what = 1) or product
// (what = 2) against the hardware one (see the header).
static amrs_status intpipe_check(amrs_handle* h, int what, uint64_t seed, int64_t count, int64_t* mismatches,
                                 double* first) {
  if (!h || !mismatches || !first) return AMRS_ERR_NULL;
  if (count < 1 || count > (1ll << 40)) return AMRS_ERR_SIZE;
  CK(cudaSetDevice(h->device));
  unsigned long long* bad = nullptr;
  double* dfirst = nullptr;
  CK(cudaMalloc(&bad, sizeof(unsigned long long)));
  cudaError_t e = cudaMalloc(&dfirst, 4 * sizeof(double));
  if (e == cudaSuccess) e = cudaMemset(bad, 0, sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaMemset(dfirst, 0, 4 * sizeof(double));
  if (e == cudaSuccess)
    e = what == 2 ? launch_dmul_check(seed, count, bad, dfirst, h->nsm, 0)
                  : (what ? launch_dsqrt_check(seed, count, bad, dfirst, h->nsm, 0)
                          : launch_ddiv_check(seed, count, bad, dfirst, h->nsm, 0));
  unsigned long long nb = 0;
  if (e == cudaSuccess) e = cudaMemcpy(&nb, bad, sizeof(nb), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(first, dfirst, 4 * sizeof(double), cudaMemcpyDeviceToHost);
  cudaFree(bad);
  if (dfirst) cudaFree(dfirst);
  if (e != cudaSuccess) return cuda_fail(e, "amrs_debug_ddiv_check");
  *mismatches = (int64_t)nb;
  return AMRS_OK;
}

amrs_status amrs_debug_ddiv_check(amrs_handle* h, uint64_t seed, int64_t count, int64_t* mismatches, double* first) {
  return intpipe_check(h, 0, seed, count, mismatches, first);
}

amrs_status amrs_debug_dsqrt_check(amrs_handle* h, uint64_t seed, int64_t count, int64_t* mismatches, double* first) {
  return intpipe_check(h, 1, seed, count, mismatches, first);
}

amrs_status amrs_debug_dmul_check(amrs_handle* h, uint64_t seed, int64_t count, int64_t* mismatches, double* first) {
  return intpipe_check(h, 2, seed, count, mismatches, first);
}

// The same probe with a timed launch of about 0.2 s.
amrs_status amrs_probe_fp64_tflops(amrs_handle* h, double* tflops) {
  return amrs_probe_fp64_tflops_timed(h, 0.2, tflops, nullptr);
}

// Per-kernel timing of one RK stage of one box (KEEP fused path): the
// primitive, viscous-cell and fused face kernels each bracketed by CUDA
// events on `stream`, averaged over `reps` stages.  ms[0..3] = prims, viscous
// cells, face kernel, whole stage.  Host-synchronising.
amrs_status amrs_profile_stage_box(amrs_handle* h, const amrs_box* bx, const double dxinv[3],
                                   const amrs_stage_prog* prog, amrs_array4 stage_in, amrs_array4 s1, amrs_array4 out,
                                   int32_t reps, void* stream, double* ms) {
  if (!h || !bx || !dxinv || !prog || !ms) return AMRS_ERR_NULL;
  if (reps < 1) return AMRS_ERR_SIZE;
  if (!covers(stage_in, *bx, NGHOST, NCONS) || !covers(s1, *bx, 0, NCONS) || !covers(out, *bx, 0, NCONS))
    return AMRS_ERR_LAYOUT;
  std::lock_guard<std::mutex> lk(h->mu);
  CK(cudaSetDevice(h->device));
  amrs_array4 slots[3] = {stage_in, s1, out};
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (amrs_status s = one_box(h, bx, dxinv, slots, 3, st)) return s;
  List& L = *h->one;
  const amrs_scheme& sc = L.sc;
  // the face-array path is profiled for WENO5 (point fluxes timed with the
  // primitives), MUSCL-Riemann (slopes timed with the faces), WENO5-Riemann
  // and the unshared KEEP baseline
  const bool plain_ok = sc.rhs_euler && !sc.art_diss && sc.flux_euler >= 0 && sc.flux_euler <= 3;
  if (!L.fused && !plain_ok) { ring_release(h, st); return AMRS_ERR_SCHEME; }
  const DProg p = to_dprog(prog);
  cudaEvent_t ev[5];
  for (int i = 0; i < 5; ++i) CK(cudaEventCreate(&ev[i]));
  double acc[4] = {0, 0, 0, 0};
  long long nf[3] = {L.tot_f[0], L.tot_f[1], L.tot_f[2]};
  amrs_status rs = AMRS_OK;
  for (int r = 0; r < reps && rs == AMRS_OK; ++r) {
    cudaError_t e = cudaEventRecord(ev[0], st);
    if (e == cudaSuccess) e = launch_prims(L.tb, 0, L.tot_p, h->nsm, st);
    if (e == cudaSuccess && !L.fused && sc.flux_euler == 2) e = launch_weno_point(L.tb, L.ft, 0, L.tot_g, h->nsm, st);
    if (e == cudaSuccess) e = cudaEventRecord(ev[1], st);
    if (e == cudaSuccess && sc.rhs_visc) e = launch_visc(L.tb, L.tot_v, h->nsm, st);
    if (e == cudaSuccess) e = cudaEventRecord(ev[2], st);
    if (e == cudaSuccess && L.fused)
      e = launch_keep_face(sc.order_keep, sc.rhs_visc != 0, L.source, L.tb, 0, 1, 2, p, 0, L.tma, h->derr,
                           L.face_grid, h->nsm, st);
    else if (e == cudaSuccess && sc.flux_euler == 2)
      e = launch_weno_faces(L.tb, L.ft, 0, nf, sc.weno_fast == 0, h->nsm, st);
    else if (e == cudaSuccess && sc.flux_euler == 3)
      e = launch_weno_riemann(L.tb, L.ft, nf, h->nsm, st);
    else if (e == cudaSuccess && sc.flux_euler == 0) {
      long long ns[3] = {L.tot_s[0], L.tot_s[1], L.tot_s[2]};
      e = launch_riemann(L.tb, L.ft, L.d_spre, ns, nf, h->nsm, st);
    } else if (e == cudaSuccess)
      e = launch_keep_faces_plain(sc.order_keep, L.tb, L.ft, nf, h->nsm, st);
    if (e == cudaSuccess) e = cudaEventRecord(ev[3], st);
    if (e == cudaSuccess && !L.fused) {
      if (sc.rhs_visc) e = launch_visc_face_add(L.tb, L.ft, nf, h->nsm, st);
      if (e == cudaSuccess) e = launch_div_stage(L.tb, L.ft, 0, 1, 2, p, 0, L.tot_valid, h->nsm, st);
    }
    if (e == cudaSuccess) e = cudaEventRecord(ev[4], st);
    if (e == cudaSuccess) e = cudaEventSynchronize(ev[4]);
    for (int i = 0; i < 3 && e == cudaSuccess; ++i) {
      float t = 0.f;
      e = cudaEventElapsedTime(&t, ev[i], ev[i + 1]);
      acc[i] += t;
    }
    if (e == cudaSuccess) {
      float t = 0.f;
      e = cudaEventElapsedTime(&t, ev[0], ev[4]);
      acc[3] += t;
    }
    if (e != cudaSuccess) rs = cuda_fail(e, "amrs_profile_stage_box");
  }
  for (int i = 0; i < 5; ++i) cudaEventDestroy(ev[i]);
  ring_release(h, st);
  if (rs) return rs;
  for (int i = 0; i < 4; ++i) ms[i] = acc[i] / reps;
  return AMRS_OK;
}

// Whether the fused face kernel of this handle's last single-box list stages
// its planes with TMA (1) or with plain loads (0).
int32_t amrs_debug_tma_enabled(amrs_handle* h) { return (h && h->one) ? h->one->tma.enabled : -1; }
int32_t amrs_boxlist_tma_enabled(amrs_boxlist* bl) { return bl ? bl->L.tma.enabled : -1; }

}  // extern "C"
