// C front end over the reference's own CNS::compute_rhs / CNS::advance /
// cns_estdt, compiled by oracle/build_ref.sh together with the reference's
// src/tim/CNS_advance.cpp and kernel headers.  TEST INFRASTRUCTURE ONLY.
//
// It exports the same orc_* entry points as the restatement in
// oracle/cns_oracle.cpp, so tests can run both on identical inputs.  This
// file supplies what the reference's src/CNS.cpp would (static members, the
// level's scratch MultiFabs as CNS::post_regrid allocates them at
// src/CNS.cpp:432-467, KEEP coefficients as at src/CNS.cpp:241-252) without
// compiling that file, which needs the full AMReX AmrLevel machinery.
#include <CNS.h>
#include <CNS_K.h>
#include <CNS_hydro_K.h>

#include <cstdint>
#include <cstring>

using namespace amrex;

// ---- static members of CNS (defined in src/CNS.cpp in the reference) ----
int CNS::num_state_data_types = 1;
int CNS::do_reflux = 0;
bool CNS::verbose = false;
Real CNS::cfl = 0.3;
int CNS::refine_max_dengrad_lev = -1;
Real CNS::refine_dengrad = 1.0e10;
Real CNS::gravity = 0.0;
Real CNS::dt_constant = 0.0;
bool CNS::dt_dynamic = false;
int CNS::nstep_screen_output = 1;
int CNS::flux_euler = 1;
int CNS::art_diss = 0;
int CNS::order_rk = 3;
int CNS::stages_rk = 3;
bool CNS::rhs_euler = true;
bool CNS::rhs_visc = true;
bool CNS::rhs_source = false;
bool CNS::ib_move = false;
bool CNS::plot_surf = false;
Vector<MultiFab> CNS::VdSdt;
Vector<MultiFab> CNS::VSborder;
Vector<MultiFab> CNS::Vprimsmf;
Vector<Array<MultiFab, AMREX_SPACEDIM>> CNS::Vnumflxmf;
Vector<Array<MultiFab, AMREX_SPACEDIM>> CNS::Vpntvflxmf;
PROB::ProbClosures* CNS::h_prob_closures = nullptr;
PROB::ProbClosures* CNS::d_prob_closures = nullptr;
PROB::ProbParm* CNS::h_prob_parm = nullptr;
PROB::ProbParm* CNS::d_prob_parm = nullptr;
BCRec* CNS::h_phys_bc = nullptr;
BCRec* CNS::d_phys_bc = nullptr;
namespace CentralKEEP {
GpuArray<Real, 3> coeffs, coeffs2;
int order_keep = 4;
}  // namespace CentralKEEP

// ---- CNS members the reference defines in src/CNS.cpp (not on this path) ----
CNS::CNS() {}
CNS::~CNS() {}
void CNS::init(AmrLevel&) {}
void CNS::init() {}
void CNS::initData() {}
void CNS::post_init(Real) {}
void CNS::computeInitialDt(int, int, Vector<int>&, const Vector<IntVect>&, Vector<Real>&, Real) {}
void CNS::computeNewDt(int, int, Vector<int>&, const Vector<IntVect>&, Vector<Real>&, Vector<Real>&, Real, int) {}
void CNS::post_timestep(int) {}
void CNS::postCoarseTimeStep(Real) {}
void CNS::post_regrid(int, int) {}
void CNS::errorEst(TagBoxArray&, int, int, Real, int, int) {}
void CNS::writePlotFile(const std::string&, std::ostream&, VisMF::How) {}
void CNS::writePlotFilePost(const std::string&, std::ostream&) {}

// ---- single-level ghost fill used by the stand-in FillPatch ----
// Periodic images first, then physical BCs direction by direction (bc
// codes of cns.lo_bc/hi_bc mapped through src/set/CNS_setup.cpp:18-31).
namespace amrex {
static int comp_bc(int phys, int comp, int dir) {
  const bool normal = (comp == UMX + dir);
  const bool vel = (comp >= UMX && comp <= UMZ);
  if (phys == 2) return BCType::foextrap;
  if (phys == 3 || phys == 4) return (vel && normal) ? BCType::reflect_odd : BCType::reflect_even;
  if (phys == 5) return vel ? BCType::reflect_odd : BCType::reflect_even;
  return BCType::int_dir;
}
void fill_level_ghosts(MultiFab& mf, const Geometry& geom, const BCRec& bc, int ng) {
  const Box& dom = geom.Domain();
  for (int b = 0; b < (int)mf.fabs.size(); ++b) {
    auto a = mf.fabs[b].array();
    Box gb = grow(mf.ba.boxes[b], ng);
    for (int d = 0; d < 3; ++d) {
      if (!geom.isPeriodic(d)) continue;
      const int n = dom.length(d);
      ParallelFor(gb, [&](int i, int j, int k) {
        int c[3] = {i, j, k};
        if (c[d] >= dom.lo[d] && c[d] <= dom.hi[d]) return;
        int s[3] = {i, j, k};
        s[d] = (c[d] < dom.lo[d]) ? c[d] + n : c[d] - n;
        for (int m = 0; m < mf.ncomp; ++m) a(i, j, k, m) = a(s[0], s[1], s[2], m);
      });
    }
    for (int d = 0; d < 3; ++d)
      for (int side = 0; side < 2; ++side) {
        const int phys = side ? bc.hi(d) : bc.lo(d);
        if (geom.isPeriodic(d) || phys == 0) continue;
        ParallelFor(gb, [&](int i, int j, int k) {
          int c[3] = {i, j, k};
          const bool out = side ? (c[d] > dom.hi[d]) : (c[d] < dom.lo[d]);
          if (!out) return;
          for (int m = 0; m < mf.ncomp; ++m) {
            const int t = comp_bc(phys, m, d);
            int s[3] = {i, j, k};
            if (t == BCType::foextrap) {
              s[d] = side ? dom.hi[d] : dom.lo[d];
              a(i, j, k, m) = a(s[0], s[1], s[2], m);
            } else if (t == BCType::reflect_even || t == BCType::reflect_odd) {
              s[d] = side ? 2 * dom.hi[d] - c[d] + 1 : 2 * dom.lo[d] - c[d] - 1;
              Real v = a(s[0], s[1], s[2], m);
              a(i, j, k, m) = (t == BCType::reflect_odd) ? -v : v;
            }
          }
        });
      }
  }
}
}  // namespace amrex

// ---- C API (same shapes as oracle/cns_oracle.cpp) ----
struct OrcClosures {
  double gamma, cv, cp, Rspec;
  int32_t visc_law, cond_law;
  double visc_ref, Tvisc_ref, cond_ref, Tcond_ref, Cshock, Cdamp;
};
struct OrcScheme {
  int32_t rhs_euler, rhs_visc, flux_euler, order_keep, art_diss, rhs_source;
  double force[3];
};

static PROB::ProbClosures g_cl;
static PROB::ProbParm g_parm;
static BCRec g_bc;

static int set_closures(const OrcClosures* c) {
  g_cl = PROB::ProbClosures{};
  g_cl.gamma = c->gamma;
  g_cl.cv = c->cv;
  g_cl.cp = c->cp;
  g_cl.Rspec = c->Rspec;
  g_cl.Cshock = c->Cshock;
  g_cl.Cdamp = c->Cdamp;
#ifdef REF_CONST_TRANSPORT
  if (c->visc_law != 0 || c->cond_law != 0) return 10;
  g_cl.visc_ref = c->visc_ref;
  g_cl.cond_ref = c->cond_ref;
#else
  // Sutherland coefficients are private constants of visc_suth_t/cond_suth_t
  if (c->visc_law != 1 || c->cond_law != 1) return 10;
  if (c->visc_ref != 1.458e-6 || c->Tvisc_ref != 110.4 || c->cond_ref != 2.495e-3 || c->Tcond_ref != 194.0)
    return 11;
#endif
  CNS::h_prob_closures = CNS::d_prob_closures = &g_cl;
  CNS::h_prob_parm = CNS::d_prob_parm = &g_parm;
  CNS::h_phys_bc = CNS::d_phys_bc = &g_bc;
  return 0;
}

static void set_scheme(const OrcScheme* s) {
  CNS::rhs_euler = s->rhs_euler != 0;
  CNS::rhs_visc = s->rhs_visc != 0;
  CNS::rhs_source = s->rhs_source != 0;
  for (int d = 0; d < 3; ++d) g_parm.force[d] = s->force[d];
  CNS::flux_euler = s->flux_euler;
  CNS::art_diss = s->art_diss;
  CentralKEEP::order_keep = s->order_keep;
  // KEEP coefficients as the reference's CPU build sets them (src/CNS.cpp:241-252)
  CentralKEEP::coeffs2 = {Real(1.0), 0.0, 0.0};
  if (CentralKEEP::order_keep == 6) CentralKEEP::coeffs = {Real(6.0) / 4, Real(-6.0) / 20, Real(2.0) / 60};
  else if (CentralKEEP::order_keep == 4) CentralKEEP::coeffs = {Real(4.0) / 3, Real(-2.0) / 12, 0.0};
  else CentralKEEP::coeffs = {Real(1.0), 0.0, 0.0};
}

// Level 0 of a single-box domain with the scratch of CNS::post_regrid.
static void setup_level(CNS& lev, Amr& amr, const int* lo, const int* hi, const double* dxinv, const int* bc_lo,
                        const int* bc_hi) {
  Box dom(IntVect(lo[0], lo[1], lo[2]), IntVect(hi[0], hi[1], hi[2]));
  lev.geom.dom = dom;
  for (int d = 0; d < 3; ++d) {
    lev.geom.cellinv[d] = dxinv[d];
    lev.geom.cell[d] = 1.0 / dxinv[d];
    lev.geom.plo[d] = 0.0;
    lev.geom.phi[d] = dom.length(d) * lev.geom.cell[d];
    lev.geom.periodic[d] = (bc_lo && bc_lo[d] == -1) ? 1 : 0;
    g_bc.setLo(d, bc_lo ? bc_lo[d] : 0);
    g_bc.setHi(d, bc_hi ? bc_hi[d] : 0);
  }
  lev.phys_bc_for_fill = g_bc;
  lev.grids = BoxArray(dom);
  lev.level = 0;
  amr.levels.assign(1, &lev);
  lev.parent = &amr;
  DistributionMapping dm;
  CNS::VdSdt.resize(1);
  CNS::VSborder.resize(1);
  CNS::Vprimsmf.resize(1);
  CNS::Vnumflxmf.resize(1);
  CNS::Vpntvflxmf.resize(1);
  CNS::VdSdt[0].define(lev.grids, dm, NCONS, 0);
  CNS::VdSdt[0].setVal(0.0);
  CNS::VSborder[0].define(lev.grids, dm, NCONS, NGHOST);
  CNS::VSborder[0].setVal(0.0);
  CNS::Vprimsmf[0].define(lev.grids, dm, NPRIM, NGHOST);
  CNS::Vprimsmf[0].setVal(0.0);
  for (int d = 0; d < 3; ++d) {
    CNS::Vnumflxmf[0][d].define(convert(lev.grids, IntVect::TheDimensionVector(d)), dm, NCONS, NGHOST);
    CNS::Vnumflxmf[0][d].setVal(0.0);
    CNS::Vpntvflxmf[0][d].define(lev.grids, dm, NCONS, NGHOST);
    CNS::Vpntvflxmf[0][d].setVal(0.0);
  }
}

static void copy_in(MultiFab& mf, const double* src) {
  std::memcpy(mf.fabs[0].data.data(), src, mf.fabs[0].data.size() * sizeof(double));
}
static void copy_valid_out(MultiFab& mf, double* dst, int ng) {
  auto a = mf.fabs[0].array();
  const Box& vb = mf.ba.boxes[0];
  Box gb = grow(vb, ng);
  long t = 0;
  for (int n = 0; n < NCONS; ++n)
    for (int k = gb.lo[2]; k <= gb.hi[2]; ++k)
      for (int j = gb.lo[1]; j <= gb.hi[1]; ++j)
        for (int i = gb.lo[0]; i <= gb.hi[0]; ++i) dst[t++] = a(i, j, k, n);
}

extern "C" {

int orc_version(void) { return 1000; }

int orc_compute_rhs(const OrcScheme* s, const OrcClosures* c, const int* lo, const int* hi, const double* dxinv,
                    const double* U, double* dSdt, int /*nthreads*/) {
  if (int rc = set_closures(c)) return rc;
  set_scheme(s);
  static CNS lev;
  static Amr amr;
  int per[3] = {-1, -1, -1};
  setup_level(lev, amr, lo, hi, dxinv, per, per);
  MultiFab& Sborder = CNS::VSborder[0];
  copy_in(Sborder, U);
  lev.compute_rhs(Sborder, CNS::VdSdt[0], 0.0, nullptr, nullptr);
  copy_valid_out(CNS::VdSdt[0], dSdt, 0);
  return 0;
}

// The same with y sides of boundary code 6 where walls4 = {wall_lo, wall_hi,
// dom_lo_y, dom_hi_y} says so (x, z periodic; a non-wall y side outflow):
// the reference's own Flux_2nd_Order_KEEP and ViscousWallFluxes branches of
// compute_rhs run.  The box must be the domain.
int orc_compute_rhs_walls(const OrcScheme* s, const OrcClosures* c, const int* lo, const int* hi,
                          const double* dxinv, const double* U, double* dSdt, int /*nthreads*/, const int* walls4) {
  if (walls4[2] != lo[1] || walls4[3] != hi[1]) return 20;
  if (int rc = set_closures(c)) return rc;
  set_scheme(s);
  static CNS lev;
  static Amr amr;
  int bl[3] = {-1, walls4[0] ? 6 : 2, -1}, bh[3] = {-1, walls4[1] ? 6 : 2, -1};
  setup_level(lev, amr, lo, hi, dxinv, bl, bh);
  MultiFab& Sborder = CNS::VSborder[0];
  copy_in(Sborder, U);
  lev.compute_rhs(Sborder, CNS::VdSdt[0], 0.0, nullptr, nullptr);
  copy_valid_out(CNS::VdSdt[0], dSdt, 0);
  return 0;
}

int orc_fill_halo(const int* lo, const int* hi, const int* bc_lo, const int* bc_hi, double* U, int ncomp) {
  Box dom(IntVect(lo[0], lo[1], lo[2]), IntVect(hi[0], hi[1], hi[2]));
  Geometry geom;
  geom.dom = dom;
  BCRec bc;
  for (int d = 0; d < 3; ++d) {
    geom.periodic[d] = bc_lo[d] == -1;
    bc.setLo(d, bc_lo[d]);
    bc.setHi(d, bc_hi[d]);
  }
  MultiFab mf(BoxArray(dom), DistributionMapping(), ncomp, NGHOST);
  copy_in(mf, U);
  fill_level_ghosts(mf, geom, bc, NGHOST);
  std::memcpy(U, mf.fabs[0].data.data(), mf.fabs[0].data.size() * sizeof(double));
  return 0;
}

double orc_est_timestep(const OrcClosures* c, const int* lo, const int* hi, const double* dx, const double* U,
                        int nghost, double cfl) {
  if (set_closures(c)) return -1.0;
  Box bx(IntVect(lo[0], lo[1], lo[2]), IntVect(hi[0], hi[1], hi[2]));
  Box gb = grow(bx, nghost);
  Array4<const Real> a(const_cast<double*>(U), {gb.lo[0], gb.lo[1], gb.lo[2]},
                       {gb.hi[0] + 1, gb.hi[1] + 1, gb.hi[2] + 1}, NCONS);
  GpuArray<Real, AMREX_SPACEDIM> dxa = {{dx[0], dx[1], dx[2]}};
  // CNS::estTimeStep (src/CNS.cpp:380-395): ReduceMin of cns_estdt, times cfl
  Real estdt = cns_estdt(bx, a, dxa, g_cl);
  estdt *= cfl;
  return estdt;
}

int orc_advance(const OrcScheme* s, const OrcClosures* c, const int* lo, const int* hi, const double* dxinv,
                const int* bc_lo, const int* bc_hi, int order_rk, int stages_rk, double dt, double* S1, double* S2,
                int /*nthreads*/) {
  if (int rc = set_closures(c)) return rc;
  set_scheme(s);
  CNS::order_rk = order_rk;
  CNS::stages_rk = stages_rk;
  static CNS lev;
  static Amr amr;
  setup_level(lev, amr, lo, hi, dxinv, bc_lo, bc_hi);
  lev.state.clear();
  lev.state.resize(1);
  lev.state[0].new_data.reset(new MultiFab(lev.grids, DistributionMapping(), NCONS, NGHOST));
  copy_in(*lev.state[0].new_data, S1);
  lev.state[0].new_time = 0.0;
  lev.state[0].old_time = 0.0;
  lev.advance(0.0, dt, 1, 1);
  copy_valid_out(*lev.state[0].new_data, S2, NGHOST);
  return 0;
}

// CNS::printTotal's primitive extrema and convective CFL table
// (src/CNS.cpp:532-611) of one ghosted box: the reference's own cons2prim
// (src/rhs/CNS_hydro_K.h:15-34) over the valid cells, the min and max of each
// primitive, and the reference's own pointCFL (src/cls/CNS_K.h:49-59) applied
// cell by cell in one thread (k, j, i order) to a zero-initialised table, as
// the CPU build runs it.  out: min[6], max[6] (rho, u, v, w, T, p), then row d
// of the table: max |u_d + c|, max |u_d - c|, CFL_d.
int orc_prim_stats(const OrcClosures* c, const int* lo, const int* hi, const double* dx, const double* U, double dt,
                   double* out) {
  if (int rc = set_closures(c)) return rc;
  Box bx(IntVect(lo[0], lo[1], lo[2]), IntVect(hi[0], hi[1], hi[2]));
  Box gb = grow(bx, NGHOST);
  Array4<const Real> u(const_cast<double*>(U), {gb.lo[0], gb.lo[1], gb.lo[2]},
                       {gb.hi[0] + 1, gb.hi[1] + 1, gb.hi[2] + 1}, NCONS);
  FArrayBox qf(bx, NPRIM);
  Array4<Real> q = qf.array();
  for (int k = bx.lo[2]; k <= bx.hi[2]; ++k)
    for (int j = bx.lo[1]; j <= bx.hi[1]; ++j)
      for (int i = bx.lo[0]; i <= bx.hi[0]; ++i) cons2prim(i, j, k, u, q, g_cl);
  for (int n = 0; n < NPRIM; ++n) {
    Real mn = q(bx.lo[0], bx.lo[1], bx.lo[2], n), mx = mn;
    for (int k = bx.lo[2]; k <= bx.hi[2]; ++k)
      for (int j = bx.lo[1]; j <= bx.hi[1]; ++j)
        for (int i = bx.lo[0]; i <= bx.hi[0]; ++i) {
          mn = amrex::min(mn, q(i, j, k, n));
          mx = amrex::max(mx, q(i, j, k, n));
        }
    out[n] = mn;
    out[NPRIM + n] = mx;
  }
  Array2D<Real, 0, 2, 0, 2> arr{};
  GpuArray<Real, AMREX_SPACEDIM> dxa = {{dx[0], dx[1], dx[2]}};
  Array4<const Real> qc = q;
  for (int k = bx.lo[2]; k <= bx.hi[2]; ++k)
    for (int j = bx.lo[1]; j <= bx.hi[1]; ++j)
      for (int i = bx.lo[0]; i <= bx.hi[0]; ++i) pointCFL(i, j, k, arr, qc, g_cl, dxa, dt);
  for (int d = 0; d < 3; ++d)
    for (int e = 0; e < 3; ++e) out[2 * NPRIM + 3 * d + e] = arr(d, e);
  return 0;
}

// The reference's own derive functions of its plotfiles (derpres, dertemp,
// dervel: src/cls/CNS_K.h:76-129, registered at src/set/CNS_setup.cpp:153-176)
// on one ghosted box's valid cells; out as orc_plot_derive's.
int orc_plot_derive(const OrcClosures* c, const int* lo, const int* hi, const double* U, double* out) {
  if (int rc = set_closures(c)) return rc;
  Box bx(IntVect(lo[0], lo[1], lo[2]), IntVect(hi[0], hi[1], hi[2]));
  Box gb = grow(bx, NGHOST);
  Array4<const Real> u(const_cast<double*>(U), {gb.lo[0], gb.lo[1], gb.lo[2]},
                       {gb.hi[0] + 1, gb.hi[1] + 1, gb.hi[2] + 1}, NCONS);
  FArrayBox dat(bx, NCONS), der(bx, 5);
  Array4<Real> d = dat.array();
  for (int n = 0; n < NCONS; ++n)
    for (int k = bx.lo[2]; k <= bx.hi[2]; ++k)
      for (int j = bx.lo[1]; j <= bx.hi[1]; ++j)
        for (int i = bx.lo[0]; i <= bx.hi[0]; ++i) d(i, j, k, n) = u(i, j, k, n);
  Geometry geom;
  derpres(bx, der, 0, 1, dat, geom, 0.0, nullptr, 0);
  dertemp(bx, der, 1, 1, dat, geom, 0.0, nullptr, 0);
  for (int v = 0; v < 3; ++v) {
    // dervel reads (density, momentum component) as its components 0 and 1
    FArrayBox dv(bx, 2);
    Array4<Real> a = dv.array();
    for (int k = bx.lo[2]; k <= bx.hi[2]; ++k)
      for (int j = bx.lo[1]; j <= bx.hi[1]; ++j)
        for (int i = bx.lo[0]; i <= bx.hi[0]; ++i) {
          a(i, j, k, 0) = u(i, j, k, URHO);
          a(i, j, k, 1) = u(i, j, k, UMX + v);
        }
    dervel(bx, der, 2 + v, 1, dv, geom, 0.0, nullptr, 0);
  }
  std::memcpy(out, der.data.data(), der.data.size() * sizeof(double));
  return 0;
}

}  // extern "C"
