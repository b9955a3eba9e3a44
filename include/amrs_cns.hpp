// amrs_cns.hpp - C++ drop-in with the reference's CNS call surface over the
// C ABI of amrs_gb300.h (header-only; link libamrs_gb300.so and cudart).
//
// Mirrors, for one level (a BoxArray tiling the domain):
//   CNS::compute_rhs(MultiFab& S, MultiFab& dSdt, Real dt, FluxRegister*, FluxRegister*)
//       src/CNS.h:51, src/tim/CNS_advance.cpp:186-427
//   CNS::advance(Real time, Real dt, int iteration, int ncycle)
//       src/CNS.h:77-80, src/tim/CNS_advance.cpp:14-183
//   CNS::estTimeStep()                      src/CNS.cpp:380-395
//   CNS::computeInitialDt / computeNewDt    src/CNS.cpp:282-377
// over a minimal MultiFab: device FArrayBoxes in the amrex::Array4 layout
// (component-major, i fastest, ghost cells included).  Errors throw
// amrs::Error carrying the C status (the C layer itself never throws).
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <limits>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "amrs_gb300.h"

namespace amrs {

using Real = double;

struct Error : std::runtime_error {
  amrs_status status;
  Error(amrs_status s, const std::string& what)
      : std::runtime_error(what + ": " + amrs_status_string(s) + " " + amrs_last_cuda_error()), status(s) {}
};
inline void check(amrs_status s, const char* what) {
  if (s != AMRS_OK) throw Error(s, what);
}

// amrex::Box (cell-centred, inclusive bounds)
struct Box {
  int lo[3], hi[3];
  int length(int d) const { return hi[d] - lo[d] + 1; }
  long long numPts() const { return (long long)length(0) * length(1) * length(2); }
  amrs_box c() const { return amrs_box{{lo[0], lo[1], lo[2]}, {hi[0], hi[1], hi[2]}}; }
};

// One device FArrayBox of a MultiFab.
class FArrayBox {
 public:
  FArrayBox(const Box& valid, int ncomp, int ngrow) : valid_(valid), ncomp_(ncomp), ngrow_(ngrow) {
    const size_t n = (size_t)(valid.length(0) + 2 * ngrow) * (valid.length(1) + 2 * ngrow) *
                     (valid.length(2) + 2 * ngrow) * ncomp;
    if (cudaMalloc(&p_, n * sizeof(Real)) != cudaSuccess) throw Error(AMRS_ERR_ALLOC, "FArrayBox");
    bytes_ = n * sizeof(Real);
  }
  ~FArrayBox() { if (p_) cudaFree(p_); }
  FArrayBox(const FArrayBox&) = delete;
  FArrayBox& operator=(const FArrayBox&) = delete;
  amrs_array4 array() const {
    amrs_array4 a{};
    const int nx = valid_.length(0) + 2 * ngrow_, ny = valid_.length(1) + 2 * ngrow_,
              nz = valid_.length(2) + 2 * ngrow_;
    a.p = p_;
    a.jstride = nx;
    a.kstride = (int64_t)nx * ny;
    a.nstride = (int64_t)nx * ny * nz;
    for (int d = 0; d < 3; ++d) {
      a.begin[d] = valid_.lo[d] - ngrow_;
      a.end[d] = valid_.hi[d] + ngrow_ + 1;
    }
    a.ncomp = ncomp_;
    return a;
  }
  Real* dataPtr() const { return p_; }
  size_t bytes() const { return bytes_; }
  const Box& box() const { return valid_; }

 private:
  Box valid_;
  int ncomp_, ngrow_;
  Real* p_ = nullptr;
  size_t bytes_ = 0;
};

// amrex::MultiFab restricted to what the RHS path uses.
class MultiFab {
 public:
  MultiFab() = default;
  MultiFab(const std::vector<Box>& grids, int ncomp, int ngrow) { define(grids, ncomp, ngrow); }
  void define(const std::vector<Box>& grids, int ncomp, int ngrow) {
    fabs_.clear();
    grids_ = grids;
    ncomp_ = ncomp;
    ngrow_ = ngrow;
    for (const Box& b : grids) fabs_.emplace_back(new FArrayBox(b, ncomp, ngrow));
  }
  int size() const { return (int)fabs_.size(); }
  int nComp() const { return ncomp_; }
  int nGrow() const { return ngrow_; }
  const Box& box(int i) const { return grids_[i]; }
  FArrayBox& fab(int i) { return *fabs_[i]; }
  amrs_array4 array(int i) const { return fabs_[i]->array(); }

 private:
  std::vector<Box> grids_;
  int ncomp_ = 0, ngrow_ = 0;
  std::vector<std::unique_ptr<FArrayBox>> fabs_;
};

// cns.lo_bc / cns.hi_bc codes and cell sizes (amrex::Geometry subset).
struct Geometry {
  Box domain;
  Real dx[3];
  int lo_bc[3] = {-1, -1, -1}, hi_bc[3] = {-1, -1, -1};
  Real ProbSize() const { return domain.length(0) * dx[0] * domain.length(1) * dx[1] * domain.length(2) * dx[2]; }
};

struct FluxRegister;  // reflux is commented out in the reference; the pointers are accepted and unused

// One level: a BoxArray `grids` tiling the domain (default: the domain as one
// box).  FillPatch is single-level FillPatch across the level (neighbour
// copies, periodic images, physical BCs: amrs_boxlist_set_domain);
// compute_rhs is the reference's MFIter loop of per-box calls; advance runs
// each RK stage over all boxes at once (amrs_rk_stage_boxlist).
class CNS {
 public:
  static constexpr int NCONS = 5;
  static constexpr int NGHOST = 3;

  // body_force: cns.rhs_source = 1 with a constant body force per unit mass
  // as the problem's user_source (the channel problem's is {fx, 0, 0});
  // nullptr: rhs_source = 0.
  CNS(const Geometry& geom, const amrs_scheme& scheme, const amrs_closures& closures, int order_rk = 3,
      int stages_rk = 3, int device = 0, const Real* body_force = nullptr)
      : CNS(geom, std::vector<Box>{geom.domain}, scheme, closures, order_rk, stages_rk, device, body_force) {}

  CNS(const Geometry& geom, const std::vector<Box>& grids, const amrs_scheme& scheme,
      const amrs_closures& closures, int order_rk = 3, int stages_rk = 3, int device = 0,
      const Real* body_force = nullptr)
      : geom_(geom), grids_(grids), order_rk_(order_rk), stages_rk_(stages_rk) {
    check(amrs_create(&h_, &scheme, &closures, device), "amrs_create");
    if (body_force) check(amrs_set_source(h_, 1, body_force), "amrs_set_source");
    for (int i = 0; i < 3; ++i) state_[i].define(grids, NCONS, NGHOST);
    for (int d = 0; d < 3; ++d) dxinv_[d] = 1.0 / geom.dx[d];
    const int n = (int)grids.size();
    std::vector<amrs_box> boxes(n);
    std::vector<double> dx3(3 * n);
    std::vector<amrs_array4> arrs(3 * n);
    for (int b = 0; b < n; ++b) {
      boxes[b] = grids[b].c();
      for (int d = 0; d < 3; ++d) dx3[3 * b + d] = dxinv_[d];
      for (int s = 0; s < 3; ++s) arrs[3 * b + s] = state_[s].array(b);
    }
    check(amrs_boxlist_create(h_, n, boxes.data(), dx3.data(), 3, arrs.data(), nullptr, 0, nullptr, &bl_),
          "amrs_boxlist_create");
    amrs_box dom = geom.domain.c();
    check(amrs_boxlist_set_domain(bl_, &dom, geom.lo_bc, geom.hi_bc), "amrs_boxlist_set_domain");
    if (cudaMalloc(&dt_dev_, n * sizeof(Real)) != cudaSuccess) throw Error(AMRS_ERR_ALLOC, "CNS");
  }
  ~CNS() {
    if (dt_dev_) cudaFree(dt_dev_);
    if (bl_) amrs_boxlist_destroy(bl_);
    if (h_) amrs_destroy(h_);
  }
  CNS(const CNS&) = delete;
  CNS& operator=(const CNS&) = delete;

  MultiFab& get_new_data() { return state_[cur_]; }
  const std::vector<Box>& boxArray() const { return grids_; }
  Real curTime() const { return time_; }
  void setStream(cudaStream_t s) { stream_ = s; }
  // The problem's bcnormal beyond code-6 y sides evaluated on the device in
  // every FillPatch of the level (amrs_bcnormal kind 1: the channel
  // problem's isothermal no-slip wall); nullptr: the ghosts stay the caller's.
  void setBcNormal(const amrs_bcnormal* bn) { check(amrs_boxlist_set_bcnormal(bl_, bn), "amrs_boxlist_set_bcnormal"); }

  // CNS::compute_rhs: S ghost-filled (3 ghosts), dSdt valid-only; the
  // reference's MFIter loop, one amrs_rhs_box per box.
  void compute_rhs(MultiFab& S, MultiFab& dSdt, Real /*dt*/, FluxRegister* = nullptr, FluxRegister* = nullptr) {
    for (int i = 0; i < S.size(); ++i) {
      amrs_box b = S.box(i).c();
      check(amrs_rhs_box(h_, &b, dxinv_, S.array(i), dSdt.array(i), stream_), "amrs_rhs_box");
    }
  }

  // Single-level FillPatch of one of this level's state MultiFabs, or of a
  // caller MultiFab made of the domain as one box.
  void FillPatch(MultiFab& S) {
    for (int s = 0; s < 3; ++s)
      if (&S == &state_[s]) {
        check(amrs_boxlist_fill_halo(bl_, s, stream_), "amrs_boxlist_fill_halo");
        return;
      }
    if (S.size() != 1) throw Error(AMRS_ERR_STATE, "FillPatch of a multi-box MultiFab outside the level");
    amrs_box d = geom_.domain.c();
    check(amrs_fill_halo_box(&d, geom_.lo_bc, geom_.hi_bc, S.array(0), stream_), "amrs_fill_halo_box");
  }

  // CNS::advance: one step of the configured SSP-RK scheme; returns dt.
  Real advance(Real time, Real dt, int /*iteration*/ = 1, int /*ncycle*/ = 1) {
    amrs_stage_prog progs[16];
    int32_t ns = 0;
    check(amrs_rk_program(order_rk_, stages_rk_, dt, progs, 16, &ns), "amrs_rk_program");
    const int s1 = cur_;
    int work[2], w = 0;
    for (int i = 0; i < 3; ++i)
      if (i != s1) work[w++] = i;
    int cur = s1, which = 0;
    for (int i = 0; i < ns; ++i) {
      const int src = progs[i].src_state == 0 ? s1 : cur;
      int out = work[which];
      if (out == src) { which ^= 1; out = work[which]; }
      check(amrs_boxlist_fill_halo(bl_, src, stream_), "amrs_boxlist_fill_halo");
      check(amrs_rk_stage_boxlist(bl_, &progs[i], src, s1, out, stream_), "amrs_rk_stage_boxlist");
      cur = out;
      which ^= 1;
    }
    cur_ = cur;
    time_ = time + dt;
    return dt;
  }

  // The reference's main loop for this level (src/main.cpp:66-75): steps
  // until stop_time or max_step, dt from cfl (computeInitialDt /
  // computeNewDt) when cfl > 0, else fixed_dt; the whole loop is one graph
  // launch on the device (amrs_rk_run_boxlist).  Returns the steps taken
  // (host-synchronising).
  int run(Real stop_time, int max_step, Real cfl, Real fixed_dt = 0.0) {
    int work[2], w = 0;
    for (int i = 0; i < 3; ++i)
      if (i != cur_) work[w++] = i;
    check(amrs_rk_run_boxlist(bl_, order_rk_, stages_rk_, cfl, fixed_dt, time_, stop_time, max_step, cur_, work[0],
                              work[1], stream_),
          "amrs_rk_run_boxlist");
    double t = 0.0, dt = 0.0;
    int32_t steps = 0;
    check(amrs_boxlist_run_state(bl_, &t, &dt, &steps, stream_), "amrs_boxlist_run_state");
    time_ = t;
    return steps;
  }

  // CNS::estTimeStep: cfl * min over the level of dx/(|u|+c) (host-synchronising).
  Real estTimeStep(Real cfl) {
    const int n = (int)grids_.size();
    for (int b = 0; b < n; ++b) {
      amrs_box bx = grids_[b].c();
      check(amrs_est_timestep_box(h_, &bx, geom_.dx, cfl, state_[cur_].array(b), dt_dev_ + b, stream_),
            "amrs_est_timestep_box");
    }
    std::vector<Real> dts(n);
    if (cudaMemcpyAsync(dts.data(), dt_dev_, n * sizeof(Real), cudaMemcpyDeviceToHost, stream_) != cudaSuccess ||
        cudaStreamSynchronize(stream_) != cudaSuccess)
      throw Error(AMRS_ERR_CUDA, "estTimeStep");
    return *std::min_element(dts.begin(), dts.end());
  }

  // CNS::computeNewDt for one level: growth capped at 1.1x, last step clamped to stop_time.
  Real computeNewDt(Real cfl, Real dt_old, Real stop_time) {
    Real dt0 = std::min(estTimeStep(cfl), 1.1 * dt_old);
    const Real eps = 0.001 * dt0;
    if (stop_time >= 0.0 && time_ + dt0 > stop_time - eps) dt0 = stop_time - time_;
    return dt0;
  }

  amrs_handle* handle() { return h_; }
  amrs_boxlist* boxlist() { return bl_; }

 private:
  Geometry geom_;
  std::vector<Box> grids_;
  int order_rk_, stages_rk_;
  amrs_handle* h_ = nullptr;
  amrs_boxlist* bl_ = nullptr;
  MultiFab state_[3];
  int cur_ = 0;
  Real time_ = 0.0;
  Real dxinv_[3];
  Real* dt_dev_ = nullptr;
  cudaStream_t stream_ = 0;
};

}  // namespace amrs
