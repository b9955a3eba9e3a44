// Launch wrappers of the device kernels (host-callable, no CUDA types in the
// C ABI: these stay internal to the library).
#pragma once
#include <cuda_runtime.h>

#include "amrs_boxes.cuh"
#include "tma.cuh"

namespace amrs {

// ---- KEEP fused path (rhs_keep.cu)
cudaError_t launch_prims(const BoxTable& tb, int s_in, long long ncells, int nsm, cudaStream_t st);
cudaError_t launch_visc(const BoxTable& tb, long long ncells, int nsm, cudaStream_t st);
cudaError_t launch_keep_face(int order, bool visc, bool src, const BoxTable& tb, int s_in, int s_s1, int s_out,
                             const DProg& prog, int rhs_only, const TmaDesc& tma, int* err, int grid, int nsm,
                             cudaStream_t st);
bool keep_tile_fits(int order, int tx, int ty);
int keep_ctas_per_sm(int order);
template <int ORDER> int keep_smem_bytes();

// ---- face-array (reference-structured) path (rhs_plain.cu)
// Face flux scratch per box: three nodal arrays, described per box in FaceRec.
struct FaceRec {
  DArr f[3];    // face fluxes, nodal in direction d, NCONS comps, over [lo,hi] (+1 in d)
  DArr pf[3];   // WENO physical fluxes over grow(box,3), NCONS comps
  DArr lam;     // WENO / JST spectral radius over grow(box,3), 3 comps
  DArr sen;     // JST sensor over grow(box,3), 3 comps
  DArr slope[3];  // MUSCL face-state terms per direction over grow(box,1), NSLOPE comps
  long long nface[3];  // faces per direction (for flattening)
};
struct FaceTable {
  const FaceRec* fr;
  const long long* fpre[3];  // prefix of face counts per direction
  const long long* gpre;     // prefix of grow(box,3) cell counts
  const long long* vpre;     // prefix of valid cell counts
};

cudaError_t launch_keep_faces_plain(int order, const BoxTable& tb, const FaceTable& ft, long long nfaces[3],
                                    int nsm, cudaStream_t st);
cudaError_t launch_weno(const BoxTable& tb, const FaceTable& ft, int s_in, long long ngcells, long long nfaces[3],
                        bool ref_order, int nsm, cudaStream_t st);
// physical fluxes and lambda only (the forward values the WENO adjoint reads)
cudaError_t launch_weno_point(const BoxTable& tb, const FaceTable& ft, int s_in, long long ngcells, int nsm,
                              cudaStream_t st);
// the WENO face kernel alone (point fluxes already current)
cudaError_t launch_weno_faces(const BoxTable& tb, const FaceTable& ft, int s_in, long long nfaces[3], bool ref_order,
                              int nsm, cudaStream_t st);
// MUSCL slopes and face-state terms alone (the reverse pass recomputes them)
cudaError_t launch_slopes(const BoxTable& tb, const FaceTable& ft, const long long* spre_d[3], long long nslope[3],
                          int nsm, cudaStream_t st);
cudaError_t launch_riemann(const BoxTable& tb, const FaceTable& ft, const long long* spre_d[3],
                           long long nslope[3], long long nfaces[3], int nsm, cudaStream_t st);
// WENO5-reconstructed primitive states + the two-shock solver (riemann_weno = 1)
cudaError_t launch_weno_riemann(const BoxTable& tb, const FaceTable& ft, long long nfaces[3], int nsm,
                                cudaStream_t st);
// JST sensor and spectral radius alone (the reverse pass recomputes them)
cudaError_t launch_jst_sensor(const BoxTable& tb, const FaceTable& ft, long long nvalid, int nsm, cudaStream_t st);
cudaError_t launch_jst(const BoxTable& tb, const FaceTable& ft, int s_in, long long ngcells, long long nvalid,
                       long long nfaces[3], int nsm, cudaStream_t st);
cudaError_t launch_visc_face_add(const BoxTable& tb, const FaceTable& ft, long long nfaces[3], int nsm,
                                 cudaStream_t st);
cudaError_t launch_div_stage(const BoxTable& tb, const FaceTable& ft, int s_in, int s_s1, int s_out,
                             const DProg& prog, int rhs_only, long long nvalid, int nsm, cudaStream_t st);

// ---- utilities (util.cu)
struct HaloBox {
  DArr u;
  int lo[3], hi[3];
  int bc_lo[3], bc_hi[3];
  int ncomp;
};
cudaError_t launch_halo(const HaloBox& hb, cudaStream_t st);

// ---- adjoint (adjoint.cu), single box (tb.box[0], Q already computed)
struct AdjRecHost {
  DArr vbar, ubar;
  DArr pair[3][3];  // [direction][separation-1], 12 comps over grow(box,3)
  DArr vg;          // 16 comps over grow(box,1)
  int n[3];
  int visc;
  double* part;     // 2 x 8 x nsm doubles: per-block parameter-cotangent sums (needed when pbar is given)
};
// order 0: viscous part and cons2prim reverse only (no KEEP pairs)
cudaError_t launch_rhs_vjp(int order, const BoxTable& tb, const AdjRecHost& ah, double* pbar, int nsm,
                           cudaStream_t st);
// MUSCL-Riemann Euler part of the RHS VJP, added to ubar (adjoint_muscl.cu)
size_t muscl_vjp_buffer_bytes(const int n[3]);
cudaError_t launch_muscl_vjp(const BoxTable& tb, const FaceRec& fr, const DArr& vbar, const DArr& ubar, double* buf,
                             const int n[3], int nsm, cudaStream_t st);
// JST part of the RHS VJP, added to ubar (adjoint_jst.cu)
size_t jst_vjp_buffer_bytes(const int n[3]);
cudaError_t launch_jst_vjp(const BoxTable& tb, const FaceRec& fr, const DArr& vbar, const DArr& ubar, double* buf,
                           const int n[3], int nsm, cudaStream_t st);
// WENO5-Riemann Euler part of the RHS VJP, added to ubar (adjoint_weno_riemann.cu)
size_t weno_riemann_vjp_buffer_bytes(const int n[3]);
cudaError_t launch_weno_riemann_vjp(const BoxTable& tb, const DArr& vbar, const DArr& ubar, double* buf,
                                    const int n[3], int nsm, cudaStream_t st);
// WENO5 Euler part of the RHS VJP, added to ubar (adjoint_weno.cu)
size_t weno_vjp_buffer_bytes(const int n[3]);
cudaError_t launch_weno_vjp(const BoxTable& tb, const FaceRec& fr, const DArr& vbar, const DArr& ubar, double* buf,
                            const int n[3], int nsm, cudaStream_t st);
cudaError_t launch_source_vjp(const BoxRec& R, const double force[3], const DArr& vbar, const DArr& ubar, int nsm,
                              cudaStream_t st);
cudaError_t launch_adj_prog(const BoxRec& R, const DProg& prog, const DArr& wbar, const DArr& s1bar, const DArr& inbar,
                            const DArr& vbar, int accumulate, int nsm, cudaStream_t st);
cudaError_t launch_adj_halo(const HaloBox& hb, int nsm, cudaStream_t st);
cudaError_t launch_halo_list(const BoxTable& tb, const long long* gpre, long long total, int slot, const int bc_lo[3],
                             const int bc_hi[3], int nsm, cudaStream_t st);
// Device state of a time loop over a box list (amrs_rk_run_boxlist); the
// list's kernels read `active` through BoxTable::active.
struct RunCtl {
  double time, dt, stop, cfl, change_max;
  int step, max_steps, use_cfl, active;
  unsigned long long bits;  // cns_estdt reduction cell (ordered bits of the minimum)
};
cudaError_t launch_run_estdt(const BoxTable& tb, int s_in, long long nvalid, RunCtl* c, int nsm, cudaStream_t st);
cudaError_t launch_run_step_done(RunCtl* c, cudaGraphConditionalHandle cond, cudaStream_t st);
cudaError_t launch_run_begin(RunCtl* c, cudaStream_t st);
cudaError_t launch_copy_slot(const BoxTable& tb, int from, int to, long long nvalid, int nsm, cudaStream_t st);
int totals_blocks(long long nvalid, int nsm);
// CNS::printTotal's primitive extrema and CFL table over the valid cells
// (slot -1: the primitive scratch of the last RHS); out: 21 device doubles
cudaError_t launch_prim_stats(const BoxTable& tb, const long long* vpre, int slot, double dt, const double dx[3],
                              long long nvalid, unsigned long long* cells, double* out, int nsm, cudaStream_t st);
// raises *flag when a valid cell of `slot` holds a NaN or an infinity
cudaError_t launch_nonfinite_check(const BoxTable& tb, const long long* vpre, int slot, long long nvalid, int* flag,
                                   int nsm, cudaStream_t st);
cudaError_t launch_totals(const BoxTable& tb, int slot, long long nvalid, double scale, double* part, double* out,
                          int nsm, cudaStream_t st);

// domain of a level whose boxes tile it, with its physical boundary codes
struct LevelDomain {
  int lo[3], hi[3];
  int bc_lo[3], bc_hi[3];
};
cudaError_t launch_halo_level(const BoxTable& tb, const long long* gpre, const int* owner, long long total, int slot,
                              const LevelDomain& dom, int nsm, cudaStream_t st);
// A problem bcnormal evaluated on the device for y sides of code 6 (kind 1:
// the channel problem's isothermal no-slip wall), after the library's fill.
struct DBcNormal {
  int kind;
  double Tw, Tmin;
  double prob_lo[3], prob_hi[3], dx[3];
};
cudaError_t launch_bcnormal_box(const DArr& u, const int lo[3], const int hi[3], const int bc_lo[3],
                                const int bc_hi[3], const DClosures& cl, const DBcNormal& bn, cudaStream_t st);
cudaError_t launch_bcnormal_list(const BoxTable& tb, int slot, const LevelDomain& dom, const DBcNormal& bn, int nsm,
                                 cudaStream_t st);
cudaError_t launch_fp64_probe(double* out, int blocks, int iters, cudaStream_t st);
cudaError_t launch_intpipe_probe(int mode, double* out, int blocks, int iters, cudaStream_t st);
// ddiv_rn (ddiv.cuh) against the hardware division over `count` generated operand pairs
cudaError_t launch_ddiv_check(unsigned long long seed, long long count, unsigned long long* bad, double* first,
                              int nsm, cudaStream_t st);
// dsqrt_rn (ddiv.cuh) against the hardware square root over `count` generated operands
cudaError_t launch_dmul_check(unsigned long long seed, long long count, unsigned long long* bad, double* first,
                              int nsm, cudaStream_t st);
cudaError_t launch_dsqrt_check(unsigned long long seed, long long count, unsigned long long* bad, double* first,
                               int nsm, cudaStream_t st);
// derived plot variables (pressure, temperature, velocities) of one box's valid cells
cudaError_t launch_plot_derive(const DArr& U, const DArr& O, const int lo[3], const int n[3], double gamma, double cv,
                               int nsm, cudaStream_t st);
// amrex::average_down of cell-centred data (coarse box lo, extents n, ratio r).
cudaError_t launch_avgdown(const DArr& fine, const DArr& crse, const int lo[3], const int n[3], const int r[3],
                           int scomp, int ncomp, double volfrac, int nsm, cudaStream_t st);
// One bounded mbarrier wait that nothing completes; raises *err.
cudaError_t launch_wait_timeout_probe(int* err, long long polls, cudaStream_t st);
cudaError_t launch_estdt(const BoxTable& tb, int s_in, long long nvalid, double cfl, unsigned long long* bits,
                         double* dt_out, int nsm, cudaStream_t st);

}  // namespace amrs
