/*
 * amrs_gb300.h - C ABI of the GB300-native compressible RHS + SSP-RK path.
 *
 * Drop-in for the per-box RHS and RK-stage calls of amrsolver:
 *   CNS::compute_rhs(MultiFab& S, MultiFab& dSdt, Real dt, FluxRegister*, FluxRegister*)
 *       (src/CNS.h:51, src/tim/CNS_advance.cpp:186-427)
 *   CNS::advance(Real time, Real dt, int iteration, int ncycle)
 *       (src/CNS.h:77-80, src/tim/CNS_advance.cpp:14-183)
 * plus the pieces of AMReX those calls rely on (FillPatch ghost fill,
 * MultiFab::LinComb/Saxpy/Xpay/Copy, ReduceMin for cns_estdt).
 *
 * All arrays are FP64 device memory in the amrex::Array4 convention:
 * element (i,j,k,n) lives at p[(i-begin[0]) + (j-begin[1])*jstride +
 * (k-begin[2])*kstride + n*nstride].  Conserved components are
 * (rho, rho u, rho v, rho w, rho E) as URHO..UET in the reference's prob.h.
 *
 * Every function returns an amrs_status; none aborts, none throws, and none
 * synchronises the host unless its comment says so.  Caller-owned buffers
 * are never freed by the library.  Scratch memory belongs to the handle.
 */
#ifndef AMRS_GB300_H
#define AMRS_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum amrs_status {
  AMRS_OK = 0,
  AMRS_ERR_NULL = 1,        /* a required pointer is NULL */
  AMRS_ERR_BOX = 2,         /* empty box, box outside its array, or 2^31+ cells with ghosts */
  AMRS_ERR_BC = 3,          /* unsupported or inconsistent boundary codes */
  AMRS_ERR_SCHEME = 4,      /* unsupported scheme switches */
  AMRS_ERR_RK = 5,          /* order_rk/stages_rk combination the reference rejects */
  AMRS_ERR_CUDA = 6,        /* a CUDA runtime call failed (see amrs_last_cuda_error) */
  AMRS_ERR_ALLOC = 7,       /* device or host allocation failed */
  AMRS_ERR_LAYOUT = 8,      /* strides/ncomp inconsistent with the box */
  AMRS_ERR_SIZE = 9,        /* request beyond a documented size limit */
  AMRS_ERR_NONFINITE = 10,  /* non-finite value detected in a checked result */
  AMRS_ERR_TIMEOUT = 11,    /* a bounded device-side wait ran out */
  AMRS_ERR_STATE = 12       /* call sequence error (e.g. graph not built) */
} amrs_status;

/* amrex::Array4<Real> */
typedef struct amrs_array4 {
  double* p;
  int64_t jstride, kstride, nstride;
  int32_t begin[3]; /* inclusive lower corner of the allocation (ghosts included) */
  int32_t end[3];   /* exclusive upper corner */
  int32_t ncomp;
} amrs_array4;

/* closures_derived_t<Visc, Cond, calorifically_perfect_gas_t>
 * (src/cls/Closures.h:72-182).  visc_law/cond_law: 0 = constant
 * (visc_const_t / cond_const_t), 1 = Sutherland (visc_suth_t / cond_suth_t). */
typedef struct amrs_closures {
  double gamma, cv, cp, Rspec;
  int32_t visc_law, cond_law;
  double visc_ref, Tvisc_ref, cond_ref, Tcond_ref;
  double Cshock, Cdamp;
} amrs_closures;

/* cns.* run-time switches read by CNS::read_params (src/CNS.cpp:85-136).
 * flux_euler: 1 = KEEP split form (src/rhs/CentralKEEP.h), 2 = WENO5-JS with
 * local Lax-Friedrichs splitting (src/rhs/High_resolution.h), any other value
 * (0 in the reference's inputs) = the Riemann path, as compute_rhs's else
 * branch (src/tim/CNS_advance.cpp:221-223): MUSCL + two-shock solver
 * (src/rhs/Riemann.h).  order_keep: 2, 4 or 6.  art_diss: JST. */
typedef struct amrs_scheme {
  int32_t rhs_euler, rhs_visc, flux_euler, order_keep, art_diss;
  /* WENO5 only (no counterpart in the reference's switches).  0: the
   * reference's operation order (src/rhs/High_resolution.h:124-159),
   * bit-identical to its CPU build.  1: each reconstruction forms its three
   * nonlinear weights over a common denominator with fused multiply-adds
   * (one division instead of four, about 1.7x faster): the same function in
   * exact arithmetic, rounding differences only, which the flux
   * differencing amplifies where the RHS is small next to the split fluxes
   * (near-incompressible flow: up to ~1e-9 relative on the mass RHS). */
  int32_t weno_fast;
  /* Riemann path only (no counterpart in the reference's switches).  0: the
   * reference's MUSCL characteristic states.  1: WENO5-Riemann, an
   * extension: rho, u_n, p and the tangential velocities reconstructed to
   * each face from both sides with the WENO5-JS stencils, fed to the same
   * two-shock solver (src/rhs/Riemann.h:123-249). */
  int32_t riemann_weno;
} amrs_scheme;

/* Cell-centred index box, inclusive bounds (amrex::Box). */
typedef struct amrs_box {
  int32_t lo[3], hi[3];
} amrs_box;

/* One RK stage as the BLAS-1 program CNS::advance runs after compute_rhs
 * (src/tim/CNS_advance.cpp:51-166).  Registers: 0 = S1 (old state),
 * 1 = S2 (new state; equal to the stage input's valid cells), 2 = dSdt.
 * kind 0 LinComb dst = a*x + b*y; 1 Saxpy dst += a*x; 2 Xpay dst = x + a*dst;
 * 3 Copy dst = x.  src_state tells which state FillPatch reads for this
 * stage (0 = S1, 1 = S2).  The stage's result is register 1. */
typedef struct amrs_rk_op {
  int32_t kind, dst, x, y;
  double a, b;
} amrs_rk_op;

typedef struct amrs_stage_prog {
  int32_t src_state;
  int32_t nops;
  amrs_rk_op ops[3];
} amrs_stage_prog;

typedef struct amrs_handle amrs_handle;

/* ---- handle ---------------------------------------------------------- */

/* Create a handle bound to CUDA device `device` with the given scheme and
 * closures (the reference's CNS::variableSetUp + read_params,
 * src/set/CNS_setup.cpp:90-104, src/CNS.cpp:85-153).  The handle owns the
 * scratch arena (primitive and viscous-flux fields, reduction cells). */
amrs_status amrs_create(amrs_handle** out, const amrs_scheme* scheme, const amrs_closures* closures, int device);
amrs_status amrs_destroy(amrs_handle* h);
amrs_status amrs_set_closures(amrs_handle* h, const amrs_closures* closures);
/* The physical domain and boundary codes (cns.lo_bc / cns.hi_bc) of the
 * level the handle's per-box calls work on; NULL arguments clear them.
 * y sides with code 6 (user-defined wall) switch on the reference's wall
 * treatment in compute_rhs (src/tim/CNS_advance.cpp:226-229, :300-333) for
 * boxes that touch them: the KEEP y faces of the order_keep/2 planes next to
 * the wall take the second-order pair (Flux_2nd_Order_KEEP,
 * src/rhs/CentralKEEP.h:232-287) and the viscous cell fluxes of the wall's
 * ghost row use one-sided y derivatives (ViscousWallFluxes,
 * src/rhs/CNS_hydro_K.h:177-251).  Ghost cells beyond code-1/6 sides are the
 * caller's (the problem's bcnormal fills them); the library's fills leave
 * them untouched.  amrs_rhs_vjp_box applies the same wall treatment in
 * reverse; amrs_rk_stage_vjp_box rejects a handle with walls (the ghost
 * values beyond a code-6 side come from the caller's bcnormal, whose
 * derivative the library does not have): such domains use
 * amrs_rk_stage_vjp_box_ghosted. */
amrs_status amrs_set_domain(amrs_handle* h, const amrs_box* domain, const int32_t bc_lo[3], const int32_t bc_hi[3]);
/* cns.rhs_source (src/CNS.cpp:22,103) with the problem's user_source being a
 * constant body force per unit mass f, the source step of compute_rhs
 * (src/tim/CNS_advance.cpp:396-407): after the flux divergence, dSdt(UMX+d)
 * += rho f_d and dSdt(UET) += m_d f_d (x, y, z order) for every d with
 * f_d != 0, from the stage input's conserved state.  The channel problem's
 * user_source (exm/Channel/prob.h:189-193) is f = (fx, 0, 0).  rhs_source 0
 * or an all-zero force: no source (problems whose user_source is empty).
 * Applies to the handle's per-box calls (forward and VJP) and to box lists
 * created afterwards. */
amrs_status amrs_set_source(amrs_handle* h, int32_t rhs_source, const double force[3]);
const char* amrs_status_string(amrs_status s);
/* Last CUDA error string recorded by the library (thread-local). */
const char* amrs_last_cuda_error(void);
/* Library version (major*10000 + minor*100 + patch) and the CUDA arch it was built for. */
int32_t amrs_version(void);
int32_t amrs_cuda_arch(void);

/* ---- RK programs ------------------------------------------------------ */

/* Fill `progs` (capacity `cap`) with the stage programs of CNS::advance for
 * (order_rk, stages_rk) and time step dt; *nstages receives the count.
 * Mirrors src/tim/CNS_advance.cpp:51-166 and the checks of
 * src/CNS.cpp:119-133.  Host only. */
amrs_status amrs_rk_program(int32_t order_rk, int32_t stages_rk, double dt, amrs_stage_prog* progs, int32_t cap,
                            int32_t* nstages);

/* ---- per-box entry points (drop-in for one MFIter iteration) ---------- */

/* dSdt over `bx` from the ghost-filled state (3 ghost cells): one box of
 * CNS::compute_rhs (src/tim/CNS_advance.cpp:186-391).  `dxinv` is
 * Geometry::InvCellSizeArray().  Asynchronous on `stream` (cudaStream_t). */
amrs_status amrs_rhs_box(amrs_handle* h, const amrs_box* bx, const double dxinv[3], amrs_array4 state,
                         amrs_array4 dsdt, void* stream);

/* amrs_rhs_box without any device allocation: no counterpart in the
 * reference.  Some callers cannot call cudaMalloc (a host whose arena or
 * memory pool owns all device memory, or one with a fixed device-memory
 * budget); this variant of the fused KEEP + viscous RHS keeps its scratch in
 * one static device array of the library instead of a handle.  Limits:
 * KEEP 2/4/6 with or without viscous terms, no JST and no source term
 * (AMRS_ERR_SCHEME otherwise, also for transport laws other than 0/1),
 * boxes of at most 32 cells per direction (AMRS_ERR_SIZE beyond); the array
 * (6.9 MB) lives on every device that loads the library until exit; every
 * call shares it, so calls that overlap on the GPU race.  The kernels run on
 * the current device: a `stream` of another device is refused
 * (AMRS_ERR_STATE).  The first call on a device looks the array's address
 * up with that device current: make it before any stream capture.  Results
 * are identical to amrs_rhs_box. */
amrs_status amrs_rhs_box_noalloc(const amrs_scheme* scheme, const amrs_closures* closures, const amrs_box* bx,
                                 const double dxinv[3], amrs_array4 state, amrs_array4 dsdt, void* stream);

/* One RK stage of one box: RHS of the ghost-filled stage input `stage_in`
 * followed by the stage's BLAS-1 program, writing register S2 into the
 * valid cells of `out`.  `s1` holds the old state S1.  `out` must not alias
 * `stage_in` (the RHS reads neighbours of cells being written); it may
 * alias `s1`'s storage only if the program never reads S1. */
amrs_status amrs_rk_stage_box(amrs_handle* h, const amrs_box* bx, const double dxinv[3],
                              const amrs_stage_prog* prog, double dt, amrs_array4 stage_in, amrs_array4 s1,
                              amrs_array4 out, void* stream);

/* Ghost fill of a box that is the whole single-box domain: periodic images
 * and the physical BC types of src/set/CNS_setup.cpp:18-31 for cns.lo_bc /
 * cns.hi_bc codes (-1 periodic, 2 outflow/foextrap, 3/4 symmetry and slip
 * wall, 5 no-slip wall).  Ghost cells beyond codes 1 and 6 (ext_dir: the
 * problem's bcnormal fills them) are left as the caller stored them. */
amrs_status amrs_fill_halo_box(const amrs_box* domain, const int32_t bc_lo[3], const int32_t bc_hi[3],
                               amrs_array4 state, void* stream);

/* A problem bcnormal the library evaluates on the device, for y sides of
 * code 6, after its own fill (the order of AMReX's FillPatch: periodic
 * images and physical BCs first, then cns_bcfill, src/set/bcs.cpp:11-106).
 * kind 0: none (the caller's bcnormal fills those ghosts).  kind 1: the
 * channel problem's isothermal no-slip wall (exm/Channel/prob.h:158-186):
 * from the first interior cell of the ghost's column, the velocity negated,
 * the pressure kept, T = max(Tw + dratio (Tw - T_int), Tmin) with dratio the
 * ghost-to-wall over first-cell-to-wall distance computed as cns_bcfill
 * does from prob_lo, prob_hi and dx (geometry.prob_lo / prob_hi, the
 * geometry's CellSize; cell centres at prob_lo + (index + 0.5) dx), and
 * rho = p / (R T).  The channel problem uses Tmin = 50. */
typedef struct amrs_bcnormal {
  int32_t kind;
  double Tw, Tmin;
  double prob_lo[3], prob_hi[3], dx[3];
} amrs_bcnormal;
/* amrs_fill_halo_box, then the bcnormal beyond code-6 y sides. */
amrs_status amrs_fill_halo_box_bcnormal(const amrs_box* domain, const int32_t bc_lo[3], const int32_t bc_hi[3],
                                        const amrs_closures* closures, const amrs_bcnormal* bn, amrs_array4 state,
                                        void* stream);

/* cfl * min over the valid box of dx_d/(|u_d|+c): CNS::estTimeStep
 * (src/CNS.cpp:380-395, kernel cns_estdt src/cls/CNS_K.h:12-47).  Writes the
 * result to *dt_device (device pointer) without a host sync. */
amrs_status amrs_est_timestep_box(amrs_handle* h, const amrs_box* bx, const double dx[3], double cfl,
                                  amrs_array4 state, double* dt_device, void* stream);
/* The derived plot variables of the reference's plotfiles
 * (src/set/CNS_setup.cpp:153-176, written by CNS::writePlotFile,
 * src/CNS.cpp:644-874) over the valid cells of `bx`: out components 0..4 =
 * pressure (derpres), temperature (dertemp: internal energy / (rho cv)), x, y
 * and z velocity (dervel: momentum / density), in the operation order of
 * src/cls/CNS_K.h:76-129.  Runs on the current device; asynchronous on
 * `stream`. */
amrs_status amrs_plot_derive_box(const amrs_closures* closures, const amrs_box* bx, amrs_array4 state, amrs_array4 out,
                                 void* stream);
/* amrs_boxlist_prim_stats for one box's state (valid cells of `state`, the
 * same 21 doubles into `out`, device memory).  Asynchronous on `stream`. */
amrs_status amrs_prim_stats_box(amrs_handle* h, const amrs_box* bx, const double dx[3], amrs_array4 state, double dt,
                                double* out, void* stream);

/* ---- box lists: one persistent launch over many boxes ---------------- */

/* A level's box list with caller-owned state arrays per box, uploaded once.
 * states[b*nslots + s] is slot s of box b (all ghosted with 3 cells);
 * out[b] receives dSdt in amrs_rhs_boxlist.  The scratch arena grows to the
 * list's needs at creation.  Optional per-box closure index (ensembles):
 * closure_index[b] selects closures[closure_index[b]].  The list uses its
 * handle until it is destroyed: destroy every list before its handle
 * (amrs_boxlist_destroy itself reads nothing from the handle). */
typedef struct amrs_boxlist amrs_boxlist;
amrs_status amrs_boxlist_create(amrs_handle* h, int32_t nboxes, const amrs_box* boxes, const double* dxinv3,
                                int32_t nslots, const amrs_array4* states, const int32_t* closure_index,
                                int32_t nclosures, const amrs_closures* closures, amrs_boxlist** out);
amrs_status amrs_boxlist_destroy(amrs_boxlist* bl);

/* Tile shape (threads per tile = tx*ty <= 256) and z-chunk per box, as
 * chosen by the autotuner; tx must be a multiple of 8.  Applies to every
 * box whose valid extents match (nx,ny,nz) exactly; nx=ny=nz=0 sets the default. */
amrs_status amrs_boxlist_set_tile(amrs_boxlist* bl, int32_t nx, int32_t ny, int32_t nz, int32_t tx, int32_t ty,
                                  int32_t kchunk);

/* Boundary codes applied to every box of the list as its own domain
 * (ensemble members, isolated boxes): periodic wrap, foextrap or
 * reflection as in amrs_fill_halo_box.  Once set, amrs_rk_step_boxlist
 * fills each stage input's ghosts before its RHS (one launch for all boxes).
 * NULL codes switch the fill off (ghosts kept as the caller set them). */
amrs_status amrs_boxlist_set_bc(amrs_boxlist* bl, const int32_t bc_lo[3], const int32_t bc_hi[3]);
/* The boxes of the list form one level tiling (part of) `domain`:
 * single-level FillPatch as the reference's stages call it
 * (src/tim/CNS_advance.cpp:54-161 with the BC mapping of
 * src/set/CNS_setup.cpp:18-31): every ghost cell reads the domain cell
 * that periodic images or the physical boundary codes map it to, from the
 * box that owns that cell (neighbour copies inside the domain).  Results
 * equal those of one box covering the same cells.  Replaces
 * amrs_boxlist_set_bc; amrs_rk_step_boxlist and amrs_boxlist_fill_halo
 * then fill the whole level in one launch.  Boxes must be disjoint, inside
 * `domain`, and cover every cell a ghost reads (AMRS_ERR_BOX otherwise).
 * Host-synchronising (uploads the owner table). */
amrs_status amrs_boxlist_set_domain(amrs_boxlist* bl, const amrs_box* domain, const int32_t bc_lo[3],
                                    const int32_t bc_hi[3]);
/* The level fill of amrs_boxlist_set_domain followed by a device bcnormal
 * beyond the domain's code-6 y sides (amrs_bcnormal; NULL or kind 0: none),
 * for every box touching such a side, in every later fill, step graph and
 * device time loop of the list.  Host-synchronising. */
amrs_status amrs_boxlist_set_bcnormal(amrs_boxlist* bl, const amrs_bcnormal* bn);
/* Ghost fill of slot `slot` of every box with the codes of
 * amrs_boxlist_set_bc or the level of amrs_boxlist_set_domain. */
amrs_status amrs_boxlist_fill_halo(amrs_boxlist* bl, int32_t slot, void* stream);

/* Per-box tiles in one call: tiles[3*b + {0,1,2}] = (tx, ty, kchunk) of
 * box b (the autotuner's output). */
amrs_status amrs_boxlist_set_tiles(amrs_boxlist* bl, const int32_t* tiles);
/* Work distribution of the fused face kernel (no counterpart in the
 * reference, whose MFIter loop launches box by box): the (tile column x
 * plane) work of all boxes is cut into `waves` x (resident CTAs) equal shares
 * (1 <= waves <= 8; default 1).  One wave gives each CTA the longest z run
 * (the fewest z prologues); more waves give shorter runs that later CTAs
 * pick up as earlier ones finish.  The autotuner sweeps it with the tile
 * shapes.  Host-synchronising; recorded graphs of the list are re-recorded. */
amrs_status amrs_boxlist_set_schedule(amrs_boxlist* bl, int32_t waves);
/* CTAs of the list's face-kernel schedule (0 for the face-array path). */
int32_t amrs_boxlist_face_grid(amrs_boxlist* bl);
/* The list's current per-box tiles, in the layout of amrs_boxlist_set_tiles. */
amrs_status amrs_boxlist_get_tiles(amrs_boxlist* bl, int32_t* tiles);

/* RK stage over all boxes: stage input slot `in`, old state slot `s1`,
 * output slot `out` (valid cells).  One launch per kernel kind. */
amrs_status amrs_rk_stage_boxlist(amrs_boxlist* bl, const amrs_stage_prog* prog, int32_t in, int32_t s1,
                                  int32_t out, void* stream);

/* Whole RK step (all stages) over all boxes, slots rotating among
 * s1/work slots as CNS::advance does; result in slot `result`.  When
 * use_graph != 0 the step is captured once into a CUDA graph and replayed.
 * Ghost cells of the work slots are left as the caller initialised them
 * (boxes of a batched level with frozen, analytically filled ghosts). */
amrs_status amrs_rk_step_boxlist(amrs_boxlist* bl, int32_t order_rk, int32_t stages_rk, double dt, int32_t s1,
                                 int32_t w1, int32_t w2, int32_t use_graph, void* stream, int32_t* result_slot);

/* The reference's main loop (src/main.cpp:66-75 with CNS::advance and the
 * single-level dt control of src/CNS.cpp:282-377) as ONE graph launch on the
 * device, no host synchronisation: steps of (order_rk, stages_rk) from time
 * `time` while step < max_steps and time < stop_time.  cfl > 0: dt from
 * cns_estdt (computeInitialDt, then computeNewDt: growth capped at 1.1x, the
 * last step clamped to stop_time); cfl <= 0: fixed dt.  The state lives in
 * slot s1 (each step's result is copied back), w1/w2 are work slots; the
 * stage kernels read dt from device memory.  A conditional WHILE graph node
 * repeats the step body; its kernels return at once after the last step.
 * No counterpart in the reference (its loop runs on the host). */
amrs_status amrs_rk_run_boxlist(amrs_boxlist* bl, int32_t order_rk, int32_t stages_rk, double cfl, double dt,
                                double time, double stop_time, int32_t max_steps, int32_t s1, int32_t w1, int32_t w2,
                                void* stream);
/* Time, current dt and step count of the last amrs_rk_run_boxlist
 * (host-synchronising on `stream`). */
amrs_status amrs_boxlist_run_state(amrs_boxlist* bl, double* time, double* dt, int32_t* steps, void* stream);
/* Conserved totals of slot `slot` (CNS::printTotal, src/CNS.cpp:532-541:
 * sum over the valid cells of every box times `scale`, the domain volume
 * there) into totals[0..4] (device memory), one reduction on the device in
 * a fixed order (deterministic; not the rounding of a serial sum). */
amrs_status amrs_boxlist_totals(amrs_boxlist* bl, int32_t slot, double scale, double* totals, void* stream);
/* The rest of CNS::printTotal (src/CNS.cpp:543-611): the min and max of each
 * primitive and the convective CFL table of pointCFL (src/cls/CNS_K.h:49-59)
 * over the valid cells of every box.  slot >= 0: primitives of that state
 * slot (cons2prim as compute_rhs forms them); slot = -1: the list's primitive
 * scratch, i.e. the primitives of the stage input the list's last RHS read,
 * which is what the reference's Vprimsmf holds when printTotal reads it.
 * out (device memory, 21 doubles): min[6] and max[6] of (rho, u, v, w, T, p),
 * then for d = x, y, z: max |u_d + c|, max |u_d - c| and CFL_d = (the larger
 * of the two) * dt / dx_d, with c = sqrt(gamma Rspec T) from each box's
 * closures.  The reference accumulates its table in one shared array from
 * every GPU thread without synchronisation; here warps reduce and fold into
 * order-preserving integer cells with atomic min/max: extrema are exact, so
 * the result is the same on every run (-0.0 counts as +0.0).  Asynchronous on
 * `stream`. */
amrs_status amrs_boxlist_prim_stats(amrs_boxlist* bl, int32_t slot, const double dx[3], double dt, double* out,
                                    void* stream);

/* ---- adjoint ----------------------------------------------------------- */

/* Vector-Jacobian product of one RHS evaluation of one box (KEEP, WENO5
 * LLF, MUSCL-Riemann, WENO5-Riemann or no Euler flux, each with or without
 * JST dissipation and viscous fluxes; no counterpart in the reference,
 * whose lib/autodiff is absent):
 * given the ghost-filled state and a cotangent `vbar` on the valid cells,
 * writes ubar = (d dSdt/d state)^T vbar into `ubar` over the ghosted box
 * (ghost entries hold the sensitivities to ghost values).  `ubar` is
 * overwritten.  If `param_bar` (device, 2 doubles) is not NULL,
 * vbar . d dSdt/d(visc_ref) and vbar . d dSdt/d(cond_ref) are added to it
 * (constant-law closures only). */
amrs_status amrs_rhs_vjp_box(amrs_handle* h, const amrs_box* bx, const double dxinv[3], amrs_array4 state,
                             amrs_array4 vbar, amrs_array4 ubar, double* param_bar, void* stream);

/* Adjoint of amrs_fill_halo_box: every valid cell of `ubar` (ghosted, in
 * place) receives the cotangents of the ghost cells filled from it.  Ghost
 * cells beyond ext_dir sides (codes 1, 6) are not filled by the library, so
 * their cotangents are left where they are: a caller whose bcnormal filled
 * them folds them back through its own derivative first. */
amrs_status amrs_fill_halo_box_adjoint(const amrs_box* domain, const int32_t bc_lo[3], const int32_t bc_hi[3],
                                       amrs_array4 ubar, void* stream);

/* VJP of one RK stage of one box (amrs_rk_stage_box preceded by
 * amrs_fill_halo_box with bc_lo/bc_hi): given the cotangent `wbar` of the
 * stage result (valid cells), ADDS the cotangent of the old state S1 to
 * `s1bar` and the cotangent of the stage input's valid cells to `inbar`
 * (ghost sensitivities folded back through the ghost fill).  `stage_in` is
 * the ghost-filled stage input of the forward stage. */
amrs_status amrs_rk_stage_vjp_box(amrs_handle* h, const amrs_box* bx, const double dxinv[3],
                                  const amrs_stage_prog* prog, const int32_t bc_lo[3], const int32_t bc_hi[3],
                                  amrs_array4 stage_in, amrs_array4 wbar, amrs_array4 s1bar, amrs_array4 inbar,
                                  double* param_bar, void* stream);
/* The same stage VJP without the ghost fold, for domains with ext_dir sides
 * (codes 1, 6; code-6 y walls included): OVERWRITES the ghosted `ubar`
 * (grow(box,3)) with the cotangent of the ghost-filled stage input and ADDS
 * the cotangent of S1 to `s1bar`.  The caller then folds the ghost
 * cotangents beyond its ext_dir sides through its bcnormal's derivative,
 * calls amrs_fill_halo_box_adjoint for the library-filled ghosts, and takes
 * the valid cells as the stage input's cotangent (AMReX's order reversed:
 * the forward fills periodic/foextrap/reflect ghosts first, then bcnormal). */
amrs_status amrs_rk_stage_vjp_box_ghosted(amrs_handle* h, const amrs_box* bx, const double dxinv[3],
                                          const amrs_stage_prog* prog, amrs_array4 stage_in, amrs_array4 wbar,
                                          amrs_array4 s1bar, amrs_array4 ubar, double* param_bar, void* stream);

/* ---- diagnostics ---------------------------------------------------- */

/* Synchronise `stream`, then report and clear one raised device flag: the
 * flag a bounded device-side wait raises when it gives up (AMRS_ERR_TIMEOUT)
 * first, else the flag of the non-finite check (AMRS_ERR_NONFINITE).
 * Host-synchronising. */
amrs_status amrs_sync_check(amrs_handle* h, void* stream);
/* Opt-in detection of non-finite results (no counterpart in the reference,
 * whose runs carry NaNs on silently).  With on = 1, every RK stage and RHS
 * the handle runs (per-box calls, box-list steps and graphs, the device time
 * loop) ends with a check of the values it wrote over the valid cells; a
 * NaN or an infinity raises a device flag that the next amrs_sync_check
 * reports as AMRS_ERR_NONFINITE.  Costs one read of the written state per
 * stage; off (0) by default.  Box-list graphs recorded before the switch
 * changed are re-recorded on their next launch. */
amrs_status amrs_set_check_nonfinite(amrs_handle* h, int32_t on);
/* amrex::average_down for cell-centred data on a Cartesian grid, the call
 * CNS::avgDown makes after a fine level's step (src/CNS.cpp:513-530): every
 * cell of `crse_box` (coarse index space) becomes the mean of its
 * ratio[0]*ratio[1]*ratio[2] fine cells, summed from zero with the fine k
 * offset outermost and i innermost, then scaled by 1/(rx*ry*rz) (AMReX's
 * amrex_avgdown order), for components scomp..scomp+ncomp-1.  `fine` must
 * cover the refined box, `crse` the coarse box; ratios 1..16.  Asynchronous
 * on `stream`, on the current device. */
amrs_status amrs_average_down(const amrs_box* crse_box, const int32_t ratio[3], amrs_array4 fine, amrs_array4 crse,
                              int32_t scomp, int32_t ncomp, void* stream);
/* Test of the failure path of the bounded device waits: launches one thread
 * that waits on an mbarrier nothing arrives at, with the face kernel's
 * bounded wait limited to `polls` polls (1..2^20), after which it raises the
 * handle's error flag and returns; the next amrs_sync_check reports
 * AMRS_ERR_TIMEOUT (and clears the flag), and the context stays usable.
 * Asynchronous on `stream`. */
amrs_status amrs_debug_wait_timeout(amrs_handle* h, int32_t polls, void* stream);
/* FP64 FMA throughput of the device (TFLOP/s, FMA = 2 flops), measured
 * by a DFMA-chain kernel (4 CTAs x 256 threads per SM, 16 independent
 * chains per thread) over one launch of about 0.2 s: a measured
 * denominator of this FP64-bound path's roofline.  Host-synchronising. */
amrs_status amrs_probe_fp64_tflops(amrs_handle* h, double* tflops);
/* The same probe with a timed launch of about `seconds` (0.01..10); *ms
 * (may be NULL) receives the launch's duration, so that a caller sampling
 * the SM clock over it can relate the rate to the clock.
 * Host-synchronising. */
amrs_status amrs_probe_fp64_tflops_timed(amrs_handle* h, double seconds, double* tflops, double* ms);
/* Check of the library's integer-pipe FP64 division (used where the kernels
 * divide; no counterpart in the reference): `count` operand pairs generated
 * on the device from `seed` (WENO weight and normalisation ranges, arbitrary
 * bit patterns, random significands) are divided both ways; *mismatches
 * receives the number of results whose bits differ from the hardware
 * division's, first[0..3] the first such (a, b, hardware, library).
 * Host-synchronising. */
amrs_status amrs_debug_ddiv_check(amrs_handle* h, uint64_t seed, int64_t count, int64_t* mismatches, double* first);
/* The same for the library's integer-pipe FP64 square root: `count`
 * arguments (arbitrary bit patterns, positive doubles over the whole
 * exponent range, squares and their neighbours) against the hardware square
 * root; first[0] = x, first[2] = hardware, first[3] = library. */
amrs_status amrs_debug_dsqrt_check(amrs_handle* h, uint64_t seed, int64_t count, int64_t* mismatches, double* first);
/* The same for the library's integer-pipe FP64 product (used for part of the
 * products of the FP64-bound kernels): `count` operand pairs (arbitrary bit
 * patterns, random significands, short significands whose products fall on
 * rounding ties, exponents at the edges of underflow and overflow, zeros,
 * subnormals and specials, the kernels' constant factors) against the
 * hardware product; first[0..3] = (a, b, hardware, library). */
amrs_status amrs_debug_dmul_check(amrs_handle* h, uint64_t seed, int64_t count, int64_t* mismatches, double* first);
/* Overlap probe of the integer-pipe product: one launch of 2 CTAs of 256
 * threads per SM, each thread running 16 FP64 FMA chains for 8000
 * iterations plus four chains of products per iteration: none (mode 0),
 * hardware products (mode 1) or the library's integer-pipe product (mode 2).
 * *ms receives the launch's time (CUDA events, mean of three after a
 * warm-up); the difference to mode 0 is what four products per 16 FMAs cost
 * a kernel whose FP64 pipe is full (AMRS_ERR_SIZE for another mode).
 * Host-synchronising. */
amrs_status amrs_probe_intpipe(amrs_handle* h, int32_t mode, double* ms);
/* Per-kernel timing of one RK stage of one box: CUDA events around the
 * kernels on `stream`, averaged over `reps`.  ms[0] primitives (plus the
 * WENO5 point fluxes), ms[1] viscous cell fluxes, ms[2] the Euler face
 * kernel (on the fused KEEP path: faces + viscous averages + divergence +
 * stage program; on the MUSCL-Riemann path: slopes + Riemann faces), ms[3]
 * the whole stage.  Host-synchronising. */
amrs_status amrs_profile_stage_box(amrs_handle* h, const amrs_box* bx, const double dxinv[3],
                                   const amrs_stage_prog* prog, amrs_array4 stage_in, amrs_array4 s1,
                                   amrs_array4 out, int32_t reps, void* stream, double* ms);
/* 1 if the fused face kernel stages planes with TMA for the handle's last
 * per-box call (resp. for the box list), 0 if with plain loads, -1 if none. */
int32_t amrs_debug_tma_enabled(amrs_handle* h);
int32_t amrs_boxlist_tma_enabled(amrs_boxlist* bl);

#ifdef __cplusplus
}
#endif
#endif /* AMRS_GB300_H */
