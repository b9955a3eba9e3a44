// Problem plugin for the oracle build of the reference sources (test
// infrastructure only).  The reference selects its closures and index
// macros at compile time through a prob.h (exm/*/prob.h); this one uses the
// reference's own closure classes from src/cls/Closures.h, chosen by the
// REF_VISC / REF_COND macros given by oracle/build_ref.sh, and the same
// component numbering as the reference examples.
#ifndef CNS_PROB_H_
#define CNS_PROB_H_

#include <AMReX_FArrayBox.H>
#include <AMReX_Geometry.H>
#include <AMReX_ParmParse.H>
#include <Closures.h>

using namespace amrex;

namespace PROB {

#define URHO 0
#define UMX 1
#define UMY 2
#define UMZ 3
#define UET 4
#define NCONS 5

#define QRHO 0
#define QU 1
#define QV 2
#define QW 3
#define QT 4
#define QPRES 5
#define NPRIM 6

#define NGHOST 3

#ifndef REF_VISC
#define REF_VISC visc_suth_t
#endif
#ifndef REF_COND
#define REF_COND cond_suth_t
#endif

inline void inputs() {}

typedef closures_derived_t<REF_VISC, REF_COND, calorifically_perfect_gas_t> ProbClosures;

struct ProbParm {
  Real force[3] = {0.0, 0.0, 0.0};  // body force per unit mass (user_source)
};

AMREX_GPU_DEVICE AMREX_FORCE_INLINE void bcnormal(const Real*, Real, const Real*, const Real*, Real*, const int,
                                                  const int, const Real, GeometryData const&, ProbClosures const&,
                                                  ProbParm const&) {
  Abort("bcnormal not available in the oracle build");
}

// A body force per unit mass, as the channel problem's user_source applies
// its x force (exm/Channel/prob.h:189-193), for each direction with a
// nonzero component.
AMREX_GPU_DEVICE AMREX_FORCE_INLINE void user_source(int i, int j, int k, const auto& state, const auto& rhs,
                                                     const ProbParm& pp, ProbClosures const&, auto const) {
  for (int d = 0; d < 3; ++d) {
    if (pp.force[d] == 0.0) continue;
    rhs(i, j, k, UMX + d) += state(i, j, k, URHO) * pp.force[d];
    rhs(i, j, k, UET) += state(i, j, k, UMX + d) * pp.force[d];
  }
}

}  // namespace PROB
#endif
