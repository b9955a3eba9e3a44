// Minimal single-process, CPU-only stand-in for the AMReX types that the
// reference's RHS path uses, written for this repository's oracle build.
// It lets oracle/build_ref.sh compile the reference's own kernel headers and
// src/tim/CNS_advance.cpp unmodified.  TEST INFRASTRUCTURE ONLY.
//
// Semantics follow AMReX's public API where the reference relies on them:
// Array4 indexing, Box/IntVect algebra, MultiFab BLAS-1 (LinComb, Saxpy,
// Xpay, Copy), ParallelFor loops, max/min as std::max/std::min, and a
// single-level FillPatch (periodic images + foextrap/reflect physical BCs).
// One tile per box (tiling does not change any value these loops produce).
#pragma once
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <type_traits>
#include <iostream>
#include <limits>
#include <memory>
#include <ostream>
#include <string>
#include <utility>
#include <vector>

#define AMREX_SPACEDIM 3
#define AMREX_GPU_DEVICE
#define AMREX_GPU_HOST
#define AMREX_GPU_HOST_DEVICE
#define AMREX_FORCE_INLINE inline
#define AMREX_D_TERM(a, b, c) a b c
#define AMREX_D_DECL(a, b, c) a, b, c
#define BL_PROFILE(x)
#define BL_PROFILE_VAR(x, y)
#define BL_PROFILE_VAR_STOP(x)

namespace amrex {

using Real = double;

constexpr Real operator"" _rt(long double x) { return Real(x); }
constexpr Real operator"" _rt(unsigned long long x) { return Real(x); }

// std::max / std::min semantics, variadic as in AMReX_Algorithm.H
template <class T> constexpr const T& max(const T& a, const T& b) noexcept { return (a < b) ? b : a; }
template <class T> constexpr const T& min(const T& a, const T& b) noexcept { return (b < a) ? b : a; }
template <class T, class... Ts> constexpr const T& max(const T& a, const T& b, const Ts&... c) noexcept {
  return max(max(a, b), c...);
}
template <class T, class... Ts> constexpr const T& min(const T& a, const T& b, const Ts&... c) noexcept {
  return min(min(a, b), c...);
}

namespace Math {
template <class T> inline T abs(T x) { return std::abs(x); }
template <class T> inline T copysign(T x, T y) { return std::copysign(x, y); }
}  // namespace Math

template <class T> using Vector = std::vector<T>;
template <class T, std::size_t N> using Array = std::array<T, N>;

template <class T, int N> struct GpuArray {
  T arr[N];
  T& operator[](int i) noexcept { return arr[i]; }
  const T& operator[](int i) const noexcept { return arr[i]; }
};

struct Dim3 { int x, y, z; };

struct IntVect {
  int v[3] = {0, 0, 0};
  IntVect() = default;
  IntVect(int a, int b, int c) { v[0] = a; v[1] = b; v[2] = c; }
  int& operator[](int d) { return v[d]; }
  const int& operator[](int d) const { return v[d]; }
  static IntVect TheDimensionVector(int d) { IntVect r; r.v[d] = 1; return r; }
  static IntVect TheZeroVector() { return IntVect(); }
};

struct IndexType {
  int nodal[3] = {0, 0, 0};
  static IndexType TheCellType() { return IndexType(); }
};

struct Box {
  IntVect lo, hi;
  IndexType typ;
  Box() = default;
  Box(const IntVect& l, const IntVect& h) : lo(l), hi(h) {}
  int smallEnd(int d) const { return lo[d]; }
  int bigEnd(int d) const { return hi[d]; }
  const IntVect& smallEnd() const { return lo; }
  const IntVect& bigEnd() const { return hi; }
  const int* loVect() const { return lo.v; }
  const int* hiVect() const { return hi.v; }
  int length(int d) const { return hi[d] - lo[d] + 1; }
  long numPts() const { return (long)length(0) * length(1) * length(2); }
  bool contains(int i, int j, int k) const {
    return i >= lo[0] && i <= hi[0] && j >= lo[1] && j <= hi[1] && k >= lo[2] && k <= hi[2];
  }
};

inline Box grow(const Box& b, int n) {
  Box r = b;
  for (int d = 0; d < 3; ++d) { r.lo[d] -= n; r.hi[d] += n; }
  return r;
}
inline Box grow(const Box& b, int dir, int n) {
  Box r = b;
  r.lo[dir] -= n;
  r.hi[dir] += n;
  return r;
}
inline Box surroundingNodes(const Box& b, int dir) {
  Box r = b;
  if (!r.typ.nodal[dir]) { r.hi[dir] += 1; r.typ.nodal[dir] = 1; }
  return r;
}
inline Box surroundingNodes(const Box& b) {
  Box r = b;
  for (int d = 0; d < 3; ++d) r = surroundingNodes(r, d);
  return r;
}
inline Dim3 lbound(const Box& b) { return {b.lo[0], b.lo[1], b.lo[2]}; }
inline Dim3 ubound(const Box& b) { return {b.hi[0], b.hi[1], b.hi[2]}; }

template <class T> struct Array4 {
  T* p = nullptr;
  long jstride = 0, kstride = 0, nstride = 0;
  Dim3 begin{0, 0, 0}, end{0, 0, 0};
  int ncomp = 0;
  Array4() = default;
  Array4(T* ptr, Dim3 b, Dim3 e, int nc)
      : p(ptr), jstride(e.x - b.x), kstride((long)(e.x - b.x) * (e.y - b.y)),
        nstride((long)(e.x - b.x) * (e.y - b.y) * (e.z - b.z)), begin(b), end(e), ncomp(nc) {}
  template <class U, class = typename std::enable_if<std::is_same<const U, T>::value>::type>
  Array4(const Array4<U>& o)
      : p(o.p), jstride(o.jstride), kstride(o.kstride), nstride(o.nstride), begin(o.begin), end(o.end),
        ncomp(o.ncomp) {}
  T& operator()(int i, int j, int k) const noexcept {
    return p[(i - begin.x) + (j - begin.y) * jstride + (k - begin.z) * kstride];
  }
  T& operator()(int i, int j, int k, int n) const noexcept {
    return p[(i - begin.x) + (j - begin.y) * jstride + (k - begin.z) * kstride + n * nstride];
  }
  T& operator()(const IntVect& iv, int n) const noexcept { return (*this)(iv[0], iv[1], iv[2], n); }
};

// Fixed-size 2-D array (AMReX_Array.H), used by the CFL logging kernel.
template <class T, int XLO, int XHI, int YLO, int YHI> struct Array2D {
  T arr[(XHI - XLO + 1) * (YHI - YLO + 1)] = {};
  T& operator()(int i, int j) noexcept { return arr[(i - XLO) + (j - YLO) * (XHI - XLO + 1)]; }
};

class FArrayBox {
 public:
  Box box;
  int nc = 0;
  std::vector<Real> data;
  FArrayBox() = default;
  FArrayBox(const Box& b, int n) { resize(b, n); }
  void resize(const Box& b, int n) {
    box = b;
    nc = n;
    data.assign((size_t)b.numPts() * n, 0.0);
  }
  Array4<Real> array() {
    return Array4<Real>(data.data(), {box.lo[0], box.lo[1], box.lo[2]},
                        {box.hi[0] + 1, box.hi[1] + 1, box.hi[2] + 1}, nc);
  }
  Array4<Real> array(int comp) {
    Array4<Real> a = array();
    a.p += comp * a.nstride;
    return a;
  }
  Array4<const Real> array() const { return const_cast<FArrayBox*>(this)->array(); }
  Array4<const Real> const_array() const { return const_cast<FArrayBox*>(this)->array(); }
  struct ElixirT { void clear() {} };
  ElixirT elixir() { return ElixirT(); }
};
using Elixir = FArrayBox::ElixirT;

struct BoxArray {
  std::vector<Box> boxes;
  IndexType typ;
  BoxArray() = default;
  explicit BoxArray(const Box& b) { boxes.push_back(b); }
  int size() const { return (int)boxes.size(); }
  const Box& operator[](int i) const { return boxes[i]; }
};
inline BoxArray convert(const BoxArray& ba, const IntVect& nodal) {
  BoxArray r = ba;
  for (int d = 0; d < 3; ++d) r.typ.nodal[d] = nodal[d];
  return r;
}
struct DistributionMapping {};
struct MFInfo {};
struct FabFactoryDummy {};

class MFIter;

class MultiFab {
 public:
  BoxArray ba;
  DistributionMapping dm;
  int ncomp = 0, ngrow = 0;
  std::vector<FArrayBox> fabs;
  MultiFab() = default;
  MultiFab(const BoxArray& b, const DistributionMapping& d, int nc, int ng, MFInfo = {}, FabFactoryDummy = {}) {
    define(b, d, nc, ng);
  }
  MultiFab(const MultiFab&) = delete;
  MultiFab& operator=(const MultiFab&) = delete;
  MultiFab(MultiFab&&) = default;
  MultiFab& operator=(MultiFab&&) = default;
  void define(const BoxArray& b, const DistributionMapping& d, int nc, int ng, MFInfo = {},
              FabFactoryDummy = {}) {
    ba = b;
    dm = d;
    ncomp = nc;
    ngrow = ng;
    fabs.clear();
    for (const Box& vb : b.boxes) {
      Box fb = vb;
      for (int dd = 0; dd < 3; ++dd)
        if (b.typ.nodal[dd]) fb.hi[dd] += 1;
      fabs.emplace_back(grow(fb, ng), nc);
    }
  }
  void clear() { fabs.clear(); }
  const BoxArray& boxArray() const { return ba; }
  const DistributionMapping& DistributionMap() const { return dm; }
  int nComp() const { return ncomp; }
  int nGrow() const { return ngrow; }
  void setVal(Real v) {
    for (auto& f : fabs) std::fill(f.data.begin(), f.data.end(), v);
  }
  MultiFab& operator=(Real v) { setVal(v); return *this; }
  Array4<Real> array(const MFIter& mfi);
  Array4<Real> array(int i) { return fabs[i].array(); }
  Array4<const Real> const_array(const MFIter& mfi) const;

  // BLAS-1 over the valid region grown by nghost (AMReX semantics)
  template <class F> static void forValid(const MultiFab& m, int nghost, F&& f) {
    for (int b = 0; b < (int)m.fabs.size(); ++b) {
      Box vb = grow(m.ba.boxes[b], nghost);
      for (int k = vb.lo[2]; k <= vb.hi[2]; ++k)
        for (int j = vb.lo[1]; j <= vb.hi[1]; ++j)
          for (int i = vb.lo[0]; i <= vb.hi[0]; ++i) f(b, i, j, k);
    }
  }
  static void LinComb(MultiFab& dst, Real a, const MultiFab& x, int xcomp, Real b, const MultiFab& y, int ycomp,
                      int dstcomp, int numcomp, int nghost) {
    forValid(dst, nghost, [&](int fb, int i, int j, int k) {
      auto d = dst.fabs[fb].array();
      auto xa = const_cast<MultiFab&>(x).fabs[fb].array();
      auto ya = const_cast<MultiFab&>(y).fabs[fb].array();
      for (int n = 0; n < numcomp; ++n)
        d(i, j, k, dstcomp + n) = a * xa(i, j, k, xcomp + n) + b * ya(i, j, k, ycomp + n);
    });
  }
  static void Saxpy(MultiFab& dst, Real a, const MultiFab& src, int srccomp, int dstcomp, int numcomp, int nghost) {
    forValid(dst, nghost, [&](int fb, int i, int j, int k) {
      auto d = dst.fabs[fb].array();
      auto s = const_cast<MultiFab&>(src).fabs[fb].array();
      for (int n = 0; n < numcomp; ++n) d(i, j, k, dstcomp + n) += a * s(i, j, k, srccomp + n);
    });
  }
  static void Xpay(MultiFab& dst, Real a, const MultiFab& src, int srccomp, int dstcomp, int numcomp, int nghost) {
    forValid(dst, nghost, [&](int fb, int i, int j, int k) {
      auto d = dst.fabs[fb].array();
      auto s = const_cast<MultiFab&>(src).fabs[fb].array();
      for (int n = 0; n < numcomp; ++n)
        d(i, j, k, dstcomp + n) = s(i, j, k, srccomp + n) + a * d(i, j, k, dstcomp + n);
    });
  }
  static void Copy(MultiFab& dst, const MultiFab& src, int srccomp, int dstcomp, int numcomp, int nghost) {
    forValid(dst, nghost, [&](int fb, int i, int j, int k) {
      auto d = dst.fabs[fb].array();
      auto s = const_cast<MultiFab&>(src).fabs[fb].array();
      for (int n = 0; n < numcomp; ++n) d(i, j, k, dstcomp + n) = s(i, j, k, srccomp + n);
    });
  }
};

class MFIter {
 public:
  const MultiFab* mf;
  int idx = 0;
  MFIter(const MultiFab& m, bool /*tiling*/ = false) : mf(&m) {}
  bool isValid() const { return idx < (int)mf->fabs.size(); }
  MFIter& operator++() { ++idx; return *this; }
  int index() const { return idx; }
  Box validbox() const { return mf->ba.boxes[idx]; }
  Box tilebox() const { return validbox(); }
  Box growntilebox(int n) const { return grow(validbox(), n); }
  Box nodaltilebox(int dir = -1) const {
    return dir < 0 ? surroundingNodes(validbox()) : surroundingNodes(validbox(), dir);
  }
  Box grownnodaltilebox(int dir = -1, int ng = 0) const { return grow(nodaltilebox(dir), ng); }
};
inline Array4<Real> MultiFab::array(const MFIter& mfi) { return fabs[mfi.idx].array(); }
inline Array4<const Real> MultiFab::const_array(const MFIter& mfi) const {
  return const_cast<MultiFab*>(this)->fabs[mfi.idx].array();
}

inline bool TilingIfNotGPU() { return true; }

template <class F> inline void ParallelFor(const Box& b, F&& f) {
  for (int k = b.lo[2]; k <= b.hi[2]; ++k)
    for (int j = b.lo[1]; j <= b.hi[1]; ++j)
      for (int i = b.lo[0]; i <= b.hi[0]; ++i) f(i, j, k);
}
template <class F> inline void ParallelFor(const Box& b, int ncomp, F&& f) {
  for (int n = 0; n < ncomp; ++n)
    for (int k = b.lo[2]; k <= b.hi[2]; ++k)
      for (int j = b.lo[1]; j <= b.hi[1]; ++j)
        for (int i = b.lo[0]; i <= b.hi[0]; ++i) f(i, j, k, n);
}
template <class F> inline void ParallelFor(int n, F&& f) {
  for (int i = 0; i < n; ++i) f(i);
}

namespace Gpu {
inline void streamSynchronize() {}
inline void htod_memcpy(void* d, const void* s, std::size_t n) { std::memcpy(d, s, n); }
}  // namespace Gpu

struct BCRec {
  int l[3] = {0, 0, 0}, h[3] = {0, 0, 0};
  int lo(int d) const { return l[d]; }
  int hi(int d) const { return h[d]; }
  const int* lo() const { return l; }
  const int* hi() const { return h; }
  void setLo(int d, int v) { l[d] = v; }
  void setHi(int d, int v) { h[d] = v; }
};

namespace BCType {
enum { reflect_odd = -1, int_dir = 0, reflect_even = 1, foextrap = 2, ext_dir = 3, hoextrap = 4 };
}

struct GeometryData {
  Real plo[3], phi[3], dx[3];
  Box dom;
  const Real* ProbLo() const { return plo; }
  const Real* ProbHi() const { return phi; }
  const Real* CellSize() const { return dx; }
  const Box& Domain() const { return dom; }
};

class Geometry {
 public:
  Box dom;
  Real plo[3] = {0, 0, 0}, phi[3] = {1, 1, 1};
  Real cell[3] = {1, 1, 1}, cellinv[3] = {1, 1, 1};
  int periodic[3] = {0, 0, 0};
  GpuArray<Real, 3> CellSizeArray() const { return {{cell[0], cell[1], cell[2]}}; }
  GpuArray<Real, 3> InvCellSizeArray() const { return {{cellinv[0], cellinv[1], cellinv[2]}}; }
  const Box& Domain() const { return dom; }
  Real ProbSize() const { return (phi[0] - plo[0]) * (phi[1] - plo[1]) * (phi[2] - plo[2]); }
  bool isPeriodic(int d) const { return periodic[d] != 0; }
};

struct FluxRegister {
  void setVal(Real) {}
};

struct TagBoxArray {};
namespace VisMF { enum How { OneFilePerCPU, NFiles }; }

class AmrLevel;
class Amr {
 public:
  std::vector<AmrLevel*> levels;
  int finestLevel() const { return (int)levels.size() - 1; }
  AmrLevel& getLevel(int l) { return *levels[l]; }
};

// Time levels of one state type (AMReX StateData): old and new data with
// their times; FillPatch picks the level whose time matches.
class StateData {
 public:
  std::unique_ptr<MultiFab> old_data, new_data;
  Real old_time = 0, new_time = 0;
  void allocOldData() {
    if (!old_data) {
      old_data.reset(new MultiFab(new_data->ba, new_data->dm, new_data->ncomp, new_data->ngrow));
    }
  }
  void swapTimeLevels(Real dt) {
    old_time = new_time;
    new_time = new_time + dt;
    std::swap(old_data, new_data);
  }
  void setOldTimeLevel(Real t) { old_time = t; }
  void setNewTimeLevel(Real t) { new_time = t; }
  Real curTime() const { return new_time; }
};

void fill_level_ghosts(MultiFab& mf, const Geometry& geom, const BCRec& bc, int ng);

class AmrLevel {
 public:
  Amr* parent = nullptr;
  int level = 0;
  Geometry geom;
  BoxArray grids;
  DistributionMapping dmap;
  Vector<StateData> state;
  BCRec phys_bc_for_fill;
  virtual ~AmrLevel() {}
  MultiFab& get_old_data(int t) { return *state[t].old_data; }
  MultiFab& get_new_data(int t) { return *state[t].new_data; }
  int nStep() const { return 0; }
  FabFactoryDummy Factory() const { return {}; }

  // Single-level FillPatch: copy the time level matching `time`, then fill
  // the ghost cells (periodic images, then physical BCs).
  static void FillPatch(AmrLevel& lev, MultiFab& dst, int ng, Real time, int idx, int scomp, int ncomp,
                        int dcomp = 0) {
    StateData& sd = lev.state[idx];
    Real teps = (sd.new_time - sd.old_time) * 1.e-3;
    if (teps < 0) teps = -teps;
    MultiFab* src = nullptr;
    if (time > sd.new_time - teps - 1e-300 && time < sd.new_time + teps + 1e-300) src = sd.new_data.get();
    else if (sd.old_data && time > sd.old_time - teps - 1e-300 && time < sd.old_time + teps + 1e-300)
      src = sd.old_data.get();
    if (!src) { std::fprintf(stderr, "FillPatch: time interpolation not supported\n"); std::abort(); }
    MultiFab::Copy(dst, *src, scomp, dcomp, ncomp, 0);
    fill_level_ghosts(dst, lev.geom, lev.phys_bc_for_fill, ng);
  }

  virtual void init(AmrLevel& old) = 0;
  virtual void init() = 0;
  virtual void initData() = 0;
  virtual void post_init(Real) {}
  virtual void computeInitialDt(int, int, Vector<int>&, const Vector<IntVect>&, Vector<Real>&, Real) {}
  virtual void computeNewDt(int, int, Vector<int>&, const Vector<IntVect>&, Vector<Real>&, Vector<Real>&, Real,
                            int) {}
  virtual Real advance(Real time, Real dt, int iteration, int ncycle) = 0;
  virtual void post_timestep(int) {}
  virtual void postCoarseTimeStep(Real) {}
  virtual void post_regrid(int, int) {}
  virtual void errorEst(TagBoxArray&, int, int, Real, int = 0, int = 0) = 0;
  virtual void writePlotFile(const std::string&, std::ostream&, VisMF::How = VisMF::NFiles) {}
  virtual void writePlotFilePost(const std::string&, std::ostream&) {}
};

struct PrintT {
  PrintT& SetPrecision(int) { return *this; }
  template <class T> PrintT& operator<<(const T&) { return *this; }
  PrintT& operator<<(std::ostream& (*)(std::ostream&)) { return *this; }
};
inline PrintT Print() { return PrintT(); }
[[noreturn]] inline void Abort(const char* msg = "") {
  std::fprintf(stderr, "amrex::Abort: %s\n", msg);
  std::abort();
}
inline Real second() { return 0.0; }

class ParmParse {
 public:
  explicit ParmParse(const std::string& = "") {}
  template <class T> void add(const char*, const T&) {}
  template <class T> void addarr(const char*, const T&) {}
  template <class T> bool query(const char*, T&) { return false; }
};

}  // namespace amrex
