// Device box table shared by every launch: one record per box of a level
// (a single-box list for the per-box entry points).
#pragma once
#include "amrs_device.cuh"

namespace amrs {

constexpr int MAX_SLOTS = 4;
constexpr int F_THREADS = 256;  // threads per CTA of the face/divergence kernel

struct BoxRec {
  int lo[3], hi[3];
  double dxinv[3];
  double dx[3];
  DArr slot[MAX_SLOTS];  // caller-owned ghosted state arrays (3 ghosts)
  DArr q;                // primitives scratch over grow(box,3), NQ comps
  DArr vf;               // viscous cell fluxes over grow(box,1), NVF comps
  int cl;                // closure index
  int tx, ty, kc;        // tile shape and z chunk of the face kernel
  int ntx, nty, nkz;     // tiles per direction
  // y walls of boundary code 6 that this box touches (walls == 0: none):
  // viscous cell fluxes of rows wrow_lo / wrow_hi use one-sided y
  // derivatives (ViscousWallFluxes); KEEP y faces j <= red_lo or
  // red_hi <= j <= hi[1] take the second-order pair (Flux_2nd_Order_KEEP)
  int walls;
  int wrow_lo, wrow_hi;
  int red_lo, red_hi;
};

// Prefix tables for flattening launches over boxes.
struct BoxTable {
  const BoxRec* box;
  const long long* pcell;  // prefix of primitive-region cells, size n+1
  const long long* vcell;  // prefix of viscous-region cells, size n+1
  const int* fwork;        // prefix of face-kernel work items, size n+1 (unused by the balanced schedule)
  const int4* seg;         // face-kernel segments: (box, tile index, k0, k1)
  const int* cta_seg;      // segments of CTA c: [cta_seg[c], cta_seg[c+1])
  const DClosures* cls;
  int n;
  int gq;                  // ghost depth of the primitive region
  // device-resident time loop: every kernel of a step returns at once while
  // *active == 0 (steps after the stop time); null outside such loops
  const int* active;
};

__device__ __forceinline__ bool list_idle(const BoxTable& tb) { return tb.active && *tb.active == 0; }

__device__ __forceinline__ int find_box_ll(const long long* pref, int n, long long x) {
  int lo = 0, hi = n;  // pref[lo] <= x < pref[hi]
  while (hi - lo > 1) {
    int mid = (lo + hi) >> 1;
    if (pref[mid] <= x) lo = mid; else hi = mid;
  }
  return lo;
}
__device__ __forceinline__ int find_box_i(const int* pref, int n, int x) {
  int lo = 0, hi = n;
  while (hi - lo > 1) {
    int mid = (lo + hi) >> 1;
    if (pref[mid] <= x) lo = mid; else hi = mid;
  }
  return lo;
}

}  // namespace amrs
