// amrs_rhs_box_noalloc: the KEEP + viscous RHS of one box without any
// device allocation.
//
// Some callers cannot call cudaMalloc: a host that owns all device memory
// through its own arena or pool (AMReX's The_Arena, PyTorch's caching
// allocator) and forbids allocations behind the pool's back, or one that
// reserves a fixed device-memory budget up front.  For them this entry point
// keeps the scratch that amrs_rhs_box takes from its handle (primitive and
// viscous-flux fields, the box table and the face-kernel schedule) in one
// fixed static device array, and needs no handle.
//
// Limits and sharing rules:
//  * boxes of at most 32 cells in every direction (the array holds
//    NQ x 38^3 + 12 x 34^3 doubles plus a 64 KiB table region, 6.9 MB);
//    larger boxes return AMRS_ERR_SIZE;
//  * the array exists once per device that loads the library and stays
//    allocated until the process exits;
//  * every call on a device uses the same array and leaves its contents
//    behind; calls that overlap on the GPU (different streams, or
//    concurrent host threads) race on it;
//  * the first call on a device looks the array's device address up
//    (cudaGetSymbolAddress) with that device current; make that first call
//    before any stream capture.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>

#include "../../include/amrs_gb300.h"
#include "amrs_kernels.h"

using namespace amrs;

namespace {

constexpr int NA_MAX_EDGE = 32;
constexpr size_t NA_Q = (size_t)NQ * (NA_MAX_EDGE + 6) * (NA_MAX_EDGE + 6) * (NA_MAX_EDGE + 6);
constexpr size_t NA_VF = (size_t)NVF * (NA_MAX_EDGE + 2) * (NA_MAX_EDGE + 2) * (NA_MAX_EDGE + 2);
constexpr size_t NA_TABLE_BYTES = 64 * 1024;
constexpr size_t NA_DOUBLES = NA_Q + NA_VF + NA_TABLE_BYTES / 8;

}  // namespace

// The scratch array.  In host code this name is only a host-side stand-in:
// its device address comes from cudaGetSymbolAddress below.
static __device__ __align__(256) double g_noalloc_scratch[NA_DOUBLES];

namespace {

std::mutex g_na_mu;
// host staging of the table region and of the schedule (no heap use)
constexpr int NA_MAX_SEGS = 2048;
alignas(128) char g_na_host[NA_TABLE_BYTES];
int4 g_na_segs[NA_MAX_SEGS];
int g_na_cta[NA_MAX_SEGS + 1];
constexpr int NA_MAX_DEVICES = 64;
double* g_na_ptr[NA_MAX_DEVICES] = {nullptr};
int g_na_nsm[NA_MAX_DEVICES] = {0};

amrs_status na_fail(cudaError_t) { return AMRS_ERR_CUDA; }

// Device address of the scratch array on the current device (looked up once
// per device, with that device current).
amrs_status na_setup(int dev, double** ptr, int* nsm) {
  if (dev < 0 || dev >= NA_MAX_DEVICES) return AMRS_ERR_SIZE;
  if (!g_na_ptr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) return na_fail(e);
    int n = 0;
    e = cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return na_fail(e);
    g_na_ptr[dev] = static_cast<double*>(p);
    g_na_nsm[dev] = n;
  }
  *ptr = g_na_ptr[dev];
  *nsm = g_na_nsm[dev];
  return AMRS_OK;
}

DArr na_view(double* p, const amrs_box& b, int g) {
  DArr a;
  a.p = p;
  const int nx = b.hi[0] - b.lo[0] + 1 + 2 * g, ny = b.hi[1] - b.lo[1] + 1 + 2 * g, nz = b.hi[2] - b.lo[2] + 1 + 2 * g;
  a.js = nx;
  a.ks = (long long)nx * ny;
  a.ns = (long long)nx * ny * nz;
  a.b0 = b.lo[0] - g;
  a.b1 = b.lo[1] - g;
  a.b2 = b.lo[2] - g;
  return a;
}

DArr na_user(const amrs_array4& a) {
  DArr d;
  d.p = a.p; d.js = a.jstride; d.ks = a.kstride; d.ns = a.nstride;
  d.b0 = a.begin[0]; d.b1 = a.begin[1]; d.b2 = a.begin[2];
  return d;
}

bool na_covers(const amrs_array4& a, const amrs_box& b, int g) {
  if (!a.p || a.ncomp < NCONS) return false;
  for (int d = 0; d < 3; ++d)
    if (a.begin[d] > b.lo[d] - g || a.end[d] < b.hi[d] + g + 1) return false;
  const long long nx = a.end[0] - a.begin[0], ny = a.end[1] - a.begin[1], nz = a.end[2] - a.begin[2];
  return a.jstride >= nx && a.kstride >= a.jstride * ny && a.nstride >= a.kstride * nz;
}

size_t al(size_t x) { return (x + 127) / 128 * 128; }

}  // namespace

extern "C" amrs_status amrs_rhs_box_noalloc(const amrs_scheme* scheme, const amrs_closures* closures,
                                            const amrs_box* bx, const double dxinv[3], amrs_array4 state,
                                            amrs_array4 dsdt, void* stream) {
  if (!scheme || !closures || !bx || !dxinv) return AMRS_ERR_NULL;
  const amrs_scheme& sc = *scheme;
  // the switches amrs_create accepts, restricted to the fused KEEP path
  if (!(sc.rhs_euler == 1 && sc.flux_euler == 1 && sc.art_diss == 0 && (sc.weno_fast == 0 || sc.weno_fast == 1) &&
        (sc.riemann_weno == 0 || sc.riemann_weno == 1) && (sc.rhs_visc == 0 || sc.rhs_visc == 1) &&
        (sc.order_keep == 2 || sc.order_keep == 4 || sc.order_keep == 6)))
    return AMRS_ERR_SCHEME;
  // transport laws: 0 constant, 1 Sutherland (src/cls/Closures.h:103-166)
  if ((closures->visc_law != 0 && closures->visc_law != 1) || (closures->cond_law != 0 && closures->cond_law != 1))
    return AMRS_ERR_SCHEME;
  for (int d = 0; d < 3; ++d)
    if (!(dxinv[d] > 0.0) || !std::isfinite(dxinv[d])) return AMRS_ERR_BOX;
  int n[3];
  for (int d = 0; d < 3; ++d) {
    n[d] = bx->hi[d] - bx->lo[d] + 1;
    if (n[d] < 1) return AMRS_ERR_BOX;
    if (n[d] > NA_MAX_EDGE) return AMRS_ERR_SIZE;
  }
  if (!na_covers(state, *bx, NGHOST) || !na_covers(dsdt, *bx, 0)) return AMRS_ERR_LAYOUT;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  std::lock_guard<std::mutex> lk(g_na_mu);
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return AMRS_ERR_CUDA;
  // the scratch address below belongs to the current device: a stream of
  // another device would run the kernels against the wrong array
  if (st) {
    int sdev = -1;
    if (cudaStreamGetDevice(st, &sdev) != cudaSuccess) return AMRS_ERR_CUDA;
    if (sdev != dev) return AMRS_ERR_STATE;
  }
  double* base = nullptr;
  int nsm = 0;
  if (amrs_status s = na_setup(dev, &base, &nsm)) return s;

  // scratch fields inside the static array
  double* qp = base;
  double* vfp = base + NA_Q;
  char* tab = reinterpret_cast<char*>(base + NA_Q + NA_VF);
  const int order = sc.order_keep;

  // box record, tile and balanced schedule (as the handle path builds them)
  BoxRec R{};
  for (int d = 0; d < 3; ++d) {
    R.lo[d] = bx->lo[d];
    R.hi[d] = bx->hi[d];
    R.dxinv[d] = dxinv[d];
    R.dx[d] = 1.0 / dxinv[d];
  }
  R.slot[0] = na_user(state);
  R.slot[1] = na_user(state);
  R.slot[2] = na_user(dsdt);
  R.q = na_view(qp, *bx, 3);
  R.vf = na_view(vfp, *bx, 1);
  R.cl = 0;
  int tx = 32, ty = 8;
  if (!keep_tile_fits(order, tx, ty)) { tx = 16; ty = 8; }
  if (n[0] <= 16 && keep_tile_fits(order, 16, 16)) { tx = 16; ty = 16; }
  if (n[0] <= 8 && keep_tile_fits(order, 8, 30)) { tx = 8; ty = 30; }
  R.tx = tx; R.ty = ty; R.kc = n[2];
  R.ntx = (n[0] + tx - 1) / tx; R.nty = (n[1] + ty - 1) / ty; R.nkz = 1;
  const int ncol = R.ntx * R.nty;
  const long long G = std::min<long long>((long long)keep_ctas_per_sm(order) * nsm, (long long)ncol * n[2]);
  int nseg = 0, ncs = 0;
  int4* segs = g_na_segs;
  int* cta_seg = g_na_cta;
  if (G + 1 > NA_MAX_SEGS) return AMRS_ERR_SIZE;
  {
    double total = 0.0;
    for (int c = 0; c < ncol; ++c) {
      const int txw = std::min(tx, n[0] - (c % R.ntx) * tx), tyw = std::min(ty, n[1] - (c / R.ntx) * ty);
      total += (double)txw * tyw * n[2];
    }
    const double per = total / (double)G;
    int cta = 0;
    double acc = 0.0;
    cta_seg[ncs++] = 0;
    for (int c = 0; c < ncol; ++c) {
      const int txw = std::min(tx, n[0] - (c % R.ntx) * tx), tyw = std::min(ty, n[1] - (c / R.ntx) * ty);
      const double w = (double)txw * tyw;
      int k = R.lo[2];
      while (k <= R.hi[2]) {
        if (nseg >= NA_MAX_SEGS) return AMRS_ERR_SIZE;
        const double boundary = (cta + 1) * per;
        long long fit = (long long)((boundary - acc) / w + 0.5);
        if (fit < 1) fit = 1;
        const int kend = (int)std::min<long long>(R.hi[2] + 1, k + fit);
        segs[nseg++] = make_int4(0, c, k, kend);
        acc += (kend - k) * w;
        k = kend;
        if (acc >= boundary - 0.5 * w && cta < G - 1) {
          ++cta;
          cta_seg[ncs++] = nseg;
        }
      }
    }
    while (ncs < G + 1) cta_seg[ncs++] = nseg;
    cta_seg[G] = nseg;
  }
  const int gq = std::max(order / 2, 2);
  long long pcell[2] = {0, (long long)(n[0] + 2 * gq) * (n[1] + 2 * gq) * (n[2] + 2 * gq)};
  long long vcell[2] = {0, (long long)(n[0] + 2) * (n[1] + 2) * (n[2] + 2)};
  int fwork[2] = {0, 0};
  DClosures cl;
  cl.gamma = closures->gamma; cl.cv = closures->cv; cl.cp = closures->cp; cl.Rspec = closures->Rspec;
  cl.visc_law = closures->visc_law; cl.cond_law = closures->cond_law;
  cl.visc_ref = closures->visc_ref; cl.Tvisc_ref = closures->Tvisc_ref;
  cl.cond_ref = closures->cond_ref; cl.Tcond_ref = closures->Tcond_ref;
  cl.Cshock = closures->Cshock; cl.Cdamp = closures->Cdamp;
  cl.source = 0;  // no source term on this path
  cl.force[0] = cl.force[1] = cl.force[2] = 0.0;

  // table region layout: box | closures | pcell | vcell | fwork | err | segs | cta_seg
  size_t t = 0;
  const size_t o_box = t; t = al(t + sizeof(BoxRec));
  const size_t o_cl = t; t = al(t + sizeof(DClosures));
  const size_t o_p = t; t = al(t + sizeof(pcell));
  const size_t o_v = t; t = al(t + sizeof(vcell));
  const size_t o_w = t; t = al(t + sizeof(fwork));
  const size_t o_err = t; t = al(t + sizeof(int));
  const size_t o_seg = t; t = al(t + sizeof(int4) * nseg);
  const size_t o_cs = t; t = al(t + sizeof(int) * ncs);
  if (t > NA_TABLE_BYTES) return AMRS_ERR_SIZE;
  char* host = g_na_host;
  std::memset(host, 0, t);
  std::memcpy(&host[o_box], &R, sizeof(BoxRec));
  std::memcpy(&host[o_cl], &cl, sizeof(DClosures));
  std::memcpy(&host[o_p], pcell, sizeof(pcell));
  std::memcpy(&host[o_v], vcell, sizeof(vcell));
  std::memcpy(&host[o_w], fwork, sizeof(fwork));
  std::memcpy(&host[o_seg], segs, sizeof(int4) * nseg);
  std::memcpy(&host[o_cs], cta_seg, sizeof(int) * ncs);
  // The copy also clears the error flag, which must start at zero.  From
  // pageable host memory it waits for the stream's earlier work and returns
  // once the staging is consumed, so the static host buffer can be reused.
  if (cudaMemcpyAsync(tab, host, t, cudaMemcpyHostToDevice, st) != cudaSuccess) return AMRS_ERR_CUDA;
  BoxTable tb{};  // every field defined: tb.active stays null (no device time loop here)
  tb.active = nullptr;
  tb.box = reinterpret_cast<const BoxRec*>(tab + o_box);
  tb.pcell = reinterpret_cast<const long long*>(tab + o_p);
  tb.vcell = reinterpret_cast<const long long*>(tab + o_v);
  tb.fwork = reinterpret_cast<const int*>(tab + o_w);
  tb.seg = reinterpret_cast<const int4*>(tab + o_seg);
  tb.cta_seg = reinterpret_cast<const int*>(tab + o_cs);
  tb.cls = reinterpret_cast<const DClosures*>(tab + o_cl);
  tb.n = 1;
  tb.gq = gq;
  TmaDesc tma{};
  tma.maps = nullptr;
  tma.enabled = 0;
  DProg prog{};
  // The face kernel takes a flag word that only its TMA staging's bounded
  // waits write; this path stages with plain loads (tma.enabled = 0), so
  // nothing can raise it and there is nothing to read back.
  int* err = reinterpret_cast<int*>(tab + o_err);
  if (launch_prims(tb, 0, pcell[1], nsm, st) != cudaSuccess) return AMRS_ERR_CUDA;
  if (sc.rhs_visc && launch_visc(tb, vcell[1], nsm, st) != cudaSuccess) return AMRS_ERR_CUDA;
  if (launch_keep_face(order, sc.rhs_visc != 0, false, tb, 0, 1, 2, prog, 1, tma, err, (int)G, nsm, st) != cudaSuccess)
    return AMRS_ERR_CUDA;
  return AMRS_OK;
}
