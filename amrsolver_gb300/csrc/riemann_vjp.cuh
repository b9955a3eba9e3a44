// Reverse of the two-shock approximate Riemann solver riemann_prob
// (src/rhs/Riemann.h:123-249), host- and device-callable so that it can be
// checked on the CPU against the oracle's dual numbers.  Non-smooth points
// follow the forward's branch (max, |.|, the state selection); the
// weak-wave switch of the iteration carries no derivative.
#pragma once
#include <cmath>

#include "ddiv.cuh"

#if defined(__CUDACC__)
#define AMRS_HD __host__ __device__ __forceinline__
#else
#define AMRS_HD inline
#endif

namespace amrs {
namespace rpvjp {

using std::copysign;
using std::fabs;
using std::sqrt;

AMRS_HD double sgn1(double x) { return x < 0.0 ? -1.0 : 1.0; }  // d|x|/dx as fabs's branch

// Square roots of the reverse solver: integer-pipe (dsqrt_rn) or hardware,
// the same correctly rounded value.
#ifndef AMRS_RV_ISQRT
#define AMRS_RV_ISQRT 0
#endif
AMRS_HD double rvsqrt(double x) { return AMRS_RV_ISQRT ? dsqrt_rn(x) : sqrt(x); }

// One iteration of riemann_prob's pressure update (src/rhs/Riemann.h:163-189)
// and its reverse.  State (P = pstar, Pm = pstnm1, UM = ustarm, UP = ustarp).
struct RPPar {
  double pl, pr, ul, ur, rl, rr, hg, cleft, cright, ccs, smallp;
};

AMRS_HD void rp_iter_fwd(const RPPar& q, double P, double Pm, double UM, double UP, double& Pn,
                                            double& UMn, double& UPn) {
  const double wl = ddiv_rn(1., rvsqrt((q.hg * (P + q.pl) + P) * q.rl));
  const double wr = ddiv_rn(1., rvsqrt((q.hg * (P + q.pr) + P) * q.rr));
  UMn = q.ur - (q.pr - P) * wr;
  UPn = q.ul + (q.pl - P) * wl;
  const double dpd = fabs(Pm - P);
  double zp = fabs(UPn - UP);
  if (zp - 1.e-3 * q.cleft < 0.0) zp = dpd * wl;
  double zm = fabs(UMn - UM);
  if (zm - 1.e-3 * q.cright < 0.0) zm = dpd * wr;
  const double zz = zp + zm;
  const double denom = ddiv_rn(dpd, ((zz < q.ccs) ? q.ccs : zz));
  const double pn = P - denom * (UMn - UPn);
  Pn = (pn < q.smallp) ? q.smallp : pn;
}

// Given the cotangents of the iteration's outputs (Pn, Pm' = P, UMn, UPn),
// add the cotangents of its inputs and of the parameters.
struct RPBar {
  double pl, pr, ul, ur, rl, rr, ccs;
};
AMRS_HD void rp_iter_vjp(const RPPar& q, double P, double Pm, double UM, double UP, double Pnb,
                                            double Pmnb, double UMnb, double UPnb, double& Pb, double& Pmb,
                                            double& UMb, double& UPb, RPBar& g) {
  const double al = q.hg * (P + q.pl) + P, ar = q.hg * (P + q.pr) + P;
  const double sl = rvsqrt(al * q.rl), sr = rvsqrt(ar * q.rr);
  const double wl = ddiv_rn(1., sl), wr = ddiv_rn(1., sr);
  const double UMn = q.ur - (q.pr - P) * wr;
  const double UPn = q.ul + (q.pl - P) * wl;
  const double draw = Pm - P, dpd = fabs(draw);
  const double zpr = UPn - UP, zp0 = fabs(zpr);
  const bool bp = zp0 - 1.e-3 * q.cleft < 0.0;
  const double zp = bp ? dpd * wl : zp0;
  const double zmr = UMn - UM, zm0 = fabs(zmr);
  const bool bm = zm0 - 1.e-3 * q.cright < 0.0;
  const double zm = bm ? dpd * wr : zm0;
  const double zz = zp + zm;
  const bool bz = zz < q.ccs;
  const double den = bz ? q.ccs : zz;
  const double denom = ddiv_rn(dpd, den);
  const double pn = P - denom * (UMn - UPn);
  const bool bpn = pn < q.smallp;
  // reverse
  double Pbar = Pmnb;  // P is also the next pstnm1
  double UMnbar = UMnb, UPnbar = UPnb, wlb = 0.0, wrb = 0.0, dpdb = 0.0;
  const double pnb = bpn ? 0.0 : Pnb;
  Pbar += pnb;
  const double denomb = -pnb * (UMn - UPn);
  UMnbar += -pnb * denom;
  UPnbar += pnb * denom;
  const double iden = ddiv_rn(1.0, den);
  dpdb += denomb * iden;
  const double denb = -denomb * denom * iden;
  if (bz) g.ccs += denb;
  const double zzb = bz ? 0.0 : denb;
  if (bp) { dpdb += zzb * wl; wlb += zzb * dpd; }
  else { const double t = zzb * sgn1(zpr); UPnbar += t; UPb += -t; }
  if (bm) { dpdb += zzb * wr; wrb += zzb * dpd; }
  else { const double t = zzb * sgn1(zmr); UMnbar += t; UMb += -t; }
  const double drb = dpdb * sgn1(draw);
  Pmb += drb;
  Pbar -= drb;
  // UMn = ur - (pr - P) wr;  UPn = ul + (pl - P) wl
  g.ur += UMnbar;
  g.pr += -UMnbar * wr;
  Pbar += UMnbar * wr;
  wrb += -UMnbar * (q.pr - P);
  g.ul += UPnbar;
  g.pl += UPnbar * wl;
  Pbar -= UPnbar * wl;
  wlb += UPnbar * (q.pl - P);
  // w = 1/rvsqrt(a r), a = hg (P + p) + P; d sqrt(x)/dx = 1/(2 sqrt(x)) = w/2
  const double slb = -wlb * wl * wl, srb = -wrb * wr * wr;
  const double wlsqb = 0.5 * slb * wl, wrsqb = 0.5 * srb * wr;
  g.rl += wlsqb * al;
  g.rr += wrsqb * ar;
  const double alb = wlsqb * q.rl, arb = wrsqb * q.rr;
  Pbar += alb * (q.hg + 1.0) + arb * (q.hg + 1.0);
  g.pl += alb * q.hg;
  g.pr += arb * q.hg;
  Pb += Pbar;
}

// Reverse of riemann_prob (src/rhs/Riemann.h:123-249): in = (rl, ul, pl,
// ut1l, ut2l, rr, ur, pr, ut1r, ut2r), fb = cotangents of (flxrho, flxu,
// flxut, flxutt, flxe); ib receives the cotangents of in.
AMRS_HD void riemann_prob_vjp(const double gamma, const double smallp, const double in[10], const double fb[5],
                                 double ib[10]) {
  const double rl = in[0], ul = in[1], pl = in[2], ut1l = in[3], ut2l = in[4];
  const double rr = in[5], ur = in[6], pr = in[7], ut1r = in[8], ut2r = in[9];
  const double small = 1.e-6;
  const double hg = 0.5 * (gamma - 1.);
  // ---- forward
  const double clsql = gamma * pl * rl, clsqr = gamma * pr * rr;
  const double wl0 = rvsqrt(clsql), wr0 = rvsqrt(clsqr);
  const double cleft = ddiv_rn(wl0, rl), cright = ddiv_rn(wr0, rr);
  const double ccs = small * (cleft + cright);
  const double dU = ur - ul;
  const double D0 = wl0 + wr0;
  const double ps0 = ddiv_rn((wl0 * pr + wr0 * pl - wr0 * wl0 * dU), D0);
  const bool m0 = !(ps0 < smallp);
  const double p0 = m0 ? ps0 : smallp;
  const double a1l = hg * (p0 + pl) + p0, a1r = hg * (p0 + pr) + p0;
  const double wl1 = rvsqrt(a1l * rl), wr1 = rvsqrt(a1r * rr);
  const double usp0 = ul - ddiv_rn((p0 - pl), wl1);
  const double usm0 = ur + ddiv_rn((p0 - pr), wr1);
  const double D1 = wl1 + wr1;
  const double ps1 = ddiv_rn((wl1 * pr + wr1 * pl - wr1 * wl1 * dU), D1);
  const bool m1 = !(ps1 < smallp);
  const double p1 = m1 ? ps1 : smallp;
  const RPPar q{pl, pr, ul, ur, rl, rr, hg, cleft, cright, ccs, smallp};
  double P[4], Pm[4], UM[4], UP[4];
  P[0] = p1; Pm[0] = p0; UM[0] = usm0; UP[0] = usp0;
#pragma unroll
  for (int it = 0; it < 3; ++it) {
    rp_iter_fwd(q, P[it], Pm[it], UM[it], UP[it], P[it + 1], UM[it + 1], UP[it + 1]);
    Pm[it + 1] = P[it];
  }
  const double pstar = P[3], ustar = 0.5 * (UM[3] + UP[3]);
  // state selection by the sign of u*
  const int side = (ustar > 0.) ? 0 : ((ustar < 0.) ? 1 : 2);
  double ro, uo, po, sgnm, utr1, utr2;
  if (side == 0) { ro = rl; uo = ul; po = pl; sgnm = 1.; utr1 = ut1l; utr2 = ut2l; }
  else if (side == 1) { ro = rr; uo = ur; po = pr; sgnm = -1.; utr1 = ut1r; utr2 = ut2r; }
  else {
    uo = 0.5 * (ur + ul); po = 0.5 * (pr + pl); ro = ddiv_rn(2. * (rl * rr), (rl + rr)); sgnm = 1.;
    utr1 = 0.5 * (ut1l + ut1r); utr2 = 0.5 * (ut2l + ut2r);
  }
  const double aw = hg * (pstar + po) + pstar;
  const double wosq = aw * ro;
  const double dpjmp = pstar - po;
  const double tt = ro * dpjmp, uu = ddiv_rn(tt, wosq), dd = 1. - uu;
  const double rstar = ddiv_rn(ro, dd);
  const double suo = sgnm * uo;
  // kind: 0 side state, 1 star state, 2 mixed (rarefaction fan)
  int kind;
  double spin = 0.0, spout = 0.0, co = 0.0, cstar = 0.0;
  if (pstar >= po) {
    spin = ddiv_rn(rvsqrt(wosq), ro) - suo;
    kind = (spin < 0.) ? 0 : ((spin >= 0.) ? 1 : 2);
    spout = spin;
  } else {
    co = rvsqrt(ddiv_rn(gamma * po, ro));
    cstar = rvsqrt(ddiv_rn(gamma * pstar, rstar));
    spout = co - suo;
    spin = cstar - suo;
    kind = (spout < 0.) ? 0 : ((spin >= 0.) ? 1 : 2);
  }
  double frac = 0.0, ssv = 0.0, den2 = 0.0;
  bool bss = false, bab = false;
  if (kind == 2) {
    const double a = spout - spin, b = spout + spin;
    bab = a < b;
    ssv = bab ? b : a;
    bss = ssv < ccs;
    den2 = bss ? ccs : ssv;
    frac = 0.5 * (1. + ddiv_rn((spin + spout), den2));
  }
  double rg, ug, pg;
  if (kind == 0) { rg = ro; ug = uo; pg = po; }
  else if (kind == 1) { rg = rstar; ug = ustar; pg = pstar; }
  else {
    rg = frac * rstar + (1. - frac) * ro;
    ug = frac * ustar + (1. - frac) * uo;
    pg = frac * pstar + (1. - frac) * po;
  }
  // ---- reverse of the fluxes
  const double K = ug * ug + utr1 * utr1 + utr2 * utr2;
  const double E = 0.5 * rg * K + ddiv_rn(pg, (gamma - 1.)) + pg;
  double rgb = fb[0] * ug + fb[1] * ug * ug + fb[2] * ug * utr1 + fb[3] * ug * utr2 + fb[4] * ug * 0.5 * K;
  double ugb = fb[0] * rg + fb[1] * 2.0 * rg * ug + fb[2] * rg * utr1 + fb[3] * rg * utr2 +
               fb[4] * (E + ug * rg * ug);
  double t1b = fb[2] * rg * ug + fb[4] * ug * rg * utr1;
  double t2b = fb[3] * rg * ug + fb[4] * ug * rg * utr2;
  double pgb = fb[1] + fb[4] * ug * (ddiv_rn(1.0, (gamma - 1.)) + 1.0);
  // ---- reverse of the selection
  double rob = 0.0, uob = 0.0, pob = 0.0, rstarb = 0.0, ustarb = 0.0, pstarb = 0.0, ccsb = 0.0;
  if (kind == 0) { rob += rgb; uob += ugb; pob += pgb; }
  else if (kind == 1) { rstarb += rgb; ustarb += ugb; pstarb += pgb; }
  else {
    rstarb += frac * rgb; rob += (1. - frac) * rgb;
    ustarb += frac * ugb; uob += (1. - frac) * ugb;
    pstarb += frac * pgb; pob += (1. - frac) * pgb;
    const double fracb = rgb * (rstar - ro) + ugb * (ustar - uo) + pgb * (pstar - po);
    const double iden2 = ddiv_rn(1.0, den2);
    const double qb = 0.5 * fracb * iden2;
    const double den2b = -0.5 * fracb * (spin + spout) * iden2 * iden2;
    double ab = 0.0, bb = 0.0;
    if (bss) ccsb += den2b;
    else if (bab) bb += den2b;
    else ab += den2b;
    const double spoutb = ab + bb + qb, spinb = -ab + bb + qb;
    if (pstar >= po) {
      // only reached with a NaN speed: the derivative is not defined there
    } else {
      const double cob = spoutb, cstarb = spinb;
      const double suob = -spoutb - spinb;
      uob += suob * sgnm;
      const double iro = ddiv_rn(1.0, ro), irst = ddiv_rn(1.0, rstar);
      const double xb = ddiv_rn(cob, (2.0 * co));
      pob += xb * gamma * iro;
      rob += -xb * gamma * po * iro * iro;
      const double yb = ddiv_rn(cstarb, (2.0 * cstar));
      pstarb += yb * gamma * irst;
      rstarb += -yb * gamma * pstar * irst * irst;
    }
  }
  // rstar = ro / (1 - ro dpjmp / wosq), wosq = (hg (pstar + po) + pstar) ro
  {
    const double idd = ddiv_rn(1.0, dd), iwo = ddiv_rn(1.0, wosq);
    rob += rstarb * idd;
    const double ddb = -rstarb * rstar * idd;
    const double uub = -ddb;
    const double ttb = uub * iwo;
    const double wosqb = -uub * uu * iwo;
    rob += ttb * dpjmp;
    const double dpb = ttb * ro;
    pstarb += dpb;
    pob -= dpb;
    const double awb = wosqb * ro;
    rob += wosqb * aw;
    pstarb += awb * (hg + 1.0);
    pob += awb * hg;
  }
  double inb[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
  if (side == 0) { inb[0] += rob; inb[1] += uob; inb[2] += pob; inb[3] += t1b; inb[4] += t2b; }
  else if (side == 1) { inb[5] += rob; inb[6] += uob; inb[7] += pob; inb[8] += t1b; inb[9] += t2b; }
  else {
    inb[6] += 0.5 * uob; inb[1] += 0.5 * uob;
    inb[7] += 0.5 * pob; inb[2] += 0.5 * pob;
    const double s = rl + rr;
    const double is2 = ddiv_rn(1.0, s * s);
    inb[0] += rob * 2.0 * rr * rr * is2;
    inb[5] += rob * 2.0 * rl * rl * is2;
    inb[3] += 0.5 * t1b; inb[8] += 0.5 * t1b;
    inb[4] += 0.5 * t2b; inb[9] += 0.5 * t2b;
  }
  // ---- reverse of the three iterations (ustar is the last one's)
  RPBar g{0, 0, 0, 0, 0, 0, 0};
  double Pnb = pstarb, Pmnb = 0.0, UMnb = 0.5 * ustarb, UPnb = 0.5 * ustarb;
#pragma unroll
  for (int it = 2; it >= 0; --it) {
    double Pb = 0.0, Pmb = 0.0, UMb = 0.0, UPb = 0.0;
    rp_iter_vjp(q, P[it], Pm[it], UM[it], UP[it], Pnb, Pmnb, UMnb, UPnb, Pb, Pmb, UMb, UPb, g);
    Pnb = Pb; Pmnb = Pmb; UMnb = UMb; UPnb = UPb;
  }
  // (Pnb, Pmnb, UMnb, UPnb) now hold the cotangents of (p1, p0, usm0, usp0)
  double wl0b = 0.0, wr0b = 0.0, dUb = 0.0;
  double p0b = Pmnb;
  {
    const double ps1b = m1 ? Pnb : 0.0;
    const double iD1 = ddiv_rn(1.0, D1);
    const double N1b = ps1b * iD1, D1b = -ps1b * ps1 * iD1;
    double wl1b = N1b * (pr - wr1 * dU) + D1b, wr1b = N1b * (pl - wl1 * dU) + D1b;
    g.pr += N1b * wl1;
    g.pl += N1b * wr1;
    dUb += -N1b * wr1 * wl1;
    // usm0 = ur + (p0 - pr)/wr1;  usp0 = ul - (p0 - pl)/wl1
    const double iwr1 = ddiv_rn(1.0, wr1), iwl1 = ddiv_rn(1.0, wl1);
    const double um = UMnb * iwr1, up = UPnb * iwl1;
    g.ur += UMnb;
    p0b += um;
    g.pr -= um;
    wr1b += -um * (p0 - pr) * iwr1;
    g.ul += UPnb;
    p0b -= up;
    g.pl += up;
    wl1b += up * (p0 - pl) * iwl1;
    // w1 = rvsqrt(a1 r), a1 = hg (p0 + p) + p0
    const double wlsqb = 0.5 * wl1b * iwl1, wrsqb = 0.5 * wr1b * iwr1;
    g.rl += wlsqb * a1l;
    g.rr += wrsqb * a1r;
    const double alb = wlsqb * rl, arb = wrsqb * rr;
    p0b += (alb + arb) * (hg + 1.0);
    g.pl += alb * hg;
    g.pr += arb * hg;
  }
  {
    const double ps0b = m0 ? p0b : 0.0;
    const double iD0 = ddiv_rn(1.0, D0);
    const double N0b = ps0b * iD0, D0b = -ps0b * ps0 * iD0;
    wl0b += N0b * (pr - wr0 * dU) + D0b;
    wr0b += N0b * (pl - wl0 * dU) + D0b;
    g.pr += N0b * wl0;
    g.pl += N0b * wr0;
    dUb += -N0b * wr0 * wl0;
  }
  // ccs = small (cleft + cright), cleft = wl0 / rl, cright = wr0 / rr
  {
    const double cb = small * (ccsb + g.ccs);
    const double irl = ddiv_rn(1.0, rl), irr = ddiv_rn(1.0, rr);
    wl0b += cb * irl;
    g.rl += -cb * cleft * irl;
    wr0b += cb * irr;
    g.rr += -cb * cright * irr;
  }
  g.ur += dUb;
  g.ul -= dUb;
  // w0 = rvsqrt(gamma p r)
  {
    const double lb = ddiv_rn(wl0b, (2.0 * wl0)), rb2 = ddiv_rn(wr0b, (2.0 * wr0));
    g.pl += lb * gamma * rl;
    g.rl += lb * gamma * pl;
    g.pr += rb2 * gamma * rr;
    g.rr += rb2 * gamma * pr;
  }
  ib[0] = inb[0] + g.rl;
  ib[1] = inb[1] + g.ul;
  ib[2] = inb[2] + g.pl;
  ib[3] = inb[3];
  ib[4] = inb[4];
  ib[5] = inb[5] + g.rr;
  ib[6] = inb[6] + g.ur;
  ib[7] = inb[7] + g.pr;
  ib[8] = inb[8];
  ib[9] = inb[9];
}

}  // namespace rpvjp
}  // namespace amrs
