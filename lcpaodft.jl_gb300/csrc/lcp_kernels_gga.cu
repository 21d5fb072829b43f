// GGA-PBE on the grid (FP64): the 27-point gradient stencil, the pointwise
// PBE functional and the divergence pass of the potential, fused with the
// effective potential and the energy-term tile sums of the grid step.
//
// Two passes over each cell:
//   1. gradient + PBE: per point, grad(rho_s + pcc) by the stencil, then
//      XC_PBE! (src/XC/XC_PBE.jl:187-476) giving the local potential
//      dE/drho_s (stored in vpot[s]), dE/d(grad rho_s) (stored in dexc) and
//      the energy per particle for Calc_EXC1's sums;
//   2. divergence: vpot[s] -= sum_a stencil_a(dexc[s][a]) (src/XC/GGA_PBE.jl:
//      325-354, 423-461), then dVHart + vxc + V_na.
// The stencil reads neighbours straight from global memory: a tile of 1024
// consecutive points spans about 11 rows of a 96-point plane, and the rows of
// the neighbouring planes it touches stay in L1/L2, so DRAM sees each field
// about once per pass.  The pointwise functional dominates: in FP64 (the
// drop-in) it is a few divisions, cube roots and logs and an exp per point,
// so the passes are bound by the FP64 pipe, not HBM; the precision forms run
// the stencils and the functional in double-float on the FP32 pipe, with
// only the sums and the stored values in FP64.
#include <cuda_runtime.h>

#include "lcp_device.h"
#include "lcp_grid_common.cuh"

namespace lcp {

namespace {

constexpr double kDenMin = 1.0e-14;  // src/LCPAODFT.jl:71
constexpr double kPi = 3.14159265358979323846;

// Reciprocals of N positive values with one division (Montgomery's
// simultaneous inversion: prefix products, one reciprocal, back-substitution;
// a few ulps each).  The callers keep the products inside the double range.
template <int N>
__device__ __forceinline__ void batch_recip(const double (&x)[N], double (&r)[N]) {
  double p[N];
  p[0] = x[0];
#pragma unroll
  for (int k = 1; k < N; ++k) p[k] = p[k - 1] * x[k];
  double inv = 1.0 / p[N - 1];
#pragma unroll
  for (int k = N - 1; k > 0; --k) {
    r[k] = inv * p[k - 1];
    inv *= x[k];
  }
  r[0] = inv;
}

// PW92 parameters of G(0), G(1), G(2) (src/XC/XC_PBE.jl:7-13).
__device__ __constant__ double kPwA[3] = {0.0310910, 0.0155450, 0.0168870};
__device__ __constant__ double kPwA1[3] = {0.2137000, 0.2054800, 0.1112500};
__device__ __constant__ double kPwB[3][4] = {{7.5957000, 3.5876000, 1.6382000, 0.4929400},
                                             {14.1189000, 6.1977000, 3.3662000, 0.6251700},
                                             {10.3570000, 3.6231000, 0.8802600, 0.4967100}};

// XC_PBE! (src/XC/XC_PBE.jl:187-476) with XC_PW92C (:1-126) and the
// spin-scaled exchange through XC_EX (:132-184), at one point: e = Exc[1] +
// Exc[2] (energy per particle), v[s] = DEXDD[s] + DECDD[s], dg[3 s + a] =
// DEXDGD + DECDGD, g = (grad up, grad down).  SYM: the "off" case (equal spin
// densities and gradients): zeta = 0, phi = 1, PW92's spin-interpolation terms
// vanish exactly (only G(0) is needed), both spins share one exchange
// evaluation, and DS = dt, GDMS = GDMT.
//
// The reference's expressions, rearranged to spend few FP64 divisions (the
// GB300's FP64 pipe is the limit of this pass):
//   - the reciprocals come in batches (batch_recip);
//   - one cube root of dt serves rs, kF and ("off") the exchange's kF;
//   - rsqrt gives sqrt(rs) and 1/sqrt(rs), and ks with 1/ks;
//   - c = 1 + 1/t and dcdrs/c = -2 A dbdrs / (t (t + 1)) share 1/(t (t + 1));
//   - f1/Ec = 1/(gamma phi^3) and DSDD/s = -(4/3)/DS: no 1/Ec or 1/s;
//   - 1/f3, 1/(1 + A f3) and 1/(1 + f4) = (1 + A f3)/(1 + A f3 + f3 beta/gamma)
//     share one division;
//   - log1p(f4) for log(1 + f4); cbrt for XC_EX's truncated power
//     D^(-0.333333333333333) (relative change <= |ln D| * 3.3e-16).
template <bool SYM>
__device__ __forceinline__ void xc_pbe_point(double d1, double d2, const double (&g)[6], double& e, double (&v)[2],
                                             double (&dg)[6]) {
  constexpr double beta = 0.06672455060314922;
  constexpr double gamma = 0.031090690869654901;  // (1 - ln 2) / pi^2
  constexpr double igamma = 1.0 / gamma;
  constexpr double bg = beta / gamma;
  constexpr double kappa = 0.8040;
  constexpr double mu = beta * kPi * kPi / 3;
  constexpr double c3pi2 = 3.0936677262801355;  // cbrt(3 pi^2)
  constexpr double COE1 = 0.6203504908994, COE2 = 0.610887057710857;
  constexpr int NS = SYM ? 1 : 2;
  constexpr int NG = SYM ? 1 : 3;  // PW92 G terms

  d1 = fmax(0.5 * kDenMin, d1);
  d2 = fmax(0.5 * kDenMin, d2);
  const double dt = d1 + d2;
  const double GDT[3] = {g[0] + g[3], g[1] + g[4], g[2] + g[5]};
  const double GDMT = fmax(1e-14, sqrt(GDT[0] * GDT[0] + GDT[1] * GDT[1] + GDT[2] * GDT[2]));
  double DS[2], GDMS[2], rcs[2], cds[2];
  const double r3 = rcbrt(dt);
  const double c3 = dt * r3 * r3;  // cbrt(dt)
  if (SYM) {
    // 2 d1 = dt >= den_min; |2 g| = 2 |g| exactly (GDT = 2 g)
    DS[0] = dt;
    GDMS[0] = GDMT;
    rcs[0] = r3;
    cds[0] = c3;
  } else {
    const double dd[2] = {d1, d2};
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      DS[s] = fmax(kDenMin, 2 * dd[s]);
      const double* gs = g + 3 * s;
      GDMS[s] = fmax(1e-14, 2 * sqrt(gs[0] * gs[0] + gs[1] * gs[1] + gs[2] * gs[2]));
      rcs[s] = rcbrt(DS[s]);
      cds[s] = DS[s] * rcs[s] * rcs[s];
    }
  }

  // XC_PW92C: its densities (reset to den_min/2 each where dt <= den_min), rs
  const bool low = dt <= kDenMin;
  const double pd1 = low ? 0.5e-14 : d1, pd2 = low ? 0.5e-14 : d2;
  const double rs = low ? 6203.504908994 : COE1 * r3;
  const double isrs = rsqrt(rs), srs = rs * isrs;
  double Gb[NG], Gdb[NG], GT[NG];
#pragma unroll
  for (int k = 0; k < NG; ++k) {
    Gb[k] = kPwB[k][0] * srs + rs * (kPwB[k][1] + kPwB[k][2] * srs + kPwB[k][3] * rs);
    Gdb[k] = kPwB[k][0] * 0.5 * isrs + kPwB[k][1] + kPwB[k][2] * 1.5 * srs + kPwB[k][3] * 2 * rs;
    GT[k] = 2 * kPwA[k] * Gb[k];
  }

  // first batch of reciprocals: dt, GDMT, the G terms' t (t + 1); "on" also DS, GDMS
  constexpr int NA = SYM ? 2 + NG : 6 + NG;
  double xa[NA], ra[NA];
  xa[0] = dt;
  xa[1] = GDMT;
#pragma unroll
  for (int k = 0; k < NG; ++k) xa[2 + k] = GT[k] * (GT[k] + 1.0);
  if (!SYM) {
    xa[2 + NG] = DS[0];
    xa[3 + NG] = DS[1];
    xa[4 + NG] = GDMS[0];
    xa[5 + NG] = GDMS[1];
  }
  batch_recip<NA>(xa, ra);
  const double idt = ra[0], iGT = ra[1];
  double iDS[2], iG[2];
  if (SYM) {
    iDS[0] = idt;
    iG[0] = iGT;
  } else {
    iDS[0] = ra[2 + NG];
    iDS[1] = ra[3 + NG];
    iG[0] = ra[4 + NG];
    iG[1] = ra[5 + NG];
  }
  const double tmp0 = low ? 1.0 / kDenMin : idt;  // 1/dtot
  const double dtot = low ? kDenMin : dt;
  double G[NG], dG[NG];
#pragma unroll
  for (int k = 0; k < NG; ++k) {
    const double r = ra[2 + k];
    const double c = 1.0 + (GT[k] + 1.0) * r;        // 1 + 1/t
    const double dcdrs_c = -Gdb[k] * 2 * kPwA[k] * r;  // dcdrs / c
    const double dum = log(c);
    const double dum1 = 1 + kPwA1[k] * rs;
    G[k] = -2 * kPwA[k] * dum1 * dum;
    dG[k] = -2 * kPwA[k] * (kPwA1[k] * dum + dum1 * dcdrs_c);
  }
  const double drsdd = -(1.0 / 3.0) * rs * tmp0;
  double Ec, Vc[2], zeta = 0.0, cz1 = 1.0, cz2 = 1.0;
  if (SYM) {
    Ec = G[0];
    Vc[0] = Vc[1] = G[0] + dtot * (dG[0] * drsdd);
  } else {
    zeta = tmp0 * (pd1 - pd2);
    zeta = zeta > 0.99 ? 0.99 : zeta;
    zeta = zeta < -1.0 ? -0.99 : zeta;
    cz1 = cbrt(1 + zeta);
    cz2 = cbrt(1 - zeta);
    constexpr double c = 1.92366105093154;
    constexpr double ifpp0 = 1.0 / 1.70992093416137;
    const double z1sq = cz1 * cz1, z2sq = cz2 * cz2;
    const double f = (z1sq * z1sq + z2sq * z2sq - 2) * c;
    const double dfdz = (4.0 / 3.0) * (cz1 - cz2) * c;
    const double z3 = zeta * zeta * zeta, z4 = z3 * zeta;
    Ec = G[0] - G[2] * f * ifpp0 * (1 - z4) + (G[1] - G[0]) * f * z4;
    const double dEcdrs = dG[0] - dG[2] * f * ifpp0 * (1 - z4) + (dG[1] - dG[0]) * f * z4;
    const double dEcdz = -G[2] * ifpp0 * (dfdz * (1 - z4) - f * 4 * z3) + (G[1] - G[0]) * (dfdz * z4 + f * 4 * z3);
    const double dum = dEcdrs * drsdd;
    Vc[0] = Ec + dtot * (dum + dEcdz * (tmp0 * (1 - zeta)));
    Vc[1] = Ec + dtot * (dum + dEcdz * (tmp0 * (-1 - zeta)));
  }

  // exchange enhancement: s and f1 per spin (src/XC/XC_PBE.jl:359-367)
  double sx[2], f1x[2];
#pragma unroll
  for (int s = 0; s < NS; ++s) {
    sx[s] = GDMS[s] * (0.5 / c3pi2) * rcs[s] * iDS[s];  // GDMS / (2 KFS DS)
    f1x[s] = 1 + mu * sx[s] * sx[s] / kappa;
  }
  // second batch: 1/f1 per spin; "on" also 1/phi, 1/cbrt(1 +- zeta)
  constexpr int NB = SYM ? 1 : 5;
  double xb[NB], rb[NB];
  xb[0] = f1x[0];
  double phi = 1.0;
  if (!SYM) {
    phi = 0.5 * (cz1 * cz1 + cz2 * cz2);  // ((1+z)^(2/3) + (1-z)^(2/3)) / 2
    xb[1] = f1x[1];
    xb[2] = phi;
    xb[3] = cz1;
    xb[4] = cz2;
  }
  batch_recip<NB>(xb, rb);
  double if1[2];
  if1[0] = rb[0];
  double iphi = 1.0, DPDZ = 0.0;
  if (!SYM) {
    if1[1] = rb[1];
    iphi = rb[2];
    DPDZ = (1.0 / 3.0) * (rb[3] - rb[4]);
  }

  // correlation gradient term H (src/XC/XC_PBE.jl:241-267)
  const double kF = c3pi2 * c3;
  const double xks = 4 * kF / kPi;
  const double iks = rsqrt(xks), ks = xks * iks;
  const double phi3 = phi * phi * phi, iphi3 = iphi * iphi * iphi;
  const double K = 0.5 * iphi * iks * idt;  // t / GDMT
  const double t = GDMT * K;
  const double f1 = Ec * igamma * iphi3;
  const double f2 = exp(-f1);
  const double E = f2 - 1;
  const double iE = 1.0 / E;
  const double A = bg * iE;
  const double t2 = t * t;
  const double f3 = t2 + A * t2 * t2;
  const double P = 1 + A * f3;  // 1 + A f3
  const double Q = P + bg * f3;  // P (1 + f4)
  double xc3[3] = {f3, P, Q}, rc3[3];
  batch_recip<3>(xc3, rc3);
  const double if3 = rc3[0], iP = rc3[1];
  const double if4 = P * rc3[2];  // 1 / (1 + f4)
  const double f4 = bg * f3 * iP;
  const double H = gamma * phi3 * log1p(f4);
  const double Fc = Ec + H;

  // correlation derivatives (:273-342)
  const double DKSDD = 0.5 * ks * (1.0 / 3.0) * idt;
  const double dt3 = 2 * t + 4 * A * t2 * t;
  double DFCDD[2];
#pragma unroll
  for (int is = 0; is < NS; ++is) {
    const double DZDD = is == 0 ? idt - zeta * idt : -idt - zeta * idt;
    const double DECUDD = (Vc[is] - Ec) * idt;
    const double DPDD = DPDZ * DZDD;
    const double DTDD = (-t) * (DPDD * iphi + DKSDD * iks + idt);
    const double DF1DD = igamma * iphi3 * DECUDD - 3 * f1 * DPDD * iphi;
    const double DF2DD = -f2 * DF1DD;
    const double DADD = -A * DF2DD * iE;
    const double DF3DD = dt3 * DTDD + DADD * t2 * t2;
    const double DF4DD = f4 * (DF3DD * if3 - (DADD * f3 + A * DF3DD) * iP);
    const double DHDD = 3 * H * DPDD * iphi + gamma * phi3 * DF4DD * if4;
    DFCDD[is] = Vc[is] + H + dt * DHDD;
  }
  if (SYM) DFCDD[1] = DFCDD[0];
  // d Fc / d GDT_x = kc * GDT_x (the reference's f4 (1/f3 - A/(1 + A f3)), kept
  // as written: for large t both terms nearly cancel)
  const double kc = dt * gamma * phi3 * f4 * (if3 - A * iP) * dt3 * K * iGT * if4;

  // exchange (:348-451): fx = DS Ex_unif F(s), Ex_unif = 0.75 VXP, VXP = -COE2/COE1 cbrt(DS)
  double fx[2], dfx[2], kx[2];
#pragma unroll
  for (int s = 0; s < NS; ++s) {
    const double f = 1 + kappa - kappa * if1[s];
    const double VXP = -(COE2 / COE1) * cds[s];
    const double EXP = 0.75 * VXP;
    fx[s] = DS[s] * EXP * f;
    const double DF1DD = 2 * (f1x[s] - 1) * (-(4.0 / 3.0) * iDS[s]);  // 2 (f1 - 1) DSDD / s
    const double DFDD = kappa * DF1DD * if1[s] * if1[s];
    dfx[s] = VXP * f + DS[s] * EXP * DFDD;
    kx[s] = DS[s] * EXP * (2 * mu * sx[s] * (sx[s] * iG[s]) * 2 * iG[s]) * if1[s] * if1[s];
  }
  if (SYM) {
    fx[1] = fx[0];
    dfx[1] = dfx[0];
    kx[1] = kx[0];
  }
  e = 0.5 * (fx[0] + fx[1]) * idt + Fc;
  v[0] = dfx[0] + DFCDD[0];
  v[1] = dfx[1] + DFCDD[1];
  dg[0] = kx[0] * g[0] + kc * GDT[0];
  dg[1] = kx[0] * g[1] + kc * GDT[1];
  dg[2] = kx[0] * g[2] + kc * GDT[2];
  dg[3] = kx[1] * g[3] + kc * GDT[0];
  dg[4] = kx[1] * g[4] + kc * GDT[1];
  dg[5] = kx[1] * g[5] + kc * GDT[2];
}

// ------------------------------------------------------------ double-float PBE (the precision forms)
//
// xc_pbe_point's expressions in double-float on the FP32 pipe (lcp_dfloat.cuh):
// reciprocals, square roots and cube roots by Newton-refined FP32 estimates,
// each reciprocal on its own (cheaper than a Montgomery batch here);
// log1p and expm1 (which keep their precision near 0) by argument reduction,
// a short series and a Newton step (lcp_dfloat.cuh).  The density tests that
// select the reference's branches are made in FP64, as in xc_pbe_point, so
// both evaluations take the same branches.  The results agree with
// xc_pbe_point to about 2^-44 relative.

__device__ __constant__ Dfl kPwAd[3] = {dflc(0.0310910), dflc(0.0155450), dflc(0.0168870)};
__device__ __constant__ Dfl kPwA1d[3] = {dflc(0.2137000), dflc(0.2054800), dflc(0.1112500)};
__device__ __constant__ Dfl kPwBd[3][4] = {{dflc(7.5957000), dflc(3.5876000), dflc(1.6382000), dflc(0.4929400)},
                                           {dflc(14.1189000), dflc(6.1977000), dflc(3.3662000), dflc(0.6251700)},
                                           {dflc(10.3570000), dflc(3.6231000), dflc(0.8802600), dflc(0.4967100)}};

__device__ __forceinline__ Dfl dsq(Dfl a) { return a * a; }
// sqrt(x) for x > 0 as x rsqrt(x)
__device__ __forceinline__ Dfl dfl_sqrt(Dfl x) { return x * dfl_rsqrt(x); }
// a < b and a > b on the double-float values (the sign of a - b)
__device__ __forceinline__ bool dlt(Dfl a, Dfl b) {
  const Dfl d = a - b;
  return d.hi < 0.f || (d.hi == 0.f && d.lo < 0.f);
}
__device__ __forceinline__ bool dgt(Dfl a, Dfl b) { return dlt(b, a); }
// max(c, 2^k sqrt(n2)) for n2 >= 0 (c > 0)
__device__ __forceinline__ Dfl norm_floor(Dfl n2, float twice, Dfl c) {
  if (n2.hi <= 1e-36f) return c;
  const Dfl r = dfl_sqrt(n2) * twice;
  return dlt(r, c) ? c : r;
}
// acc + f w, the high product exact, not renormalised (stencil sums)
__device__ __forceinline__ Dfl fma_acc(Dfl acc, Dfl f, Dfl w) {
  const float p = f.hi * w.hi;
  const float pe = fmaf(f.hi, w.hi, -p) + fmaf(f.hi, w.lo, f.lo * w.hi);
  const float s = acc.hi + p;
  const float bb = s - acc.hi;
  return {s, acc.lo + (((acc.hi - (s - bb)) + (p - bb)) + pe)};
}

template <bool SYM>
__device__ __forceinline__ void xc_pbe_point_df(double d1, double d2, const Dfl (&g)[6], double& e_out,
                                                double (&v_out)[2], double (&dg_out)[6]) {
  constexpr double beta = 0.06672455060314922;
  constexpr double gamma = 0.031090690869654901;  // (1 - ln 2) / pi^2
  constexpr double kappa = 0.8040;
  constexpr double mu = beta * kPi * kPi / 3;
  constexpr double c3pi2 = 3.0936677262801355;  // cbrt(3 pi^2)
  constexpr double COE1 = 0.6203504908994, COE2 = 0.610887057710857;
  constexpr int NS = SYM ? 1 : 2;
  constexpr int NG = SYM ? 1 : 3;
  const Dfl one = dflc(1.0);

  d1 = fmax(0.5 * kDenMin, d1);
  d2 = fmax(0.5 * kDenMin, d2);
  const bool low = d1 + d2 <= kDenMin;
  const Dfl D1 = dfl_of(d1), D2 = dfl_of(d2);
  const Dfl dt = D1 + D2;
  const Dfl GDT[3] = {g[0] + g[3], g[1] + g[4], g[2] + g[5]};
  const Dfl GDMT = norm_floor(dot2(GDT[0], GDT[0], GDT[1], GDT[1]) + dsq(GDT[2]), 1.0f, dflc(1e-14));
  Dfl DS[2], GDMS[2], rcs[2], cds[2];
  const Dfl r3 = dfl_rcbrt(dt);
  const Dfl c3 = dt * dsq(r3);  // cbrt(dt)
  if (SYM) {
    DS[0] = dt;
    GDMS[0] = GDMT;
    rcs[0] = r3;
    cds[0] = c3;
  } else {
    const Dfl dd[2] = {D1, D2};
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      DS[s] = dd[s] * 2.0f;
      if (dlt(DS[s], dflc(kDenMin))) DS[s] = dflc(kDenMin);
      const Dfl* gs = g + 3 * s;
      GDMS[s] = norm_floor(dot2(gs[0], gs[0], gs[1], gs[1]) + dsq(gs[2]), 2.0f, dflc(1e-14));
      rcs[s] = dfl_rcbrt(DS[s]);
      cds[s] = DS[s] * dsq(rcs[s]);
    }
  }

  // XC_PW92C
  const Dfl pd1 = low ? dflc(0.5e-14) : D1, pd2 = low ? dflc(0.5e-14) : D2;
  const Dfl rs = low ? dflc(6203.504908994) : r3 * dflc(COE1);
  const Dfl isrs = dfl_rsqrt(rs), srs = rs * isrs;
  const Dfl idt = dfl_rcp(dt);
  const Dfl tmp0 = low ? dflc(1.0 / kDenMin) : idt;  // 1/dtot
  const Dfl dtot = low ? dflc(kDenMin) : dt;
  Dfl G[NG], dG[NG];
#pragma unroll
  for (int k = 0; k < NG; ++k) {
    const Dfl Gb = dot2(kPwBd[k][0], srs, rs, dot2(kPwBd[k][2], srs, kPwBd[k][3], rs) + kPwBd[k][1]);
    const Dfl Gdb = dot2(kPwBd[k][0] * 0.5f, isrs, kPwBd[k][2] * 1.5f, srs) + dot2(kPwBd[k][3] * 2.0f, rs, one,
                                                                                  kPwBd[k][1]);
    const Dfl A2 = kPwAd[k] * 2.0f;
    const Dfl GT = A2 * Gb;
    const Dfl r = dfl_rcp(GT * (GT + one));
    const Dfl it = (GT + one) * r;            // 1/t: c = 1 + 1/t
    const Dfl dcdrs_c = -(Gdb * A2) * r;      // dcdrs / c
    const Dfl dum = dfl_log1p(it);            // log(c)
    const Dfl dum1 = one + kPwA1d[k] * rs;
    G[k] = -(A2 * dum1 * dum);
    dG[k] = -(A2 * dot2(kPwA1d[k], dum, dum1, dcdrs_c));
  }
  const Dfl drsdd = -(rs * tmp0) * dflc(1.0 / 3.0);
  Dfl Ec, Vc[2], zeta = dflc(0.0), cz1 = one, cz2 = one;
  if (SYM) {
    Ec = G[0];
    Vc[0] = Vc[1] = G[0] + dtot * (dG[0] * drsdd);
  } else {
    zeta = tmp0 * (pd1 - pd2);
    if (dgt(zeta, dflc(0.99))) zeta = dflc(0.99);
    if (zeta < -1.0f) zeta = dflc(-0.99);
    const Dfl p1 = one + zeta, m1 = one - zeta;
    cz1 = dfl_cbrt(p1);
    cz2 = dfl_cbrt(m1);
    const Dfl c = dflc(1.92366105093154);
    const Dfl ifpp0 = dflc(1.0 / 1.70992093416137);
    const Dfl z1sq = dsq(cz1), z2sq = dsq(cz2);
    const Dfl f = (dsq(z1sq) + dsq(z2sq) - dflc(2.0)) * c;
    const Dfl dfdz = (cz1 - cz2) * c * dflc(4.0 / 3.0);
    const Dfl z3 = zeta * zeta * zeta, z4 = z3 * zeta;
    const Dfl omz4 = one - z4;
    const Dfl G2f = G[2] * f * ifpp0, G10 = G[1] - G[0];
    Ec = G[0] - G2f * omz4 + G10 * f * z4;
    const Dfl dEcdrs = dG[0] - dG[2] * f * ifpp0 * omz4 + (dG[1] - dG[0]) * f * z4;
    const Dfl dEcdz = -(G[2] * ifpp0) * (dfdz * omz4 - f * z3 * 4.0f) + G10 * dot2(dfdz, z4, f * 4.0f, z3);
    const Dfl dum = dEcdrs * drsdd;
    Vc[0] = Ec + dtot * (dum + dEcdz * (tmp0 * m1));
    Vc[1] = Ec + dtot * (dum - dEcdz * (tmp0 * p1));
  }

  // exchange enhancement: s and f1 per spin
  Dfl sx[2], f1x[2], if1[2];
#pragma unroll
  for (int s = 0; s < NS; ++s) {
    sx[s] = GDMS[s] * dflc(0.5 / c3pi2) * rcs[s] * dfl_rcp(DS[s]);  // GDMS / (2 KFS DS)
    f1x[s] = one + dsq(sx[s]) * dflc(mu / kappa);
    if1[s] = dfl_rcp(f1x[s]);
  }
  Dfl phi = one, iphi = one, DPDZ = dflc(0.0);
  if (!SYM) {
    phi = (dsq(cz1) + dsq(cz2)) * 0.5f;
    iphi = dfl_rcp(phi);
    DPDZ = (dfl_rcp(cz1) - dfl_rcp(cz2)) * dflc(1.0 / 3.0);
  }

  // correlation gradient term H
  const Dfl kF = c3 * dflc(c3pi2);
  const Dfl xks = kF * dflc(4 / kPi);
  const Dfl iks = dfl_rsqrt(xks), ks = xks * iks;
  const Dfl phi3 = phi * phi * phi, iphi3 = iphi * iphi * iphi;
  const Dfl K = iphi * iks * idt * 0.5f;  // t / GDMT
  const Dfl t = GDMT * K;
  const Dfl f1 = Ec * dflc(1.0 / gamma) * iphi3;
  const Dfl E = dfl_expm1(-f1);  // exp(-f1) - 1
  const Dfl f2 = E + one;
  const Dfl iE = dfl_rcp(E);
  const Dfl A = iE * dflc(beta / gamma);
  const Dfl t2 = dsq(t);
  const Dfl f3 = t2 + A * dsq(t2);
  const Dfl P = one + A * f3;
  const Dfl Q = P + f3 * dflc(beta / gamma);
  const Dfl if3 = dfl_rcp(f3), iP = dfl_rcp(P);
  const Dfl if4 = P * dfl_rcp(Q);  // 1 / (1 + f4)
  const Dfl f4 = f3 * dflc(beta / gamma) * iP;
  const Dfl H = dflc(gamma) * phi3 * dfl_log1p(f4);
  const Dfl Fc = Ec + H;

  // correlation derivatives
  const Dfl DKSDD = ks * idt * dflc(0.5 / 3.0);
  const Dfl dt3 = t * 2.0f + A * t2 * t * 4.0f;
  Dfl DFCDD[2];
#pragma unroll
  for (int is = 0; is < NS; ++is) {
    const Dfl DZDD = is == 0 ? idt - zeta * idt : -(idt + zeta * idt);
    const Dfl DECUDD = (Vc[is] - Ec) * idt;
    const Dfl DPDD = DPDZ * DZDD;
    const Dfl DTDD = -(t * (DPDD * iphi + DKSDD * iks + idt));
    const Dfl DF1DD = dflc(1.0 / gamma) * iphi3 * DECUDD - f1 * DPDD * iphi * 3.0f;
    const Dfl DF2DD = -(f2 * DF1DD);
    const Dfl DADD = -(A * DF2DD * iE);
    const Dfl DF3DD = dot2(dt3, DTDD, DADD, dsq(t2));
    const Dfl DF4DD = f4 * (DF3DD * if3 - dot2(DADD, f3, A, DF3DD) * iP);
    const Dfl DHDD = H * DPDD * iphi * 3.0f + dflc(gamma) * phi3 * DF4DD * if4;
    DFCDD[is] = Vc[is] + H + dt * DHDD;
  }
  if (SYM) DFCDD[1] = DFCDD[0];
  const Dfl kc = dt * dflc(gamma) * phi3 * f4 * (if3 - A * iP) * dt3 * K * dfl_rcp(GDMT) * if4;

  // exchange
  Dfl fx[2], dfx[2], kx[2];
#pragma unroll
  for (int s = 0; s < NS; ++s) {
    const Dfl f = dflc(1 + kappa) - if1[s] * dflc(kappa);
    const Dfl VXP = -(cds[s] * dflc(COE2 / COE1));
    const Dfl EXP = VXP * 0.75f;
    const Dfl DSE = DS[s] * EXP;
    fx[s] = DSE * f;
    const Dfl iDS = dfl_rcp(DS[s]);
    const Dfl DF1DD = (f1x[s] - one) * iDS * dflc(-8.0 / 3.0);  // 2 (f1 - 1) DSDD / s
    const Dfl DFDD = DF1DD * dsq(if1[s]) * dflc(kappa);
    dfx[s] = dot2(VXP, f, DSE, DFDD);
    const Dfl iG = dfl_rcp(GDMS[s]);
    kx[s] = DSE * (dsq(sx[s]) * dsq(iG) * dflc(4 * mu)) * dsq(if1[s]);
  }
  if (SYM) {
    fx[1] = fx[0];
    dfx[1] = dfx[0];
    kx[1] = kx[0];
  }
  e_out = dbl_of((fx[0] + fx[1]) * idt * 0.5f + Fc);
  v_out[0] = dbl_of(dfx[0] + DFCDD[0]);
  v_out[1] = dbl_of(dfx[1] + DFCDD[1]);
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    dg_out[a] = dbl_of(dot2(kx[0], g[a], kc, GDT[a]));
    dg_out[3 + a] = dbl_of(dot2(kx[1], g[3 + a], kc, GDT[a]));
  }
}

struct GgaArgs {
  GridCell cell0;
  GridBatch batch;
  int spinpol;  // LCP_SPIN_OFF or LCP_SPIN_ON ("nc" runs as "on" plus a rotation)
};

__device__ __forceinline__ int wrap_index(int i, int n) { return i < 0 ? i + n : (i >= n ? i - n : i); }

// The 27 neighbours of point x (transform2primcell, src/XC/GGA_PBE.jl:42-50)
// in the reference's order: i1, j1, k1 in -1..1, k1 fastest
// (src/XC/GGA_PBE.jl:77-90).  Neighbour p = 9 a + q lies in plane a
// (i + a - 1) at row q / 3 (j + q/3 - 1) and column q % 3 (k + q%3 - 1).
struct Stencil {
  int i, n1;
  int64_t plane;
  int64_t jr[3];  // (j - 1, j, j + 1) wrapped, times n3
  int k[3];       // k - 1, k, k + 1 wrapped
  __device__ __forceinline__ Stencil(int64_t x, const int32_t* ng) {
    const int n2 = ng[1], n3 = ng[2];
    n1 = ng[0];
    plane = (int64_t)n2 * n3;
    i = (int)(x / plane);
    const int64_t rem = x - (int64_t)i * plane;
    const int j = (int)(rem / n3);
    const int kc = (int)(rem - (int64_t)j * n3);
#pragma unroll
    for (int b = 0; b < 3; ++b) {
      jr[b] = (int64_t)wrap_index(j + b - 1, n2) * n3;
      k[b] = wrap_index(kc + b - 1, n3);
    }
  }
  __device__ __forceinline__ int64_t plane_base(int a) const { return (int64_t)wrap_index(i + a - 1, n1) * plane; }
  // q = 0..8 must be a compile-time constant at the call site
  __device__ __forceinline__ int64_t at(int64_t base, int q) const { return base + jr[q / 3] + k[q % 3]; }
};

__device__ __forceinline__ void load_coef(const GridCell& c, double* dc) {
  for (int q = threadIdx.x; q < 81; q += blockDim.x) dc[q] = c.dcoef[q];
  __syncthreads();
}

// Pass 1: Set_dDensity_Grid! (src/XC/GGA_PBE.jl:53-159) and the pointwise
// part of Set_Vxc_GGA_PBE! (src/XC/GGA_PBE.jl:274-322, 358-420); where the
// cell has tile partials, also Calc_EH1 / Calc_EXC1's terms (src/Energy.jl:
// 655-700, the GGA energy per particle of src/XC/XC_Func.jl:193-215), over the
// same tiles and in the same order as the LDA/LSDA pass.
// The masks are the reference's: gradient where den_min < t, local potential
// where t >= den_min ("off") / t > den_min ("on"), energy where t > den_min,
// with t = 2 rho ("off") or rho_up + rho_down, before the PCC is added.
// DF: the stencil and the functional in double-float (the precision forms).
template <bool SYM, bool DF>
__global__ void __launch_bounds__(kRedThreads) gga_point_g_kernel(const __grid_constant__ GgaArgs a) {
  int64_t t;
  const GridCell& c = grid_cell(a.cell0, a.batch, blockIdx.x, t);
  __shared__ double dc[81];
  __shared__ Dfl dcf[DF ? 81 : 1];
  load_coef(c, dc);
  if (DF) {
    for (int q = threadIdx.x; q < 81; q += blockDim.x) dcf[q] = dfl_of(dc[q]);
    __syncthreads();
  }
  const int64_t nn = c.nn;
  const int64_t x0 = t * kRedTile, x1 = min(nn, x0 + kRedTile);
  const double* r0p = c.rho[0];
  const double* r1p = SYM ? c.rho[0] : c.rho[1];
  const double* pcp = c.pcc;
  double acc[3] = {0, 0, 0};
  for (int64_t x = x0 + threadIdx.x; x < x1; x += kRedThreads) {
    const double pc = pcp ? pcp[x] : 0.0;
    const double r0 = r0p[x];
    const double r1 = SYM ? r0 : r1p[x];
    const double test = SYM ? 2 * r0 : r0 + r1;
    double g[6] = {0, 0, 0, 0, 0, 0};
    Dfl gd[6] = {};
    if (kDenMin < test) {
      const Stencil nb(x, c.ng);
#pragma unroll 1
      for (int pa = 0; pa < 3; ++pa) {
        const int64_t base = nb.plane_base(pa);
        const double* w = dc + 9 * pa;
        const Dfl* wf = dcf + (DF ? 9 * pa : 0);
#pragma unroll
        for (int q = 0; q < 9; ++q) {
          const int64_t y = nb.at(base, q);
          if (DF) {
            const Dfl py = pcp ? dfl_of(pcp[y]) : Dfl{0.f, 0.f};
            const Dfl fu = pcp ? dfl_of(r0p[y]) + py : dfl_of(r0p[y]);
            gd[0] = fma_acc(gd[0], fu, wf[q]);
            gd[1] = fma_acc(gd[1], fu, wf[27 + q]);
            gd[2] = fma_acc(gd[2], fu, wf[54 + q]);
            if (!SYM) {
              const Dfl fd = pcp ? dfl_of(r1p[y]) + py : dfl_of(r1p[y]);
              gd[3] = fma_acc(gd[3], fd, wf[q]);
              gd[4] = fma_acc(gd[4], fd, wf[27 + q]);
              gd[5] = fma_acc(gd[5], fd, wf[54 + q]);
            }
          } else {
            const double py = pcp ? pcp[y] : 0.0;
            const double fu = r0p[y] + py;
            g[0] += fu * w[q];
            g[1] += fu * w[27 + q];
            g[2] += fu * w[54 + q];
            if (!SYM) {
              const double fd = r1p[y] + py;
              g[3] += fd * w[q];
              g[4] += fd * w[27 + q];
              g[5] += fd * w[54 + q];
            }
          }
        }
      }
    }
    if (DF) {
#pragma unroll
      for (int q = 0; q < 6; ++q) gd[q] = quick_two_sum(gd[q].hi, gd[q].lo);
      if (SYM) {
        gd[3] = gd[0];
        gd[4] = gd[1];
        gd[5] = gd[2];
      }
    } else if (SYM) {
      g[3] = g[0];
      g[4] = g[1];
      g[5] = g[2];
    }
    double e = 0.0, v[2] = {0.0, 0.0}, dg[6] = {0, 0, 0, 0, 0, 0};
    const bool act = SYM ? test >= kDenMin : test > kDenMin;
    if (DF) {
      if (act) xc_pbe_point_df<SYM>(r0 + pc, r1 + pc, gd, e, v, dg);
      if (c.dden)
#pragma unroll
        for (int q = 0; q < 6; ++q) g[q] = dbl_of(gd[q]);
    } else if (act) {
      xc_pbe_point<SYM>(r0 + pc, r1 + pc, g, e, v, dg);
    }
#pragma unroll
    for (int s = 0; s < (SYM ? 1 : 2); ++s) {
      c.vpot[s][x] = v[s];
#pragma unroll
      for (int q = 0; q < 3; ++q) c.dexc[(3 * s + q) * nn + x] = dg[3 * s + q];
      if (c.dden)
#pragma unroll
        for (int q = 0; q < 3; ++q) c.dden[(3 * s + q) * nn + x] = g[3 * s + q];
    }
    if (c.part) {
      const double eu = test > kDenMin ? e : 0.0;
      energy_terms<DF>(SYM ? LCP_XC_LDA : LCP_XC_LSDA, a.spinpol, r0, r1, c.aden ? c.aden[x] : 0.0, pc,
                       c.dvh ? c.dvh[x] : 0.0, eu, acc);
    }
  }
  if (c.part) block_reduce_store<3>(acc, c.part + t * 3);
}

// Pass 2: the divergence term of Set_Vxc_GGA_PBE! (src/XC/GGA_PBE.jl:325-354,
// 423-461), vxc_s -= sum_a stencil_a(dexc[s][a]) where t > den_min, then, if
// the cell has a Hartree potential, Set_Vpot_Grid! (src/Matrix/
// Set_Vpot_Grid.jl:1-19) plus V_na in place.
template <bool SYM, bool DF>
__global__ void __launch_bounds__(kRedThreads) gga_div_g_kernel(const __grid_constant__ GgaArgs a) {
  int64_t t;
  const GridCell& c = grid_cell(a.cell0, a.batch, blockIdx.x, t);
  __shared__ double dc[81];
  __shared__ Dfl dcf[DF ? 81 : 1];
  load_coef(c, dc);
  if (DF) {
    for (int q = threadIdx.x; q < 81; q += blockDim.x) dcf[q] = dfl_of(dc[q]);
    __syncthreads();
  }
  const int64_t nn = c.nn;
  const int64_t x0 = t * kRedTile, x1 = min(nn, x0 + kRedTile);
  constexpr int ns = SYM ? 1 : 2;
  for (int64_t x = x0 + threadIdx.x; x < x1; x += kRedThreads) {
    const double r0 = c.rho[0][x];
    const double test = SYM ? 2 * r0 : r0 + c.rho[1][x];
    double v[2];
#pragma unroll
    for (int s = 0; s < ns; ++s) v[s] = c.vpot[s][x];
    if (test > kDenMin) {
      const Stencil nb(x, c.ng);
#pragma unroll
      for (int s = 0; s < ns; ++s) {
        const double* fx = c.dexc + (3 * s) * nn;
        const double* fy = fx + nn;
        const double* fz = fy + nn;
        double sx = 0.0, sy = 0.0, sz = 0.0;
        Dfl dx = {}, dy = {}, dz = {};
#pragma unroll 1
        for (int pa = 0; pa < 3; ++pa) {
          const int64_t base = nb.plane_base(pa);
          const double* w = dc + 9 * pa;
          const Dfl* wf = dcf + (DF ? 9 * pa : 0);
#pragma unroll
          for (int q = 0; q < 9; ++q) {
            const int64_t y = nb.at(base, q);
            if (DF) {
              dx = fma_acc(dx, dfl_of(fx[y]), wf[q]);
              dy = fma_acc(dy, dfl_of(fy[y]), wf[27 + q]);
              dz = fma_acc(dz, dfl_of(fz[y]), wf[54 + q]);
            } else {
              sx += fx[y] * w[q];
              sy += fy[y] * w[27 + q];
              sz += fz[y] * w[54 + q];
            }
          }
        }
        if (DF) v[s] -= dbl_of((add_lazy(dx, dy)) + dz);
        else v[s] -= (sx + sy) + sz;
      }
    }
    if (c.dvh) {
      const double dv = c.dvh[x];
      const double na = c.vna ? c.vna[x] : 0.0;
#pragma unroll
      for (int s = 0; s < ns; ++s) c.vpot[s][x] = dv + v[s] + na;
    } else {
#pragma unroll
      for (int s = 0; s < ns; ++s) c.vpot[s][x] = v[s];
    }
  }
}

}  // namespace

template <bool SYM, bool DF>
cudaError_t launch_gga_t(const GgaArgs& a, int64_t n, bool potential, cudaStream_t st) {
  gga_point_g_kernel<SYM, DF><<<(unsigned)n, kRedThreads, 0, st>>>(a);
  LCP_CUDA_TRY(cudaGetLastError());
  if (potential) gga_div_g_kernel<SYM, DF><<<(unsigned)n, kRedThreads, 0, st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_gga_g(int spinpol, const GridCell& c0, const GridBatch& b, bool potential, bool dfl,
                         cudaStream_t st) {
  const int64_t n = b.cells ? b.nblocks : red_tiles(c0.nn);
  if (n == 0) return cudaSuccess;
  GgaArgs a;
  a.cell0 = c0;
  a.batch = b;
  a.spinpol = spinpol == LCP_SPIN_OFF ? LCP_SPIN_OFF : LCP_SPIN_ON;
  if (a.spinpol == LCP_SPIN_OFF)
    return dfl ? launch_gga_t<true, true>(a, n, potential, st) : launch_gga_t<true, false>(a, n, potential, st);
  return dfl ? launch_gga_t<false, true>(a, n, potential, st) : launch_gga_t<false, false>(a, n, potential, st);
}

}  // namespace lcp
