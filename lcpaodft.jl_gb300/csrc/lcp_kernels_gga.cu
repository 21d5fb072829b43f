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
// about once per pass.  The pointwise functional dominates: it is FP64
// arithmetic (a few divisions, cube roots and logs and an exp per point), so
// the passes are bound by the FP64 pipe, not HBM.
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
template <bool SYM>
__global__ void __launch_bounds__(kRedThreads) gga_point_g_kernel(const __grid_constant__ GgaArgs a) {
  int64_t t;
  const GridCell& c = grid_cell(a.cell0, a.batch, blockIdx.x, t);
  __shared__ double dc[81];
  load_coef(c, dc);
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
    if (kDenMin < test) {
      const Stencil nb(x, c.ng);
#pragma unroll 1
      for (int pa = 0; pa < 3; ++pa) {
        const int64_t base = nb.plane_base(pa);
        const double* w = dc + 9 * pa;
#pragma unroll
        for (int q = 0; q < 9; ++q) {
          const int64_t y = nb.at(base, q);
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
    if (SYM) {
      g[3] = g[0];
      g[4] = g[1];
      g[5] = g[2];
    }
    double e = 0.0, v[2] = {0.0, 0.0}, dg[6] = {0, 0, 0, 0, 0, 0};
    const bool act = SYM ? test >= kDenMin : test > kDenMin;
    if (act) xc_pbe_point<SYM>(r0 + pc, r1 + pc, g, e, v, dg);
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
      energy_terms(SYM ? LCP_XC_LDA : LCP_XC_LSDA, a.spinpol, r0, r1, c.aden ? c.aden[x] : 0.0, pc,
                   c.dvh ? c.dvh[x] : 0.0, eu, acc);
    }
  }
  if (c.part) block_reduce_store<3>(acc, c.part + t * 3);
}

// Pass 2: the divergence term of Set_Vxc_GGA_PBE! (src/XC/GGA_PBE.jl:325-354,
// 423-461), vxc_s -= sum_a stencil_a(dexc[s][a]) where t > den_min, then, if
// the cell has a Hartree potential, Set_Vpot_Grid! (src/Matrix/
// Set_Vpot_Grid.jl:1-19) plus V_na in place.
template <bool SYM>
__global__ void __launch_bounds__(kRedThreads) gga_div_g_kernel(const __grid_constant__ GgaArgs a) {
  int64_t t;
  const GridCell& c = grid_cell(a.cell0, a.batch, blockIdx.x, t);
  __shared__ double dc[81];
  load_coef(c, dc);
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
#pragma unroll 1
        for (int pa = 0; pa < 3; ++pa) {
          const int64_t base = nb.plane_base(pa);
          const double* w = dc + 9 * pa;
#pragma unroll
          for (int q = 0; q < 9; ++q) {
            const int64_t y = nb.at(base, q);
            sx += fx[y] * w[q];
            sy += fy[y] * w[27 + q];
            sz += fz[y] * w[54 + q];
          }
        }
        v[s] -= (sx + sy) + sz;
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

cudaError_t launch_gga_g(int spinpol, const GridCell& c0, const GridBatch& b, bool potential, cudaStream_t st) {
  const int64_t n = b.cells ? b.nblocks : red_tiles(c0.nn);
  if (n == 0) return cudaSuccess;
  GgaArgs a;
  a.cell0 = c0;
  a.batch = b;
  a.spinpol = spinpol == LCP_SPIN_OFF ? LCP_SPIN_OFF : LCP_SPIN_ON;
  if (a.spinpol == LCP_SPIN_OFF) {
    gga_point_g_kernel<true><<<(unsigned)n, kRedThreads, 0, st>>>(a);
    LCP_CUDA_TRY(cudaGetLastError());
    if (potential) gga_div_g_kernel<true><<<(unsigned)n, kRedThreads, 0, st>>>(a);
  } else {
    gga_point_g_kernel<false><<<(unsigned)n, kRedThreads, 0, st>>>(a);
    LCP_CUDA_TRY(cudaGetLastError());
    if (potential) gga_div_g_kernel<false><<<(unsigned)n, kRedThreads, 0, st>>>(a);
  }
  return cudaGetLastError();
}

}  // namespace lcp
