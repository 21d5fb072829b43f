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
// arithmetic (about 40 divisions' worth of reciprocals, 4 logs, 1 exp and 6
// cube roots per point), so the passes are bound by the FP64 pipe, not HBM.
#include <cuda_runtime.h>

#include "lcp_device.h"
#include "lcp_grid_common.cuh"

namespace lcp {

namespace {

constexpr double kDenMin = 1.0e-14;  // src/LCPAODFT.jl:71
constexpr double kPi = 3.14159265358979323846;

// One PW92 G(rs) term and its rs-derivative (src/XC/XC_PBE.jl:41-90).  With
// t = 2 A b, the reference's c = 1 + 1/t and dcdrs/c = -dbdrs / (t + 1) share
// one reciprocal r = 1 / (t (t + 1)).
__device__ __forceinline__ void pw92_g(double rs, double srs, double isrs, double A, double a1, double b1,
                                       double b2, double b3, double b4, double& G, double& dG) {
  const double b = b1 * srs + rs * (b2 + b3 * srs + b4 * rs);
  const double dbdrs = b1 * 0.5 * isrs + b2 + b3 * 1.5 * srs + b4 * 2 * rs;
  const double t = 2 * A * b;
  const double r = 1.0 / (t * (t + 1.0));
  const double c = 1.0 + (t + 1.0) * r;  // 1 + 1/t
  const double dcdrs_c = -dbdrs * 2 * A * r;  // dcdrs / c = -(c-1) dbdrs / (b c) = -2 A dbdrs / (t (t+1))
  const double dum = log(c);
  const double dum1 = 1 + a1 * rs;
  G = -2 * A * dum1 * dum;
  dG = -2 * A * (a1 * dum + dum1 * dcdrs_c);
}

// XC_PW92C (src/XC/XC_PBE.jl:1-126): Ec and Vc1/Vc2 of the densities d1, d2,
// which it writes back as den_min/2 each where their sum is <= den_min.
// SYM: d1 == d2 (zeta = 0), where the spin interpolation terms vanish exactly
// and only G(0) is needed.
template <bool SYM>
__device__ __forceinline__ void pw92c(double& d1, double& d2, double& Ec, double& Vc1, double& Vc2, double& cz1,
                                      double& cz2) {
  double dtot = d1 + d2;
  double rs;
  if (dtot <= kDenMin) {
    rs = 6203.504908994;
    d1 = d2 = 0.5e-14;
    dtot = kDenMin;
  } else {
    rs = 0.6203504908994 * rcbrt(dtot);
  }
  const double tmp0 = 1.0 / dtot;
  const double srs = sqrt(rs), isrs = 1.0 / srs;
  const double drsdd = -(1.0 / 3.0) * rs * tmp0;
  double G0, dG0;
  pw92_g(rs, srs, isrs, 0.0310910, 0.2137000, 7.5957000, 3.5876000, 1.6382000, 0.4929400, G0, dG0);
  if (SYM) {
    Ec = G0;
    Vc1 = Vc2 = G0 + dtot * (dG0 * drsdd);
    cz1 = cz2 = 1.0;
    return;
  }
  double zeta = tmp0 * (d1 - d2);
  zeta = zeta > 0.99 ? 0.99 : zeta;
  zeta = zeta < -1.0 ? -0.99 : zeta;
  const double dzdd1 = tmp0 * (1 - zeta);
  const double dzdd2 = tmp0 * (-1 - zeta);
  double G1, dG1, G2, dG2;
  pw92_g(rs, srs, isrs, 0.0155450, 0.2054800, 14.1189000, 6.1977000, 3.3662000, 0.6251700, G1, dG1);
  pw92_g(rs, srs, isrs, 0.0168870, 0.1112500, 10.3570000, 3.6231000, 0.8802600, 0.4967100, G2, dG2);
  const double c = 1.92366105093154;
  const double ifpp0 = 1.0 / 1.70992093416137;
  cz1 = cbrt(1 + zeta);
  cz2 = cbrt(1 - zeta);
  const double z1sq = cz1 * cz1, z2sq = cz2 * cz2;
  const double f = (z1sq * z1sq + z2sq * z2sq - 2) * c;
  const double dfdz = (4.0 / 3.0) * (cz1 - cz2) * c;
  const double z3 = zeta * zeta * zeta, z4 = z3 * zeta;
  Ec = G0 - G2 * f * ifpp0 * (1 - z4) + (G1 - G0) * f * z4;
  const double dEcdrs = dG0 - dG2 * f * ifpp0 * (1 - z4) + (dG1 - dG0) * f * z4;
  const double dEcdz = -G2 * ifpp0 * (dfdz * (1 - z4) - f * 4 * z3) + (G1 - G0) * (dfdz * z4 + f * 4 * z3);
  const double dum = dEcdrs * drsdd;
  Vc1 = Ec + dtot * (dum + dEcdz * dzdd1);
  Vc2 = Ec + dtot * (dum + dEcdz * dzdd2);
}

// Spin-scaled PBE exchange of one spin channel (src/XC/XC_PBE.jl:356-448):
// fx = DS * Ex_unif * F(s), dfx/dDS and the gradient factor k with
// dfx/d(grad rho_s)_x = k * grad(rho_s)_x.  XC_EX with NSP = 1
// (src/XC/XC_PBE.jl:132-184) gives Ex_unif = 0.75 VXP, VXP = -COE2 / RS.
__device__ __forceinline__ void pbe_x_spin(double d, double gx, double gy, double gz, double& fx, double& dfx,
                                           double& k) {
  constexpr double kappa = 0.8040;
  constexpr double mu = 0.06672455060314922 * kPi * kPi / 3;
  const double DS = fmax(kDenMin, 2 * d);
  const double GDMS = fmax(1e-14, 2 * sqrt(gx * gx + gy * gy + gz * gz));
  const double cds = cbrt(DS);
  const double KFS = 3.0936677262801355 * cds;  // cbrt(3 pi^2) cbrt(DS)
  const double iDS = 1.0 / DS;
  const double s = GDMS / (2 * KFS * DS);
  const double f1 = 1 + mu * s * s / kappa;
  const double if1 = 1.0 / f1;
  const double f = 1 + kappa - kappa * if1;
  // RS = COE1 DS^(-1/3): VXP = -COE2 / RS
  const double VXP = -0.610887057710857 / (0.6203504908994 / cds);
  const double EXP = 0.75 * VXP;
  fx = DS * EXP * f;
  const double DSDD = s * (-(1.0 / 3.0) * iDS - iDS);
  const double DF1DD = 2 * (f1 - 1) * DSDD / s;
  const double DFDD = kappa * DF1DD * if1 * if1;
  dfx = VXP * f + DS * EXP * DFDD;
  // DSDGD = (s / GDMS) 2 g / GDMS; DFDGD = kappa (2 mu s DSDGD / kappa) / f1^2
  const double iG = 1.0 / GDMS;
  k = DS * EXP * (2 * mu * s * (s * iG) * 2 * iG) * if1 * if1;
}

// XC_PBE! (src/XC/XC_PBE.jl:187-476) at one point: e = Exc[1] + Exc[2] (the
// energy per particle), v[s] = DEXDD[s] + DECDD[s], and dg[3 s + a] =
// DEXDGD + DECDGD, with g = (grad up, grad down).  SYM: the "off" case
// (equal spin densities and gradients), where both spins share one exchange
// evaluation and zeta = 0.
template <bool SYM>
__device__ __forceinline__ void xc_pbe_point(double d1, double d2, const double (&g)[6], double& e, double (&v)[2],
                                             double (&dg)[6]) {
  constexpr double beta = 0.06672455060314922;
  constexpr double gamma = 0.031090690869654901;  // (1 - ln 2) / pi^2
  constexpr double bg = beta / gamma;
  d1 = fmax(0.5 * kDenMin, d1);
  d2 = fmax(0.5 * kDenMin, d2);
  const double dt = d1 + d2;
  const double idt = 1.0 / dt;
  const double GDT0 = g[0] + g[3], GDT1 = g[1] + g[4], GDT2 = g[2] + g[5];
  const double GDMT = fmax(1e-14, sqrt(GDT0 * GDT0 + GDT1 * GDT1 + GDT2 * GDT2));

  double Ec, Vc1, Vc2, cz1, cz2;
  pw92c<SYM>(d1, d2, Ec, Vc1, Vc2, cz1, cz2);

  // correlation energy (:241-267)
  const double kF = 3.0936677262801355 * cbrt(dt);  // cbrt(3 pi^2 dt)
  const double ks = sqrt(4 * kF / kPi);
  double zeta = 0.0, phi = 1.0, DPDZ = 0.0;
  if (!SYM) {
    zeta = (d1 - d2) * idt;
    zeta = zeta > 0.99 ? 0.99 : zeta;
    zeta = zeta < -1.0 ? -0.99 : zeta;
    // pw92c's cube roots cbrt(1 +- zeta) are of this same clamped zeta (where
    // it reset the densities, zeta is 0 there and here)
    phi = 0.5 * (cz1 * cz1 + cz2 * cz2);
    DPDZ = (1.0 / 3.0) * (1.0 / cz1 - 1.0 / cz2);
  }
  const double iphi = 1.0 / phi;
  const double phi3 = phi * phi * phi;
  const double t = GDMT / (2 * phi * ks * dt);
  const double f1 = Ec / (gamma * phi3);
  const double f2 = exp(-f1);
  const double A = bg / (f2 - 1);
  const double t2 = t * t;
  const double f3 = t2 + A * t2 * t2;
  const double iAf3 = 1.0 / (1 + A * f3);
  const double f4 = bg * f3 * iAf3;
  const double if4 = 1.0 / (1 + f4);
  const double H = gamma * phi3 * log1p(f4);
  const double Fc = Ec + H;

  // correlation derivatives (:273-342)
  const double iks = 1.0 / ks;
  const double DKSDD = 0.5 * ks * (1.0 / 3.0) * idt;  // 0.5 ks DKFDD / kF, DKFDD = kF / (3 dt)
  const double if3 = 1.0 / f3;
  const double dt3 = 2 * t + 4 * A * t2 * t;
  const double iEc = 1.0 / Ec;
  const double if2m1 = 1.0 / (f2 - 1);
  double DFCDD[2];
#pragma unroll
  for (int is = 0; is < (SYM ? 1 : 2); ++is) {
    const double Vc = is == 0 ? Vc1 : Vc2;
    const double DZDD = is == 0 ? idt - zeta * idt : -idt - zeta * idt;
    const double DECUDD = (Vc - Ec) * idt;
    const double DPDD = DPDZ * DZDD;
    const double DTDD = (-t) * (DPDD * iphi + DKSDD * iks + idt);
    const double DF1DD = f1 * (DECUDD * iEc - 3 * DPDD * iphi);
    const double DF2DD = -f2 * DF1DD;
    const double DADD = -A * DF2DD * if2m1;
    const double DF3DD = dt3 * DTDD + DADD * t2 * t2;
    const double DF4DD = f4 * (DF3DD * if3 - (DADD * f3 + A * DF3DD) * iAf3);
    const double DHDD = 3 * H * DPDD * iphi + gamma * phi3 * DF4DD * if4;
    DFCDD[is] = Vc + H + dt * DHDD;
  }
  if (SYM) DFCDD[1] = DFCDD[0];
  // d Fc / d GDT_x = dt * gamma phi^3 f4 (1/f3 - A/(1 + A f3)) dt3 (t / GDMT^2) GDT_x / (1 + f4)
  const double iGT = 1.0 / GDMT;
  const double kc = dt * gamma * phi3 * f4 * (if3 - A * iAf3) * dt3 * (t * iGT) * iGT * if4;

  // exchange (:348-451)
  double fx0, dfx0, kx0, fx1, dfx1, kx1;
  pbe_x_spin(d1, g[0], g[1], g[2], fx0, dfx0, kx0);
  if (SYM) {
    fx1 = fx0;
    dfx1 = dfx0;
    kx1 = kx0;
  } else {
    pbe_x_spin(d2, g[3], g[4], g[5], fx1, dfx1, kx1);
  }
  const double Fx = 0.5 * (fx0 + fx1) * idt;
  e = Fx + Fc;
  v[0] = dfx0 + DFCDD[0];
  v[1] = dfx1 + DFCDD[1];
  // DEXDGD = DS Ex_unif DFDGD with GDS = 2 g: k * 2 g
  dg[0] = kx0 * g[0] + kc * GDT0;
  dg[1] = kx0 * g[1] + kc * GDT1;
  dg[2] = kx0 * g[2] + kc * GDT2;
  dg[3] = kx1 * g[3] + kc * GDT0;
  dg[4] = kx1 * g[4] + kc * GDT1;
  dg[5] = kx1 * g[5] + kc * GDT2;
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
