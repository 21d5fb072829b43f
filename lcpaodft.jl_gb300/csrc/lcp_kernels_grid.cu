// Pointwise grid kernels (FP64): Poisson source and reciprocal-space scaling,
// LDA/LSDA exchange-correlation, effective potential, and deterministic
// energy reductions.
#include <cuda_runtime.h>
#include <cuComplex.h>

#include "lcp_device.h"
#include "lcp_grid_common.cuh"
#include "lcp_pdl.cuh"

namespace lcp {

namespace {

constexpr double kPi = 3.14159265358979323846;

int grid_blocks(int64_t n, int threads) {
  int64_t b = (n + threads - 1) / threads;
  return (int)std::max<int64_t>(1, std::min<int64_t>(b, 152 * 32));
}

// ------------------------------------------------------------ Poisson

// Set_Density_xyz! (src/Poisson.jl:10-26): 2rho - 2rho_a ("off") or
// rho_up + rho_down - 2rho_a ("on", "nc"), as a real array.
__global__ void poisson_prep_kernel(int spinpol, int64_t nn, const double* __restrict__ r0,
                                    const double* __restrict__ r1, const double* __restrict__ aden,
                                    double* __restrict__ out) {
  for (int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; x < nn; x += (int64_t)gridDim.x * blockDim.x) {
    double a = aden ? aden[x] : 0.0;
    out[x] = spinpol == LCP_SPIN_OFF ? 2 * r0[x] - 2 * a : r0[x] + r1[x] - 2 * a;
  }
}

__device__ __forceinline__ int signed_freq(int i, int n) { return i < n / 2 ? i : i - n; }

__device__ __forceinline__ double inv_g2_scale(int i, int j, int k, const int* ng, const double* rv) {
  const int s1 = signed_freq(i, ng[0]), s2 = signed_freq(j, ng[1]), s3 = signed_freq(k, ng[2]);
  const double gx = s1 * rv[0] + s2 * rv[3] + s3 * rv[6];
  const double gy = s1 * rv[1] + s2 * rv[4] + s3 * rv[7];
  const double gz = s1 * rv[2] + s2 * rv[5] + s3 * rv[8];
  return 4 * kPi / (gx * gx + gy * gy + gz * gz);
}

// 4*pi/|G|^2 with the reference's signed frequencies s = i < N/2 ? i : i-N
// (src/Poisson.jl:60-76) on the R2C half spectrum, G = 0 set to zero, the
// inverse transform's 1/NN folded in.  The reference keeps the real part of a
// full complex inverse transform; with a real source that equals the C2R
// transform of the spectrum scaled by (S(k) + S(-k))/2.  For even N the two
// terms agree; for odd N the reference's map sends index (N-1)/2 to
// -(N+1)/2, and the average reproduces exactly what its real part keeps.
struct PoissonArgs {
  int ng[3];
  double rv[9];
  double inv_nn;
};
__global__ void poisson_scale_kernel(PoissonArgs a, cuDoubleComplex* __restrict__ spec) {
  const int N1 = a.ng[0], N2 = a.ng[1], N3 = a.ng[2];
  const int H3 = N3 / 2 + 1;
  const int64_t total = (int64_t)N1 * N2 * H3;
  for (int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; x < total; x += (int64_t)gridDim.x * blockDim.x) {
    const int k = (int)(x % H3);
    const int64_t ij = x / H3;
    const int j = (int)(ij % N2);
    const int i = (int)(ij / N2);
    double s;
    if (i == 0 && j == 0 && k == 0) {
      s = 0.0;
    } else {
      const int mi = (N1 - i) % N1, mj = (N2 - j) % N2, mk = (N3 - k) % N3;
      s = 0.5 * (inv_g2_scale(i, j, k, a.ng, a.rv) + inv_g2_scale(mi, mj, mk, a.ng, a.rv)) * a.inv_nn;
    }
    cuDoubleComplex v = spec[x];
    spec[x] = make_cuDoubleComplex(v.x * s, v.y * s);
  }
}

// ------------------------------------------------------------ exchange-correlation

// LSDA_CA (src/XC/LSDA_CA.jl:1-138): switch 0 (exc, both spins equal) and
// switch 1 (vxc up/down).
__device__ __forceinline__ void lsda_ca(double up, double dn, double& exc, double& vu, double& vd) {
  const double tden = up + dn;
  const double min_den = 1e-15;
  if (tden <= min_den) {
    exc = vu = vd = 0.0;
    return;
  }
  double zeta = (up - dn) / tden;
  zeta = zeta > 1.0 ? 1 - min_den : zeta;
  zeta = zeta < -1.0 ? -1 + min_den : zeta;
  const double coe = 0.6203504908994;
  const double rs = tden < min_den ? 62035.04908994 : coe * rcbrt(tden);
  const double tmp0 = 0.458165293632163 / rs;
  const double ExP = -tmp0, dExP = tmp0 / rs;
  const double ExF = 1.25992104989487 * ExP, dExF = 1.25992104989487 * dExP;
  double EcP, dEcP, EcF, dEcF;
  if (rs >= 1.0) {
    const double t = sqrt(rs);
    double dum = 1.0 + 1.0529 * t + 0.3334 * rs;
    double t1 = 0.1423 / dum;
    EcP = -t1;
    dEcP = t1 / dum * (0.52645 / t + 0.3334);
    dum = 1.0 + 1.3981 * t + 0.2611 * rs;
    t1 = 0.0843 / dum;
    EcF = -t1;
    dEcF = t1 / dum * (0.69905 / t + 0.2611);
  } else {
    const double lr = log(rs);
    EcP = -0.0480 + 0.0311 * lr + rs * (0.0020 * lr - 0.0116);
    dEcP = 0.0311 / rs + 0.0020 * lr - 0.0096;
    EcF = -0.0269 + 0.01555 * lr + rs * (0.0007 * lr - 0.0048);
    dEcF = 0.01555 / rs + 0.0007 * lr - 0.0041;
  }
  const double z0 = cbrt(1 + zeta), z1 = cbrt(1 - zeta);
  const double z02 = z0 * z0, z04 = z02 * z02, z12 = z1 * z1, z14 = z12 * z12;
  // switch 0 uses (1 +- zeta)^(4/3) directly
  const double fz0 = 1.92366105093154 * ((1 + zeta) * z0 + (1 - zeta) * z1 - 2.0);
  exc = ExP + EcP + (ExF + EcF - ExP - EcP) * fz0;
  const double fz = 1.92366105093154 * (z04 + z14 - 2.0);
  const double dfz = 2.56488140124205 * (z0 - z1);
  const double t0 = ExF + EcF - ExP - EcP;
  const double e1 = ExP + EcP + t0 * fz;
  const double de = dExP + dEcP + (dExF + dEcF - dExP - dEcP) * fz;
  const double v = e1 - 1.0 / 3.0 * rs * de;
  vu = v + t0 * (1 - zeta) * dfz;
  vd = v + t0 * (-1 - zeta) * dfz;
}

// LSDA_CA in double-float for the precision forms (as lda_ca_df): the same
// expressions, zeta from a refined reciprocal (exactly +-1 when a spin is
// empty), 1 +- zeta as 2 up / tden and 2 dn / tden, (1 +- zeta)^(1/3) as
// x rcbrt(x)^2, the rs < 1 logarithm in double-float, the results rounded to
// FP64 once.
__device__ __forceinline__ void lsda_ca_df(double up, double dn, double& exc, double& vu, double& vd) {
  const double tden = up + dn;
  const double min_den = 1e-15;
  if (tden <= min_den) {
    exc = vu = vd = 0.0;
    return;
  }
  const Dfl T = dfl_of(tden), iT = dfl_rcp(T);
  const Dfl U2 = dfl_of(up) * 2.0f, D2 = dfl_of(dn) * 2.0f;
  // one spin empty: zeta is exactly +-1, as the FP64 division gives it
  Dfl zeta = dn == 0.0 ? dflc(1.0) : (up == 0.0 ? dflc(-1.0) : dfl_of(up - dn) * iT);
  bool clamped = false;
  if (!(zeta < 1.0f) && !(zeta.hi == 1.0f && zeta.lo == 0.0f)) {
    zeta = dflc(1 - min_den);
    clamped = true;
  }
  if (zeta < -1.0f) {
    zeta = dflc(-1 + min_den);
    clamped = true;
  }
  const Dfl rs = dfl_rcbrt(T) * dflc(0.6203504908994);
  const Dfl irs = dfl_rcp(rs);
  const Dfl tmp0 = irs * dflc(0.458165293632163);
  const Dfl ExP = -tmp0, dExP = tmp0 * irs;
  const Dfl ExF = ExP * dflc(1.25992104989487), dExF = dExP * dflc(1.25992104989487);
  Dfl EcP, dEcP, EcF, dEcF;
  if (!(rs < 1.0f)) {
    const Dfl it = dfl_rsqrt(rs), t = rs * it;
    Dfl idum = dfl_rcp(dflc(1.0) + dot2(dflc(1.0529), t, dflc(0.3334), rs));
    Dfl t1 = idum * dflc(0.1423);
    EcP = -t1;
    dEcP = (t1 * idum) * dot2(dflc(0.52645), it, dflc(1.0), dflc(0.3334));
    idum = dfl_rcp(dflc(1.0) + dot2(dflc(1.3981), t, dflc(0.2611), rs));
    t1 = idum * dflc(0.0843);
    EcF = -t1;
    dEcF = (t1 * idum) * dot2(dflc(0.69905), it, dflc(1.0), dflc(0.2611));
  } else {
    const Dfl lr = dfl_log(rs);
    EcP = dflc(-0.0480) + dot2(dflc(0.0311), lr, rs, dot2(dflc(0.0020), lr, dflc(1.0), dflc(-0.0116)));
    dEcP = dot2(dflc(0.0311), irs, dflc(0.0020), lr) + dflc(-0.0096);
    EcF = dflc(-0.0269) + dot2(dflc(0.01555), lr, rs, dot2(dflc(0.0007), lr, dflc(1.0), dflc(-0.0048)));
    dEcF = dot2(dflc(0.01555), irs, dflc(0.0007), lr) + dflc(-0.0041);
  }
  // 1 +- zeta as 2 up / tden and 2 dn / tden (no cancellation near full
  // polarisation), from the clamped zeta where a negative spin density pushed it past 1
  const Dfl p1 = clamped ? dflc(1.0) + zeta : U2 * iT, m1 = clamped ? dflc(1.0) - zeta : D2 * iT;
  const Dfl z0 = dfl_cbrt(p1), z1 = dfl_cbrt(m1);  // (1 +- zeta)^(1/3)
  const Dfl z02 = z0 * z0, z04 = z02 * z02, z12 = z1 * z1, z14 = z12 * z12;
  const Dfl t0 = (ExF + EcF) - (ExP + EcP);
  // switch 0 uses (1 +- zeta)^(4/3) directly
  const Dfl fz0 = (dot2(p1, z0, m1, z1) - dflc(2.0)) * dflc(1.92366105093154);
  exc = dbl_of((ExP + EcP) + t0 * fz0);
  const Dfl fz = ((z04 + z14) - dflc(2.0)) * dflc(1.92366105093154);
  const Dfl dfz = (z0 - z1) * dflc(2.56488140124205);
  const Dfl e1 = (ExP + EcP) + t0 * fz;
  const Dfl de = (dExP + dEcP) + ((dExF + dEcF) - (dExP + dEcP)) * fz;
  const Dfl v = e1 - rs * de * dflc(1.0 / 3.0);
  const Dfl tz = t0 * dfz;
  vu = dbl_of(v + tz * m1);
  vd = dbl_of(v - tz * p1);
}

template <bool DF>
__device__ __forceinline__ void lsda_eval(double up, double dn, double& exc, double& vu, double& vd) {
  if (DF) lsda_ca_df(up, dn, exc, vu, vd);
  else lsda_ca(up, dn, exc, vu, vd);
}

struct XcArgs {
  int xc, spinpol;
  int64_t nn;
  const double* pcc;
  const double* rho[4];
  const double* dvh;
  const double* vna;
  double* vxc[4];
  double* vpot[4];
};

// Set_XC_Grid! (src/XC/XC_Func.jl:111-145) and, where vpot is given,
// Set_Vpot_Grid! (src/Matrix/Set_Vpot_Grid.jl:1-19) in the same pass.
__global__ void xc_vpot_kernel(XcArgs a) {
  for (int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; x < a.nn; x += (int64_t)gridDim.x * blockDim.x) {
    const double pc = a.pcc ? a.pcc[x] : 0.0;
    double v[4] = {0, 0, 0, 0};
    if (a.xc == LCP_XC_LDA) {
      double e;
      lda_ca(2 * (a.rho[0][x] + pc), e, v[0]);
    } else {
      double e;
      lsda_ca(a.rho[0][x] + pc, a.rho[1][x] + pc, e, v[0], v[1]);
      if (a.spinpol == LCP_SPIN_NC) {
        const double th = a.rho[2][x], ph = a.rho[3][x];
        const double t0 = 0.5 * (v[0] + v[1]), t1 = 0.5 * (v[0] - v[1]);
        v[3] = -t1 * sin(th) * sin(ph);
        v[2] = t1 * sin(th) * cos(ph);
        v[1] = t0 - t1 * cos(th);
        v[0] = t0 + t1 * cos(th);
      }
    }
    const int nv = a.spinpol == LCP_SPIN_OFF ? 1 : (a.spinpol == LCP_SPIN_ON ? 2 : 4);
    for (int c = 0; c < nv; ++c)
      if (a.vxc[c]) a.vxc[c][x] = v[c];
    if (a.vpot[0]) {
      const double dv = a.dvh[x];
      const double na = a.vna ? a.vna[x] : 0.0;
      for (int c = 0; c < nv; ++c) a.vpot[c][x] = c < 2 ? dv + v[c] + na : v[c];
    }
  }
}

struct VpotArgs {
  int spinpol;
  int64_t nn;
  const double* dvh;
  const double* vxc[4];
  const double* vna;
  double* vpot[4];
};
__global__ void vpot_kernel(VpotArgs a) {
  const int nv = a.spinpol == LCP_SPIN_OFF ? 1 : (a.spinpol == LCP_SPIN_ON ? 2 : 4);
  for (int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; x < a.nn; x += (int64_t)gridDim.x * blockDim.x) {
    const double na = a.vna ? a.vna[x] : 0.0;
    for (int c = 0; c < nv; ++c) a.vpot[c][x] = c < 2 ? a.dvh[x] + a.vxc[c][x] + na : a.vxc[c][x];
  }
}

// ------------------------------------------------------------ "nc" channels

// diagonalize_nc_density! (src/Matrix/Set_Density_Grid.jl:243-261): per point
// EulerAngle_Spin (src/utils/EulerAngle_Spin.jl:1-6) of the spin density
// matrix, through xyz_to_spherical (src/utils/xyz_to_spherical.jl:1-31) of
// (2 Re12, -2 Im12, Re11 - Re22).
__global__ void nc_diagonalize_kernel(int64_t nn, double* __restrict__ d0, double* __restrict__ d1,
                                      double* __restrict__ d2, double* __restrict__ d3) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nn; i += (int64_t)gridDim.x * blockDim.x) {
    const double re11 = d0[i], re22 = d1[i], re12 = d2[i], im12 = d3[i];
    const double x = 2 * re12, y = -2 * im12, z = re11 - re22;
    // each product and sum rounded on its own (no FMA contraction), as the
    // reference evaluates them: theta = acos(z/r) amplifies a 1-ulp change
    // of r near the poles to ~1e-8
    const double dum = __dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y));
    const double r = sqrt(__dadd_rn(dum, __dmul_rn(z, z)));
    const double r1 = sqrt(dum);
    double theta = 0.5 * kPi, phi = 0.0;
    if (1e-14 <= r) {
      const double c = r < fabs(z) ? (z > 0 ? 1.0 : (z < 0 ? -1.0 : 0.0)) : z / r;
      theta = acos(c);
      if (1e-14 <= r1) {
        const double sy = r1 < fabs(y) ? (y > 0 ? 1.0 : (y < 0 ? -1.0 : 0.0)) : y / r1;
        phi = x >= 0.0 ? asin(sy) : kPi - asin(sy);
      }
    }
    d0[i] = 0.5 * __dadd_rn(__dadd_rn(re11, re22), r);
    d1[i] = 0.5 * __dadd_rn(__dadd_rn(re11, re22), -r);
    d2[i] = theta;
    d3[i] = phi;
  }
}

// The "nc" potentials from the collinear pair (vu, vd) and the local angles;
// each point's inputs are read before its outputs are written, so out[0..1]
// may be the vu/vd buffers.
__global__ void nc_rotate_kernel(int64_t nn, const double* vu, const double* vd, const double* theta,
                                 const double* phi, double sign3, double* o0, double* o1, double* o2, double* o3) {
  for (int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; x < nn; x += (int64_t)gridDim.x * blockDim.x) {
    const double tmp0 = 0.5 * (vu[x] + vd[x]);
    const double tmp1 = 0.5 * (vu[x] - vd[x]);
    double sit, cot, sip, cop;
    sincos(theta[x], &sit, &cot);
    sincos(phi[x], &sip, &cop);
    o3[x] = -tmp1 * sit * sip;
    o2[x] = sign3 * tmp1 * sit * cop;
    o1[x] = tmp0 - cot * tmp1;
    o0[x] = tmp0 + cot * tmp1;
  }
}

struct EnergyArgs {
  int xc, spinpol;
  int64_t nn;
  const double* aden;
  const double* pcc;
  const double* rho[2];
  const double* dvh;
  double* partials;  // [red_tiles(nn)][3]
};

// Per-tile partial sums of the energy terms (one block per tile).
__global__ void __launch_bounds__(kRedThreads) energy_partials_kernel(EnergyArgs a) {
  double v[3] = {0, 0, 0};
  const int64_t x0 = (int64_t)blockIdx.x * kRedTile, x1 = min(a.nn, x0 + kRedTile);
  for (int64_t x = x0 + threadIdx.x; x < x1; x += kRedThreads) {
    const double ad = a.aden ? a.aden[x] : 0.0;
    const double pc = a.pcc ? a.pcc[x] : 0.0;
    const double r0 = a.rho[0][x];
    double e, vv, r1 = 0.0;
    if (a.xc == LCP_XC_LDA) {
      lda_ca(2 * (r0 + pc), e, vv);
    } else {
      double vd;
      r1 = a.rho[1][x];
      lsda_ca(r0 + pc, r1 + pc, e, vv, vd);
    }
    energy_terms(a.xc, a.spinpol, r0, r1, ad, pc, a.dvh ? a.dvh[x] : 0.0, e, v);
  }
  block_reduce_store<3>(v, a.partials + (size_t)blockIdx.x * 3);
}

template <int NV>
__global__ void __launch_bounds__(kRedThreads) finish_sums_kernel(const double* __restrict__ partials, int64_t nblocks,
                                                                  double* out) {
  double v[NV];
  for (int c = 0; c < NV; ++c) v[c] = 0.0;
  for (int64_t b = threadIdx.x; b < nblocks; b += blockDim.x)
    for (int c = 0; c < NV; ++c) v[c] += partials[b * NV + c];
  block_reduce_store<NV>(v, out);
}

struct GridArgs {
  GridCell cell0;
  GridBatch batch;
  int xc, spinpol, nspin;
};

// Poisson source 2rho - 2rho_a / rho_up + rho_down - 2rho_a (as
// poisson_prep_kernel), one tile of one cell per block.
__global__ void __launch_bounds__(kRedThreads) poisson_prep_g_kernel(const __grid_constant__ GridArgs a) {
  int64_t t;
  const GridCell& c = grid_cell(a.cell0, a.batch, blockIdx.x, t);
  const int64_t x0 = t * kRedTile, x1 = min(c.nn, x0 + kRedTile);
  const double* r0 = c.rho[0];
  const double* r1 = c.rho[1];
  const double* ad = c.aden;
  for (int64_t x = x0 + threadIdx.x; x < x1; x += kRedThreads) {
    const double aa = ad ? ad[x] : 0.0;
    c.real[x] = a.spinpol == LCP_SPIN_OFF ? 2 * r0[x] - 2 * aa : r0[x] + r1[x] - 2 * aa;
  }
}

// 4*pi/|G|^2 scaling of the half spectrum (as poisson_scale_kernel), one
// tile of one cell per block.
// The scale of half-spectrum element x of a cell (as poisson_scale_kernel).
__device__ __forceinline__ double poisson_factor(int64_t x, const int* ng, const double* rv, double inv_nn) {
  const int N1 = ng[0], N2 = ng[1], N3 = ng[2], H3 = N3 / 2 + 1;
  const int k = (int)(x % H3);
  const int64_t ij = x / H3;
  const int j = (int)(ij % N2);
  const int i = (int)(ij / N2);
  if (i == 0 && j == 0 && k == 0) return 0.0;
  const int mi = (N1 - i) % N1, mj = (N2 - j) % N2, mk = (N3 - k) % N3;
  return 0.5 * (inv_g2_scale(i, j, k, ng, rv) + inv_g2_scale(mi, mj, mk, ng, rv)) * inv_nn;
}

// A cell's Poisson factors, tabulated once: the step's scaling pass is then
// a streaming multiply instead of FP64 divisions per element.
__global__ void __launch_bounds__(kRedThreads) poisson_table_kernel(PoissonArgs a, double* __restrict__ out) {
  const int64_t total = (int64_t)a.ng[0] * a.ng[1] * (a.ng[2] / 2 + 1);
  for (int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; x < total; x += (int64_t)gridDim.x * blockDim.x)
    out[x] = poisson_factor(x, a.ng, a.rv, a.inv_nn);
}

__global__ void __launch_bounds__(kRedThreads) poisson_scale_g_kernel(const __grid_constant__ GridArgs a) {
  int64_t t;
  const GridCell& c = grid_cell(a.cell0, a.batch, blockIdx.x, t);
  if (c.pfac) {  // tabulated factors
    const int64_t total = (int64_t)c.ng[0] * c.ng[1] * (c.ng[2] / 2 + 1);
    const int64_t x0 = t * kRedTile, x1 = min(total, x0 + kRedTile);
    double2* spec = reinterpret_cast<double2*>(c.spec);
    for (int64_t x = x0 + threadIdx.x; x < x1; x += kRedThreads) {
      const double f = c.pfac[x];
      const double2 v = spec[x];
      spec[x] = make_double2(v.x * f, v.y * f);
    }
    return;
  }
  const int ng[3] = {c.ng[0], c.ng[1], c.ng[2]};
  double rv[9];
  for (int d = 0; d < 9; ++d) rv[d] = c.rv[d];
  const double inv_nn = 1.0 / ((double)ng[0] * ng[1] * ng[2]);
  const int64_t total = (int64_t)ng[0] * ng[1] * (ng[2] / 2 + 1);
  const int64_t x0 = t * kRedTile, x1 = min(total, x0 + kRedTile);
  cuDoubleComplex* spec = reinterpret_cast<cuDoubleComplex*>(c.spec);
  for (int64_t x = x0 + threadIdx.x; x < x1; x += kRedThreads) {
    const double s = poisson_factor(x, ng, rv, inv_nn);
    const cuDoubleComplex v = spec[x];
    spec[x] = make_cuDoubleComplex(v.x * s, v.y * s);
  }
}

// The grid step's fused pass: Set_XC_Grid! + Set_Vpot_Grid! (as
// xc_vpot_kernel) and the energy-term partial sums (as
// energy_partials_kernel, over the same tiles in the same order, so the sums
// are the same bits), evaluating the xc functional once per point.
// DF: the functional in double-float (the precision forms), FP64 otherwise.
template <bool DF>
__global__ void __launch_bounds__(kRedThreads) xc_vpot_energy_g_kernel(const __grid_constant__ GridArgs a) {
  int64_t t;
  const GridCell& c = grid_cell(a.cell0, a.batch, blockIdx.x, t);
  const int64_t x0 = t * kRedTile, x1 = min(c.nn, x0 + kRedTile);
  double acc[3] = {0, 0, 0};
  const int nv = a.spinpol == LCP_SPIN_OFF ? 1 : 2;
  for (int64_t x = x0 + threadIdx.x; x < x1; x += kRedThreads) {
    const double pc = c.pcc ? c.pcc[x] : 0.0;
    const double r0 = c.rho[0][x];
    double v[2] = {0, 0};
    double e, r1 = 0.0;
    if (a.xc == LCP_XC_LDA) {
      lda_eval<DF>(2 * (r0 + pc), e, v[0]);
    } else {
      r1 = c.rho[1][x];
      lsda_eval<DF>(r0 + pc, r1 + pc, e, v[0], v[1]);
    }
    if (c.dvh) {
      const double dvh = c.dvh[x];
      const double na = c.vna ? c.vna[x] : 0.0;
      for (int s = 0; s < nv; ++s) c.vpot[s][x] = dvh + v[s] + na;
      energy_terms<DF>(a.xc, a.spinpol, r0, r1, c.aden ? c.aden[x] : 0.0, pc, dvh, e, acc);
    } else {
      // ahead of the Hartree potential: vxc only, the E_H1 term left to vpot_eh_g_kernel
      for (int s = 0; s < nv; ++s) c.vpot[s][x] = v[s];
      energy_terms<DF>(a.xc, a.spinpol, r0, r1, c.aden ? c.aden[x] : 0.0, pc, 0.0, e, acc);
    }
  }
  block_reduce_store<3>(acc, c.part + t * 3);
}

// After an xc pass run without the Hartree potential (vpot holding vxc):
// vpot = dVHart + vxc + V_na and the E_H1 tile partials, over the same tiles
// and in the same order as the fused pass, so every sum keeps its bits.
__global__ void __launch_bounds__(kRedThreads) vpot_eh_g_kernel(const __grid_constant__ GridArgs a) {
  int64_t t;
  const GridCell& c = grid_cell(a.cell0, a.batch, blockIdx.x, t);
  const int64_t x0 = t * kRedTile, x1 = min(c.nn, x0 + kRedTile);
  double acc[1] = {0.0};
  const int nv = a.spinpol == LCP_SPIN_OFF ? 1 : 2;
  for (int64_t x = x0 + threadIdx.x; x < x1; x += kRedThreads) {
    const double dvh = c.dvh[x];
    const double na = c.vna ? c.vna[x] : 0.0;
    for (int s = 0; s < nv; ++s) c.vpot[s][x] = dvh + c.vpot[s][x] + na;
    const double r0 = c.rho[0][x];
    const double ad = c.aden ? c.aden[x] : 0.0;
    const double drho = a.spinpol == LCP_SPIN_OFF ? 2 * (r0 - ad) : r0 + c.rho[1][x] - 2 * ad;
    acc[0] += drho * dvh;
  }
  block_reduce_store<1>(acc, c.part + t * 3);
}

// Sums of each cell's energy tile partials: sums[0..2] (one block per cell).
__global__ void __launch_bounds__(kRedThreads) grid_sums_g_kernel(const __grid_constant__ GridArgs a) {
  pdl_trigger();
  pdl_wait();
  const GridCell& c = a.batch.cells ? a.batch.cells[blockIdx.x] : a.cell0;
  const int64_t nt = red_tiles(c.nn);
  double v[3] = {0, 0, 0};
  for (int64_t b = threadIdx.x; b < nt; b += blockDim.x)
    for (int k = 0; k < 3; ++k) v[k] += c.part[b * 3 + k];
  block_reduce_store<3>(v, c.sums);
}

// Tile partials of sum_s <D_s, H_s> (one block per tile of matrix entries).
__global__ void __launch_bounds__(kRedThreads) dot_g_kernel(const __grid_constant__ GridArgs a) {
  pdl_trigger();
  pdl_wait();
  int64_t t;
  const GridCell& c = grid_cell(a.cell0, a.batch, blockIdx.x, t);
  const int64_t x0 = t * kRedTile, x1 = min(c.hsize, x0 + kRedTile);
  double v[1] = {0.0};
  for (int s = 0; s < a.nspin; ++s) {
    const double* dm = c.dm[s];
    const double* hk = c.hks[s];
    for (int64_t x = x0 + threadIdx.x; x < x1; x += kRedThreads) v[0] += dm[x] * hk[x];
  }
  block_reduce_store<1>(v, c.part + t);
}

// sums[3] = sum_s <D_s, H_s> and the step's energies (one block per cell):
// sums[8..12] = E_H1, E_xc1 (up), E_xc1 (down), sum <D,H>,
// f_s sum <D,H> + E_H1 + E_xc1, with f_s = 2 for SpinPol "off".
__global__ void __launch_bounds__(kRedThreads) dot_energy_g_kernel(const __grid_constant__ GridArgs a) {
  pdl_trigger();
  pdl_wait();
  const GridCell& c = a.batch.cells ? a.batch.cells[blockIdx.x] : a.cell0;
  const int64_t nt = red_tiles(c.hsize);
  double v[1] = {0.0};
  for (int64_t b = threadIdx.x; b < nt; b += blockDim.x) v[0] += c.part[b];
  block_reduce_store<1>(v, c.sums + 3);
  if (threadIdx.x == 0) {
    double* sc = c.sums;
    const double eh1 = sc[0] * c.gridvol * 0.5;
    const double x1 = sc[1] * c.gridvol;
    const double x2 = a.spinpol == LCP_SPIN_OFF ? x1 : sc[2] * c.gridvol;
    const double fs = a.spinpol == LCP_SPIN_OFF ? 2.0 : 1.0;
    sc[8] = eh1;
    sc[9] = x1;
    sc[10] = x2;
    sc[11] = sc[3];
    sc[12] = fs * sc[3] + eh1 + x1 + x2;
  }
}

// FP64 FMA throughput probe: 8 independent dependency chains per thread.
__global__ void fp64_probe_kernel(double* out, int iters, double a, double b) {
  double x[8];
  for (int k = 0; k < 8; ++k) x[k] = threadIdx.x * 1e-3 + k;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = fma(x[k], a, b);
  }
  double s = 0;
  for (int k = 0; k < 8; ++k) s += x[k];
  if (s == 1234.5) out[0] = s;  // keeps the chains live
}

}  // namespace

cudaError_t launch_fp64_probe(double* out, int blocks, int threads, int iters, cudaStream_t st) {
  fp64_probe_kernel<<<blocks, threads, 0, st>>>(out, iters, 0.999999, 1e-7);
  return cudaGetLastError();
}

cudaError_t launch_poisson_prep(int spinpol, int64_t nn, const double* rho0, const double* rho1, const double* aden,
                                double* out, cudaStream_t st) {
  poisson_prep_kernel<<<grid_blocks(nn, 256), 256, 0, st>>>(spinpol, nn, rho0, rho1, aden, out);
  return cudaGetLastError();
}

cudaError_t launch_poisson_scale(const int32_t* ngrid, const double* recvecs, void* spectrum, cudaStream_t st) {
  PoissonArgs a;
  for (int d = 0; d < 3; ++d) a.ng[d] = ngrid[d];
  for (int d = 0; d < 9; ++d) a.rv[d] = recvecs[d];
  a.inv_nn = 1.0 / ((double)ngrid[0] * ngrid[1] * ngrid[2]);
  int64_t total = (int64_t)ngrid[0] * ngrid[1] * (ngrid[2] / 2 + 1);
  poisson_scale_kernel<<<grid_blocks(total, 256), 256, 0, st>>>(a, reinterpret_cast<cuDoubleComplex*>(spectrum));
  return cudaGetLastError();
}

cudaError_t launch_xc_vpot(int xc, int spinpol, int64_t nn, const double* pcc, const double* const* rho,
                           const double* dvh, const double* vna, double* const* vxc_out, double* const* vpot_out,
                           cudaStream_t st) {
  XcArgs a{};
  a.xc = xc;
  a.spinpol = spinpol;
  a.nn = nn;
  a.pcc = pcc;
  const int nr = spinpol == LCP_SPIN_OFF ? 1 : (spinpol == LCP_SPIN_ON ? 2 : 4);
  for (int c = 0; c < nr; ++c) {
    a.rho[c] = rho[c];
    a.vxc[c] = vxc_out ? vxc_out[c] : nullptr;
    a.vpot[c] = vpot_out ? vpot_out[c] : nullptr;
  }
  a.dvh = dvh;
  a.vna = vna;
  xc_vpot_kernel<<<grid_blocks(nn, 256), 256, 0, st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_vpot(int spinpol, int64_t nn, const double* dvh, const double* const* vxc, const double* vna,
                        double* const* vpot, cudaStream_t st) {
  VpotArgs a{};
  a.spinpol = spinpol;
  a.nn = nn;
  a.dvh = dvh;
  a.vna = vna;
  const int nv = spinpol == LCP_SPIN_OFF ? 1 : (spinpol == LCP_SPIN_ON ? 2 : 4);
  for (int c = 0; c < nv; ++c) {
    a.vxc[c] = vxc[c];
    a.vpot[c] = vpot[c];
  }
  vpot_kernel<<<grid_blocks(nn, 256), 256, 0, st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_energy_sums(int xc, int spinpol, int64_t nn, const double* aden, const double* pcc,
                               const double* const* rho, const double* dvh, double* partials, double* out,
                               cudaStream_t st) {
  EnergyArgs a{};
  a.xc = xc;
  a.spinpol = spinpol;
  a.nn = nn;
  a.aden = aden;
  a.pcc = pcc;
  a.rho[0] = rho[0];
  a.rho[1] = spinpol == LCP_SPIN_OFF ? nullptr : rho[1];
  a.dvh = dvh;
  a.partials = partials;
  const int64_t nt = red_tiles(nn);
  energy_partials_kernel<<<(unsigned)nt, kRedThreads, 0, st>>>(a);
  LCP_CUDA_TRY(cudaGetLastError());
  finish_sums_kernel<3><<<1, kRedThreads, 0, st>>>(partials, nt, out);
  return cudaGetLastError();
}

cudaError_t launch_nc_diagonalize(int64_t nn, double* const* rho, cudaStream_t st) {
  nc_diagonalize_kernel<<<grid_blocks(nn, 256), 256, 0, st>>>(nn, rho[0], rho[1], rho[2], rho[3]);
  return cudaGetLastError();
}

cudaError_t launch_nc_rotate(int64_t nn, const double* vu, const double* vd, const double* theta, const double* phi,
                             double sign3, double* const* out, cudaStream_t st) {
  nc_rotate_kernel<<<grid_blocks(nn, 256), 256, 0, st>>>(nn, vu, vd, theta, phi, sign3, out[0], out[1], out[2],
                                                         out[3]);
  return cudaGetLastError();
}

namespace {
GridArgs grid_args(const GridCell& c0, const GridBatch& b, int xc, int spinpol, int nspin) {
  GridArgs a;
  a.cell0 = c0;
  a.batch = b;
  a.xc = xc;
  a.spinpol = spinpol;
  a.nspin = nspin;
  return a;
}
// blocks of a tiled launch: the batch's total, or the single cell's tiles
unsigned tiled_blocks(const GridBatch& b, int64_t single) { return (unsigned)(b.cells ? b.nblocks : single); }
unsigned cell_blocks(const GridBatch& b) { return (unsigned)(b.cells ? b.ncells : 1); }
int64_t spec_size(const GridCell& c) { return (int64_t)c.ng[0] * c.ng[1] * (c.ng[2] / 2 + 1); }
}  // namespace

cudaError_t launch_poisson_prep_g(int spinpol, const GridCell& c0, const GridBatch& b, cudaStream_t st) {
  const unsigned n = tiled_blocks(b, red_tiles(c0.nn));
  if (n == 0) return cudaSuccess;
  poisson_prep_g_kernel<<<n, kRedThreads, 0, st>>>(grid_args(c0, b, 0, spinpol, 0));
  return cudaGetLastError();
}

cudaError_t launch_poisson_table(const int32_t* ngrid, const double* recvecs, double* out, cudaStream_t st) {
  PoissonArgs a;
  for (int d = 0; d < 3; ++d) a.ng[d] = ngrid[d];
  for (int d = 0; d < 9; ++d) a.rv[d] = recvecs[d];
  a.inv_nn = 1.0 / ((double)ngrid[0] * ngrid[1] * ngrid[2]);
  const int64_t total = (int64_t)ngrid[0] * ngrid[1] * (ngrid[2] / 2 + 1);
  poisson_table_kernel<<<grid_blocks(total, kRedThreads), kRedThreads, 0, st>>>(a, out);
  return cudaGetLastError();
}

cudaError_t launch_poisson_scale_g(const GridCell& c0, const GridBatch& b, cudaStream_t st) {
  const unsigned n = tiled_blocks(b, red_tiles(spec_size(c0)));
  if (n == 0) return cudaSuccess;
  poisson_scale_g_kernel<<<n, kRedThreads, 0, st>>>(grid_args(c0, b, 0, 0, 0));
  return cudaGetLastError();
}

cudaError_t launch_xc_vpot_energy_g(int xc, int spinpol, const GridCell& c0, const GridBatch& b, bool dfl,
                                    cudaStream_t st) {
  const unsigned n = tiled_blocks(b, red_tiles(c0.nn));
  if (n == 0) return cudaSuccess;
  if (dfl)
    xc_vpot_energy_g_kernel<true><<<n, kRedThreads, 0, st>>>(grid_args(c0, b, xc, spinpol, 0));
  else
    xc_vpot_energy_g_kernel<false><<<n, kRedThreads, 0, st>>>(grid_args(c0, b, xc, spinpol, 0));
  return cudaGetLastError();
}

// Per point: the LDA (xc LCP_XC_LDA, density 2 (up + pcc)) or LSDA functional
// in FP64 or double-float: out[3 x] = exc, out[3 x + 1..2] = vxc (up, down).
template <bool DF>
__global__ void xc_selftest_kernel(int xc, int64_t nn, const double* up, const double* dn, const double* pcc,
                                   double* out) {
  for (int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; x < nn; x += (int64_t)gridDim.x * blockDim.x) {
    const double pc = pcc ? pcc[x] : 0.0;
    double e, v0, v1 = 0.0;
    if (xc == LCP_XC_LDA) lda_eval<DF>(2 * (up[x] + pc), e, v0);
    else lsda_eval<DF>(up[x] + pc, dn[x] + pc, e, v0, v1);
    out[3 * x] = e;
    out[3 * x + 1] = v0;
    out[3 * x + 2] = v1;
  }
}

cudaError_t launch_xc_selftest(int xc, bool dfl, int64_t nn, const double* up, const double* dn, const double* pcc,
                               double* out, cudaStream_t st) {
  if (nn <= 0) return cudaSuccess;
  const unsigned g = grid_blocks(nn, 256);
  if (dfl) xc_selftest_kernel<true><<<g, 256, 0, st>>>(xc, nn, up, dn, pcc, out);
  else xc_selftest_kernel<false><<<g, 256, 0, st>>>(xc, nn, up, dn, pcc, out);
  return cudaGetLastError();
}

cudaError_t launch_vpot_eh_g(int spinpol, const GridCell& c0, const GridBatch& b, cudaStream_t st) {
  const unsigned n = tiled_blocks(b, red_tiles(c0.nn));
  if (n == 0) return cudaSuccess;
  vpot_eh_g_kernel<<<n, kRedThreads, 0, st>>>(grid_args(c0, b, 0, spinpol, 0));
  return cudaGetLastError();
}

cudaError_t launch_grid_sums_g(const GridCell& c0, const GridBatch& b, cudaStream_t st) {
  return launch_pdl(grid_sums_g_kernel, dim3(cell_blocks(b)), dim3(kRedThreads), 0, st, grid_args(c0, b, 0, 0, 0));
}

cudaError_t launch_dot_energy_g(int spinpol, int nspin, const GridCell& c0, const GridBatch& tiles,
                                const GridBatch& cells, cudaStream_t st) {
  const unsigned n = tiled_blocks(tiles, red_tiles(c0.hsize));
  if (n > 0) {
    LCP_CUDA_TRY(launch_pdl(dot_g_kernel, dim3(n), dim3(kRedThreads), 0, st, grid_args(c0, tiles, 0, spinpol, nspin)));
  }
  return launch_pdl(dot_energy_g_kernel, dim3(cell_blocks(cells)), dim3(kRedThreads), 0, st,
                    grid_args(c0, cells, 0, spinpol, nspin));
}

}  // namespace lcp
