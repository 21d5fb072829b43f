// Device helpers shared by the grid kernels: the LDA functional, the
// deterministic tile reductions, the cell lookup of batched launches and the
// per-point energy terms.
#pragma once
#include <cuda_runtime.h>

#include "lcp_device.h"
#include "lcp_dfloat.cuh"

namespace lcp {
namespace {

// LDA_CA (src/XC/LDA_CA.jl:4-41): exc (switch 0) and vxc (switch 1).
__device__ __forceinline__ void lda_ca(double den, double& exc, double& vxc) {
  if (den <= 1e-15) {
    exc = 0.0;
    vxc = 0.0;
    return;
  }
  // The reference's expressions with the divisions by rs, sqrt(rs) and the
  // correlation denominator each taken once as a reciprocal (FP64 division is
  // a multi-instruction sequence on this GPU's narrow FP64 pipe).
  const double coe = 0.6203504908994;
  const double rs = coe * rcbrt(den);
  const double irs = 1.0 / rs;
  const double tmp0 = 0.458165293632163 * irs;
  const double Ex = -tmp0, dEx = tmp0 * irs;
  double Ec, dEc;
  if (rs >= 1.0) {
    const double it = rsqrt(rs), t = rs * it;
    const double dum = 1.0 + 1.0529 * t + 0.3334 * rs;
    const double idum = 1.0 / dum;
    const double t1 = 0.1423 * idum;
    Ec = -t1;
    dEc = t1 * idum * (0.52645 * it + 0.3334);
  } else {
    const double lr = log(rs);
    Ec = -0.0480 + 0.0311 * lr + rs * (0.0020 * lr - 0.0116);
    dEc = 0.0311 * irs + 0.0020 * lr - 0.0096;
  }
  exc = Ex + Ec;
  vxc = Ex + Ec - 1.0 / 3.0 * rs * (dEx + dEc);
}

// The same functional in double-float for the precision forms: rs from the
// Newton-refined reciprocal cube root, the reciprocals, the square root and
// the logarithm of the rs < 1 branch refined the same way (lcp_dfloat.cuh),
// the results rounded to FP64 once.  It agrees with the FP64 evaluation to
// about 2^-45 relative and issues a few FP64 instructions (conversions back,
// the density test) instead of about a hundred.
__device__ __forceinline__ void lda_ca_df(double den, double& exc, double& vxc) {
  if (den <= 1e-15) {
    exc = 0.0;
    vxc = 0.0;
    return;
  }
  const Dfl rs = dfl_rcbrt(dfl_of(den)) * dflc(0.6203504908994);
  const Dfl irs = dfl_rcp(rs);
  const Dfl tmp0 = irs * dflc(0.458165293632163);
  const Dfl Ex = -tmp0, dEx = tmp0 * irs;
  Dfl Ec, dEc;
  if (!(rs < 1.0f)) {
    const Dfl it = dfl_rsqrt(rs), t = rs * it;
    const Dfl dum = dflc(1.0) + dot2(dflc(1.0529), t, dflc(0.3334), rs);
    const Dfl idum = dfl_rcp(dum);
    const Dfl t1 = idum * dflc(0.1423);
    Ec = -t1;
    dEc = (t1 * idum) * dot2(dflc(0.52645), it, dflc(1.0), dflc(0.3334));
  } else {
    const Dfl lr = dfl_log(rs);
    Ec = dflc(-0.0480) + dot2(dflc(0.0311), lr, rs, dot2(dflc(0.0020), lr, dflc(1.0), dflc(-0.0116)));
    dEc = dot2(dflc(0.0311), irs, dflc(0.0020), lr) + dflc(-0.0096);
  }
  const Dfl e = Ex + Ec;
  exc = dbl_of(e);
  vxc = dbl_of(e - rs * (dEx + dEc) * dflc(1.0 / 3.0));
}

template <bool DF>
__device__ __forceinline__ void lda_eval(double den, double& exc, double& vxc) {
  if (DF) lda_ca_df(den, exc, vxc);
  else lda_ca(den, exc, vxc);
}

// ------------------------------------------------------------ deterministic reductions
//
// Every reduction runs over fixed tiles of kRedTile points (or matrix
// entries): one block per tile, thread t summing the tile's elements t,
// t + 256, ... in order, then a fixed tree over the block; one block per cell
// then sums the cell's tile partials the same way.  The partition depends only
// on the cell's own sizes, so a cell's sums are the same bits whether it runs
// alone or in a batch of cells.

constexpr int kRedThreads = 256;

template <int NV>
__device__ __forceinline__ void block_reduce_store(double (&v)[NV], double* out) {
  __shared__ double sh[NV][kRedThreads];
  for (int c = 0; c < NV; ++c) sh[c][threadIdx.x] = v[c];
  __syncthreads();
  for (int s = kRedThreads / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s)
      for (int c = 0; c < NV; ++c) sh[c][threadIdx.x] += sh[c][threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int c = 0; c < NV; ++c) out[c] = sh[c][0];
}

// Cell and cell-local block of block g of a grid launch.
__device__ __forceinline__ const GridCell& grid_cell(const GridCell& c0, const GridBatch& b, int64_t g, int64_t& lb) {
  if (!b.cells) {
    lb = g;
    return c0;
  }
  int lo = 0, hi = b.ncells;  // cell with start[lo] <= g < start[lo+1]
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (b.start[mid] <= g) lo = mid;
    else hi = mid;
  }
  lb = g - b.start[lo];
  return b.cells[lo];
}

// Calc_EH1 (src/Energy.jl:655-666) and Calc_EXC1 (src/Energy.jl:669-700, with
// Calc_Vxc_Grid switch 0 of src/XC/XC_Func.jl:164-189) terms of one point;
// e is the xc energy density at the point's density (DF: the atomic
// density's LDA term in double-float, as the precision forms' xc pass).
template <bool DF = false>
__device__ __forceinline__ void energy_terms(int xc, int spinpol, double r0, double r1, double ad, double pc,
                                             double dvh, double e, double (&acc)[3]) {
  const double drho = spinpol == LCP_SPIN_OFF ? 2 * (r0 - ad) : r0 + r1 - 2 * ad;
  acc[0] += drho * dvh;
  const double temp = ad + pc;
  double eat, vat;
  lda_eval<DF>(2 * temp, eat, vat);
  acc[1] += (r0 + pc) * e - temp * eat;
  if (xc != LCP_XC_LDA) acc[2] += (r1 + pc) * e - temp * eat;
}

}  // namespace
}  // namespace lcp
