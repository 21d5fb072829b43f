// Pseudo-atomic orbital tabulation on the grid (FP64).
//
//   phi_{l,p,m}(r) = R_{lp}(|r - tau|) * Y_lm(angles of r - tau)
//
// on every point of each atom's cutoff-sphere list, and with GRAD the
// gradient tables of Set_dOrbitals_Grid.  Follows
// src/Matrix/Set_Orbitals_Grid.jl:94-274 and
// src/Matrix/Set_dOrbitals_Grid.jl:88-359: the same radial spline (binary
// search on the PAO log mesh + 4-point Hermite cubic, polynomial extrapolation
// below RV[1], zero beyond RV[end]), real Y_lm for l <= 3 in the reference's
// m order, and the reference's derivative chain rule with the 1e-13 shift of
// points that sit on the atom.
//
// The angles enter only through sin/cos, which are taken from the Cartesian
// components (sin(theta) = r_xy/r, cos(phi) = x/r_xy, ...) instead of
// acos/asin followed by sin/cos; the edge conventions of
// src/utils/xyz_to_spherical.jl (r < 1e-14: theta = pi/2, phi = 0;
// r_xy < 1e-14: phi = 0) are kept.
//
// The value tables (tabulate_values_kernel) take the spline from per-interval
// cubic coefficients computed once per species on the host (the same Hermite
// interpolant: value and slope at both mesh nodes of the interval, written as
// c0 + c1 u + c2 u^2 + c3 u^3 in u = (R - RV[m-1]) / (RV[m] - RV[m-1])), find
// the interval from a table of log2(R) buckets and a short forward scan
// instead of a binary search, and form Y_lm from the unit vector (x, y, z)/R.
// That takes the FP64 work per point from the spline's divisions and the
// per-function Hermite set-up to one Horner evaluation per radial function.
// The gradient tables keep the reference's per-point evaluation.
//
// One thread per sphere point; a block stages its points x NO values per
// table in shared memory and writes them back as contiguous, 16-byte
// vectorised stores (the table is point-major, NO values per point).
#include <cuda_runtime.h>

#include <cmath>
#include <vector>

#include "lcp_device.h"

namespace lcp {

namespace {

constexpr int kTabPoints = 64;
constexpr double kPi = 3.14159265358979323846;

// Real spherical harmonics of one l in the orbital order of
// src/Matrix/Set_Orbitals_Grid.jl:242-268 (src/utils/Ylm_real.jl:1-53) and
// their theta / phi derivatives (src/utils/Ylm_real.jl:56-162).
template <bool GRAD>
__device__ __forceinline__ void ylm_l(int l, double siQ, double coQ, double siP, double coP, double* Y,
                                      double* dQ, double* dP) {
  const double pi = kPi;
  if (l == 0) {
    Y[0] = 0.5 * sqrt(1 / pi);
    if (GRAD) {
      dQ[0] = 0.0;
      dP[0] = 0.0;
    }
  } else if (l == 1) {
    const double c = sqrt(3 / 4.0 / pi);
    Y[0] = c * siQ * coP;  // px (m = 1)
    Y[1] = c * siQ * siP;  // py (m = -1)
    Y[2] = c * coQ;        // pz (m = 0)
    if (GRAD) {
      dQ[0] = c * coQ * coP;
      dQ[1] = c * coQ * siP;
      dQ[2] = -c * siQ;
      dP[0] = -c * siP;
      dP[1] = c * coP;
      dP[2] = 0.0;
    }
  } else if (l == 2) {
    const double s = sqrt(15 / pi);
    Y[0] = 0.25 * sqrt(5 / pi) * (3 * coQ * coQ - 1);          // m = 0
    Y[1] = 0.25 * s * siQ * siQ * (1 - 2 * siP * siP);         // m = 2
    Y[2] = 0.5 * s * siQ * siQ * siP * coP;                    // m = -2
    Y[3] = 0.5 * s * siQ * coQ * coP;                          // m = 1
    Y[4] = 0.5 * s * siQ * coQ * siP;                          // m = -1
    if (GRAD) {
      dQ[0] = -1.5 * sqrt(5 / pi) * siQ * coQ;
      dQ[1] = 0.5 * s * siQ * coQ * (1 - 2 * siP * siP);
      dQ[2] = s * siQ * coQ * siP * coP;
      dQ[3] = 0.5 * s * (1 - 2 * siQ * siQ) * coP;
      dQ[4] = 0.5 * s * (1 - 2 * siQ * siQ) * siP;
      dP[0] = 0.0;
      dP[1] = -s * siQ * siP * coP;
      dP[2] = 0.5 * s * siQ * (1 - 2 * siP * siP);
      dP[3] = -0.5 * s * coQ * siP;
      dP[4] = 0.5 * s * coQ * coP;
    }
  } else {
    const double a = sqrt(35 / 2.0 / pi), b = sqrt(105 / pi), c = sqrt(21 / 2.0 / pi), d = sqrt(7 / pi);
    Y[0] = 0.25 * d * (5 * coQ * coQ * coQ - 3 * coQ);                          // m = 0
    Y[1] = 0.25 * c * siQ * (5 * coQ * coQ - 1) * coP;                          // m = 1
    Y[2] = 0.25 * c * siQ * (5 * coQ * coQ - 1) * siP;                          // m = -1
    Y[3] = 0.25 * b * siQ * siQ * coQ * (coP * coP - siP * siP);                // m = 2
    Y[4] = 0.5 * b * siQ * siQ * coQ * siP * coP;                               // m = -2
    Y[5] = 0.25 * a * siQ * siQ * siQ * (4 * coP * coP * coP - 3 * coP);        // m = 3
    Y[6] = 0.25 * a * siQ * siQ * siQ * (3 * siP - 4 * siP * siP * siP);        // m = -3
    if (GRAD) {
      dQ[0] = 0.25 * d * siQ * (-15 * coQ * coQ + 3);
      dQ[1] = 0.25 * c * coP * coQ * (15 * coQ * coQ - 11);
      dQ[2] = 0.25 * c * siP * coQ * (15 * coQ * coQ - 11);
      dQ[3] = 0.25 * b * (coP * coP - siP * siP) * siQ * (2 * coQ * coQ - siQ * siQ);
      dQ[4] = 0.5 * b * coP * siP * siQ * (2 * coQ * coQ - siQ * siQ);
      dQ[5] = 0.75 * a * coP * coQ * siQ * siQ * (-3 + 4 * coP * coP);
      dQ[6] = 0.75 * a * siQ * siQ * coQ * siP * (3 - 4 * siP * siP);
      dP[0] = 0.0;
      dP[1] = 0.25 * c * siP * (-5 * coQ * coQ + 1);
      dP[2] = 0.25 * c * coP * (5 * coQ * coQ - 1);
      dP[3] = -b * coP * coQ * siP * siQ;
      dP[4] = 0.5 * b * coQ * siQ * (coP * coP - siP * siP);
      dP[5] = 0.75 * a * siP * siQ * siQ * (1 - 4 * coP * coP);
      dP[6] = 0.75 * a * coP * siQ * siQ * (1 - 4 * siP * siP);
    }
  }
}

// xyz_to_spherical (src/utils/xyz_to_spherical.jl:1-31) expressed through
// sin/cos of the angles.
__device__ __forceinline__ void spherical_trig(double x, double y, double z, double& r, double& siQ,
                                               double& coQ, double& siP, double& coP) {
  const double min_r = 1e-14;
  double dum = x * x + y * y;
  r = sqrt(dum + z * z);
  double r1 = sqrt(dum);
  if (min_r <= r) {
    coQ = (r < fabs(z)) ? copysign(1.0, z) : z / r;
    siQ = (r < fabs(z)) ? 0.0 : r1 / r;
    if (min_r <= r1) {
      siP = (r1 < fabs(y)) ? copysign(1.0, y) : y / r1;
      coP = (r1 < fabs(y)) ? 0.0 : x / r1;
    } else {
      siP = 0.0;
      coP = 1.0;
    }
  } else {
    // theta = pi/2, phi = 0
    siQ = 1.0;
    coQ = 6.123233995736766e-17;  // cos(pi/2) in double precision
    siP = 0.0;
    coP = 1.0;
  }
}

// Values (WPHI) and/or gradients (WGRAD) of one point's orbitals, written to
// the staging rows.  (R, siQ, coQ, siP, coP) describe the point relative to
// the atom.
template <bool WPHI, bool WGRAD>
__device__ __forceinline__ void eval_point(const DevSpecies& sp, const double* __restrict__ rv,
                                           const double* __restrict__ rwf, double R, double siQ, double coQ,
                                           double siP, double coP, double* srow, double* sx, double* sy,
                                           double* sz) {
  const int n = sp.nmesh;
  const bool outside = rv[n - 1] < R;
  const bool inner = R < rv[0];

  // spline geometry (src/Matrix/Set_Orbitals_Grid.jl:187-214); below RV[1]
  // the geometry of 0-based mesh point 4 (:126-145)
  int m = 0;
  double h1 = 0, h2 = 1, h3 = 0, y1 = 0, y2 = 0, dum1 = 0, dum2 = 0, dum3 = 0, dum4 = 0;
  const int me = 4;
  const double rm = rv[me];
  if (!outside) {
    if (inner) {
      m = me;
    } else {
      int lo = 1, hi = n - 1;  // first index >= 1 with rv[idx] >= R
      while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (rv[mid] < R) lo = mid + 1;
        else hi = mid;
      }
      m = min(max(lo, 2), n - 2);
    }
    h1 = rv[m - 1] - rv[m - 2];
    h2 = rv[m] - rv[m - 1];
    h3 = rv[m + 1] - rv[m];
    const double xr = inner ? rm : R;
    y1 = (xr - rv[m - 1]) / h2;
    y2 = (xr - rv[m]) / h2;
    double dum = h1 + h2;
    dum1 = h1 / h2 / dum;
    dum2 = h2 / h1 / dum;
    dum = h2 + h3;
    dum3 = h2 / h3 / dum;
    dum4 = h3 / h2 / dum;
  }
  const double y12 = y1 * y1, y22 = y2 * y2;

  double dRx = 0, dRy = 0, dRz = 0, dQx = 0, dQy = 0, dQz = 0, dPx = 0, dPy = 0;
  if (WGRAD && !outside) {  // src/Matrix/Set_dOrbitals_Grid.jl:257-280
    dRx = siQ * coP;
    dRy = siQ * siP;
    dRz = coQ;
    if (R > 1.0e-13) {
      dQx = coQ * coP / R;
      dQy = coQ * siP / R;
      dQz = -siQ / R;
      dPx = -siP / R;
      dPy = coP / R;
    }
  }

  int ist = 0;
  int rad = 0;
  for (int l = 0; l <= sp.max_l; ++l) {
    double Y[7], dQ[7], dP[7];
    ylm_l<WGRAD>(l, siQ, coQ, siP, coP, Y, dQ, dP);
    for (int p = 0; p < sp.nb[l]; ++p, ++rad) {
      const double* w = rwf + (size_t)rad * n;
      double rf = 0.0, drf = 0.0, rfd = 0.0;
      if (!outside) {
        const double f1 = w[m - 2], f2 = w[m - 1], f3 = w[m];
        double f4 = w[m + 1];
        const double dum = f3 - f2;
        const double g1 = dum * dum1 + (f2 - f1) * dum2;
        double g2 = (f4 - f3) * dum3 + dum * dum4;
        const double A = 3 * f2 + h2 * g1, B = 2 * f2 + h2 * g1;
        double C = 3 * f3 - h2 * g2, D = 2 * f3 - h2 * g2;
        const double E = A + B * y2;
        double F = C - D * y1;
        const double f = y22 * E + y12 * F;
        if (inner) {
          // Set_Orbitals_Grid's derivative expression (:165) and
          // Set_dOrbitals_Grid's (:168) round differently; each table uses its own
          for (int which = 0; which < 2; ++which) {
            if ((which == 0 && !WPHI) || (which == 1 && !WGRAD)) continue;
            const double df = which == 0
                                  ? (2 * y2 / h2) * E + y22 * B / h2 + (2 * y1 / h2) * F - y12 * D / h2
                                  : (2 * y2 * E + y22 * B + 2.0 * y1 * F - y12 * D) / h2;
            double a, b, c, d;
            if (l == 0) {
              a = 0.0; b = 0.5 * df / rm; c = 0.0; d = f - b * (rm * rm);
            } else if (l == 1) {
              a = (rm * df - f) / (2 * (rm * rm * rm)); b = 0.0; c = df - 3 * a * (rm * rm); d = 0.0;
            } else {
              b = (3 * f - rm * df) / (rm * rm); a = (f - b * (rm * rm)) / (rm * rm * rm); c = 0.0; d = 0.0;
            }
            const double val = a * (R * R * R) + b * (R * R) + c * R + d;
            if (which == 0) {
              rf = val;
            } else {
              rfd = val;
              drf = 3 * a * (R * R) + 2 * b * R + c;
            }
          }
        } else {
          rfd = f;
          if (WGRAD) drf = (2 * y2 * E + y22 * B + 2.0 * y1 * F - y12 * D) / h2;
          if (WPHI && m == n - 2) {
            // Set_Orbitals_Grid substitutes f4 = f1 here (:226-229)
            f4 = f1;
            g2 = (f4 - f3) * dum3 + dum * dum4;
            C = 3 * f3 - h2 * g2;
            D = 2 * f3 - h2 * g2;
            F = C - D * y1;
            rf = y22 * E + y12 * F;
          } else {
            rf = f;
          }
        }
      }
      for (int mm = 0; mm < 2 * l + 1; ++mm, ++ist) {
        if (WPHI) srow[ist] = outside ? 0.0 : rf * Y[mm];
        if (WGRAD) {
          const double dchidr = drf * Y[mm];
          const double dchidt = rfd * dQ[mm];
          const double dchidp = rfd * dP[mm];
          sx[ist] = outside ? 0.0 : -dRx * dchidr - dQx * dchidt - dPx * dchidp;
          sy[ist] = outside ? 0.0 : -dRy * dchidr - dQy * dchidt - dPy * dchidp;
          sz[ist] = outside ? 0.0 : -dRz * dchidr - dQz * dchidt;
        }
      }
    }
  }
}

// Real Y_lm of one l in the orbital order of src/Matrix/Set_Orbitals_Grid.jl:242-268
// (src/utils/Ylm_real.jl:1-53), from the unit vector u = (x, y, z) / R:
// sin(theta) cos(phi) = ux, sin(theta) sin(phi) = uy, cos(theta) = uz.
__device__ __forceinline__ void ylm_unit(int l, double ux, double uy, double uz, double* Y) {
  const double pi = kPi;
  if (l == 0) {
    Y[0] = 0.5 * sqrt(1 / pi);
  } else if (l == 1) {
    const double c = sqrt(3 / 4.0 / pi);
    Y[0] = c * ux;
    Y[1] = c * uy;
    Y[2] = c * uz;
  } else if (l == 2) {
    const double s = sqrt(15 / pi);
    Y[0] = 0.25 * sqrt(5 / pi) * (3 * uz * uz - 1);
    Y[1] = 0.25 * s * (ux * ux - uy * uy);
    Y[2] = 0.5 * s * ux * uy;
    Y[3] = 0.5 * s * ux * uz;
    Y[4] = 0.5 * s * uy * uz;
  } else {
    const double a = sqrt(35 / 2.0 / pi), b = sqrt(105 / pi), c = sqrt(21 / 2.0 / pi), d = sqrt(7 / pi);
    const double z2 = uz * uz;
    Y[0] = 0.25 * d * (5 * z2 * uz - 3 * uz);
    Y[1] = 0.25 * c * ux * (5 * z2 - 1);
    Y[2] = 0.25 * c * uy * (5 * z2 - 1);
    Y[3] = 0.25 * b * uz * (ux * ux - uy * uy);
    Y[4] = 0.5 * b * uz * ux * uy;
    Y[5] = 0.25 * a * (ux * ux * ux - 3 * ux * uy * uy);
    Y[6] = 0.25 * a * (3 * ux * ux * uy - uy * uy * uy);
  }
}

// Value tables: one thread per sphere point, kTabBlock points per block.
__global__ void __launch_bounds__(kTabBlock) tabulate_values_kernel(DevGeom g, const DevSpecies* __restrict__ spes,
                                                                     const double* __restrict__ radial,
                                                                     const int32_t* __restrict__ buckets,
                                                                     const int32_t* __restrict__ block_atom,
                                                                     const int64_t* __restrict__ block_start,
                                                                     double* phi) {
  extern __shared__ double stage[];
  const int atom = block_atom[blockIdx.x];
  const int64_t first = block_start[blockIdx.x];
  const int64_t s0 = g.sph_off[atom], s1 = g.sph_off[atom + 1];
  const int npts = (int)((s1 - first) < kTabBlock ? (s1 - first) : kTabBlock);
  const DevSpecies sp = spes[g.spe[atom]];
  const int NO = sp.no;
  const int t = threadIdx.x;
  if (t < npts) {
    const int64_t k = first + t;
    const int gn = g.glist[k];
    const int cell = g.clist[k];
    const int N2 = g.ngrid[1], N3 = g.ngrid[2];
    const int n1 = gn / (N2 * N3);
    const int n2 = (gn - n1 * N2 * N3) / N3;
    const int n3 = gn - n1 * N2 * N3 - n2 * N3;
    double xyz[3];
    for (int d = 0; d < 3; ++d) {
      double c = n1 * g.glat[0 * 3 + d] + n2 * g.glat[1 * 3 + d] + n3 * g.glat[2 * 3 + d] + g.origin[d];
      xyz[d] = c + g.atv[cell * 3 + d] - g.gxyz[atom * 3 + d];
    }
    const double r2 = xyz[0] * xyz[0] + xyz[1] * xyz[1] + xyz[2] * xyz[2];
    double R, ux, uy, uz;
    if (r2 < 1e-28) {
      // R < 1e-14: theta = pi/2, phi = 0 (src/utils/xyz_to_spherical.jl)
      R = sqrt(r2);
      ux = 1.0;
      uy = 0.0;
      uz = 6.123233995736766e-17;  // cos(pi/2) in double precision
    } else {
      const double ir = rsqrt(r2);
      R = r2 * ir;
      ux = xyz[0] * ir;
      uy = xyz[1] * ir;
      uz = xyz[2] * ir;
    }
    const int n = sp.nmesh;
    const double* rv = radial + sp.rv_off;
    double* srow = stage + (size_t)t * NO;
    const bool outside = rv[n - 1] < R;
    const bool inner = R < rv[0];
    const double* rec = nullptr;
    double u = 0.0;
    if (!outside && !inner) {
      // the interval: first mesh index >= 1 with RV >= R, from one bucket down
      int b = (int)((__log2f((float)R) - sp.bk_lo) * sp.bk_inv) - 1;
      b = min(max(b, 0), kSplineBuckets - 1);
      int i = buckets[sp.bk_off + b];
      while (i < n - 1 && rv[i] < R) ++i;
      const int m = min(max(i, 2), n - 2);
      rec = radial + sp.iv_off + (size_t)m * (2 + 4 * sp.nrad);
      u = (R - rec[0]) * rec[1];
    }
    int ist = 0, rad = 0;
    for (int l = 0; l <= sp.max_l; ++l) {
      double Y[7];
      ylm_unit(l, ux, uy, uz, Y);
      for (int p = 0; p < sp.nb[l]; ++p, ++rad) {
        double rf = 0.0;
        if (rec) {
          const double* c = rec + 2 + 4 * rad;
          rf = ((c[3] * u + c[2]) * u + c[1]) * u + c[0];
        } else if (inner) {
          const double* e = radial + sp.ex_off + 4 * rad;
          rf = ((e[0] * R + e[1]) * R + e[2]) * R + e[3];
        }
        for (int mm = 0; mm < 2 * l + 1; ++mm, ++ist) srow[ist] = rf * Y[mm];
      }
    }
  }
  __syncthreads();
  const int64_t base = g.phi_off[atom] + (first - s0) * NO;
  const int total = npts * NO;
  double* dst = phi + base;
  const int head = (int)(((uintptr_t)dst & 15) ? 1 : 0);
  if (t == 0 && head && total > 0) dst[0] = stage[0];
  const int nvec = (total - head) / 2;
  double2* dv = reinterpret_cast<double2*>(dst + head);
  for (int i = t; i < nvec; i += blockDim.x) dv[i] = make_double2(stage[head + 2 * i], stage[head + 2 * i + 1]);
  const int tail = head + 2 * nvec;
  if (t == 0 && tail < total) dst[tail] = stage[tail];
}

template <bool GRAD>
__global__ void __launch_bounds__(kTabPoints) tabulate_kernel(DevGeom g, const DevSpecies* __restrict__ spes,
                                                              const double* __restrict__ radial,
                                                              const int32_t* __restrict__ block_atom,
                                                              const int64_t* __restrict__ block_start, double* phi,
                                                              double* dpx, double* dpy, double* dpz) {
  extern __shared__ double stage[];
  const int atom = block_atom[blockIdx.x];
  const int64_t first = block_start[blockIdx.x];
  const int64_t s0 = g.sph_off[atom], s1 = g.sph_off[atom + 1];
  const int npts = (int)((s1 - first) < kTabPoints ? (s1 - first) : kTabPoints);
  const DevSpecies sp = spes[g.spe[atom]];
  const int NO = sp.no;
  const double* rv = radial + sp.rv_off;
  const double* rwf = radial + sp.rwf_off;
  const int t = threadIdx.x;

  if (t < npts) {
    const int64_t k = first + t;
    const int gn = g.glist[k];
    const int cell = g.clist[k];
    const int N2 = g.ngrid[1], N3 = g.ngrid[2];
    const int n1 = gn / (N2 * N3);
    const int n2 = (gn - n1 * N2 * N3) / N3;
    const int n3 = gn - n1 * N2 * N3 - n2 * N3;
    double xyz[3];
    for (int d = 0; d < 3; ++d) {
      double c = n1 * g.glat[0 * 3 + d] + n2 * g.glat[1 * 3 + d] + n3 * g.glat[2 * 3 + d] + g.origin[d];
      xyz[d] = c + g.atv[cell * 3 + d] - g.gxyz[atom * 3 + d];
    }
    double* srow = stage + (size_t)t * NO;
    double* sx = stage + (size_t)kTabPoints * NO + (size_t)t * NO;
    double* sy = sx + (size_t)kTabPoints * NO;
    double* sz = sy + (size_t)kTabPoints * NO;
    double R, siQ, coQ, siP, coP;
    spherical_trig(xyz[0], xyz[1], xyz[2], R, siQ, coQ, siP, coP);
    if (!GRAD) {
      eval_point<true, false>(sp, rv, rwf, R, siQ, coQ, siP, coP, srow, sx, sy, sz);
    } else if (R < 1.0e-13) {
      // the gradient tables shift points that sit on the atom
      // (src/Matrix/Set_dOrbitals_Grid.jl:107-112); the values do not
      eval_point<true, false>(sp, rv, rwf, R, siQ, coQ, siP, coP, srow, sx, sy, sz);
      spherical_trig(xyz[0] + 1.0e-13, xyz[1] + 1.0e-13, xyz[2] + 1.0e-13, R, siQ, coQ, siP, coP);
      eval_point<false, true>(sp, rv, rwf, R, siQ, coQ, siP, coP, srow, sx, sy, sz);
    } else {
      eval_point<true, true>(sp, rv, rwf, R, siQ, coQ, siP, coP, srow, sx, sy, sz);
    }
  }
  __syncthreads();

  // contiguous write-back: the block's points occupy rows [first-s0, +npts)
  const int64_t base = g.phi_off[atom] + (first - s0) * NO;
  const int total = npts * NO;
  const int ntab = GRAD ? 4 : 1;
  double* outs[4] = {phi, dpx, dpy, dpz};
  for (int tab = 0; tab < ntab; ++tab) {
    const double* src = stage + (size_t)tab * kTabPoints * NO;
    double* dst = outs[tab] + base;
    // 16-byte stores where the destination is 16-byte aligned
    const int head = (int)(((uintptr_t)dst & 15) ? 1 : 0);
    if (t == 0 && head && total > 0) dst[0] = src[0];
    const int nvec = (total - head) / 2;
    double2* dv = reinterpret_cast<double2*>(dst + head);
    for (int i = t; i < nvec; i += blockDim.x) dv[i] = make_double2(src[head + 2 * i], src[head + 2 * i + 1]);
    const int tail = head + 2 * nvec;
    if (t == 0 && tail < total) dst[tail] = src[tail];
  }
}

__global__ void f64_to_f32_kernel(const double* __restrict__ s, float* __restrict__ d, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    d[i] = (float)s[i];
}

}  // namespace

cudaError_t launch_tabulate(const DevGeom& g, const DevSpecies* dspe, const double* radial, const int32_t* buckets,
                            int64_t nblocks, const int32_t* block_atom, const int64_t* block_start, double* phi,
                            double* dphi_x, double* dphi_y, double* dphi_z, int max_no, cudaStream_t st) {
  if (nblocks == 0) return cudaSuccess;
  const bool grad = dphi_x != nullptr;
  if (!grad) {
    const size_t smem = (size_t)kTabBlock * max_no * sizeof(double);
    LCP_CUDA_TRY(raise_smem(tabulate_values_kernel, smem));
    tabulate_values_kernel<<<(unsigned)nblocks, kTabBlock, smem, st>>>(g, dspe, radial, buckets, block_atom,
                                                                        block_start, phi);
    return cudaGetLastError();
  }
  // the gradient kernel takes blocks of kTabPoints points
  const size_t smem = (size_t)kTabPoints * max_no * sizeof(double) * 4;
  LCP_CUDA_TRY(raise_smem(tabulate_kernel<true>, smem));
  tabulate_kernel<true><<<(unsigned)nblocks, kTabPoints, smem, st>>>(g, dspe, radial, block_atom, block_start, phi,
                                                                     dphi_x, dphi_y, dphi_z);
  return cudaGetLastError();
}

// Per-interval cubic of the value tables' spline for interval m of one
// radial function w (src/Matrix/Set_Orbitals_Grid.jl:187-238): the Hermite
// interpolant through (RV[m-1], f2) and (RV[m], f3) with the slopes g1, g2 of
// the reference, as coefficients of u = (R - RV[m-1]) / h2; at m = N-2 the
// reference substitutes f4 = f1 (:226-229).
static void interval_cubic(const double* rv, const double* w, int n, int m, double* c) {
  const double h1 = rv[m - 1] - rv[m - 2], h2 = rv[m] - rv[m - 1], h3 = rv[m + 1] - rv[m];
  const double f1 = w[m - 2], f2 = w[m - 1], f3 = w[m];
  const double f4 = m == n - 2 ? f1 : w[m + 1];
  double dum = h1 + h2;
  const double dum1 = h1 / h2 / dum, dum2 = h2 / h1 / dum;
  dum = h2 + h3;
  const double dum3 = h2 / h3 / dum, dum4 = h3 / h2 / dum;
  const double g1 = (f3 - f2) * dum1 + (f2 - f1) * dum2;
  const double g2 = (f4 - f3) * dum3 + (f3 - f2) * dum4;
  c[0] = f2;
  c[1] = h2 * g1;
  c[2] = 3 * (f3 - f2) - 2 * h2 * g1 - h2 * g2;
  c[3] = 2 * (f2 - f3) + h2 * g1 + h2 * g2;
}

// The polynomial continuation below RV[0] (src/Matrix/Set_Orbitals_Grid.jl:122-185):
// value and slope of the spline at rm = RV[4] (mesh point 4, 0-based), then
// a R^3 + b R^2 + c R + d by l.
static void inner_cubic(const double* rv, const double* w, int l, double* e) {
  const int m = 4;
  const double rm = rv[m];
  const double h1 = rv[m - 1] - rv[m - 2], h2 = rv[m] - rv[m - 1], h3 = rv[m + 1] - rv[m];
  const double y1 = (rm - rv[m - 1]) / h2, y2 = (rm - rv[m]) / h2;
  double dum = h1 + h2;
  const double dum1 = h1 / h2 / dum, dum2 = h2 / h1 / dum;
  dum = h2 + h3;
  const double dum3 = h2 / h3 / dum, dum4 = h3 / h2 / dum;
  const double f1 = w[m - 2], f2 = w[m - 1], f3 = w[m], f4 = w[m + 1];
  const double d32 = f3 - f2;
  const double g1 = d32 * dum1 + (f2 - f1) * dum2;
  const double g2 = (f4 - f3) * dum3 + d32 * dum4;
  const double A = 3 * f2 + h2 * g1, B = 2 * f2 + h2 * g1, C = 3 * f3 - h2 * g2, D = 2 * f3 - h2 * g2;
  const double E = A + B * y2, F = C - D * y1;
  const double y12 = y1 * y1, y22 = y2 * y2;
  const double f = y22 * E + y12 * F;
  const double df = (2 * y2 / h2) * E + y22 * B / h2 + (2 * y1 / h2) * F - y12 * D / h2;
  double a = 0, b = 0, c = 0, d = 0;
  if (l == 0) {
    b = 0.5 * df / rm;
    d = f - b * (rm * rm);
  } else if (l == 1) {
    a = (rm * df - f) / (2 * (rm * rm * rm));
    c = df - 3 * a * (rm * rm);
  } else {
    b = (3 * f - rm * df) / (rm * rm);
    a = (f - b * (rm * rm)) / (rm * rm * rm);
  }
  e[0] = a;
  e[1] = b;
  e[2] = c;
  e[3] = d;
}

void append_spline_tables(const double* rv, const double* rwf, int n, const int* num_basis, int max_l,
                          DevSpecies& d, std::vector<double>& radial, std::vector<int32_t>& buckets) {
  int nrad = 0;
  for (int l = 0; l <= max_l; ++l) nrad += num_basis[l];
  const int rec = 2 + 4 * nrad;
  d.iv_off = (int64_t)radial.size();
  radial.resize(radial.size() + (size_t)n * rec, 0.0);
  for (int m = 2; m <= n - 2; ++m) {
    double* r = radial.data() + d.iv_off + (size_t)m * rec;
    r[0] = rv[m - 1];
    r[1] = 1.0 / (rv[m] - rv[m - 1]);
    for (int q = 0; q < nrad; ++q) interval_cubic(rv, rwf + (size_t)q * n, n, m, r + 2 + 4 * q);
  }
  d.ex_off = (int64_t)radial.size();
  radial.resize(radial.size() + (size_t)4 * nrad, 0.0);
  int q = 0;
  for (int l = 0; l <= max_l; ++l)
    for (int p = 0; p < num_basis[l]; ++p, ++q) inner_cubic(rv, rwf + (size_t)q * n, l, radial.data() + d.ex_off + 4 * q);
  // buckets of log2(R) over [log2 RV[1], log2 RV[n-1]]: each holds the first
  // mesh index >= 1 whose RV reaches the bucket's lower edge
  const double lo = std::log2(rv[1]), hi = std::log2(rv[n - 1]);
  const double inv = kSplineBuckets / std::max(hi - lo, 1e-30);
  d.bk_lo = (float)lo;
  d.bk_inv = (float)inv;
  d.bk_off = (int64_t)buckets.size();
  int i = 1;
  for (int b = 0; b < kSplineBuckets; ++b) {
    // the edge as the device computes bucket numbers (in float), lowered by
    // a bucket's width of margin through the device's b - 1
    const double edge = std::exp2((double)d.bk_lo + b / (double)d.bk_inv);
    while (i < n - 1 && rv[i] < edge) ++i;
    buckets.push_back(i);
  }
}

cudaError_t launch_convert_f32(const double* src, float* dst, int64_t n, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  int blocks = (int)std::min<int64_t>((n + 255) / 256, 152 * 16);
  f64_to_f32_kernel<<<blocks, 256, 0, st>>>(src, dst, n);
  return cudaGetLastError();
}

}  // namespace lcp
