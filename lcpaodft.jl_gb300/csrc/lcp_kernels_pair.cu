// Exact-lens pair contractions on CUDA cores: density assembly and grid
// matrix elements in FP64 (the drop-in) or FP32 (comparison form).
//
// The reference walks every ordered pair (i, j, R) of the neighbour list over
// the pair's overlap ("lens") points in 512-point blocks, with a small dgemm
// per block (src/Matrix/Set_Density_Grid.jl:268-304,
// src/Hamiltonian.jl:384-429).  Here each unordered pair {(i,j,R), (j,i,-R)}
// is visited once:
//   density: rho(p) += phi_i(p)^T (D_(i,j,R) + D_(j,i,-R)^T) phi_j(p)
//            -- exactly the sum of the two ordered contributions for any D;
//   H:       Hm[a][b] = sum_p phi_i,a(p) V(p) phi_j,b(p) is written to both
//            blocks, H_(i,j,R)[b,a] and H_(j,i,-R)[a,b] (V real).
// The lens lists are the reference's GListTAtoms1/2 of the kept orientation.
// Work items are 512-entry chunks of those lists; a persistent grid walks the
// items.  FP64 results reach the grids/blocks through FP64 atomics.
#include <cuda_runtime.h>

#include "lcp_bounds.cuh"
#include "lcp_device.h"

namespace lcp {

namespace {

constexpr int kPairThreads = 256;
constexpr int kTile = 64;  // lens points staged per H tile

template <typename T>
__device__ __forceinline__ T ldg(const T* p) {
  return __ldg(p);
}

struct Ptr4 {
  const double* c[4];
};
struct MPtr4 {
  double* c[4];
};

// ---------------------------------------------------------------- density

template <typename T, int NOMAX>
__global__ void __launch_bounds__(kPairThreads) density_pairs_kernel(DevGeom g, DevPairs pr, int nspin,
                                                                     const T* __restrict__ phi, Ptr4 dm,
                                                                     MPtr4 rho) {
  __shared__ T Ds[4][NOMAX * NOMAX];
  for (int64_t item = blockIdx.x; item < pr.nitems; item += gridDim.x) {
    const int64_t q = pr.item_pair[item];
    const int i = pr.atom[q], j = pr.jatom[q];
    const int noi = g.numorbs[i], noj = g.numorbs[j];
    const int64_t bp = pr.boff_p[q], bq = pr.boff_q[q];
    const bool self = pr.self[q] != 0;
    // check build: the pair's D blocks lie inside DM (else they read as zero)
    const bool okp = bounds_ok(bp + (int64_t)noi * noj - 1, pr.hsize, 1);
    const bool okq = self || bounds_ok(bq + (int64_t)noi * noj - 1, pr.hsize, 2);
    __syncthreads();
    // the whole NOMAX x NOMAX tile is written (zeros outside NOi x NOj): the
    // contraction below reads every column, multiplying the padding by zero
    for (int e = threadIdx.x; e < NOMAX * NOMAX; e += blockDim.x) {
      const int a = e / NOMAX, b = e - a * NOMAX;
      for (int s = 0; s < nspin; ++s) {
        double v = 0.0;
        if (a < noi && b < noj) {
          if (okp) v = dm.c[s][bp + (int64_t)a * noj + b];
          if (!self && okq) v += dm.c[s][bq + (int64_t)b * noi + a];
        }
        Ds[s][a * NOMAX + b] = (T)v;
      }
    }
    __syncthreads();
    const int64_t start = pr.item_start[item];
    const int count = pr.item_count[item];
    const T* phi_i = phi + g.phi_off[i];
    const T* phi_j = phi + g.phi_off[j];
    const int32_t* gl_i = g.glist + g.sph_off[i];
    const int64_t gn_i = g.sph_off[i + 1] - g.sph_off[i], gn_j = g.sph_off[j + 1] - g.sph_off[j];
    const int64_t nn = (int64_t)g.ngrid[0] * g.ngrid[1] * g.ngrid[2];
    for (int pt = threadIdx.x; pt < count; pt += blockDim.x) {
      const int64_t k = start + pt;
      const int g1 = pr.g1[k], g2 = pr.g2[k];
      // check build: lens entries inside both spheres, the point inside the grid
      if (!bounds_ok(g1, gn_i, 3) || !bounds_ok(g2, gn_j, 4) || !bounds_ok(gl_i[g1], nn, 5)) continue;
      T pi[NOMAX], pj[NOMAX];
#pragma unroll
      for (int a = 0; a < NOMAX; ++a) pi[a] = a < noi ? ldg(phi_i + (int64_t)g1 * noi + a) : T(0);
#pragma unroll
      for (int b = 0; b < NOMAX; ++b) pj[b] = b < noj ? ldg(phi_j + (int64_t)g2 * noj + b) : T(0);
      const int gidx = gl_i[g1];
      for (int s = 0; s < nspin; ++s) {
        T acc = T(0);
#pragma unroll
        for (int a = 0; a < NOMAX; ++a) {
          if (a < noi) {
            T t = T(0);
#pragma unroll
            for (int b = 0; b < NOMAX; ++b) t += Ds[s][a * NOMAX + b] * pj[b];
            acc += pi[a] * t;
          }
        }
        atomicAdd(rho.c[s] + gidx, (double)acc);
      }
    }
  }
}

// ---------------------------------------------------------------- grid H

// Per item (a 512-entry chunk of a pair's lens list) the block stages kTile
// lens points at a time -- phi_i V (per channel) and phi_j, NOMAX orbitals
// each -- into shared memory, and thread e accumulates entry (a, b) =
// (e / NOMAX, e % NOMAX) over them.  The gathers of the next tile are issued
// into registers before the current tile's FMAs, so their latency overlaps
// the FP64 arithmetic; MAXC is the largest channel count the instance serves
// (1 for SpinPol "off", else 4), so the spin-off case keeps only one V value
// per staged entry in registers.
template <typename T, int NOMAX, int MAXC>
__global__ void __launch_bounds__(kPairThreads) hamiltonian_pairs_kernel(DevGeom g, DevPairs pr, int nch,
                                                                         const T* __restrict__ phi, Ptr4 vpot,
                                                                         MPtr4 hks) {
  constexpr int kSlots = (NOMAX * NOMAX + kPairThreads - 1) / kPairThreads;
  constexpr int kStage = (kTile * NOMAX + kPairThreads - 1) / kPairThreads;  // staged entries per thread
  extern __shared__ unsigned char smem_raw[];
  T* W = reinterpret_cast<T*>(smem_raw);           // [MAXC][kTile][NOMAX]
  T* P = W + (size_t)MAXC * kTile * NOMAX;         // [kTile][NOMAX]
  for (int64_t item = blockIdx.x; item < pr.nitems; item += gridDim.x) {
    const int64_t q = pr.item_pair[item];
    const int i = pr.atom[q], j = pr.jatom[q];
    const int noi = g.numorbs[i], noj = g.numorbs[j];
    const int64_t start = pr.item_start[item];
    const int count = pr.item_count[item];
    const T* phi_i = phi + g.phi_off[i];
    const T* phi_j = phi + g.phi_off[j];
    const int32_t* gl_i = g.glist + g.sph_off[i];
    T acc[MAXC][kSlots];
#pragma unroll
    for (int c = 0; c < MAXC; ++c)
#pragma unroll
      for (int s = 0; s < kSlots; ++s) acc[c][s] = T(0);
    // this thread's staged entries of one tile: idx = threadIdx.x + r kPairThreads
    T rwi[kStage], rwj[kStage];
    double rv[kStage][MAXC];
    auto gather = [&](int t0) {
      const int nt = min(kTile, count - t0);
#pragma unroll
      for (int r = 0; r < kStage; ++r) {
        const int idx = threadIdx.x + r * kPairThreads;
        const int pt = idx / NOMAX, a = idx - pt * NOMAX;
        rwi[r] = T(0);
        rwj[r] = T(0);
#pragma unroll
        for (int c = 0; c < MAXC; ++c) rv[r][c] = 0.0;
        if (idx < kTile * NOMAX && pt < nt) {
          const int64_t k = start + t0 + pt;
          const int g1 = pr.g1[k], g2 = pr.g2[k];
          // check build: an entry outside its sphere or grid contributes nothing
          const bool ok = bounds_ok(g1, g.sph_off[i + 1] - g.sph_off[i], 3) &&
                          bounds_ok(g2, g.sph_off[j + 1] - g.sph_off[j], 4) &&
                          bounds_ok(gl_i[g1], (int64_t)g.ngrid[0] * g.ngrid[1] * g.ngrid[2], 5);
          if (ok && a < noi) {
            rwi[r] = ldg(phi_i + (int64_t)g1 * noi + a);
            const int gidx = gl_i[g1];
#pragma unroll
            for (int c = 0; c < MAXC; ++c)
              if (c < nch) rv[r][c] = ldg(vpot.c[c] + gidx);
          }
          if (ok && a < noj) rwj[r] = ldg(phi_j + (int64_t)g2 * noj + a);
        }
      }
    };
    gather(0);
    for (int t0 = 0; t0 < count; t0 += kTile) {
      const int nt = min(kTile, count - t0);
      __syncthreads();  // the previous tile's readers are done
#pragma unroll
      for (int r = 0; r < kStage; ++r) {
        const int idx = threadIdx.x + r * kPairThreads;
        if (idx < kTile * NOMAX) {
          const int pt = idx / NOMAX, a = idx - pt * NOMAX;
#pragma unroll
          for (int c = 0; c < MAXC; ++c)
            if (c < nch) W[((size_t)c * kTile + pt) * NOMAX + a] = rwi[r] * (T)rv[r][c];
          P[pt * NOMAX + a] = rwj[r];
        }
      }
      __syncthreads();
      if (t0 + kTile < count) gather(t0 + kTile);  // in flight during the FMAs below
#pragma unroll
      for (int s = 0; s < kSlots; ++s) {
        const int e = threadIdx.x + s * kPairThreads;
        if (e < NOMAX * NOMAX) {
          const int a = e / NOMAX, b = e - (e / NOMAX) * NOMAX;
          if (a < noi && b < noj) {
#pragma unroll
            for (int c = 0; c < MAXC; ++c) {
              if (c < nch) {
                T sum = T(0);
                const T* wr = W + (size_t)c * kTile * NOMAX + a;
                const T* pr_ = P + b;
                for (int pt = 0; pt < nt; ++pt) sum += wr[pt * NOMAX] * pr_[pt * NOMAX];
                acc[c][s] += sum;
              }
            }
          }
        }
      }
    }
    const bool self = pr.self[q] != 0;
    const int64_t bp = pr.boff_p[q], bq = pr.boff_q[q];
    // check build: the pair's H blocks lie inside H (else nothing is written)
    const bool okp = bounds_ok(bp + (int64_t)noi * noj - 1, pr.hsize, 6);
    const bool okq = self || bounds_ok(bq + (int64_t)noi * noj - 1, pr.hsize, 7);
#pragma unroll
    for (int s = 0; s < kSlots; ++s) {
      const int e = threadIdx.x + s * kPairThreads;
      if (e < NOMAX * NOMAX) {
        const int a = e / NOMAX, b = e - (e / NOMAX) * NOMAX;
        if (a < noi && b < noj) {
#pragma unroll
          for (int c = 0; c < MAXC; ++c) {
            if (c < nch) {
              const double val = (double)acc[c][s] * g.gridvol;
              if (okp) atomicAdd(hks.c[c] + bp + (int64_t)a * noj + b, val);
              if (!self && okq) atomicAdd(hks.c[c] + bq + (int64_t)b * noi + a, val);
            }
          }
        }
      }
    }
  }
}

int persistent_blocks(int64_t nitems, int per_sm) {
  int dev = 0, sms = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  int64_t b = (int64_t)sms * per_sm;
  return (int)std::max<int64_t>(1, std::min<int64_t>(b, nitems));
}

template <typename T, int NOMAX>
cudaError_t run_density(const DevGeom& g, const DevPairs& pr, int nspin, const T* phi, const double* const* dm,
                        double* const* rho, cudaStream_t st) {
  Ptr4 d{};
  MPtr4 r{};
  for (int s = 0; s < nspin; ++s) {
    d.c[s] = dm[s];
    r.c[s] = rho[s];
  }
  density_pairs_kernel<T, NOMAX><<<persistent_blocks(pr.nitems, 8), kPairThreads, 0, st>>>(g, pr, nspin, phi, d, r);
  return cudaGetLastError();
}

// ---------------------------------------------------------------- grid force term

// Force3 (src/Force.jl:405-566, 3344-3394): for every ordered pair (i, j, R)
// the sum over its lens points of V(p) grad phi_i(p) . D_(i,j,R) phi_j(p),
// weighted per channel.  Each folded pair item gives both orientations: the
// kept one to atom i, the partner (j, i, -R) over the same points to atom j
// (once for a pair that is its own partner).  Per item a fixed-order block
// sum of the six components; force3_reduce_kernel then adds each atom's item
// sums in item order (deterministic, no atomics).
struct Coef4 {
  double w[4];
};

template <int NOMAX>
__global__ void __launch_bounds__(kPairThreads) force3_pairs_kernel(DevGeom g, DevPairs pr, int nch,
                                                                    const double* __restrict__ phi,
                                                                    const double* __restrict__ dpx,
                                                                    const double* __restrict__ dpy,
                                                                    const double* __restrict__ dpz, Ptr4 vpot,
                                                                    Ptr4 dm, Coef4 w, double* __restrict__ out) {
  extern __shared__ double fsm[];
  double* Dp = fsm;                          // [nch][a][b]: kept pair's block
  double* Dq = fsm + nch * NOMAX * NOMAX;    // [nch][b][a]: partner's block
  __shared__ double red[6][kPairThreads];
  for (int64_t item = blockIdx.x; item < pr.nitems; item += gridDim.x) {
    const int64_t q = pr.item_pair[item];
    const int i = pr.atom[q], j = pr.jatom[q];
    const int noi = g.numorbs[i], noj = g.numorbs[j];
    const int64_t bp = pr.boff_p[q], bq = pr.boff_q[q];
    const bool self = pr.self[q] != 0;
    __syncthreads();
    for (int e = threadIdx.x; e < NOMAX * NOMAX; e += blockDim.x) {
      const int a = e / NOMAX, b = e - a * NOMAX;
      for (int c = 0; c < nch; ++c) {
        Dp[c * NOMAX * NOMAX + a * NOMAX + b] = (a < noi && b < noj) ? dm.c[c][bp + (int64_t)a * noj + b] : 0.0;
        Dq[c * NOMAX * NOMAX + b * NOMAX + a] =
            (a < noi && b < noj && !self) ? dm.c[c][bq + (int64_t)b * noi + a] : 0.0;
      }
    }
    __syncthreads();
    double acc[6] = {0, 0, 0, 0, 0, 0};
    const int64_t start = pr.item_start[item];
    const int count = pr.item_count[item];
    const int64_t oi = g.phi_off[i], oj = g.phi_off[j];
    const int32_t* gl_i = g.glist + g.sph_off[i];
    for (int pt = threadIdx.x; pt < count; pt += blockDim.x) {
      const int64_t k = start + pt;
      const int64_t r1 = oi + (int64_t)pr.g1[k] * noi, r2 = oj + (int64_t)pr.g2[k] * noj;
      double pi[NOMAX], pj[NOMAX];
#pragma unroll
      for (int a = 0; a < NOMAX; ++a) pi[a] = a < noi ? ldg(phi + r1 + a) : 0.0;
#pragma unroll
      for (int b = 0; b < NOMAX; ++b) pj[b] = b < noj ? ldg(phi + r2 + b) : 0.0;
      const int gidx = gl_i[pr.g1[k]];
      for (int c = 0; c < nch; ++c) {
        const double v = w.w[c] * ldg(vpot.c[c] + gidx);
        double sx = 0, sy = 0, sz = 0;
        for (int a = 0; a < noi; ++a) {  // grad phi_i . D_p phi_j
          double t = 0;
#pragma unroll
          for (int b = 0; b < NOMAX; ++b) t += Dp[c * NOMAX * NOMAX + a * NOMAX + b] * pj[b];
          sx += ldg(dpx + r1 + a) * t;
          sy += ldg(dpy + r1 + a) * t;
          sz += ldg(dpz + r1 + a) * t;
        }
        acc[0] += v * sx;
        acc[1] += v * sy;
        acc[2] += v * sz;
        if (!self) {
          double ux = 0, uy = 0, uz = 0;
          for (int b = 0; b < noj; ++b) {  // grad phi_j . D_q phi_i
            double t = 0;
#pragma unroll
            for (int a = 0; a < NOMAX; ++a) t += Dq[c * NOMAX * NOMAX + b * NOMAX + a] * pi[a];
            ux += ldg(dpx + r2 + b) * t;
            uy += ldg(dpy + r2 + b) * t;
            uz += ldg(dpz + r2 + b) * t;
          }
          acc[3] += v * ux;
          acc[4] += v * uy;
          acc[5] += v * uz;
        }
      }
    }
    for (int k = 0; k < 6; ++k) red[k][threadIdx.x] = acc[k];
    __syncthreads();
    for (int s2 = kPairThreads / 2; s2 > 0; s2 >>= 1) {
      if (threadIdx.x < s2)
        for (int k = 0; k < 6; ++k) red[k][threadIdx.x] += red[k][threadIdx.x + s2];
      __syncthreads();
    }
    if (threadIdx.x < 6) out[item * 6 + threadIdx.x] = red[threadIdx.x][0];
  }
}

// force[atom][x,y,z] = gridvol * sum over the atom's entries (item * 2 + half)
// of the item sums, in entry order (one block per atom).
__global__ void __launch_bounds__(kPairThreads) force3_reduce_kernel(int natom, const int64_t* __restrict__ off,
                                                                     const int64_t* __restrict__ code,
                                                                     const double* __restrict__ part, double gridvol,
                                                                     double* __restrict__ force) {
  __shared__ double red[3][kPairThreads];
  for (int atom = blockIdx.x; atom < natom; atom += gridDim.x) {
    double v[3] = {0, 0, 0};
    for (int64_t e = off[atom] + threadIdx.x; e < off[atom + 1]; e += blockDim.x) {
      const int64_t c = code[e];
      const double* src = part + (c >> 1) * 6 + (c & 1) * 3;
      for (int k = 0; k < 3; ++k) v[k] += src[k];
    }
    __syncthreads();
    for (int k = 0; k < 3; ++k) red[k][threadIdx.x] = v[k];
    __syncthreads();
    for (int s2 = kPairThreads / 2; s2 > 0; s2 >>= 1) {
      if (threadIdx.x < s2)
        for (int k = 0; k < 3; ++k) red[k][threadIdx.x] += red[k][threadIdx.x + s2];
      __syncthreads();
    }
    if (threadIdx.x < 3) force[atom * 3 + threadIdx.x] = red[threadIdx.x][0] * gridvol;
  }
}

template <int NOMAX>
cudaError_t run_force3(const DevGeom& g, const DevPairs& pr, int nch, const double* phi, const double* const* dphi,
                       const double* const* vp, const double* const* dm, const double* coef, double* part,
                       cudaStream_t st) {
  Ptr4 v{}, d{};
  Coef4 w{};
  for (int c = 0; c < nch; ++c) {
    v.c[c] = vp[c];
    d.c[c] = dm[c];
    w.w[c] = coef[c];
  }
  const size_t smem = (size_t)2 * nch * NOMAX * NOMAX * sizeof(double);
  LCP_CUDA_TRY(raise_smem(force3_pairs_kernel<NOMAX>, smem));
  force3_pairs_kernel<NOMAX><<<persistent_blocks(pr.nitems, 4), kPairThreads, smem, st>>>(
      g, pr, nch, phi, dphi[0], dphi[1], dphi[2], v, d, w, part);
  return cudaGetLastError();
}

template <typename T, int NOMAX, int MAXC>
cudaError_t run_hamiltonian_c(const DevGeom& g, const DevPairs& pr, int nch, const T* phi, const Ptr4& v,
                              const MPtr4& o, cudaStream_t st) {
  const size_t smem = (size_t)(MAXC + 1) * kTile * NOMAX * sizeof(T);
  LCP_CUDA_TRY(raise_smem(hamiltonian_pairs_kernel<T, NOMAX, MAXC>, smem));
  hamiltonian_pairs_kernel<T, NOMAX, MAXC><<<persistent_blocks(pr.nitems, 4), kPairThreads, smem, st>>>(
      g, pr, nch, phi, v, o);
  return cudaGetLastError();
}

template <typename T, int NOMAX>
cudaError_t run_hamiltonian(const DevGeom& g, const DevPairs& pr, int nch, const T* phi, const double* const* vp,
                            double* const* h, cudaStream_t st) {
  Ptr4 v{};
  MPtr4 o{};
  for (int c = 0; c < nch; ++c) {
    v.c[c] = vp[c];
    o.c[c] = h[c];
  }
  if (nch == 1) return run_hamiltonian_c<T, NOMAX, 1>(g, pr, nch, phi, v, o, st);
  return run_hamiltonian_c<T, NOMAX, 4>(g, pr, nch, phi, v, o, st);
}

}  // namespace

cudaError_t launch_density_pairs(int prec, const DevGeom& g, const DevPairs& pr, int nspin, const double* phi64,
                                 const float* phi32, const double* const* dm, double* const* rho, int max_no,
                                 cudaStream_t st) {
  if (pr.nitems == 0) return cudaSuccess;
  // NOMAX: the per-point tiles' orbital bound, exact for the common 13 (s2p2d1)
  // and 18 (s2p2d2) orbital sets, else padded to 16 or 32 (padding costs FMAs
  // on zeros: 16 for 13 orbitals is 23 % more density work)
  if (prec == LCP_PREC_FP32) {
    if (max_no == 13) return run_density<float, 13>(g, pr, nspin, phi32, dm, rho, st);
    if (max_no <= 16) return run_density<float, 16>(g, pr, nspin, phi32, dm, rho, st);
    if (max_no <= 18) return run_density<float, 18>(g, pr, nspin, phi32, dm, rho, st);
    return run_density<float, 32>(g, pr, nspin, phi32, dm, rho, st);
  }
  if (max_no == 13) return run_density<double, 13>(g, pr, nspin, phi64, dm, rho, st);
  if (max_no <= 16) return run_density<double, 16>(g, pr, nspin, phi64, dm, rho, st);
  if (max_no <= 18) return run_density<double, 18>(g, pr, nspin, phi64, dm, rho, st);
  return run_density<double, 32>(g, pr, nspin, phi64, dm, rho, st);
}

cudaError_t launch_force3_pairs(const DevGeom& g, const DevPairs& pr, int nch, const double* phi,
                                const double* const* dphi, const double* const* vpot, const double* const* dm,
                                const double* coef, double* partials, int max_no, cudaStream_t st) {
  if (pr.nitems == 0) return cudaSuccess;
  if (max_no == 13) return run_force3<13>(g, pr, nch, phi, dphi, vpot, dm, coef, partials, st);
  if (max_no <= 16) return run_force3<16>(g, pr, nch, phi, dphi, vpot, dm, coef, partials, st);
  if (max_no <= 18) return run_force3<18>(g, pr, nch, phi, dphi, vpot, dm, coef, partials, st);
  return run_force3<32>(g, pr, nch, phi, dphi, vpot, dm, coef, partials, st);
}

cudaError_t launch_force3_reduce(int natom, const int64_t* off, const int64_t* code, const double* partials,
                                 double gridvol, double* force, cudaStream_t st) {
  if (natom == 0) return cudaSuccess;
  force3_reduce_kernel<<<natom, kPairThreads, 0, st>>>(natom, off, code, partials, gridvol, force);
  return cudaGetLastError();
}

cudaError_t launch_hamiltonian_pairs(int prec, const DevGeom& g, const DevPairs& pr, int nch, const double* phi64,
                                     const float* phi32, const double* const* vpot, double* const* hks, int max_no,
                                     cudaStream_t st) {
  if (pr.nitems == 0) return cudaSuccess;
  if (prec == LCP_PREC_FP32) {
    if (max_no == 13) return run_hamiltonian<float, 13>(g, pr, nch, phi32, vpot, hks, st);
    if (max_no <= 16) return run_hamiltonian<float, 16>(g, pr, nch, phi32, vpot, hks, st);
    if (max_no <= 18) return run_hamiltonian<float, 18>(g, pr, nch, phi32, vpot, hks, st);
    return run_hamiltonian<float, 32>(g, pr, nch, phi32, vpot, hks, st);
  }
  if (max_no == 13) return run_hamiltonian<double, 13>(g, pr, nch, phi64, vpot, hks, st);
  if (max_no <= 16) return run_hamiltonian<double, 16>(g, pr, nch, phi64, vpot, hks, st);
  if (max_no <= 18) return run_hamiltonian<double, 18>(g, pr, nch, phi64, vpot, hks, st);
  return run_hamiltonian<double, 32>(g, pr, nch, phi64, vpot, hks, st);
}

cudaError_t bounds_take_pairs(unsigned long long* word) {
#ifdef LCP_BOUNDS_CHECK
  return bounds_take(word);
#else
  *word = 0;
  return cudaErrorNotSupported;
#endif
}

}  // namespace lcp
