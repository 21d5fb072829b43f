// Grid setup on the device: the sphere lists of Calc_AtomsGrid, the overlap
// lists of Calc_AtomOverlap_Grid and Set_AdenPCC_Grid.
//
// Sphere lists.  Each atom scans a box of grid coordinates n (n = nn + l N,
// nn the grid index along an axis, l the image cell); the reference keeps the
// points within the cutoff and stable-sorts them by flat grid index, so the
// list order is (nn1, nn2, nn3) and, for the images of one grid point, the
// scan order (n1, n2, n3).  Here every candidate computes its position in that
// order directly from small per-axis tables (the rank of its residue nn among
// the box's residues, its image number, and per residue the image count and
// the count before it), so a flag array in list order plus one exclusive scan
// gives every kept point its list index: no sort.  The same pass leaves a
// box-shaped table (box coordinate -> list index or -1) per atom.
//
// Overlap lists.  For a folded pair (atom i, neighbour j, cell R), a point of
// j's list at box coordinate n (image l) is the point of i's list at box
// coordinate nn + (l + R) N; the box table of i answers in one load.  Two
// passes over chunks of j's list (count, then scan and write) keep the
// reference's order (j's list order).
//
// Set_AdenPCC_Grid.  Each grid point gathers its sphere entries through a
// point -> entries index and adds them in the reference's order (atom, then
// list position), so the sums are the same bits whatever the schedule.
//
// Every distance is evaluated with each product and sum rounded on its own
// (no FMA contraction), as the reference and the host build round them, so
// the lists are bit-identical to the host's.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <vector>

#include "lcp_api_state.h"
#include "lcp_device.h"
#include "lcp_internal.h"

namespace lcp {
namespace {

// ------------------------------------------------------------ exclusive scan
//
// out[i] = sum_{k<i} in[i] (int64), out[n] = the total; three passes: block
// totals, a one-block scan of the totals, block-local scans.

constexpr int kScanThreads = 256;
constexpr int kScanPer = 8;                        // elements per thread
constexpr int kScanTile = kScanThreads * kScanPer;  // elements per block

__device__ __forceinline__ int64_t block_exclusive_scan(int64_t v, int64_t* total) {
  __shared__ int64_t warp_sums[kScanThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int64_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int64_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_sums[warp] = x;
  __syncthreads();
  if (warp == 0) {
    int64_t w = lane < kScanThreads / 32 ? warp_sums[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int64_t y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < kScanThreads / 32) warp_sums[lane] = w;
  }
  __syncthreads();
  const int64_t before = (warp > 0 ? warp_sums[warp - 1] : 0) + x - v;
  if (total) *total = warp_sums[kScanThreads / 32 - 1];
  __syncthreads();
  return before;
}

__global__ void __launch_bounds__(kScanThreads) scan_totals_kernel(const int32_t* __restrict__ in, int64_t n,
                                                                   int64_t* __restrict__ totals) {
  const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanPer;
  int64_t s = 0;
#pragma unroll
  for (int k = 0; k < kScanPer; ++k)
    if (base + k < n) s += in[base + k];
  int64_t tot;
  block_exclusive_scan(s, &tot);
  if (threadIdx.x == 0) totals[blockIdx.x] = tot;
}

// One block: exclusive scan of the block totals in place, grand total at [nb].
__global__ void __launch_bounds__(kScanThreads) scan_offsets_kernel(int64_t* __restrict__ totals, int64_t nb) {
  __shared__ int64_t carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int64_t b0 = 0; b0 < nb; b0 += kScanThreads) {
    const int64_t b = b0 + threadIdx.x;
    const int64_t v = b < nb ? totals[b] : 0;
    int64_t tot;
    const int64_t before = block_exclusive_scan(v, &tot);
    if (b < nb) totals[b] = carry + before;
    __syncthreads();
    if (threadIdx.x == 0) carry += tot;
    __syncthreads();
  }
  if (threadIdx.x == 0) totals[nb] = carry;
}

__global__ void __launch_bounds__(kScanThreads) scan_write_kernel(const int32_t* __restrict__ in, int64_t n,
                                                                  const int64_t* __restrict__ offsets,
                                                                  int64_t* __restrict__ out) {
  const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanPer;
  int32_t v[kScanPer];
  int64_t s = 0;
#pragma unroll
  for (int k = 0; k < kScanPer; ++k) {
    v[k] = base + k < n ? in[base + k] : 0;
    s += v[k];
  }
  int64_t run = offsets[blockIdx.x] + block_exclusive_scan(s, nullptr);
#pragma unroll
  for (int k = 0; k < kScanPer; ++k)
    if (base + k < n) {
      out[base + k] = run;
      run += v[k];
    }
  if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) out[n] = offsets[gridDim.x];
}

}  // namespace

// out: n + 1 int64; totals: scan_blocks(n) + 1 int64 of scratch.
int64_t scan_blocks(int64_t n) { return std::max<int64_t>(1, (n + kScanTile - 1) / kScanTile); }

cudaError_t exclusive_scan_i32(const int32_t* in, int64_t n, int64_t* out, int64_t* totals, cudaStream_t st) {
  const int64_t nb = scan_blocks(n);
  scan_totals_kernel<<<(unsigned)nb, kScanThreads, 0, st>>>(in, n, totals);
  LCP_CUDA_TRY(cudaGetLastError());
  scan_offsets_kernel<<<1, kScanThreads, 0, st>>>(totals, nb);
  LCP_CUDA_TRY(cudaGetLastError());
  scan_write_kernel<<<(unsigned)nb, kScanThreads, 0, st>>>(in, n, totals, out);
  return cudaGetLastError();
}

namespace {

// ------------------------------------------------------------ sphere lists

struct SetupGeom {
  int32_t ng[3];
  int32_t cpy, ncdim;  // CpyCell, 2 CpyCell + 1
  double glat[3][3];   // grid vectors (rows)
  double origin[3];
  const double* atv;       // [ncell][3]
  const int32_t* atv_ijk;  // [ncell][3]
  const int32_t* ratv;     // [(2C+1)^3]
};

// One atom's scan box and its per-axis order tables (see the file comment).
struct SphereAtom {
  int32_t nmin[3], len[3], nres[3];
  int32_t tab;   // offset of the tables: per axis rank[len], image[len]; then per axis count[nres], before[nres]
  int64_t cand;  // offset of the atom's box points among all atoms'
  double g[3], cut;
};

__device__ __forceinline__ int floor_div(int a, int n) {
  int q = a / n;
  if ((a % n != 0) && ((a < 0) != (n < 0))) --q;
  return q;
}

__device__ __forceinline__ int atom_of(const int64_t* __restrict__ off, int natom, int64_t idx) {
  int lo = 0, hi = natom;  // off[lo] <= idx < off[hi]
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (off[mid] <= idx) lo = mid;
    else hi = mid;
  }
  return lo;
}

// Box point t (scan order) of atom A: its position in the atom's sorted list
// order, its flat grid index, image cell and whether it is within the cutoff
// (Calc_AtomsGrid, src/UCell.jl:365-400, with Find_CGrids!,
// src/utils/Find_CGrid.jl:1-49).
struct BoxPoint {
  int64_t s;
  int32_t g, rn;
  bool keep;
};

__device__ __forceinline__ BoxPoint box_point(const SetupGeom& G, const SphereAtom& A, const int32_t* __restrict__ tabs,
                                              int64_t t) {
  const int L1 = A.len[1], L2 = A.len[2];
  const int t3 = (int)(t % L2);
  const int64_t t12 = t / L2;
  const int t2 = (int)(t12 % L1);
  const int t1 = (int)(t12 / L1);
  const int tt[3] = {t1, t2, t3};
  int rank[3], img[3], cnt[3], bef[3];
  int o = A.tab;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    rank[d] = tabs[o + tt[d]];
    img[d] = tabs[o + A.len[d] + tt[d]];
    o += 2 * A.len[d];
  }
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    cnt[d] = tabs[o + rank[d]];
    bef[d] = tabs[o + A.nres[d] + rank[d]];
    o += 2 * A.nres[d];
  }
  BoxPoint p;
  p.s = (int64_t)bef[0] * A.len[1] * A.len[2] +
        (int64_t)cnt[0] * ((int64_t)bef[1] * A.len[2] + (int64_t)cnt[1] * bef[2]) +
        ((int64_t)img[0] * cnt[1] + img[1]) * cnt[2] + img[2];
  int nn[3], l[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const int n = A.nmin[d] + tt[d];
    l[d] = floor_div(n, G.ng[d]);
    nn[d] = n - l[d] * G.ng[d];
  }
  const int C = G.cpy;
  p.rn = G.ratv[((C + l[0]) * G.ncdim + (C + l[1])) * G.ncdim + (C + l[2])];
  p.g = (nn[0] * G.ng[1] + nn[1]) * G.ng[2] + nn[2];
  double dd[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    double c = G.atv[p.rn * 3 + d];
    c = __dadd_rn(c, __dmul_rn((double)nn[0], G.glat[0][d]));
    c = __dadd_rn(c, __dmul_rn((double)nn[1], G.glat[1][d]));
    c = __dadd_rn(c, __dmul_rn((double)nn[2], G.glat[2][d]));
    c = __dadd_rn(c, G.origin[d]);
    dd[d] = __dsub_rn(c, A.g[d]);
  }
  const double R = sqrt(__dadd_rn(__dadd_rn(__dmul_rn(dd[0], dd[0]), __dmul_rn(dd[1], dd[1])), __dmul_rn(dd[2], dd[2])));
  p.keep = R <= A.cut;
  return p;
}

__global__ void sphere_flag_kernel(const __grid_constant__ SetupGeom G, const SphereAtom* __restrict__ atoms,
                                   const int64_t* __restrict__ cand_off, int natom, const int32_t* __restrict__ tabs,
                                   int32_t* __restrict__ flags) {
  const int64_t total = cand_off[natom];
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int a = atom_of(cand_off, natom, idx);
    const SphereAtom& A = atoms[a];
    const BoxPoint p = box_point(G, A, tabs, idx - A.cand);
    flags[A.cand + p.s] = p.keep ? 1 : 0;
  }
}

// pos: exclusive scan of the flags (list position of every kept point among
// all atoms'); lut[idx]: the box table, the point's index in its atom's list
// or -1.
__global__ void sphere_write_kernel(const __grid_constant__ SetupGeom G, const SphereAtom* __restrict__ atoms,
                                    const int64_t* __restrict__ cand_off, int natom, const int32_t* __restrict__ tabs,
                                    const int32_t* __restrict__ flags, const int64_t* __restrict__ pos,
                                    int32_t* __restrict__ glist, int32_t* __restrict__ clist,
                                    int32_t* __restrict__ lut) {
  const int64_t total = cand_off[natom];
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int a = atom_of(cand_off, natom, idx);
    const SphereAtom& A = atoms[a];
    const BoxPoint p = box_point(G, A, tabs, idx - A.cand);
    const int64_t f = A.cand + p.s;
    if (flags[f]) {
      const int64_t o = pos[f];
      glist[o] = p.g;
      clist[o] = p.rn;
      lut[idx] = (int32_t)(o - pos[A.cand]);
    } else {
      lut[idx] = -1;
    }
  }
}

}  // namespace

namespace {

// ------------------------------------------------------------ overlap lists

constexpr int kOvThreads = 256;
constexpr int kOvPer = 8;
constexpr int kOvChunk = kOvThreads * kOvPer;  // entries of j's list per block

struct OvPair {
  int32_t i, j;  // atom, neighbour (0-based)
  int32_t r[3];  // image cell R of the neighbour
};

// Index in atom i's list of the point at entry e of j's list seen through the
// pair's cell R, or -1 (Calc_AtomOverlap_Grid, src/UCell.jl:439-512).
__device__ __forceinline__ int32_t twin(const SetupGeom& G, const SphereAtom& Ai, const OvPair& P,
                                        const int32_t* __restrict__ glist, const int32_t* __restrict__ clist,
                                        const int32_t* __restrict__ lut, int64_t e) {
  const int cell = clist[e];
  const int C = G.cpy;
  int l[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    l[d] = G.atv_ijk[cell * 3 + d] + P.r[d];
    if (l[d] > C || l[d] < -C) return -1;
  }
  const int g = glist[e];
  const int plane = G.ng[1] * G.ng[2];
  const int nn0 = g / plane;
  const int rem = g - nn0 * plane;
  const int nn1 = rem / G.ng[2];
  const int nn2 = rem - nn1 * G.ng[2];
  const int nn[3] = {nn0, nn1, nn2};
  int t[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    t[d] = nn[d] + l[d] * G.ng[d] - Ai.nmin[d];
    if (t[d] < 0 || t[d] >= Ai.len[d]) return -1;
  }
  return lut[Ai.cand + ((int64_t)t[0] * Ai.len[1] + t[1]) * Ai.len[2] + t[2]];
}

// Block b covers entries [k0, k0 + kOvChunk) of pair q's j list; thread t its
// entries k0 + t*kOvPer .. + kOvPer - 1, in order.  WRITE = false: the block's
// number of hits into cnt[b]; WRITE = true: the hits (index in i's list, index
// in j's list) at boff[b] + the hits before them in the block.
template <bool WRITE>
__global__ void __launch_bounds__(kOvThreads) overlap_kernel(const __grid_constant__ SetupGeom G,
                                                             const SphereAtom* __restrict__ atoms,
                                                             const OvPair* __restrict__ pairs,
                                                             const int32_t* __restrict__ blk_pair,
                                                             const int64_t* __restrict__ blk_k0,
                                                             const int64_t* __restrict__ sphere_off,
                                                             const int32_t* __restrict__ glist,
                                                             const int32_t* __restrict__ clist,
                                                             const int32_t* __restrict__ lut, int32_t* __restrict__ cnt,
                                                             const int64_t* __restrict__ boff, int32_t* __restrict__ g1,
                                                             int32_t* __restrict__ g2) {
  const OvPair P = pairs[blk_pair[blockIdx.x]];
  const SphereAtom& Ai = atoms[P.i];
  const int64_t base = sphere_off[P.j];
  const int64_t nj = sphere_off[P.j + 1] - base;
  const int64_t k0 = blk_k0[blockIdx.x] + (int64_t)threadIdx.x * kOvPer;
  int32_t hit[kOvPer];
  int64_t mine = 0;
#pragma unroll
  for (int m = 0; m < kOvPer; ++m) {
    hit[m] = k0 + m < nj ? twin(G, Ai, P, glist, clist, lut, base + k0 + m) : -1;
    mine += hit[m] >= 0 ? 1 : 0;
  }
  int64_t tot;
  const int64_t before = block_exclusive_scan(mine, &tot);
  if (!WRITE) {
    if (threadIdx.x == 0) cnt[blockIdx.x] = (int32_t)tot;
    return;
  }
  int64_t o = boff[blockIdx.x] + before;
#pragma unroll
  for (int m = 0; m < kOvPer; ++m)
    if (hit[m] >= 0) {
      g1[o] = hit[m];
      g2[o] = (int32_t)(k0 + m);
      ++o;
    }
}

}  // namespace

namespace {

// ------------------------------------------------------------ Set_AdenPCC_Grid

struct Radial {
  int32_t n;         // mesh points
  const double* xv;  // log mesh [n]
  const double* rv;  // radii [n]
  const double* yv;  // values in the (n + 4)-long layout
};

// KumoF (src/utils/KumoF.jl:1-60): cubic interpolation on the uniform log
// mesh, and below the first mesh point a + b r^2 fitted to the spline's value
// and slope at the fifth point.
__device__ double kumof(const Radial& T, double x) {
  const double* xv = T.xv;
  const double* rv = T.rv;
  const double* yv = T.yv;
  if (x < xv[0]) {
    const double r = exp(x);
    const int m = 4;  // the reference's m = 5, 1-based
    const double rm = rv[m];
    const double h1 = rv[m - 1] - rv[m - 2];
    const double h2 = rv[m] - rv[m - 1];
    const double h3 = rv[m + 1] - rv[m];
    const double f1 = yv[m - 2], f2 = yv[m - 1], f3 = yv[m], f4 = yv[m + 1];
    const double g1 = ((f3 - f2) * h1 / h2 + (f2 - f1) * h2 / h1) / (h1 + h2);
    const double g2 = ((f4 - f3) * h2 / h3 + (f3 - f2) * h3 / h2) / (h2 + h3);
    const double x1 = rm - rv[m - 1];
    const double x2 = rm - rv[m];
    const double y1 = x1 / h2, y2 = x2 / h2;
    const double y12 = y1 * y1, y22 = y2 * y2;
    const double A = 2 * f2 + h2 * g1;
    const double B = 2 * f3 - h2 * g2;
    const double Cc = 3 * f2 + h2 * g1;
    const double D = 3 * f3 - h2 * g2;
    const double E = Cc + A * y2;
    const double F = D - B * y1;
    const double f = y22 * E + y12 * F;
    const double df = (2 * y2 / h2) * E + y22 * A / h2 + (2 * y1 / h2) * F - y12 * B / h2;
    const double a = 0.5 * df / rm;
    const double b = f - a * rm * rm;
    return a * r * r + b;
  }
  const double xmin = xv[0], xmax = xv[T.n - 1];
  double xx = fmin(x, xmax);
  xx = fmax(xx, xmin);
  const double tmp = (T.n - 1) * (xx - xmin) / (xmax - xmin);
  const int i0 = (int)floor(tmp);
  const double dt = tmp - i0;
  const int i = i0 + 1;  // 1-based i; yv[i + 1] (1-based) is yv[i] here
  const double d0 = yv[i] - yv[i - 1];
  const double d1 = yv[i + 1] - yv[i];
  const double d2 = yv[i + 2] - yv[i + 1];
  const double a = d0 - 2 * d1 + d2;
  const double b = -2 * d0 + 3 * d1 - d2;
  const double c = d0 + d1;
  return yv[i] + 0.5 * (((a * dt + b) * dt + c) * dt);
}

struct AdenAtom {
  double g[3];
  double ou, od;      // occupancies Nu / Nele, Nd / Nele (0 for Nele <= 1e-15)
  double sit, cot, sip, cop;  // sin and cos of the initial spin angles theta, phi
  int32_t spe;        // 0-based species
};

struct AdenArgs {
  int32_t ng[3];
  int32_t spinpol, natom;
  int64_t nn;
  double glat[3][3];
  double origin[3];
  const double* atv;
  const AdenAtom* atoms;
  const Radial* den;  // per species: Spe_Atomic_Den on the PAO mesh
  const Radial* pcc;  // per species: Spe_Atomic_PCC on the VPS mesh
  const int64_t* sphere_off;
  const int32_t* glist;
  const int32_t* clist;
  const int64_t* start;  // point -> entries index: entries of point g at idx[start[g] .. start[g+1])
  const int32_t* idx;
  double* aden;
  double* pccd;
  double* rho[4];
};

__global__ void entry_count_kernel(const int32_t* __restrict__ glist, int64_t total, int32_t* __restrict__ cnt) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x)
    atomicAdd(&cnt[glist[e]], 1);
}

__global__ void entry_fill_kernel(const int32_t* __restrict__ glist, int64_t total, const int64_t* __restrict__ start,
                                  int32_t* __restrict__ cursor, int32_t* __restrict__ idx) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int g = glist[e];
    idx[start[g] + atomicAdd(&cursor[g], 1)] = (int32_t)e;
  }
}

// Set_AdenPCC_Grid (src/Matrix/Set_AdenPCC_Grid.jl:58-140) gathered per grid
// point: its entries are taken in increasing entry index (atom, then list
// position: the reference's loop order) by repeated minimum selection.
__global__ void adenpcc_gather_kernel(const __grid_constant__ AdenArgs a) {
  const int plane = a.ng[1] * a.ng[2];
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < a.nn; g += (int64_t)gridDim.x * blockDim.x) {
    const int64_t s0 = a.start[g], s1 = a.start[g + 1];
    const int n1 = (int)(g / plane);
    const int n2 = (int)((g - (int64_t)n1 * plane) / a.ng[2]);
    const int n3 = (int)(g - (int64_t)n1 * plane - (int64_t)n2 * a.ng[2]);
    double cxyz[3];
#pragma unroll
    for (int d = 0; d < 3; ++d)
      cxyz[d] = __dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn((double)n1, a.glat[0][d]), __dmul_rn((double)n2, a.glat[1][d])),
                                    __dmul_rn((double)n3, a.glat[2][d])),
                          a.origin[d]);
    double ad = 0.0, pc = 0.0, r0 = 0.0, r1 = 0.0, r2 = 0.0, r3 = 0.0;
    int32_t prev = -1;
    for (int64_t k = s0; k < s1; ++k) {
      int32_t e = 0x7fffffff;
      for (int64_t q = s0; q < s1; ++q) {
        const int32_t v = a.idx[q];
        if (v > prev && v < e) e = v;
      }
      prev = e;
      const int atom = atom_of(a.sphere_off, a.natom, e);
      const AdenAtom& A = a.atoms[atom];
      const int grc = a.clist[e];
      const double dx = __dsub_rn(__dadd_rn(cxyz[0], a.atv[grc * 3 + 0]), A.g[0]);
      const double dy = __dsub_rn(__dadd_rn(cxyz[1], a.atv[grc * 3 + 1]), A.g[1]);
      const double dz = __dsub_rn(__dadd_rn(cxyz[2], a.atv[grc * 3 + 2]), A.g[2]);
      const double x = 0.5 * log(__dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz)));
      const double den = kumof(a.den[A.spe], x);
      const double pcv = kumof(a.pcc[A.spe], x);
      ad += 0.5 * den;
      pc += 0.5 * pcv;
      if (a.spinpol == LCP_SPIN_OFF) {
        r0 += 0.5 * den;
      } else if (a.spinpol == LCP_SPIN_ON) {
        r0 += A.ou * den;
        r1 += A.od * den;
      } else {
        const double mag = (A.ou - A.od) * den;
        r0 += den;
        r1 += mag * A.sit * A.cop;
        r2 += mag * A.sit * A.sip;
        r3 += mag * A.cot;
      }
    }
    a.aden[g] = ad;
    a.pccd[g] = pc;
    if (a.spinpol == LCP_SPIN_OFF) {
      a.rho[0][g] = r0;
    } else if (a.spinpol == LCP_SPIN_ON) {
      a.rho[0][g] = r0;
      a.rho[1][g] = r1;
    } else {
      // (rho, mx, my, mz) -> the four "nc" channels (:127-138)
      a.rho[0][g] = 0.5 * (r0 + r3);
      a.rho[1][g] = 0.5 * (r0 - r3);
      a.rho[2][g] = 0.5 * r1;
      a.rho[3][g] = -0.5 * r2;
    }
  }
}

}  // namespace

namespace {

__global__ void gather_offsets_kernel(const int64_t* __restrict__ pos, const int64_t* __restrict__ at, int n,
                                      int64_t* __restrict__ out) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) out[k] = pos[at[k]];
}

int grid_for(int64_t n, int threads) { return (int)std::max<int64_t>(1, std::min<int64_t>((n + threads - 1) / threads, 152 * 16)); }

// Host -> device copy on the stream without waiting for it (unlike upload):
// the callers keep `v` alive until they synchronise the stream.
template <class T>
cudaError_t to_device(DBuf& b, const std::vector<T>& v, cudaStream_t st) {
  cudaError_t e = b.ensure(std::max<size_t>(v.size(), 1) * sizeof(T));
  if (e || v.empty()) return e;
  return cudaMemcpyAsync(b.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, st);
}

// Per-axis order tables of a box [nmin, nmin + len) on a grid of n points:
// rank of each box coordinate's residue among the box's residues, its image
// number, and per rank the image count and the count before it.
void axis_tables(int nmin, int len, int n, std::vector<int32_t>& rank, std::vector<int32_t>& img,
                 std::vector<int32_t>& cnt, std::vector<int32_t>& before) {
  std::vector<int32_t> res(len);
  for (int t = 0; t < len; ++t) {
    int r = (nmin + t) % n;
    res[t] = r < 0 ? r + n : r;
  }
  std::vector<int32_t> distinct(res);
  std::sort(distinct.begin(), distinct.end());
  distinct.erase(std::unique(distinct.begin(), distinct.end()), distinct.end());
  std::vector<int32_t> rank_of(n, -1);
  for (size_t k = 0; k < distinct.size(); ++k) rank_of[distinct[k]] = (int32_t)k;
  rank.resize(len);
  img.resize(len);
  cnt.assign(distinct.size(), 0);
  for (int t = 0; t < len; ++t) {
    rank[t] = rank_of[res[t]];
    img[t] = cnt[rank[t]]++;
  }
  before.assign(distinct.size(), 0);
  for (size_t k = 1; k < distinct.size(); ++k) before[k] = before[k - 1] + cnt[k - 1];
}

struct SetupBuffers {
  DBuf atoms, tabs, cand, atv, ijk, ratv, flags, pos, scan, offs, at, glist, clist, lut;
  DBuf pairs, bpair, bk0, bcnt, boff, g1, g2;
};

}  // namespace

// Calc_AtomsGrid and Calc_AtomOverlap_Grid on the device for a UCell whose
// head (image cells, neighbour and pair lists) is built; fills the sphere and
// overlap lists of u exactly as build_spheres_host / build_overlaps_host.
lcp_status build_ucell_device(lcp_ctx* ctx, UCell& u) {
  cudaStream_t st = ctx->stream;
  const int natom = u.natom;
  const int C = u.cpycell;
  SetupBuffers B;
  std::vector<SphereAtom> atoms(natom);
  std::vector<int32_t> tabs;
  std::vector<int64_t> cand_off(natom + 1, 0);
  for (int a = 0; a < natom; ++a) {
    int nmin[3], nmax[3];
    atom_box(u, a, nmin, nmax);
    SphereAtom& A = atoms[a];
    std::vector<int32_t> rk[3], im[3], ct[3], bf[3];
    int64_t vol = 1;
    for (int d = 0; d < 3; ++d) {
      const int n = u.ngrid[d];
      const int llo = nmin[d] >= 0 ? nmin[d] / n : -((-nmin[d] + n - 1) / n);
      const int lhi = nmax[d] >= 0 ? nmax[d] / n : -((-nmax[d] + n - 1) / n);
      // image cells the reference indexes without leaving ratv and without
      // its out-of-range branch: -CpyCell <= l <= CpyCell - 1
      if (llo < -C || lhi > C - 1)
        return fail(LCP_ENOTSUP, "an atom's grid box reaches image cells beyond CpyCell; build the UCell on the host");
      A.nmin[d] = nmin[d];
      A.len[d] = nmax[d] - nmin[d] + 1;
      axis_tables(nmin[d], A.len[d], n, rk[d], im[d], ct[d], bf[d]);
      A.nres[d] = (int32_t)ct[d].size();
      vol *= A.len[d];
    }
    A.tab = (int32_t)tabs.size();
    for (int d = 0; d < 3; ++d) {
      tabs.insert(tabs.end(), rk[d].begin(), rk[d].end());
      tabs.insert(tabs.end(), im[d].begin(), im[d].end());
    }
    for (int d = 0; d < 3; ++d) {
      tabs.insert(tabs.end(), ct[d].begin(), ct[d].end());
      tabs.insert(tabs.end(), bf[d].begin(), bf[d].end());
    }
    A.cand = cand_off[a];
    cand_off[a + 1] = cand_off[a] + vol;
    for (int d = 0; d < 3; ++d) A.g[d] = u.gxyz[a * 3 + d];
    A.cut = u.cut[a];
  }
  const int64_t total = cand_off[natom];
  if (total >= ((int64_t)1 << 31)) return fail(LCP_ENOTSUP, "grid boxes too large for the device build");
  SetupGeom G{};
  for (int d = 0; d < 3; ++d) {
    G.ng[d] = u.ngrid[d];
    G.origin[d] = u.origin[d];
    for (int e = 0; e < 3; ++e) G.glat[d][e] = u.glat[d][e];
  }
  G.cpy = C;
  G.ncdim = 2 * C + 1;
  API_CUDA(to_device(B.atoms, atoms, st), "H2D");
  API_CUDA(to_device(B.tabs, tabs, st), "H2D");
  API_CUDA(to_device(B.cand, cand_off, st), "H2D");
  API_CUDA(to_device(B.atv, u.atv, st), "H2D");
  API_CUDA(to_device(B.ijk, u.atv_ijk, st), "H2D");
  API_CUDA(to_device(B.ratv, u.ratv, st), "H2D");
  G.atv = B.atv.as<double>();
  G.atv_ijk = B.ijk.as<int32_t>();
  G.ratv = B.ratv.as<int32_t>();
  API_CUDA(B.flags.ensure(std::max<int64_t>(total, 1) * sizeof(int32_t)), "alloc");
  API_CUDA(B.pos.ensure((total + 1) * sizeof(int64_t)), "alloc");
  API_CUDA(B.lut.ensure(std::max<int64_t>(total, 1) * sizeof(int32_t)), "alloc");
  API_CUDA(B.scan.ensure((scan_blocks(total) + 1) * sizeof(int64_t)), "alloc");
  const SphereAtom* dA = B.atoms.as<SphereAtom>();
  const int64_t* dC = B.cand.as<int64_t>();
  sphere_flag_kernel<<<grid_for(total, 256), 256, 0, st>>>(G, dA, dC, natom, B.tabs.as<int32_t>(),
                                                             B.flags.as<int32_t>());
  API_CUDA(cudaGetLastError(), "sphere flags");
  API_CUDA(exclusive_scan_i32(B.flags.as<int32_t>(), total, B.pos.as<int64_t>(), B.scan.as<int64_t>(), st),
           "sphere scan");
  // sphere_off[a] = pos[cand_off[a]]
  API_CUDA(B.offs.ensure((natom + 1) * sizeof(int64_t)), "alloc");
  gather_offsets_kernel<<<(natom + 1 + 127) / 128, 128, 0, st>>>(B.pos.as<int64_t>(), dC, natom + 1,
                                                                   B.offs.as<int64_t>());
  API_CUDA(cudaGetLastError(), "sphere offsets");
  u.sphere_off.assign(natom + 1, 0);
  API_CUDA(cudaMemcpyAsync(u.sphere_off.data(), B.offs.p, (natom + 1) * sizeof(int64_t), cudaMemcpyDeviceToHost, st),
           "D2H");
  API_CUDA(cudaStreamSynchronize(st), "sphere lists");
  const int64_t nent = u.sphere_off[natom];
  API_CUDA(B.glist.ensure(std::max<int64_t>(nent, 1) * sizeof(int32_t)), "alloc");
  API_CUDA(B.clist.ensure(std::max<int64_t>(nent, 1) * sizeof(int32_t)), "alloc");
  sphere_write_kernel<<<grid_for(total, 256), 256, 0, st>>>(G, dA, dC, natom, B.tabs.as<int32_t>(),
                                                              B.flags.as<int32_t>(), B.pos.as<int64_t>(),
                                                              B.glist.as<int32_t>(), B.clist.as<int32_t>(),
                                                              B.lut.as<int32_t>());
  API_CUDA(cudaGetLastError(), "sphere write");
  ctx->launches += 6;
  u.glist.resize(nent);
  u.clist.resize(nent);
  if (nent) {
    API_CUDA(cudaMemcpyAsync(u.glist.data(), B.glist.p, nent * sizeof(int32_t), cudaMemcpyDeviceToHost, st), "D2H");
    API_CUDA(cudaMemcpyAsync(u.clist.data(), B.clist.p, nent * sizeof(int32_t), cudaMemcpyDeviceToHost, st), "D2H");
  }

  // overlap lists of the folded pairs
  const int64_t nu = (int64_t)u.uniq_pair.size();
  std::vector<OvPair> pairs(nu);
  std::vector<int32_t> bpair;
  std::vector<int64_t> bk0, qfirst(nu + 1, 0);
  for (int64_t q = 0; q < nu; ++q) {
    const int p = u.uniq_pair[q];
    OvPair& P = pairs[q];
    P.i = u.pair_atom[p];
    P.j = u.pair_jatom[p];
    for (int d = 0; d < 3; ++d) P.r[d] = u.atv_ijk[u.pair_cell[p] * 3 + d];
    qfirst[q] = (int64_t)bpair.size();
    const int64_t nj = u.sphere_off[P.j + 1] - u.sphere_off[P.j];
    for (int64_t k0 = 0; k0 < nj; k0 += kOvChunk) {
      bpair.push_back((int32_t)q);
      bk0.push_back(k0);
    }
  }
  const int64_t nblk = (int64_t)bpair.size();
  qfirst[nu] = nblk;
  API_CUDA(to_device(B.pairs, pairs, st), "H2D");
  API_CUDA(to_device(B.bpair, bpair, st), "H2D");
  API_CUDA(to_device(B.bk0, bk0, st), "H2D");
  API_CUDA(B.bcnt.ensure(std::max<int64_t>(nblk, 1) * sizeof(int32_t)), "alloc");
  API_CUDA(B.boff.ensure((nblk + 1) * sizeof(int64_t)), "alloc");
  API_CUDA(B.scan.ensure((scan_blocks(nblk) + 1) * sizeof(int64_t)), "alloc");
  if (nblk > 0) {
    overlap_kernel<false><<<(unsigned)nblk, kOvThreads, 0, st>>>(
        G, dA, B.pairs.as<OvPair>(), B.bpair.as<int32_t>(), B.bk0.as<int64_t>(), B.offs.as<int64_t>(),
        B.glist.as<int32_t>(), B.clist.as<int32_t>(), B.lut.as<int32_t>(), B.bcnt.as<int32_t>(), nullptr, nullptr,
        nullptr);
    API_CUDA(cudaGetLastError(), "overlap count");
  }
  API_CUDA(exclusive_scan_i32(B.bcnt.as<int32_t>(), nblk, B.boff.as<int64_t>(), B.scan.as<int64_t>(), st),
           "overlap scan");
  std::vector<int64_t> boff(nblk + 1);
  API_CUDA(cudaMemcpyAsync(boff.data(), B.boff.p, (nblk + 1) * sizeof(int64_t), cudaMemcpyDeviceToHost, st), "D2H");
  API_CUDA(cudaStreamSynchronize(st), "overlap counts");
  const int64_t nhit = boff[nblk];
  API_CUDA(B.g1.ensure(std::max<int64_t>(nhit, 1) * sizeof(int32_t)), "alloc");
  API_CUDA(B.g2.ensure(std::max<int64_t>(nhit, 1) * sizeof(int32_t)), "alloc");
  if (nblk > 0) {
    overlap_kernel<true><<<(unsigned)nblk, kOvThreads, 0, st>>>(
        G, dA, B.pairs.as<OvPair>(), B.bpair.as<int32_t>(), B.bk0.as<int64_t>(), B.offs.as<int64_t>(),
        B.glist.as<int32_t>(), B.clist.as<int32_t>(), B.lut.as<int32_t>(), nullptr, B.boff.as<int64_t>(),
        B.g1.as<int32_t>(), B.g2.as<int32_t>());
    API_CUDA(cudaGetLastError(), "overlap write");
  }
  ctx->launches += 5;
  u.uniq_off.assign(nu + 1, 0);
  for (int64_t q = 0; q <= nu; ++q) u.uniq_off[q] = boff[qfirst[q]];
  u.uniq_g1.resize(nhit);
  u.uniq_g2.resize(nhit);
  if (nhit) {
    API_CUDA(cudaMemcpyAsync(u.uniq_g1.data(), B.g1.p, nhit * sizeof(int32_t), cudaMemcpyDeviceToHost, st), "D2H");
    API_CUDA(cudaMemcpyAsync(u.uniq_g2.data(), B.g2.p, nhit * sizeof(int32_t), cudaMemcpyDeviceToHost, st), "D2H");
  }
  API_CUDA(cudaStreamSynchronize(st), "overlap lists");
  u.numolg.assign(u.nloop, 0);
  for (int64_t q = 0; q < nu; ++q) {
    const int p = u.uniq_pair[q];
    u.numolg[p] = u.uniq_off[q + 1] - u.uniq_off[q];
    u.numolg[u.partner[p]] = u.numolg[p];
  }
  return LCP_OK;
}

}  // namespace lcp

extern "C" {

lcp_status lcp_ucell_create_device(lcp_ctx* ctx, int32_t nspin, const double* latvecs, int32_t natom,
                                   const int32_t* atom2spe, const double* gxyz, const double* atoms_cut1,
                                   const int32_t* ngrid, const double* grid_origin, const int32_t* total_numorbs,
                                   lcp_ucell** out) {
  lcp_status s = check_ctx(ctx);
  if (s) return s;
  if (!out || !latvecs || !atom2spe || !gxyz || !atoms_cut1 || !ngrid) return fail(LCP_EINVAL, "NULL argument");
  *out = nullptr;
  std::unique_ptr<lcp_ucell> u(new (std::nothrow) lcp_ucell());
  if (!u) return fail(LCP_ENOMEM, "out of host memory");
  try {
    std::string err = lcp::build_ucell_head(u->u, nspin, latvecs, natom, atom2spe, gxyz, atoms_cut1, ngrid,
                                            grid_origin, total_numorbs);
    if (!err.empty()) return fail(LCP_EINVAL, err);
    if ((s = lcp::build_ucell_device(ctx, u->u))) return s;
  } catch (const std::bad_alloc&) {
    return fail(LCP_ENOMEM, "out of host memory building UCell");
  }
  *out = u.release();
  return LCP_OK;
}

lcp_status lcp_set_adenpcc_grid(lcp_ctx* ctx, const lcp_ucell* ucell, int32_t spinpol, const double* init_atoms_nspin,
                                const double* init_atoms_angle, int32_t nspecies, const lcp_radial* atomic_den,
                                const lcp_radial* atomic_pcc, double* adensity_grid, double* pccdensity_grid,
                                double* const* density_grid) {
  using namespace lcp;
  lcp_status s = check_ctx(ctx);
  if (s) return s;
  if (!ucell || !init_atoms_nspin || !atomic_den || !atomic_pcc || !adensity_grid || !pccdensity_grid ||
      !density_grid)
    return fail(LCP_EINVAL, "NULL argument");
  if (spinpol < LCP_SPIN_OFF || spinpol > LCP_SPIN_NC) return fail(LCP_EINVAL, "please check SpinPol");
  if (spinpol == LCP_SPIN_NC && !init_atoms_angle) return fail(LCP_EINVAL, "NULL Init_Atoms_Angle");
  const UCell& u = ucell->u;
  const int natom = u.natom;
  const int nch = spinpol == LCP_SPIN_OFF ? 1 : (spinpol == LCP_SPIN_ON ? 2 : 4);
  for (int c = 0; c < nch; ++c)
    if (!density_grid[c]) return fail(LCP_EINVAL, "NULL channel");
  cudaStream_t st = ctx->stream;
  // species tables
  std::vector<Radial> den(nspecies), pcc(nspecies);
  std::vector<std::unique_ptr<DBuf>> keep;
  auto put = [&](const lcp_radial& r, Radial& out) -> lcp_status {
    if (r.num_mesh < 8 || !r.xv || !r.rv || !r.yv) return fail(LCP_EINVAL, "radial table needs >= 8 mesh points");
    const double* src[3] = {r.xv, r.rv, r.yv};
    const int64_t len[3] = {r.num_mesh, r.num_mesh, r.num_mesh + 4};
    const double* dst[3];
    for (int k = 0; k < 3; ++k) {
      keep.emplace_back(new DBuf());
      API_CUDA(keep.back()->ensure(len[k] * sizeof(double)), "alloc");
      API_CUDA(cudaMemcpyAsync(keep.back()->p, src[k], len[k] * sizeof(double), cudaMemcpyHostToDevice, st), "H2D");
      dst[k] = keep.back()->as<double>();
    }
    out = Radial{r.num_mesh, dst[0], dst[1], dst[2]};
    return LCP_OK;
  };
  for (int k = 0; k < nspecies; ++k) {
    if ((s = put(atomic_den[k], den[k]))) return s;
    if ((s = put(atomic_pcc[k], pcc[k]))) return s;
  }
  std::vector<AdenAtom> atoms(natom);
  for (int a = 0; a < natom; ++a) {
    const int spe = u.atom2spe[a] - 1;
    if (spe < 0 || spe >= nspecies) return fail(LCP_EINVAL, "atom2spe out of the species range");
    AdenAtom& A = atoms[a];
    for (int d = 0; d < 3; ++d) A.g[d] = u.gxyz[a * 3 + d];
    const double nu = init_atoms_nspin[2 * a], nd = init_atoms_nspin[2 * a + 1];
    const double nele = nu + nd;
    A.ou = nele > 1e-15 ? nu / nele : 0.0;
    A.od = nele > 1e-15 ? nd / nele : 0.0;
    const double th = init_atoms_angle ? init_atoms_angle[2 * a] : 0.0;
    const double ph = init_atoms_angle ? init_atoms_angle[2 * a + 1] : 0.0;
    A.sit = std::sin(th);
    A.cot = std::cos(th);
    A.sip = std::sin(ph);
    A.cop = std::cos(ph);
    A.spe = spe;
  }
  const int64_t nn = u.nn();
  const int64_t nent = u.sphere_off[natom];
  DBuf d_atoms, d_den, d_pcc, d_off, d_gl, d_cl, d_atv, d_cnt, d_start, d_scan, d_idx, d_out[6];
  API_CUDA(to_device(d_atoms, atoms, st), "H2D");
  API_CUDA(to_device(d_den, den, st), "H2D");
  API_CUDA(to_device(d_pcc, pcc, st), "H2D");
  API_CUDA(to_device(d_off, u.sphere_off, st), "H2D");
  API_CUDA(to_device(d_gl, u.glist, st), "H2D");
  API_CUDA(to_device(d_cl, u.clist, st), "H2D");
  API_CUDA(to_device(d_atv, u.atv, st), "H2D");
  API_CUDA(d_cnt.ensure(nn * sizeof(int32_t)), "alloc");
  API_CUDA(d_start.ensure((nn + 1) * sizeof(int64_t)), "alloc");
  API_CUDA(d_scan.ensure((scan_blocks(nn) + 1) * sizeof(int64_t)), "alloc");
  API_CUDA(d_idx.ensure(std::max<int64_t>(nent, 1) * sizeof(int32_t)), "alloc");
  API_CUDA(cudaMemsetAsync(d_cnt.p, 0, nn * sizeof(int32_t), st), "memset");
  entry_count_kernel<<<grid_for(nent, 256), 256, 0, st>>>(d_gl.as<int32_t>(), nent, d_cnt.as<int32_t>());
  API_CUDA(cudaGetLastError(), "entry count");
  API_CUDA(exclusive_scan_i32(d_cnt.as<int32_t>(), nn, d_start.as<int64_t>(), d_scan.as<int64_t>(), st), "scan");
  API_CUDA(cudaMemsetAsync(d_cnt.p, 0, nn * sizeof(int32_t), st), "memset");
  entry_fill_kernel<<<grid_for(nent, 256), 256, 0, st>>>(d_gl.as<int32_t>(), nent, d_start.as<int64_t>(),
                                                          d_cnt.as<int32_t>(), d_idx.as<int32_t>());
  API_CUDA(cudaGetLastError(), "entry fill");
  AdenArgs a{};
  for (int d = 0; d < 3; ++d) {
    a.ng[d] = u.ngrid[d];
    a.origin[d] = u.origin[d];
    for (int e = 0; e < 3; ++e) a.glat[d][e] = u.glat[d][e];
  }
  a.spinpol = spinpol;
  a.natom = natom;
  a.nn = nn;
  a.atv = d_atv.as<double>();
  a.atoms = d_atoms.as<AdenAtom>();
  a.den = d_den.as<Radial>();
  a.pcc = d_pcc.as<Radial>();
  a.sphere_off = d_off.as<int64_t>();
  a.glist = d_gl.as<int32_t>();
  a.clist = d_cl.as<int32_t>();
  a.start = d_start.as<int64_t>();
  a.idx = d_idx.as<int32_t>();
  for (int k = 0; k < 2 + nch; ++k) API_CUDA(d_out[k].ensure(nn * sizeof(double)), "alloc");
  a.aden = d_out[0].as<double>();
  a.pccd = d_out[1].as<double>();
  for (int c = 0; c < nch; ++c) a.rho[c] = d_out[2 + c].as<double>();
  adenpcc_gather_kernel<<<grid_for(nn, 128), 128, 0, st>>>(a);
  API_CUDA(cudaGetLastError(), "adenpcc");
  ctx->launches += 6;
  API_CUDA(cudaMemcpyAsync(adensity_grid, a.aden, nn * sizeof(double), cudaMemcpyDeviceToHost, st), "D2H");
  API_CUDA(cudaMemcpyAsync(pccdensity_grid, a.pccd, nn * sizeof(double), cudaMemcpyDeviceToHost, st), "D2H");
  for (int c = 0; c < nch; ++c)
    API_CUDA(cudaMemcpyAsync(density_grid[c], a.rho[c], nn * sizeof(double), cudaMemcpyDeviceToHost, st), "D2H");
  API_CUDA(cudaStreamSynchronize(st), "adenpcc");
  return LCP_OK;
}

}  // extern "C"
