// Hand-written 3-D FFT Poisson solve (src/Poisson.jl:1-108):
//
//   dV_H = IFFT[ S(G) * FFT(drho) ],  S = 4 pi / |G|^2 symmetrised, S(0) = 0,
//
// with drho = 2 rho - 2 rho_a ("off") or rho_up + rho_down - 2 rho_a.  The
// factors S (FP64, with the inverse's 1/NN folded in) come from the cell's
// tabulated half-spectrum table (GridCell::pfac, launch_poisson_table).
//
// Five passes over the half spectrum X[i][j][k'] (k' < N3/2 + 1, the layout of
// a real-to-complex transform of a C-order grid):
//   1. rows:  the real transform along k of two grid rows at once (row a as
//      the real part, row b as the imaginary part of one complex transform of
//      length N3, separated by the conjugate symmetry of real inputs), with
//      the source drho formed on load;
//   2. j:     complex transforms along j, W columns k' per block;
//   3. i:     forward along i, times S (FP64), inverse along i, in one pass;
//   4. j:     inverse along j;
//   5. rows:  the inverse real transform of two rows at once, written to dV_H.
// Every pencil is transformed in shared memory by one warp: a mixed-radix
// Stockham autosort FFT (radix 4, 2 and 3 butterflies in registers, any other
// prime radix by its direct DFT), natural order in and out, with the
// pencil length's roots of unity from a host-built table.
//
// Arithmetic: FP64 for the FP64 drop-in form; double-float (pairs of FP32,
// about 48 significant bits, on the FP32 pipe) for the precision forms, where
// only the G = 0 handling and the reciprocal-space scaling stay FP64.  Both
// store the spectrum as 16-byte complex elements.
#include <cuda_runtime.h>

#include <cmath>
#include <map>
#include <mutex>
#include <type_traits>
#include <utility>
#include <vector>

#include "lcp_device.h"
#include "lcp_dfloat.cuh"
#include "lcp_pdl.cuh"

namespace lcp {

namespace {

// ------------------------------------------------------------ arithmetic
//
// Double-float (lcp_dfloat.cuh) for the precision forms, FP64 for the
// drop-in; the same butterflies serve both through these overloads.

__device__ __forceinline__ double add_lazy(double a, double b) { return a + b; }
__device__ __forceinline__ double dot2(double a, double b, double c, double d) { return fma(a, b, c * d); }

template <class T>
struct Num;
template <>
struct Num<double> {
  __device__ static double from(double x) { return x; }
  __device__ static double to(double x) { return x; }
  __device__ static double half(double x) { return 0.5 * x; }
  __device__ static double twice(double x) { return x + x; }
  __device__ static double zero() { return 0.0; }
};
template <>
struct Num<Dfl> {
  __device__ static Dfl from(double x) { return dfl_of(x); }
  __device__ static double to(Dfl x) { return dbl_of(x); }  // one FP64 add
  __device__ static Dfl half(Dfl x) { return {0.5f * x.hi, 0.5f * x.lo}; }
  __device__ static Dfl twice(Dfl x) { return {x.hi + x.hi, x.lo + x.lo}; }
  __device__ static Dfl zero() { return {0.f, 0.f}; }
};

template <class T>
struct Cx {
  T x, y;
};
template <class T>
__device__ __forceinline__ Cx<T> operator+(Cx<T> a, Cx<T> b) { return {a.x + b.x, a.y + b.y}; }
template <class T>
__device__ __forceinline__ Cx<T> operator-(Cx<T> a, Cx<T> b) { return {a.x - b.x, a.y - b.y}; }
template <class T>
__device__ __forceinline__ Cx<T> cadd_l(Cx<T> a, Cx<T> b) { return {add_lazy(a.x, b.x), add_lazy(a.y, b.y)}; }
template <class T>
__device__ __forceinline__ Cx<T> csub_l(Cx<T> a, Cx<T> b) { return {add_lazy(a.x, -b.x), add_lazy(a.y, -b.y)}; }
template <class T>
__device__ __forceinline__ Cx<T> cmul(Cx<T> a, Cx<T> b) {
  return {dot2(a.x, b.x, -a.y, b.y), dot2(a.x, b.y, a.y, b.x)};
}
template <class T>
__device__ __forceinline__ Cx<T> conj(Cx<T> a) { return {a.x, -a.y}; }
// renormalised (double-float): the passes store normalised elements
__device__ __forceinline__ Cx<double> norm(Cx<double> a) { return a; }
__device__ __forceinline__ Cx<Dfl> norm(Cx<Dfl> a) {
  return {quick_two_sum(a.x.hi, a.x.lo), quick_two_sum(a.y.hi, a.y.lo)};
}
// -i * a and +i * a
template <class T>
__device__ __forceinline__ Cx<T> mul_mi(Cx<T> a) { return {a.y, -a.x}; }
template <class T>
__device__ __forceinline__ Cx<T> mul_pi(Cx<T> a) { return {-a.y, a.x}; }
template <class T>
__device__ __forceinline__ Cx<T> scale(Cx<T> a, T s) { return {a.x * s, a.y * s}; }

static_assert(sizeof(Cx<double>) == 16 && sizeof(Cx<Dfl>) == 16, "16-byte spectrum elements");

// ------------------------------------------------------------ one pencil in shared memory

// Roots of unity of the pencil length n: w[m] = exp(-2 pi i m / n); the
// inverse transform uses their conjugates.
template <class T, bool INV>
__device__ __forceinline__ Cx<T> root(const Cx<T>* w, int m) {
  const Cx<T> r = w[m];
  return INV ? conj(r) : r;
}

// One butterfly of a Stockham stage: inputs a[j + r nb] (r < R), each times
// its twiddle omega_n^(r k tstep) when tw (ns > 1), outputs b[o + s ns].  In
// double-float the outputs are left unnormalised (a stage's sums feed the
// next stage's sums and FMA-based products, which take them as they are);
// the passes renormalise what they store.
template <class T, bool INV>
__device__ __forceinline__ void bfly2(const Cx<T>* a, Cx<T>* b, int j, int nb, int o, int ns, bool tw, int m,
                                      const Cx<T>* w) {
  const Cx<T> v0 = a[j];
  Cx<T> v1 = a[j + nb];
  if (tw) v1 = cmul(v1, root<T, INV>(w, m));
  b[o] = cadd_l(v0, v1);
  b[o + ns] = csub_l(v0, v1);
}

template <class T, bool INV>
__device__ __forceinline__ void bfly4(const Cx<T>* a, Cx<T>* b, int j, int nb, int o, int ns, bool tw, int m,
                                      const Cx<T>* w) {
  const Cx<T> v0 = a[j];
  Cx<T> v1 = a[j + nb], v2 = a[j + 2 * nb], v3 = a[j + 3 * nb];
  if (tw) {
    v1 = cmul(v1, root<T, INV>(w, m));
    v2 = cmul(v2, root<T, INV>(w, 2 * m));
    v3 = cmul(v3, root<T, INV>(w, 3 * m));
  }
  const Cx<T> t0 = cadd_l(v0, v2), t1 = csub_l(v0, v2), t2 = cadd_l(v1, v3), t3 = csub_l(v1, v3);
  const Cx<T> r3 = INV ? mul_pi(t3) : mul_mi(t3);  // omega_4 * t3
  b[o] = cadd_l(t0, t2);
  b[o + ns] = cadd_l(t1, r3);
  b[o + 2 * ns] = csub_l(t0, t2);
  b[o + 3 * ns] = csub_l(t1, r3);
}

template <class T, bool INV>
__device__ __forceinline__ void bfly3(const Cx<T>* a, Cx<T>* b, int j, int nb, int o, int ns, bool tw, int m,
                                      const Cx<T>* w, int n) {
  const Cx<T> v0 = a[j];
  Cx<T> v1 = a[j + nb], v2 = a[j + 2 * nb];
  if (tw) {
    v1 = cmul(v1, root<T, INV>(w, m));
    v2 = cmul(v2, root<T, INV>(w, 2 * m));
  }
  // omega_3 = -1/2 -+ i sqrt(3)/2: Im(w[n/3]) = -sqrt(3)/2
  const T s = w[n / 3].y;
  const Cx<T> t = cadd_l(v1, v2), d = csub_l(v1, v2);
  const Cx<T> mm = csub_l(v0, Cx<T>{Num<T>::half(t.x), Num<T>::half(t.y)});
  const Cx<T> q = scale(INV ? mul_mi(d) : mul_pi(d), s);  // -+ i sqrt(3)/2 * d
  b[o] = cadd_l(v0, t);
  b[o + ns] = cadd_l(mm, q);
  b[o + 2 * ns] = csub_l(mm, q);
}

// radix 5: with t1 = v1 + v4, t2 = v2 + v3, t3 = v1 - v4, t4 = v2 - v3,
// y0 = v0 + t1 + t2, y1,4 = a1 -+ i b1, y2,3 = a2 -+ i b2 (forward; the
// inverse swaps the signs), a1 = v0 + c1 t1 + c2 t2, a2 = v0 + c2 t1 + c1 t2,
// b1 = s1 t3 + s2 t4, b2 = s2 t3 - s1 t4, with omega_5^k = c_k - i s_k.
template <class T, bool INV>
__device__ __forceinline__ void bfly5(const Cx<T>* a, Cx<T>* b, int j, int nb, int o, int ns, bool tw, int m,
                                      const Cx<T>* w, int n) {
  const Cx<T> v0 = a[j];
  Cx<T> v1 = a[j + nb], v2 = a[j + 2 * nb], v3 = a[j + 3 * nb], v4 = a[j + 4 * nb];
  if (tw) {
    v1 = cmul(v1, root<T, INV>(w, m));
    v2 = cmul(v2, root<T, INV>(w, 2 * m));
    v3 = cmul(v3, root<T, INV>(w, 3 * m));
    v4 = cmul(v4, root<T, INV>(w, 4 * m));
  }
  const Cx<T> w1 = w[n / 5], w2 = w[2 * (n / 5)];
  const T c1 = w1.x, c2 = w2.x, s1 = -w1.y, s2 = -w2.y;
  const Cx<T> t1 = cadd_l(v1, v4), t2 = cadd_l(v2, v3), t3 = csub_l(v1, v4), t4 = csub_l(v2, v3);
  const Cx<T> a1 = cadd_l(v0, Cx<T>{dot2(c1, t1.x, c2, t2.x), dot2(c1, t1.y, c2, t2.y)});
  const Cx<T> a2 = cadd_l(v0, Cx<T>{dot2(c2, t1.x, c1, t2.x), dot2(c2, t1.y, c1, t2.y)});
  const Cx<T> b1 = {dot2(s1, t3.x, s2, t4.x), dot2(s1, t3.y, s2, t4.y)};
  const Cx<T> b2 = {dot2(s2, t3.x, -s1, t4.x), dot2(s2, t3.y, -s1, t4.y)};
  const Cx<T> ib1 = INV ? mul_pi(b1) : mul_mi(b1), ib2 = INV ? mul_pi(b2) : mul_mi(b2);
  b[o] = cadd_l(v0, cadd_l(t1, t2));
  b[o + ns] = cadd_l(a1, ib1);
  b[o + 4 * ns] = csub_l(a1, ib1);
  b[o + 2 * ns] = cadd_l(a2, ib2);
  b[o + 3 * ns] = csub_l(a2, ib2);
}

// any other radix: the twiddles applied in place (the lane owns these
// inputs), then the direct DFT with the inputs read from shared memory.
template <class T, bool INV>
__device__ void bfly_dft(Cx<T>* a, Cx<T>* b, int j, int nb, int o, int ns, bool tw, int m, const Cx<T>* w, int n,
                         int R) {
  if (tw)
    for (int r = 1; r < R; ++r) a[j + r * nb] = cmul(a[j + r * nb], root<T, INV>(w, r * m));
  const int wstep = n / R;  // omega_R = w[n / R]
  for (int s = 0; s < R; ++s) {
    Cx<T> acc = a[j];
    int rs = 0;
    for (int r = 1; r < R; ++r) {
      rs += s;
      if (rs >= R) rs -= R;  // (r s) mod R
      acc = acc + cmul(a[j + r * nb], root<T, INV>(w, rs * wstep));
    }
    b[o + s * ns] = acc;
  }
}

// Stockham autosort FFT of length n on a (natural order), b scratch; returns
// the buffer holding the result.  One warp per pencil (lane = 0..31); both
// buffers may be overwritten.
template <class T, bool INV>
__device__ Cx<T>* fft_warp(Cx<T>* a, Cx<T>* b, int n, const int* fac, int nfac, const Cx<T>* w, int lane) {
  int ns = 1;
  for (int st = 0; st < nfac; ++st) {
    const int R = fac[st];
    const int nb = n / R;
    const int tstep = n / (ns * R);  // root index step of this stage's twiddles
    const bool tw = ns > 1;
    for (int j = lane; j < nb; j += 32) {
      const int k = j % ns;
      const int o = (j - k) * R + k;  // (j / ns) * ns * R + k
      const int m = k * tstep;
      if (R == 4)
        bfly4<T, INV>(a, b, j, nb, o, ns, tw, m, w);
      else if (R == 2)
        bfly2<T, INV>(a, b, j, nb, o, ns, tw, m, w);
      else if (R == 3)
        bfly3<T, INV>(a, b, j, nb, o, ns, tw, m, w, n);
      else if (R == 5)
        bfly5<T, INV>(a, b, j, nb, o, ns, tw, m, w, n);
      else
        bfly_dft<T, INV>(a, b, j, nb, o, ns, tw, m, w, n, R);
    }
    __syncwarp();
    Cx<T>* t = a;
    a = b;
    b = t;
    ns *= R;
  }
  return a;
}

// ------------------------------------------------------------ passes

struct FftArgs {
  FftGeom g;
  GridCell c0;            // the cell when cells == nullptr
  const GridCell* cells;  // else blockIdx.y selects the cell
  int spinpol;            // source: LCP_SPIN_OFF / ON (rho_up + rho_down); -1: the cell's real array as is
  int W;                  // passes 2-4: pencils (warps) per block
  int colstride;          // their shared-memory stride in elements (odd: no bank conflicts)
  int pfstride;           // the factors' stride in doubles (pass 3)
};

__device__ __forceinline__ const GridCell& fft_cell(const FftArgs& a) { return a.cells ? a.cells[blockIdx.y] : a.c0; }

template <class T>
__device__ __forceinline__ const Cx<T>* roots_of(const FftGeom& g, int axis) {
  return reinterpret_cast<const Cx<T>*>(std::is_same<T, double>::value ? g.roots64[axis] : g.roots32[axis]);
}

// The passes are chained by programmatic dependent launch (lcp_pdl.cuh): a
// pass loads its roots before it waits for the previous pass's writes.

// Copies the pencil length's roots into shared memory.
template <class T>
__device__ __forceinline__ void load_roots(Cx<T>* dst, const Cx<T>* src, int n) {
  for (int m = threadIdx.x; m < n; m += blockDim.x) dst[m] = src[m];
}

// The source at grid point x: 2 rho - 2 rho_a ("off"), rho_up + rho_down -
// 2 rho_a ("on"), or the cell's real array.  FP64 for the FP64 form; for
// double-float, each term converted and summed in double-float.
template <class T>
__device__ __forceinline__ T source_at(const GridCell& c, int spinpol, int64_t x) {
  if (spinpol < 0) return Num<T>::from(c.real[x]);
  if (std::is_same<T, double>::value) {
    const double aa = c.aden ? c.aden[x] : 0.0;
    return Num<T>::from(spinpol == LCP_SPIN_OFF ? 2 * c.rho[0][x] - 2 * aa : c.rho[0][x] + c.rho[1][x] - 2 * aa);
  }
  T v = spinpol == LCP_SPIN_OFF ? Num<T>::twice(Num<T>::from(c.rho[0][x]))
                                : Num<T>::from(c.rho[0][x]) + Num<T>::from(c.rho[1][x]);
  if (c.aden) v = v - Num<T>::twice(Num<T>::from(c.aden[x]));
  return v;
}

constexpr int kRowWarps = 4;

// Pass 1: the source rows (two per warp) to their half spectra.
template <class T>
__global__ void __launch_bounds__(32 * kRowWarps, 8) fft_rows_fwd_kernel(const __grid_constant__ FftArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  const GridCell& c = fft_cell(a);
  const int n = a.g.n[2], h = n / 2 + 1;
  const int64_t nrows = (int64_t)a.g.n[0] * a.g.n[1];
  Cx<T>* w = reinterpret_cast<Cx<T>*>(smem);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  Cx<T>* buf = w + n + (size_t)warp * 2 * n;
  pdl_trigger();
  load_roots(w, roots_of<T>(a.g, 2), n);
  pdl_wait();
  __syncthreads();
  const int64_t pair = (int64_t)blockIdx.x * (blockDim.x >> 5) + warp;
  const int64_t ra = 2 * pair, rb = ra + 1;
  if (ra >= nrows) return;
  const bool has_b = rb < nrows;
  for (int k = lane; k < n; k += 32) {
    const T va = source_at<T>(c, a.spinpol, ra * n + k);
    const T vb = has_b ? source_at<T>(c, a.spinpol, rb * n + k) : Num<T>::zero();
    buf[k] = {va, vb};
  }
  __syncwarp();
  const Cx<T>* z = fft_warp<T, false>(buf, buf + n, n, a.g.fac[2], a.g.nfac[2], w, lane);
  Cx<T>* spec = reinterpret_cast<Cx<T>*>(c.spec);
  for (int k = lane; k < h; k += 32) {
    const Cx<T> p = z[k], q = conj(z[k == 0 ? 0 : n - k]);
    const Cx<T> s = p + q, d = p - q;
    spec[ra * h + k] = {Num<T>::half(s.x), Num<T>::half(s.y)};  // (z + conj z(-k)) / 2
    if (has_b) spec[rb * h + k] = {Num<T>::half(d.y), Num<T>::half(-d.x)};  // (z - conj z(-k)) / 2i
  }
}

// Pass 5: the half spectra of two rows to the real output rows.
template <class T>
__global__ void __launch_bounds__(32 * kRowWarps, 8) fft_rows_inv_kernel(const __grid_constant__ FftArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  const GridCell& c = fft_cell(a);
  const int n = a.g.n[2], h = n / 2 + 1;
  const int64_t nrows = (int64_t)a.g.n[0] * a.g.n[1];
  Cx<T>* w = reinterpret_cast<Cx<T>*>(smem);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  Cx<T>* buf = w + n + (size_t)warp * 2 * n;
  pdl_trigger();
  load_roots(w, roots_of<T>(a.g, 2), n);
  pdl_wait();
  __syncthreads();
  const int64_t pair = (int64_t)blockIdx.x * (blockDim.x >> 5) + warp;
  const int64_t ra = 2 * pair, rb = ra + 1;
  if (ra >= nrows) return;
  const bool has_b = rb < nrows;
  const Cx<T>* spec = reinterpret_cast<const Cx<T>*>(c.spec);
  for (int k = lane; k < n; k += 32) {
    const bool lower = k < h;
    const int kk = lower ? k : n - k;
    Cx<T> p = spec[ra * h + kk];
    Cx<T> q = has_b ? spec[rb * h + kk] : Cx<T>{Num<T>::zero(), Num<T>::zero()};
    if (kk == 0 || 2 * kk == n) {  // the real rows' spectra are real there
      p.y = Num<T>::zero();
      q.y = Num<T>::zero();
    }
    if (!lower) {
      p = conj(p);
      q = conj(q);
    }
    buf[k] = p + mul_pi(q);  // row a + i row b
  }
  __syncwarp();
  const Cx<T>* z = fft_warp<T, true>(buf, buf + n, n, a.g.fac[2], a.g.nfac[2], w, lane);
  double* out = const_cast<double*>(c.dvh);
  for (int k = lane; k < n; k += 32) {
    const Cx<T> v = z[k];
    out[ra * n + k] = Num<T>::to(v.x);
    if (has_b) out[rb * n + k] = Num<T>::to(v.y);
  }
}

// Passes 2-4: pencils along axis 1 (j) or 0 (i) of the half spectrum.  The
// pencils are numbered c = outer * h + k' (outer = i for axis 1, j for axis
// 0), and a block takes W consecutive ones, one warp each, so every block is
// full.  Thread t of the block stages column t mod W (consecutive addresses
// for consecutive threads) into a shared-memory stride that is odd in 16-byte
// elements, so these stores hit distinct banks.  MODE 0 forward, 1 inverse, 2
// forward, times the FP64 factors, inverse.
template <class T, int MODE>
__global__ void __launch_bounds__(256, 4) fft_cols_kernel(const __grid_constant__ FftArgs a, int axis) {
  extern __shared__ __align__(16) unsigned char smem[];
  const GridCell& c = fft_cell(a);
  const int n2 = a.g.n[1], h = a.g.n[2] / 2 + 1;
  const int n = a.g.n[axis];
  const int W = a.W, S = a.colstride;
  const int64_t ncols = (int64_t)(axis == 1 ? a.g.n[0] : n2) * h;
  const int64_t estride = axis == 1 ? h : (int64_t)n2 * h;
  Cx<T>* w = reinterpret_cast<Cx<T>*>(smem);
  Cx<T>* bufs = w + n;  // [W][S], S >= 2n
  double* pf = reinterpret_cast<double*>(bufs + (size_t)W * S);  // MODE 2: [W][pfstride]
  pdl_trigger();
  load_roots(w, roots_of<T>(a.g, axis), n);
  pdl_wait();
  Cx<T>* spec = reinterpret_cast<Cx<T>*>(c.spec);
  const int col = threadIdx.x % W;
  const int64_t cid = (int64_t)blockIdx.x * W + col;
  const bool live = cid < ncols;
  const int64_t base = axis == 1 ? (cid / h) * n2 * h + cid % h : cid;
  const int rows = blockDim.x / W;  // elements staged per thread step
  if (live)
    for (int e = threadIdx.x / W; e < n; e += rows) {
      const int64_t x = base + e * estride;
      bufs[(size_t)col * S + e] = spec[x];
      if (MODE == 2) pf[(size_t)col * a.pfstride + e] = c.pfac[x];
    }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int* fac = a.g.fac[axis];
  const int nfac = a.g.nfac[axis];
  if ((int64_t)blockIdx.x * W + warp < ncols) {
    Cx<T>* p = bufs + (size_t)warp * S;
    Cx<T>* q = p + n;
    Cx<T>* r = fft_warp<T, MODE == 1>(p, q, n, fac, nfac, w, lane);
    if (MODE == 2) {
      const double* f = pf + (size_t)warp * a.pfstride;
      for (int e = lane; e < n; e += 32) {
        const Cx<T> v = r[e];
        r[e] = {Num<T>::from(Num<T>::to(v.x) * f[e]), Num<T>::from(Num<T>::to(v.y) * f[e])};
      }
      __syncwarp();
      fft_warp<T, true>(r, r == p ? q : p, n, fac, nfac, w, lane);
    }
  }
  __syncthreads();
  // every warp's result sits in the same half of its buffer pair
  const int passes = MODE == 2 ? 2 * nfac : nfac;
  const size_t res = (passes & 1) ? (size_t)n : 0;
  if (live)
    for (int e = threadIdx.x / W; e < n; e += rows) spec[base + e * estride] = norm(bufs[(size_t)col * S + res + e]);
}

// Shared-memory budget of a pass 2-4 block: four blocks per SM.
constexpr size_t kColsSmem = 54 * 1024;

// The factors' stride: 2 mod 16 doubles, so the 16 lanes of one 8-byte
// shared-memory wavefront (eight columns, two elements) hit distinct banks.
int pf_stride(int n) { return n + (18 - n % 16) % 16; }

int cols_width(int n, bool with_pf) {
  const size_t roots = (size_t)n * 16;
  const size_t per = (size_t)(2 * n + 1) * 16 + (with_pf ? (size_t)pf_stride(n) * 8 : 0);
  const size_t w = roots < kColsSmem ? (kColsSmem - roots) / per : 0;
  return (int)std::max<size_t>(1, std::min<size_t>(8, w));
}

// The preferred shared-memory carveout, set once per kernel and device.
cudaError_t prefer_shared(const void* kernel) {
  static std::mutex mu;
  static std::map<std::pair<const void*, int>, bool> done;
  int dev = 0;
  LCP_CUDA_TRY(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(mu);
  bool& d = done[std::make_pair(kernel, dev)];
  if (d) return cudaSuccess;
  LCP_CUDA_TRY(cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                                    (int)cudaSharedmemCarveoutMaxShared));
  d = true;
  return cudaSuccess;
}

template <class T>
cudaError_t launch_fft_t(const FftGeom& g, FftArgs args, int ncells, cudaStream_t st) {
  const int n1 = g.n[0], n2 = g.n[1], n3 = g.n[2], h = n3 / 2 + 1;
  const int64_t pairs = ((int64_t)n1 * n2 + 1) / 2;
  const dim3 rgrid((unsigned)((pairs + kRowWarps - 1) / kRowWarps), (unsigned)ncells);
  const size_t rsm = (size_t)n3 * 16 * (1 + 2 * kRowWarps);
  LCP_CUDA_TRY(raise_smem(fft_rows_fwd_kernel<T>, rsm));
  LCP_CUDA_TRY(raise_smem(fft_rows_inv_kernel<T>, rsm));
  LCP_CUDA_TRY(prefer_shared(reinterpret_cast<const void*>(fft_rows_fwd_kernel<T>)));
  LCP_CUDA_TRY(prefer_shared(reinterpret_cast<const void*>(fft_rows_inv_kernel<T>)));
  LCP_CUDA_TRY(launch_pdl(fft_rows_fwd_kernel<T>, rgrid, dim3(32 * kRowWarps), rsm, st, args));
  auto cols = [&](auto kern, int axis, bool with_pf) -> cudaError_t {
    const int n = g.n[axis];
    const int W = cols_width(n, with_pf);
    args.W = W;
    args.colstride = 2 * n + 1;
    args.pfstride = pf_stride(n);
    const int64_t ncols = (int64_t)(axis == 1 ? n1 : n2) * h;
    const size_t sm = (size_t)n * 16 + (size_t)W * args.colstride * 16 +
                      (with_pf ? (size_t)W * args.pfstride * 8 : 0);
    LCP_CUDA_TRY(raise_smem(kern, sm));
    LCP_CUDA_TRY(prefer_shared(reinterpret_cast<const void*>(kern)));
    return launch_pdl(kern, dim3((unsigned)((ncols + W - 1) / W), (unsigned)ncells), dim3(32 * W), sm, st, args,
                      axis);
  };
  LCP_CUDA_TRY(cols(fft_cols_kernel<T, 0>, 1, false));
  LCP_CUDA_TRY(cols(fft_cols_kernel<T, 2>, 0, true));
  LCP_CUDA_TRY(cols(fft_cols_kernel<T, 1>, 1, false));
  return launch_pdl(fft_rows_inv_kernel<T>, rgrid, dim3(32 * kRowWarps), rsm, st, args);
}

}  // namespace

cudaError_t raise_smem_limit(const void* kernel, size_t bytes) {
  static std::mutex mu;
  static std::map<std::pair<const void*, int>, size_t> set;
  int dev = 0;
  LCP_CUDA_TRY(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(mu);
  size_t& cur = set[std::make_pair(kernel, dev)];
  if (bytes <= cur) return cudaSuccess;
  LCP_CUDA_TRY(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
  cur = bytes;
  return cudaSuccess;
}

// Radices of a pencil length: fours first, then a two, then threes, fives,
// sevens and any larger primes.
int fft_factor(int n, int* fac) {
  int k = 0;
  while (n % 4 == 0 && k < kFftMaxFactors) {
    fac[k++] = 4;
    n /= 4;
  }
  for (int p = 2; n > 1 && k < kFftMaxFactors; ++p) {
    while (n % p == 0 && k < kFftMaxFactors) {
      fac[k++] = p;
      n /= p;
    }
    if (p * p > n && n > 1 && k < kFftMaxFactors) {
      fac[k++] = n;
      n = 1;
    }
  }
  return n == 1 ? k : -1;
}

bool fft_supported(const int32_t* ng) {
  int fac[kFftMaxFactors];
  for (int d = 0; d < 3; ++d)
    if (ng[d] < 1 || ng[d] > kFftMaxN || fft_factor(ng[d], fac) < 0) return false;
  return true;
}

// The roots of unity of one pencil length: exp(-2 pi i m / n), m < n, in
// double (re, im) and in double-float (re.hi, re.lo, im.hi, im.lo), from the
// host's long double sine and cosine.
void fft_roots(int n, std::vector<double>& r64, std::vector<float>& r32) {
  r64.resize((size_t)2 * n);
  r32.resize((size_t)4 * n);
  const long double two_pi = 6.283185307179586476925286766559005768L;
  for (int m = 0; m < n; ++m) {
    const long double t = two_pi * (long double)m / (long double)n;
    const long double c = cosl(t), s = -sinl(t);
    const long double v[2] = {c, s};
    for (int q = 0; q < 2; ++q) {
      const double d = (double)v[q];
      r64[2 * m + q] = d;
      const float hi = (float)v[q];
      r32[4 * m + 2 * q] = hi;
      r32[4 * m + 2 * q + 1] = (float)(v[q] - (long double)hi);
    }
  }
}

cudaError_t launch_poisson_fft(const FftGeom& g, bool fp64, int spinpol, const GridCell& c0, const GridCell* cells,
                               int ncells, cudaStream_t st) {
  if (ncells <= 0) return cudaSuccess;
  FftArgs a{};
  a.g = g;
  a.c0 = c0;
  a.cells = cells;
  a.spinpol = spinpol;
  return fp64 ? launch_fft_t<double>(g, a, ncells, st) : launch_fft_t<Dfl>(g, a, ncells, st);
}

}  // namespace lcp
