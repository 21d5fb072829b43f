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

namespace lcp {

namespace {

// ------------------------------------------------------------ double-float arithmetic
//
// A value is hi + lo with |lo| <= ulp(hi)/2: Dekker's exact product (here
// with an FMA) and Knuth's two-sum, renormalised after every operation.

struct Dfl {
  float hi, lo;
};

__device__ __forceinline__ Dfl quick_two_sum(float s, float e) {
  const float r = s + e;
  return {r, e - (r - s)};
}

__device__ __forceinline__ Dfl operator+(Dfl a, Dfl b) {
  const float s = a.hi + b.hi;
  const float bb = s - a.hi;
  const float e = (a.hi - (s - bb)) + (b.hi - bb) + (a.lo + b.lo);
  return quick_two_sum(s, e);
}
__device__ __forceinline__ Dfl operator-(Dfl a) { return {-a.hi, -a.lo}; }
__device__ __forceinline__ Dfl operator-(Dfl a, Dfl b) { return a + (-b); }
__device__ __forceinline__ Dfl operator*(Dfl a, Dfl b) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  return quick_two_sum(p, e);
}

template <class T>
struct Num;
template <>
struct Num<double> {
  __device__ static double from(double x) { return x; }
  __device__ static double to(double x) { return x; }
  __device__ static double half(double x) { return 0.5 * x; }
  __device__ static double zero() { return 0.0; }
};
template <>
struct Num<Dfl> {
  __device__ static Dfl from(double x) {
    const float h = (float)x;
    return {h, (float)(x - (double)h)};
  }
  __device__ static double to(Dfl x) { return (double)x.hi + (double)x.lo; }
  __device__ static Dfl half(Dfl x) { return {0.5f * x.hi, 0.5f * x.lo}; }
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
__device__ __forceinline__ Cx<T> operator*(Cx<T> a, Cx<T> b) {
  return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x};
}
template <class T>
__device__ __forceinline__ Cx<T> conj(Cx<T> a) { return {a.x, -a.y}; }
// -i * a and +i * a
template <class T>
__device__ __forceinline__ Cx<T> mul_mi(Cx<T> a) { return {a.y, -a.x}; }
template <class T>
__device__ __forceinline__ Cx<T> mul_pi(Cx<T> a) { return {-a.y, a.x}; }
template <class T>
__device__ __forceinline__ Cx<T> scale(Cx<T> a, T s) { return {a.x * s, a.y * s}; }

static_assert(sizeof(Cx<double>) == 16 && sizeof(Cx<Dfl>) == 16, "16-byte spectrum elements");

// ------------------------------------------------------------ one pencil in shared memory

constexpr int kRegRadix = 8;  // radices up to this size keep their points in registers

// Roots of unity of the pencil length n: w[m] = exp(-2 pi i m / n); the
// inverse transform uses their conjugates.
template <class T, bool INV>
__device__ __forceinline__ Cx<T> root(const Cx<T>* w, int m) {
  const Cx<T> r = w[m];
  return INV ? conj(r) : r;
}

// Stockham autosort FFT of length n on a (natural order), b scratch; returns
// the buffer holding the result.  One warp per pencil (lane = 0..31).
template <class T, bool INV>
__device__ Cx<T>* fft_warp(Cx<T>* a, Cx<T>* b, int n, const int* fac, int nfac, const Cx<T>* w, int lane) {
  int ns = 1;
  for (int st = 0; st < nfac; ++st) {
    const int R = fac[st];
    const int nb = n / R;
    const int tstep = n / (ns * R);  // root index step of this stage's twiddles
    for (int j = lane; j < nb; j += 32) {
      const int k = j % ns;
      const int o = (j - k) * R + k;  // (j / ns) * ns * R + k
      if (R == 2) {
        Cx<T> v0 = a[j], v1 = a[j + nb];
        if (k) v1 = v1 * root<T, INV>(w, k * tstep);
        b[o] = v0 + v1;
        b[o + ns] = v0 - v1;
      } else if (R == 4) {
        Cx<T> v0 = a[j], v1 = a[j + nb], v2 = a[j + 2 * nb], v3 = a[j + 3 * nb];
        if (k) {
          v1 = v1 * root<T, INV>(w, k * tstep);
          v2 = v2 * root<T, INV>(w, 2 * k * tstep);
          v3 = v3 * root<T, INV>(w, 3 * k * tstep);
        }
        const Cx<T> t0 = v0 + v2, t1 = v0 - v2, t2 = v1 + v3, t3 = v1 - v3;
        const Cx<T> r3 = INV ? mul_pi(t3) : mul_mi(t3);  // omega_4 * t3
        b[o] = t0 + t2;
        b[o + ns] = t1 + r3;
        b[o + 2 * ns] = t0 - t2;
        b[o + 3 * ns] = t1 - r3;
      } else if (R == 3) {
        Cx<T> v0 = a[j], v1 = a[j + nb], v2 = a[j + 2 * nb];
        if (k) {
          v1 = v1 * root<T, INV>(w, k * tstep);
          v2 = v2 * root<T, INV>(w, 2 * k * tstep);
        }
        // omega_3 = -1/2 -+ i sqrt(3)/2: Im(w[n/3]) = -sqrt(3)/2
        const T s = w[n / 3].y;
        const Cx<T> t = v1 + v2, d = v1 - v2;
        const Cx<T> m = {v0.x - Num<T>::half(t.x), v0.y - Num<T>::half(t.y)};
        const Cx<T> q = scale(INV ? mul_mi(d) : mul_pi(d), s);  // -+ i sqrt(3)/2 * d
        b[o] = v0 + t;
        b[o + ns] = m + q;
        b[o + 2 * ns] = m - q;
      } else if (R <= kRegRadix) {
        Cx<T> v[kRegRadix];
#pragma unroll
        for (int r = 0; r < kRegRadix; ++r)
          if (r < R) {
            v[r] = a[j + r * nb];
            if (k && r) v[r] = v[r] * root<T, INV>(w, r * k * tstep);
          }
        const int wstep = n / R;  // omega_R = w[n / R]
#pragma unroll
        for (int s = 0; s < kRegRadix; ++s)
          if (s < R) {
            Cx<T> acc = v[0];
            for (int r = 1; r < R; ++r) acc = acc + v[r] * root<T, INV>(w, ((r * s) % R) * wstep);
            b[o + s * ns] = acc;
          }
      } else {
        // a larger prime radix: its direct DFT, points read from shared memory
        const int wstep = n / R;
        for (int s = 0; s < R; ++s) {
          Cx<T> acc = a[j];
          for (int r = 1; r < R; ++r) {
            Cx<T> x = a[j + r * nb];
            if (k) x = x * root<T, INV>(w, r * k * tstep);
            acc = acc + x * root<T, INV>(w, ((r * s) % R) * wstep);
          }
          b[o + s * ns] = acc;
        }
      }
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
};

__device__ __forceinline__ const GridCell& fft_cell(const FftArgs& a) { return a.cells ? a.cells[blockIdx.y] : a.c0; }

template <class T>
__device__ __forceinline__ const Cx<T>* roots_of(const FftGeom& g, int axis) {
  return reinterpret_cast<const Cx<T>*>(std::is_same<T, double>::value ? g.roots64[axis] : g.roots32[axis]);
}

// Copies the pencil length's roots into shared memory.
template <class T>
__device__ __forceinline__ void load_roots(Cx<T>* dst, const Cx<T>* src, int n) {
  for (int m = threadIdx.x; m < n; m += blockDim.x) dst[m] = src[m];
}

// Pass 1: the source rows (two per warp) to their half spectra.
template <class T>
__global__ void fft_rows_fwd_kernel(const __grid_constant__ FftArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  const GridCell& c = fft_cell(a);
  const int n = a.g.n[2], h = n / 2 + 1;
  const int64_t nrows = (int64_t)a.g.n[0] * a.g.n[1];
  Cx<T>* w = reinterpret_cast<Cx<T>*>(smem);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  Cx<T>* buf = w + n + (size_t)warp * 2 * n;
  load_roots(w, roots_of<T>(a.g, 2), n);
  __syncthreads();
  const int64_t pair = (int64_t)blockIdx.x * (blockDim.x >> 5) + warp;
  const int64_t ra = 2 * pair, rb = ra + 1;
  if (ra >= nrows) return;
  const bool has_b = rb < nrows;
  const double* r0 = c.rho[0];
  const double* r1 = c.rho[1];
  const double* ad = c.aden;
  for (int k = lane; k < n; k += 32) {
    double v[2] = {0.0, 0.0};
    for (int q = 0; q < 2; ++q) {
      if (q == 1 && !has_b) break;
      const int64_t x = (ra + q) * n + k;
      if (a.spinpol < 0) {
        v[q] = c.real[x];
      } else {
        const double aa = ad ? ad[x] : 0.0;
        v[q] = a.spinpol == LCP_SPIN_OFF ? 2 * r0[x] - 2 * aa : r0[x] + r1[x] - 2 * aa;
      }
    }
    buf[k] = {Num<T>::from(v[0]), Num<T>::from(v[1])};
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
__global__ void fft_rows_inv_kernel(const __grid_constant__ FftArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  const GridCell& c = fft_cell(a);
  const int n = a.g.n[2], h = n / 2 + 1;
  const int64_t nrows = (int64_t)a.g.n[0] * a.g.n[1];
  Cx<T>* w = reinterpret_cast<Cx<T>*>(smem);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  Cx<T>* buf = w + n + (size_t)warp * 2 * n;
  load_roots(w, roots_of<T>(a.g, 2), n);
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

// Passes 2-4: pencils along axis 1 (j) or 0 (i) of the half spectrum, W
// consecutive k' columns per block (one warp each).  MODE 0 forward, 1
// inverse, 2 forward, times the FP64 factors, inverse.
template <class T, int MODE>
__global__ void fft_cols_kernel(const __grid_constant__ FftArgs a, int axis, int W) {
  extern __shared__ __align__(16) unsigned char smem[];
  const GridCell& c = fft_cell(a);
  const int n1 = a.g.n[0], n2 = a.g.n[1], h = a.g.n[2] / 2 + 1;
  const int n = a.g.n[axis];
  const int64_t estride = axis == 1 ? h : (int64_t)n2 * h;
  const int ntile = (h + W - 1) / W;
  const int outer = blockIdx.x / ntile;  // i for axis 1, j for axis 0
  const int k0 = (blockIdx.x % ntile) * W;
  const int64_t base = axis == 1 ? (int64_t)outer * n2 * h + k0 : (int64_t)outer * h + k0;
  const int cols = min(W, h - k0);
  Cx<T>* w = reinterpret_cast<Cx<T>*>(smem);
  Cx<T>* bufs = w + n;  // [W][2][n]
  double* pf = reinterpret_cast<double*>(bufs + (size_t)W * 2 * n);  // MODE 2: [W][n]
  load_roots(w, roots_of<T>(a.g, axis), n);
  Cx<T>* spec = reinterpret_cast<Cx<T>*>(c.spec);
  const int total = n * cols;
  for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
    const int e = idx / cols, col = idx - e * cols;
    const int64_t x = base + e * estride + col;
    bufs[(size_t)col * 2 * n + e] = spec[x];
    if (MODE == 2) pf[(size_t)col * n + e] = c.pfac[x];
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int* fac = a.g.fac[axis];
  const int nfac = a.g.nfac[axis];
  if (warp < cols) {
    Cx<T>* p = bufs + (size_t)warp * 2 * n;
    Cx<T>* q = p + n;
    Cx<T>* r = fft_warp<T, MODE == 1>(p, q, n, fac, nfac, w, lane);
    if (MODE == 2) {
      const double* f = pf + (size_t)warp * n;
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
  for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
    const int e = idx / cols, col = idx - e * cols;
    spec[base + e * estride + col] = bufs[(size_t)col * 2 * n + res + e];
  }
}

constexpr int kRowWarps = 4;

int cols_width(int n) {
  const int w = (int)(96 * 1024 / (2 * (size_t)n * 16));
  return std::max(1, std::min(8, w));
}

template <class T>
cudaError_t launch_fft_t(const FftGeom& g, const FftArgs& args, int ncells, cudaStream_t st) {
  const int n1 = g.n[0], n2 = g.n[1], n3 = g.n[2], h = n3 / 2 + 1;
  const int64_t pairs = ((int64_t)n1 * n2 + 1) / 2;
  const dim3 rgrid((unsigned)((pairs + kRowWarps - 1) / kRowWarps), (unsigned)ncells);
  const size_t rsm = (size_t)n3 * 16 * (1 + 2 * kRowWarps);
  LCP_CUDA_TRY(raise_smem(fft_rows_fwd_kernel<T>, rsm));
  LCP_CUDA_TRY(raise_smem(fft_rows_inv_kernel<T>, rsm));
  fft_rows_fwd_kernel<T><<<rgrid, 32 * kRowWarps, rsm, st>>>(args);
  LCP_CUDA_TRY(cudaGetLastError());
  auto cols = [&](auto kern, int axis, bool with_pf) -> cudaError_t {
    const int n = g.n[axis];
    const int W = cols_width(n);
    const int ntile = (h + W - 1) / W;
    const int outer = axis == 1 ? n1 : n2;
    const size_t sm = (size_t)n * 16 * (1 + 2 * W) + (with_pf ? (size_t)W * n * 8 : 0);
    LCP_CUDA_TRY(raise_smem(kern, sm));
    kern<<<dim3((unsigned)(outer * ntile), (unsigned)ncells), 32 * W, sm, st>>>(args, axis, W);
    return cudaGetLastError();
  };
  LCP_CUDA_TRY(cols(fft_cols_kernel<T, 0>, 1, false));
  LCP_CUDA_TRY(cols(fft_cols_kernel<T, 2>, 0, true));
  LCP_CUDA_TRY(cols(fft_cols_kernel<T, 1>, 1, false));
  fft_rows_inv_kernel<T><<<rgrid, 32 * kRowWarps, rsm, st>>>(args);
  return cudaGetLastError();
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
