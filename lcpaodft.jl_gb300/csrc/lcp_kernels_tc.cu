// Tensor-core (tcgen05, BF16 in / FP32 accumulate in TMEM) kernels.
//
// tc_selftest_kernel: one 128 x N x K product with both operands staged in
// shared memory in a chosen canonical layout (K-major or MN-major); used to
// check the descriptor and layout conventions on the device before the grid
// kernels rely on them.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "lcp_device.h"
#include "lcp_tc.cuh"

namespace lcp {

namespace {

constexpr int kSelfM = 128;

__global__ void __launch_bounds__(128) tc_selftest_kernel(const float* __restrict__ A, const float* __restrict__ B,
                                                          float* __restrict__ D, int N, int K, int a_mn, int b_mn,
                                                          int order, int* __restrict__ status) {
  extern __shared__ __align__(1024) uint8_t smem[];
  __shared__ uint64_t mbar;
  __shared__ uint32_t tslot;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  uint8_t* sa = smem;
  uint8_t* sb = smem + kSelfM * K * 2;
  // order 0: [k-group][mn-group][128 B core matrix]: SBO = 128 B, LBO = rows/8 * 128 B
  // order 1: [mn-group][k-group][128 B core matrix]: LBO = 128 B, SBO = K/8 * 128 B
  const uint32_t lbo_a = order ? 128 : (kSelfM / 8) * 128, lbo_b = order ? 128 : (N / 8) * 128;
  const uint32_t sbo_a = order ? (K / 8) * 128 : 128, sbo_b = sbo_a;
  const uint32_t sbo = sbo_a;
  for (int idx = tid; idx < kSelfM * K; idx += blockDim.x) {
    const int m = idx / K, k = idx - m * K;
    const uint32_t off = a_mn ? tc::mnmajor_off(m, k, lbo_a, sbo_a) : tc::kmajor_off(m, k, lbo_a, sbo_a);
    *reinterpret_cast<__nv_bfloat16*>(sa + off) = __float2bfloat16_rn(A[idx]);
  }
  for (int idx = tid; idx < N * K; idx += blockDim.x) {
    const int n = idx / K, k = idx - n * K;
    const uint32_t off = b_mn ? tc::mnmajor_off(n, k, lbo_b, sbo_b) : tc::kmajor_off(n, k, lbo_b, sbo_b);
    *reinterpret_cast<__nv_bfloat16*>(sb + off) = __float2bfloat16_rn(B[idx]);
  }
  tc::fence_proxy_async_smem();
  if (warp == 0) tc::tmem_alloc(&tslot, 256);
  if (tid == 0) {
    tc::mbar_init(&mbar, 1);
    tc::fence_mbar_init();
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tslot;
  if (tid == 0) {
    const uint32_t idesc = tc::idesc_bf16_f32(kSelfM, N, a_mn, b_mn);
    for (int ks = 0; ks < K / 16; ++ks) {
      const uint64_t da = tc::smem_desc(tc::smem_u32(sa + 2 * ks * lbo_a), lbo_a, sbo_a);
      const uint64_t db = tc::smem_desc(tc::smem_u32(sb + 2 * ks * lbo_b), lbo_b, sbo_b);
      tc::mma_bf16(tmem, da, db, idesc, ks > 0 ? 1u : 0u);
    }
    tc::mma_commit(&mbar);
  }
  bool ok = tc::mbar_wait(&mbar, 0);
  if (!ok) {
    if (tid == 0) atomicExch(status, LCP_ETIMEDOUT);
    tc::mbar_wait(&mbar, 0);  // give in-flight MMAs a second bounded window before freeing TMEM
  }
  tc::fence_after_sync();
  if (ok) {
    for (int c = 0; c < N / 16; ++c) {
      float v[16];
      tc::tmem_ld16(tc::tmem_addr(tmem, warp * 32, c * 16), v);
      const int row = warp * 32 + lane;
#pragma unroll
      for (int i = 0; i < 16; ++i) D[row * N + c * 16 + i] = v[i];
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, 256);
}

}  // namespace

cudaError_t launch_tc_selftest(const float* A, const float* B, float* D, int N, int K, int a_mn, int b_mn,
                               int order, int* status, cudaStream_t st) {
  const size_t smem = (size_t)(kSelfM + N) * K * 2;
  LCP_CUDA_TRY(cudaFuncSetAttribute(tc_selftest_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  tc_selftest_kernel<<<1, 128, smem, st>>>(A, B, D, N, K, a_mn, b_mn, order, status);
  return cudaGetLastError();
}

// ==========================================================================
// Fixed-point BF16 splitting with exact tensor-core accumulation.
//
// tcgen05's FP32 accumulation aligns each MMA's products to the largest one
// and truncates toward zero; sums whose terms share one quantum are exact as
// long as they stay below 2^24 quanta, while mixing magnitudes in one
// accumulator biases long same-sign sums.  Every operand is therefore put on
// a shared fixed-point grid: with a power-of-two scale S >= max|x|,
// u = x / S in [-1, 1] is split as
//
//   u = hi + mid + lo + e,  hi = q1/2^7, mid = q2/2^15, lo = q3/2^23, |q| <= 128,
//
// so every part is an exact BF16 value and |e| <= 2^-24.  All nine part
// products are formed (the mid*lo and lo*lo terms carry the small tails of
// the orbitals, which a six-term product loses).  hi*hi' (integer multiples
// of 2^-14) has its own accumulator, exact up to 1024 terms; the rest are
// 2^-8 and smaller and go to one accumulator (density) or three more, one
// per quantum (matrix elements).  What remains is the input quantisation e.
// ==========================================================================

// ==========================================================================

namespace {

constexpr int kPart = 2048;                    // bf16 per part of a table block
constexpr int kBlockElems = 3 * kPart;         // table block: hi, mid, lo
constexpr int kDsymElems = 768;                // D block: hi, mid, lo (256 each)
constexpr uint32_t kALbo = 2048, kASbo = 128;  // table block [h][g][8 pt][8 orb] as K-major A
constexpr int kDWin = 16;                      // density: images per column window
constexpr uint32_t kBLbo = kDWin * 2 * 128;    // B: [kh][n-group (<= 32)][8 n][8 k]
constexpr int kASmem = 3 * 4096;               // hi, mid, lo
constexpr int kBSmem = 3 * 2 * kBLbo;          // (hi, mid, lo) x (kh) x LBO
constexpr uint32_t kCross = 256;               // TMEM column of the cross-term accumulator

__device__ __forceinline__ void fx_split(double u, __nv_bfloat16& hi, __nv_bfloat16& mid, __nv_bfloat16& lo) {
  const double h = rint(u * 128.0) * (1.0 / 128.0);
  const double r1 = u - h;
  const double m = rint(r1 * 32768.0) * (1.0 / 32768.0);
  const double l = rint((r1 - m) * 8388608.0) * (1.0 / 8388608.0);
  hi = __float2bfloat16_rn((float)h);
  mid = __float2bfloat16_rn((float)m);
  lo = __float2bfloat16_rn((float)l);
}

// Same split for a float p (|p| <= 1) carrying a small correction e
// (|e| <= 2^-23 |p|): every step but the last rounding is exact in FP32 --
// p - hi and r1 - mid are multiples of ulp(p) (resp. ulp(r1)) below 2^24 of
// them -- so the parts are those of p + e up to |lo residual| <= 2^-24.
__device__ __forceinline__ void fx_split_f(float p, float e, __nv_bfloat16& hi, __nv_bfloat16& mid,
                                           __nv_bfloat16& lo) {
  const float h = rintf(p * 128.0f) * 0.0078125f;
  const float r1 = p - h;
  const float m = rintf(r1 * 32768.0f) * (1.0f / 32768.0f);
  const float r2 = (r1 - m) + e;
  const float l = rintf(r2 * 8388608.0f) * (1.0f / 8388608.0f);
  hi = __float2bfloat16_rn(h);
  mid = __float2bfloat16_rn(m);
  lo = __float2bfloat16_rn(l);
}

// Float-float accumulation (Knuth's TwoSum): hi + lo carries the running sum
// with ~2^-48 relative error, at a handful of FP32 operations per term.
__device__ __forceinline__ void ff_add(float& hi, float& lo, float x) {
  const float s = hi + x;
  const float bb = s - hi;
  const float err = (hi - (s - bb)) + (x - bb);
  hi = s;
  lo += err;
}

__device__ __forceinline__ double pow2_ceil(double x) {
  if (!(x > 0.0)) return 1.0;
  int e;
  const double m = frexp(x, &e);  // x = m * 2^e, m in [0.5, 1)
  return m == 0.5 ? ldexp(1.0, e - 1) : ldexp(1.0, e);
}

__device__ __forceinline__ void cp_async16(void* sdst, const void* gsrc) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(tc::smem_u32(sdst)), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory");
}

// max |x| over n doubles (non-negative doubles order like their bit patterns)
__global__ void absmax_kernel(const double* __restrict__ x, int64_t n, unsigned long long* out) {
  double m = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    m = fmax(m, fabs(x[i]));
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0 && m > 0.0) atomicMax(out, (unsigned long long)__double_as_longlong(m));
}

// scale[0] = power of two >= factor * max, scale[1] = its inverse
__global__ void pow2_scale_kernel(const unsigned long long* mx, double factor, double* scale) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    const double s = pow2_ceil(__longlong_as_double((long long)*mx) * factor);
    scale[0] = s;
    scale[1] = 1.0 / s;
  }
}

__global__ void brick_table_kernel(const double* __restrict__ phi, const int64_t* __restrict__ phi_off,
                                   const int32_t* __restrict__ numorbs, const int64_t* __restrict__ sph_off,
                                   int natom, const int32_t* __restrict__ point_code, int64_t npoints,
                                   const double* __restrict__ scale, __nv_bfloat16* __restrict__ tab) {
  const double inv = scale[1];
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < npoints; k += (int64_t)gridDim.x * blockDim.x) {
    int lo = 0, hi = natom;  // atom with sph_off[atom] <= k < sph_off[atom+1]
    while (hi - lo > 1) {
      int mid = (lo + hi) >> 1;
      if (sph_off[mid] <= k) lo = mid;
      else hi = mid;
    }
    const int atom = lo;
    const int no = numorbs[atom];
    const double* src = phi + phi_off[atom] + (k - sph_off[atom]) * no;
    const int code = point_code[k];
    const int64_t blk = code >> 7;
    const int slot = code & 127, g = slot >> 3, r = slot & 7;
    __nv_bfloat16* base = tab + blk * kBlockElems;
    for (int a = 0; a < no && a < 16; ++a) {
      __nv_bfloat16 h, m, l;
      fx_split(src[a] * inv, h, m, l);
      const int off = ((a >> 3) * 16 + g) * 64 + r * 8 + (a & 7);
      base[off] = h;
      base[kPart + off] = m;
      base[2 * kPart + off] = l;
    }
  }
}

// Dsym blocks in the K-major B layout [kh][nh][8 n][8 k]: n = orbital a of the
// pair's atom, k = orbital b of its jatom; fixed-point with scale[0].
__global__ void dsym_kernel(int nloop, const int32_t* __restrict__ pair_atom, const int32_t* __restrict__ pair_jatom,
                            const int64_t* __restrict__ boff, const int32_t* __restrict__ partner,
                            const int32_t* __restrict__ numorbs, const double* __restrict__ dm,
                            const double* __restrict__ scale, __nv_bfloat16* __restrict__ out) {
  const double inv = scale[1];
  const int64_t total = (int64_t)(nloop + 1) * 256;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int p = (int)(e >> 8);
    const int w = (int)(e & 255);
    const int kh = w >> 7, nh = (w >> 6) & 1, rr = (w >> 3) & 7, cc = w & 7;
    const int a = nh * 8 + rr, b = kh * 8 + cc;
    double v = 0.0;
    if (p < nloop) {
      const int i = pair_atom[p], j = pair_jatom[p];
      const int noi = numorbs[i], noj = numorbs[j];
      if (a < noi && b < noj) {
        v = dm[boff[p] + (int64_t)a * noj + b];
        const int q = partner[p];
        if (q != p) v += dm[boff[q] + (int64_t)b * noi + a];
      }
    }
    __nv_bfloat16 h, mm, l;
    const double x = v * inv;
    const float xf = (float)x;
    fx_split_f(xf, (float)(x - (double)xf), h, mm, l);
    out[(int64_t)p * kDsymElems + w] = h;
    out[(int64_t)p * kDsymElems + 256 + w] = mm;
    out[(int64_t)p * kDsymElems + 512 + w] = l;
  }
}

__device__ __forceinline__ int64_t brick_point_index(int64_t hb, int p, const int32_t* bdim, const int32_t* nb,
                                                     const int32_t* ngrid) {
  const int l2 = p % bdim[2], l1 = (p / bdim[2]) % bdim[1], l0 = p / (bdim[1] * bdim[2]);
  const int64_t h2 = hb % nb[2], h1 = (hb / nb[2]) % nb[1], h0 = hb / ((int64_t)nb[1] * nb[2]);
  const int64_t x = h0 * bdim[0] + l0, y = h1 * bdim[1] + l1, z = h2 * bdim[2] + l2;
  return (x * ngrid[1] + y) * ngrid[2] + z;
}

// Sum of the three parts of 8 consecutive values (one 16-byte chunk per part).
__device__ __forceinline__ void load_chunk3(const __nv_bfloat16* p0, double* u) {
  const uint4 vh = *reinterpret_cast<const uint4*>(p0);
  const uint4 vm = *reinterpret_cast<const uint4*>(p0 + kPart);
  const uint4 vl = *reinterpret_cast<const uint4*>(p0 + 2 * kPart);
  const __nv_bfloat16* bh = reinterpret_cast<const __nv_bfloat16*>(&vh);
  const __nv_bfloat16* bm = reinterpret_cast<const __nv_bfloat16*>(&vm);
  const __nv_bfloat16* bl = reinterpret_cast<const __nv_bfloat16*>(&vl);
#pragma unroll
  for (int c = 0; c < 8; ++c)
    u[c] = (double)__bfloat162float(bh[c]) + (double)__bfloat162float(bm[c]) + (double)__bfloat162float(bl[c]);
}

// FP32 form: hi + mid + lo is a multiple of 2^-23 of magnitude <= 1, so the
// sum is exact in FP32.
__device__ __forceinline__ void load_chunk3f(const __nv_bfloat16* p0, float* u) {
  const uint4 vh = *reinterpret_cast<const uint4*>(p0);
  const uint4 vm = *reinterpret_cast<const uint4*>(p0 + kPart);
  const uint4 vl = *reinterpret_cast<const uint4*>(p0 + 2 * kPart);
  const __nv_bfloat16* bh = reinterpret_cast<const __nv_bfloat16*>(&vh);
  const __nv_bfloat16* bm = reinterpret_cast<const __nv_bfloat16*>(&vm);
  const __nv_bfloat16* bl = reinterpret_cast<const __nv_bfloat16*>(&vl);
#pragma unroll
  for (int c = 0; c < 8; ++c) u[c] = (__bfloat162float(bh[c]) + __bfloat162float(bm[c])) + __bfloat162float(bl[c]);
}

// The 16 fixed-point values of one point of a table block.
__device__ __forceinline__ void load_point_row(const __nv_bfloat16* blk, int p, float* u) {
  const int g = p >> 3, r = p & 7;
#pragma unroll
  for (int h = 0; h < 2; ++h) load_chunk3f(blk + (h * 16 + g) * 64 + r * 8, u + h * 8);
}

// ==========================================================================
// Density on grid bricks.
//
// For brick b with atom images S_b (every image whose cutoff sphere touches
// b; m = |S_b|):
//
//   rho(p) = sum_{s <= t} phi_s(p)^T Dsym_st phi_t(p),
//   Dsym_st = D_(s,t) + D_(t,s)^T  (s != t),   D_(s,s) for the same image,
//
// the reference's sum over the ordered pairs of the neighbour list restricted
// to the brick (src/Matrix/Set_Density_Grid.jl:268-304).  Points are the MMA M
// dimension (128 slots), image t's 16 (padded) orbitals one K step:
//
//   Y[p, (s,a)] = sum_{t >= s} sum_b phi_t(p)_b Dsym_st[a][b],
//   rho(p)      = sum_{s,a} phi_s(p)_a Y[p, (s,a)],
//
// with Y in TMEM, 16 columns per image of a window of up to 16 images s.  K
// steps run t = m-1 ... c0 so the first step writes every column of the
// window.  The epilogue (one thread per point) sums in FP64; every grid point
// lies in one brick, so rho is written once, without atomics.
// ==========================================================================

struct TcDensArgs {
  int64_t nbricks;
  int32_t bdim[3], nb[3], ngrid[3];
  int32_t npts;
  int32_t zero_pair;
  double phi_scale;      // S_phi
  const double* dscale;  // [S_D, 1/S_D]
  const int64_t* img_off;
  const int32_t* img_block;
  const int64_t* tab_off;
  const int32_t* tab_pair;
  const __nv_bfloat16* tab;
  const __nv_bfloat16* dsym;
  double* rho;
  int* status;
};

__global__ void __launch_bounds__(128) density_tc_kernel(TcDensArgs args) {
  extern __shared__ __align__(1024) uint8_t smem[];
  __shared__ uint64_t mbar[2];
  __shared__ uint32_t tslot;
  __shared__ int abort_flag;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  uint8_t* sA[2] = {smem, smem + kASmem};
  uint8_t* sB[2] = {smem + 2 * kASmem, smem + 2 * kASmem + kBSmem};
  if (warp == 0) tc::tmem_alloc(&tslot, 512);
  if (tid == 0) {
    tc::mbar_init(&mbar[0], 1);
    tc::mbar_init(&mbar[1], 1);
    tc::fence_mbar_init();
    abort_flag = 0;
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tslot;
  const double out_scale = args.phi_scale * args.phi_scale * args.dscale[0];
  uint32_t uses[2] = {0, 0};
  bool pending[2] = {false, false};

  for (int64_t hb = blockIdx.x; hb < args.nbricks && !abort_flag; hb += gridDim.x) {
    const int64_t i0 = args.img_off[hb];
    const int m = (int)(args.img_off[hb + 1] - i0);
    const int32_t* ptab = args.tab_pair + args.tab_off[hb];
    const int p = warp * 32 + lane;
    float acc_hi = 0.0f, acc_lo = 0.0f;
    for (int c0 = 0; c0 < m && !abort_flag; c0 += kDWin) {
      const int c1 = min(c0 + kDWin, m);
      const int nsteps = m - c0;
      for (int k = 0; k < nsteps; ++k) {
        const int t = m - 1 - k;
        const int s_hi = min(t, c1 - 1);
        const int buf = k & 1;
        if (pending[buf]) {
          if (!tc::mbar_wait(&mbar[buf], (uses[buf] - 1) & 1)) {
            if (tid == 0) atomicExch(args.status, LCP_ETIMEDOUT);
            abort_flag = 1;
          }
          pending[buf] = false;
        }
        __syncthreads();
        if (abort_flag) break;
        const uint8_t* gA = reinterpret_cast<const uint8_t*>(args.tab + (int64_t)args.img_block[i0 + t] * kBlockElems);
        for (int c = tid; c < kASmem / 16; c += blockDim.x) cp_async16(sA[buf] + c * 16, gA + c * 16);
        const int nimg = s_hi - c0 + 1;
        for (int c = tid; c < nimg * 96; c += blockDim.x) {
          const int si = c / 96, w = c - si * 96;  // 96 x 16 B per image: (part, kh, 16 chunks)
          const int part = w >> 5, kh = (w >> 4) & 1, q = w & 15;
          int pr = ptab[(c0 + si) * m + t];
          if (pr < 0) pr = args.zero_pair;
          const uint8_t* src = reinterpret_cast<const uint8_t*>(args.dsym + (int64_t)pr * kDsymElems) +
                               part * 512 + kh * 256 + q * 16;
          uint8_t* dst = sB[buf] + part * (2 * kBLbo) + kh * kBLbo + si * 256 + q * 16;
          cp_async16(dst, src);
        }
        cp_async_wait_all();
        tc::fence_proxy_async_smem();
        __syncthreads();
        if (tid == 0) {
          tc::fence_after_sync();
          const uint32_t idesc = tc::idesc_bf16_f32(128, 16 * nimg, 0, 0);
          const uint32_t a0 = tc::smem_u32(sA[buf]), b0 = tc::smem_u32(sB[buf]);
          const uint64_t dah = tc::smem_desc(a0, kALbo, kASbo), dam = tc::smem_desc(a0 + 4096, kALbo, kASbo),
                         dal = tc::smem_desc(a0 + 8192, kALbo, kASbo);
          const uint64_t dbh = tc::smem_desc(b0, kBLbo, 128), dbm = tc::smem_desc(b0 + 2 * kBLbo, kBLbo, 128),
                         dbl = tc::smem_desc(b0 + 4 * kBLbo, kBLbo, 128);
          tc::mma_bf16(tmem, dah, dbh, idesc, k > 0 ? 1u : 0u);
          tc::mma_bf16(tmem + kCross, dah, dbm, idesc, k > 0 ? 1u : 0u);
          tc::mma_bf16(tmem + kCross, dam, dbh, idesc, 1u);
          tc::mma_bf16(tmem + kCross, dah, dbl, idesc, 1u);
          tc::mma_bf16(tmem + kCross, dal, dbh, idesc, 1u);
          tc::mma_bf16(tmem + kCross, dam, dbm, idesc, 1u);
          tc::mma_bf16(tmem + kCross, dam, dbl, idesc, 1u);
          tc::mma_bf16(tmem + kCross, dal, dbm, idesc, 1u);
          tc::mma_bf16(tmem + kCross, dal, dbl, idesc, 1u);
          tc::mma_commit(&mbar[buf]);
        }
        uses[buf]++;
        pending[buf] = true;
      }
      bool ok = !abort_flag;
      for (int b = 0; b < 2; ++b) {
        if (pending[b]) {
          if (!tc::mbar_wait(&mbar[b], (uses[b] - 1) & 1)) ok = false;
          pending[b] = false;
        }
      }
      if (!ok) {
        if (tid == 0) atomicExch(args.status, LCP_ETIMEDOUT);
        abort_flag = 1;
      }
      tc::fence_after_sync();
      __syncthreads();
      if (abort_flag) break;
      for (int s = c0; s < c1; ++s) {
        float ym[16], yc[16];
        tc::tmem_ld16(tc::tmem_addr(tmem, warp * 32, 16 * (s - c0)), ym);
        tc::tmem_ld16(tc::tmem_addr(tmem, warp * 32, kCross + 16 * (s - c0)), yc);
        float u[16];
        load_point_row(args.tab + (int64_t)args.img_block[i0 + s] * kBlockElems, p, u);
        float d = 0.0f;
#pragma unroll
        for (int c = 0; c < 16; ++c) d = fmaf(u[c], ym[c] + yc[c], d);
        ff_add(acc_hi, acc_lo, d);
      }
      tc::fence_before_sync();
      __syncthreads();
    }
    if (p < args.npts && !abort_flag) args.rho[brick_point_index(hb, p, args.bdim, args.nb, args.ngrid)] =
          ((double)acc_hi + (double)acc_lo) * out_scale;
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, 512);
}

// ==========================================================================
// Grid matrix elements on grid bricks.
//
// For brick b every image pair s <= t that is a neighbour pair gets the
// partial block
//
//   G_st[a][b] = sum_{p in brick} phi_s(p)_a V(p) phi_t(p)_b
//
// (src/Hamiltonian.jl:384-429 restricted to the brick).  M = 128 rows are the
// orbitals of 8 images s (V-weighted, built in shared memory with a per-brick
// scale of V), N the orbitals of a window of up to 16 images t >= s (the
// brick tables as stored), K the brick's 128 point slots.  Both operands are
// MN-major: the table block [h][g][8 pt][8 orb] is that layout with
// LBO = 128 B (point groups) and SBO = 2048 B (orbital halves; images 4096 B
// apart).  Partial blocks go to a scratch array (FP32); h_reduce_kernel sums
// them per folded pair in FP64 in a fixed order and writes both orientations
// of H -- no atomics.
// ==========================================================================

constexpr int kHWin = 8;                   // t images per window
constexpr int kHGroup = 8;                 // s images per M tile
constexpr int kImgBytes = 4096;            // one part of an image block
constexpr int kHBBytes = kHWin * kImgBytes;
constexpr int kHABytes = kHGroup * kImgBytes;
constexpr size_t kHSmem = 3 * kHBBytes + 3 * kHABytes;  // 192 KB
// TMEM columns of the four accumulators (N <= 16 * kHWin = 128 each), one per
// quantum of the products: hi*hi (2^-14), hi*mid + mid*hi (2^-22),
// hi*lo + lo*hi + mid*mid (2^-30), mid*lo + lo*mid + lo*lo (2^-38; lo*lo is
// the only term finer than its quantum).  Over the 128 points of a brick the
// first three sums stay below 2^24 of their quanta, so they are exact in FP32.
constexpr uint32_t kHAcc1 = 128, kHAcc2 = 256, kHAcc3 = 384;

struct TcHamArgs {
  int64_t nbricks;
  int32_t bdim[3], nb[3], ngrid[3];
  int32_t npts;
  double phi_scale;
  const int64_t* img_off;
  const int32_t* img_block;
  const int64_t* tab_off;
  const int32_t* tab_slot;
  const int64_t* slot_base;
  const __nv_bfloat16* tab;
  const double* vpot;
  float* scratch;
  int* status;
};

__global__ void __launch_bounds__(128) hamiltonian_tc_kernel(TcHamArgs args) {
  extern __shared__ __align__(1024) uint8_t smem[];
  __shared__ uint64_t mbar;
  __shared__ uint32_t tslot;
  __shared__ float sVh[128], sVl[128];
  __shared__ double sVmax[4];
  __shared__ int abort_flag;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  uint8_t* sB = smem;                 // [part][image][4096 B]
  uint8_t* sA = smem + 3 * kHBBytes;  // [part][image][4096 B]
  if (warp == 0) tc::tmem_alloc(&tslot, 512);
  if (tid == 0) {
    tc::mbar_init(&mbar, 1);
    tc::fence_mbar_init();
    abort_flag = 0;
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tslot;
  uint32_t commits = 0;
  for (int64_t hb = blockIdx.x; hb < args.nbricks && !abort_flag; hb += gridDim.x) {
    const int64_t i0 = args.img_off[hb];
    const int m = (int)(args.img_off[hb + 1] - i0);
    const int64_t t0 = args.tab_off[hb];
    const int64_t sbase = args.slot_base[hb];
    const double v = tid < args.npts ? args.vpot[brick_point_index(hb, tid, args.bdim, args.nb, args.ngrid)] : 0.0;
    double vm = fabs(v);
    for (int o = 16; o > 0; o >>= 1) vm = fmax(vm, __shfl_xor_sync(0xffffffffu, vm, o));
    if (lane == 0) sVmax[warp] = vm;
    __syncthreads();
    const double sv = pow2_ceil(fmax(fmax(sVmax[0], sVmax[1]), fmax(sVmax[2], sVmax[3])));
    {
      const double vs = v / sv;  // exact: sv is a power of two
      const float vh = (float)vs;
      sVh[tid] = vh;
      sVl[tid] = (float)(vs - (double)vh);
    }
    const float out_scale = (float)(sv * args.phi_scale * args.phi_scale);  // a power of two
    for (int w0 = 0; w0 < m && !abort_flag; w0 += kHWin) {
      const int w1 = min(w0 + kHWin, m);
      __syncthreads();
      for (int c = tid; c < (w1 - w0) * 768; c += blockDim.x) {
        const int img = c / 768, q = c - img * 768;  // q: 16-byte chunk of the 12 KB block
        const int part = q >> 8;
        const uint8_t* src =
            reinterpret_cast<const uint8_t*>(args.tab + (int64_t)args.img_block[i0 + w0 + img] * kBlockElems) + q * 16;
        uint8_t* dst = sB + part * kHBBytes + img * kImgBytes + (q & 255) * 16;
        cp_async16(dst, src);
      }
      cp_async_wait_all();
      for (int s0 = 0; s0 < w1 && !abort_flag; s0 += kHGroup) {
        const int tstart = max(w0, s0);
        for (int c = tid; c < kHGroup * 256; c += blockDim.x) {
          const int img = c >> 8, q = c & 255;  // q = (h*16 + g)*8 + r: 8 orbitals of slot g*8 + r
          const int s = s0 + img;
          uint4 oh = make_uint4(0, 0, 0, 0), om = make_uint4(0, 0, 0, 0), ol = make_uint4(0, 0, 0, 0);
          if (s < m) {
            const int pt = ((q >> 3) & 15) * 8 + (q & 7);
            const float vh = sVh[pt], vl = sVl[pt];
            float u[8];
            load_chunk3f(args.tab + (int64_t)args.img_block[i0 + s] * kBlockElems + q * 8, u);
            __nv_bfloat16* xh = reinterpret_cast<__nv_bfloat16*>(&oh);
            __nv_bfloat16* xm = reinterpret_cast<__nv_bfloat16*>(&om);
            __nv_bfloat16* xl = reinterpret_cast<__nv_bfloat16*>(&ol);
#pragma unroll
            for (int e = 0; e < 8; ++e) {
              // u * (vh + vl) = pr + er exactly up to u*vl's rounding (~2^-48)
              const float pr = u[e] * vh;
              const float er = fmaf(u[e], vh, -pr) + u[e] * vl;
              fx_split_f(pr, er, xh[e], xm[e], xl[e]);
            }
          }
          *reinterpret_cast<uint4*>(sA + img * kImgBytes + q * 16) = oh;
          *reinterpret_cast<uint4*>(sA + kHABytes + img * kImgBytes + q * 16) = om;
          *reinterpret_cast<uint4*>(sA + 2 * kHABytes + img * kImgBytes + q * 16) = ol;
        }
        tc::fence_proxy_async_smem();
        __syncthreads();
        const int nimg = w1 - tstart;
        if (tid == 0) {
          tc::fence_after_sync();
          const uint32_t idesc = tc::idesc_bf16_f32(128, 16 * nimg, 1, 1);
          const uint32_t a0 = tc::smem_u32(sA);
          const uint32_t b0 = tc::smem_u32(sB) + (tstart - w0) * kImgBytes;
          for (int ks = 0; ks < 8; ++ks) {
            const uint32_t ko = ks * 256;
            const uint64_t dah = tc::smem_desc(a0 + ko, 128, 2048), dam = tc::smem_desc(a0 + kHABytes + ko, 128, 2048),
                           dal = tc::smem_desc(a0 + 2 * kHABytes + ko, 128, 2048);
            const uint64_t dbh = tc::smem_desc(b0 + ko, 128, 2048), dbm = tc::smem_desc(b0 + kHBBytes + ko, 128, 2048),
                           dbl = tc::smem_desc(b0 + 2 * kHBBytes + ko, 128, 2048);
            const uint32_t acc = ks > 0 ? 1u : 0u;
            tc::mma_bf16(tmem, dah, dbh, idesc, acc);
            tc::mma_bf16(tmem + kHAcc1, dah, dbm, idesc, acc);
            tc::mma_bf16(tmem + kHAcc1, dam, dbh, idesc, 1u);
            tc::mma_bf16(tmem + kHAcc2, dah, dbl, idesc, acc);
            tc::mma_bf16(tmem + kHAcc2, dal, dbh, idesc, 1u);
            tc::mma_bf16(tmem + kHAcc2, dam, dbm, idesc, 1u);
            tc::mma_bf16(tmem + kHAcc3, dam, dbl, idesc, acc);
            tc::mma_bf16(tmem + kHAcc3, dal, dbm, idesc, 1u);
            tc::mma_bf16(tmem + kHAcc3, dal, dbl, idesc, 1u);
          }
          tc::mma_commit(&mbar);
        }
        if (!tc::mbar_wait(&mbar, commits & 1)) {
          if (tid == 0) atomicExch(args.status, LCP_ETIMEDOUT);
          abort_flag = 1;
          tc::mbar_wait(&mbar, commits & 1);  // second bounded window for MMAs still in flight
        }
        ++commits;
        tc::fence_after_sync();
        const int row = warp * 32 + lane;
        const int s = s0 + (row >> 4), a = row & 15;
        for (int t = tstart; t < w1; ++t) {
          float y0[16], y1[16], y2[16], y3[16];
          tc::tmem_ld16(tc::tmem_addr(tmem, warp * 32, 16 * (t - tstart)), y0);
          tc::tmem_ld16(tc::tmem_addr(tmem, warp * 32, kHAcc1 + 16 * (t - tstart)), y1);
          tc::tmem_ld16(tc::tmem_addr(tmem, warp * 32, kHAcc2 + 16 * (t - tstart)), y2);
          tc::tmem_ld16(tc::tmem_addr(tmem, warp * 32, kHAcc3 + 16 * (t - tstart)), y3);
          if (s < m && s <= t) {
            const int slot = args.tab_slot[t0 + s * m + t];
            if (slot >= 0) {
              float o[16];
#pragma unroll
              for (int c = 0; c < 16; ++c) o[c] = (y0[c] + (y1[c] + (y2[c] + y3[c]))) * out_scale;
              float4* dst = reinterpret_cast<float4*>(args.scratch + (sbase + slot) * 256 + a * 16);
              dst[0] = make_float4(o[0], o[1], o[2], o[3]);
              dst[1] = make_float4(o[4], o[5], o[6], o[7]);
              dst[2] = make_float4(o[8], o[9], o[10], o[11]);
              dst[3] = make_float4(o[12], o[13], o[14], o[15]);
            }
          }
        }
        tc::fence_before_sync();
        __syncthreads();
      }
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, 512);
}

// Float-float sum of the partial blocks of each folded pair in a fixed order,
// written (x dV, as FP64) to both blocks.
__global__ void __launch_bounds__(256) h_reduce_kernel(int64_t nu, const int64_t* __restrict__ red_off,
                                                       const int64_t* __restrict__ red_slot,
                                                       const float* __restrict__ scratch, DevPairs pr,
                                                       const int32_t* __restrict__ numorbs, double dv, double* H) {
  const int e = threadIdx.x, a = e >> 4, b = e & 15;
  for (int64_t u = blockIdx.x; u < nu; u += gridDim.x) {
    float acc_hi = 0.0f, acc_lo = 0.0f;
    for (int64_t k = red_off[u]; k < red_off[u + 1]; ++k) {
      const int64_t code = red_slot[k];
      const int64_t slot = code >> 1;
      ff_add(acc_hi, acc_lo, scratch[slot * 256 + ((code & 1) ? b * 16 + a : a * 16 + b)]);
    }
    const double acc = (double)acc_hi + (double)acc_lo;
    const int i = pr.atom[u], j = pr.jatom[u];
    const int noi = numorbs[i], noj = numorbs[j];
    if (a < noi && b < noj) {
      const double v = acc * dv;
      H[pr.boff_p[u] + (int64_t)a * noj + b] = v;
      if (!pr.self[u]) H[pr.boff_q[u] + (int64_t)b * noi + a] = v;
    }
  }
}

int sm_count() {
  int dev = 0, sms = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return sms;
}

}  // namespace

cudaError_t launch_absmax_scale(const double* x, int64_t n, double factor, unsigned long long* tmp, double* scale,
                                cudaStream_t st) {
  LCP_CUDA_TRY(cudaMemsetAsync(tmp, 0, sizeof(unsigned long long), st));
  if (n > 0) {
    const int blocks = (int)std::min<int64_t>((n + 255) / 256, (int64_t)sm_count() * 8);
    absmax_kernel<<<blocks, 256, 0, st>>>(x, n, tmp);
    LCP_CUDA_TRY(cudaGetLastError());
  }
  pow2_scale_kernel<<<1, 32, 0, st>>>(tmp, factor, scale);
  return cudaGetLastError();
}

cudaError_t launch_brick_table(const double* phi, const int64_t* phi_off, const int32_t* numorbs,
                               const int64_t* sph_off, int natom, const int32_t* point_code, int64_t npoints,
                               const double* scale, __nv_bfloat16* tab, int64_t nblocks, cudaStream_t st) {
  LCP_CUDA_TRY(cudaMemsetAsync(tab, 0, (size_t)nblocks * kBlockElems * sizeof(__nv_bfloat16), st));
  if (npoints == 0) return cudaSuccess;
  int blocks = (int)std::min<int64_t>((npoints + 255) / 256, (int64_t)sm_count() * 16);
  brick_table_kernel<<<blocks, 256, 0, st>>>(phi, phi_off, numorbs, sph_off, natom, point_code, npoints, scale, tab);
  return cudaGetLastError();
}

cudaError_t launch_dsym(int nloop, const int32_t* pair_atom, const int32_t* pair_jatom, const int64_t* boff,
                        const int32_t* partner, const int32_t* numorbs, const double* dm, const double* scale,
                        __nv_bfloat16* out, cudaStream_t st) {
  int64_t total = (int64_t)(nloop + 1) * 256;
  int blocks = (int)std::min<int64_t>((total + 255) / 256, (int64_t)sm_count() * 16);
  dsym_kernel<<<blocks, 256, 0, st>>>(nloop, pair_atom, pair_jatom, boff, partner, numorbs, dm, scale, out);
  return cudaGetLastError();
}

cudaError_t launch_density_tc(const TcBrickGeom& bg, const __nv_bfloat16* tab, double phi_scale,
                              const __nv_bfloat16* dsym, const double* dscale, int zero_pair, double* rho,
                              int* status, cudaStream_t st) {
  if (bg.max_images > 32) return cudaErrorInvalidValue;
  TcDensArgs a{};
  a.nbricks = bg.nbricks;
  for (int d = 0; d < 3; ++d) {
    a.bdim[d] = bg.bdim[d];
    a.nb[d] = bg.nb[d];
    a.ngrid[d] = bg.ngrid[d];
  }
  a.npts = bg.npts;
  a.zero_pair = zero_pair;
  a.phi_scale = phi_scale;
  a.dscale = dscale;
  a.img_off = bg.img_off;
  a.img_block = bg.img_block;
  a.tab_off = bg.tab_off;
  a.tab_pair = bg.tab_pair;
  a.tab = tab;
  a.dsym = dsym;
  a.rho = rho;
  a.status = status;
  // 512 TMEM columns per CTA: reserve enough shared memory to keep one CTA per SM
  const size_t smem = std::max<size_t>(2 * kASmem + 2 * kBSmem, 120 * 1024);
  LCP_CUDA_TRY(cudaFuncSetAttribute(density_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(bg.nbricks, sm_count()));
  density_tc_kernel<<<grid, 128, smem, st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_hamiltonian_tc(const TcBrickGeom& bg, const int32_t* tab_slot, const int64_t* slot_base,
                                  const __nv_bfloat16* tab, double phi_scale, const double* vpot, float* scratch,
                                  int* status, cudaStream_t st) {
  TcHamArgs a{};
  a.nbricks = bg.nbricks;
  for (int d = 0; d < 3; ++d) {
    a.bdim[d] = bg.bdim[d];
    a.nb[d] = bg.nb[d];
    a.ngrid[d] = bg.ngrid[d];
  }
  a.npts = bg.npts;
  a.phi_scale = phi_scale;
  a.img_off = bg.img_off;
  a.img_block = bg.img_block;
  a.tab_off = bg.tab_off;
  a.tab_slot = tab_slot;
  a.slot_base = slot_base;
  a.tab = tab;
  a.vpot = vpot;
  a.scratch = scratch;
  a.status = status;
  LCP_CUDA_TRY(cudaFuncSetAttribute(hamiltonian_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kHSmem));
  const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(bg.nbricks, sm_count()));
  hamiltonian_tc_kernel<<<grid, 128, kHSmem, st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_h_reduce(int64_t nu, const int64_t* red_off, const int64_t* red_slot, const float* scratch,
                            const DevPairs& pr, const int32_t* numorbs, double dv, double* H, cudaStream_t st) {
  if (nu == 0) return cudaSuccess;
  const int grid = (int)std::min<int64_t>(nu, (int64_t)sm_count() * 8);
  h_reduce_kernel<<<grid, 256, 0, st>>>(nu, red_off, red_slot, scratch, pr, numorbs, dv, H);
  return cudaGetLastError();
}

}  // namespace lcp
