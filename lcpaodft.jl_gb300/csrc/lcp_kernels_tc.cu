// Tensor-core (tcgen05, BF16 in / FP32 accumulate in TMEM) kernels.
//
// tc_selftest_kernel: one 128 x N x K product with both operands staged in
// shared memory in a chosen canonical layout (K-major or MN-major); used to
// check the descriptor and layout conventions on the device before the grid
// kernels rely on them.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "lcp_bounds.cuh"
#include "lcp_device.h"
#include "lcp_pdl.cuh"
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
//   u = hi + mid + lo + e,  hi = q1/2^8, mid = q2/2^17, lo = q3/2^26, |q| <= 256,
//
// so every part is an exact BF16 value (BF16 holds every integer up to 256
// in magnitude: 8 significant bits, and 256 = 2^8) and |e| <= 2^-27.  The
// quantisation error of the energies scales with the last part's quantum,
// so nine bits per part (27 in all) instead of eight cut it by 8x at no
// cost.  Eight of the nine part products are formed: mid*lo and lo*mid carry
// the small tails of the orbitals, which a six-term product loses, while
// lo*lo is at most 2^-36 of the scales' product, 2^-9 of the bound 2^-27 on
// the inputs' own quantisation, and is not formed.  hi*hi'
// (integer multiples of 2^-16) has its own accumulator, exact while the sum
// stays below 256 in magnitude (2^24 quanta: 512 terms of the largest size
// for D, whose scale is twice its maximum, and 256 for the matrix elements);
// the rest are 2^-9 and smaller and go to one accumulator (density) or
// three more, one
// per quantum (matrix elements).  What remains is the input quantisation e.
// ==========================================================================

namespace {

constexpr int kPart = 2048;                    // bf16 per part of a table block (hi, mid, lo parts)
// The tables are part-major: part p of block b at tab + (p * nblocks + b) * kPart.
constexpr int kDsymElems = 768;                // D block: hi, mid, lo (256 each)
constexpr uint32_t kALbo = 2048, kASbo = 128;  // table block [h][g][8 pt][8 orb] as K-major A

// The split above (hi, mid, lo: multiples of 2^-8, 2^-17, 2^-26) of a float
// p (|p| <= 1) carrying a small correction e
// (|e| <= 2^-23 |p|), in full-rate FP32 additions only.  Adding and
// subtracting C = 1.5 * 2^k rounds x (|x| <= 2^(k-1)) to the nearest multiple
// of ulp(C) = 2^(k-23) (ties to even), exactly: x + C lies in [2^k, 2^(k+1))
// where that is the spacing.  So C = 1.5 * 2^15, 1.5 * 2^6 and 1.5 * 2^-3
// give the multiples of 2^-8, 2^-17 and 2^-26 directly (the __fadd_rn forms
// keep the compiler from folding the pair away).
//   - r1 = p - hi is exact: hi is a multiple of 2^-8, itself a multiple of
//     ulp(p), and |r1| <= 2^-9.
//   - e joins r1 before mid is taken (one rounding, <= 2^-34), so that
//     |r1 + e| * 2^17 <= 256 + 2^-6 and |mid| stays within 256 quanta.
//   - r2 = (r1 + e) - mid is exact by the same argument, |r2| <= 2^-18, so
//     |2^26 * r2| <= 256 and lo is exact too.
// The parts are those of p + e up to |lo residual| <= 2^-27 + 2^-34.
__device__ __forceinline__ void fx_split_f(float p, float e, __nv_bfloat16& hi, __nv_bfloat16& mid,
                                           __nv_bfloat16& lo) {
  constexpr float C8 = 49152.0f, C17 = 96.0f, C26 = 0.1875f;
  const float h = __fadd_rn(__fadd_rn(p, C8), -C8);    // multiple of 2^-8, |h| <= 1
  const float r1 = __fadd_rn(__fadd_rn(p, -h), e);      // p - hi exact, then + e
  const float m = __fadd_rn(__fadd_rn(r1, C17), -C17);  // multiple of 2^-17
  const float r2 = __fadd_rn(r1, -m);                   // exact
  const float l = __fadd_rn(__fadd_rn(r2, C26), -C26);  // multiple of 2^-26
  hi = __float2bfloat16_rn(h);
  mid = __float2bfloat16_rn(m);
  lo = __float2bfloat16_rn(l);
}

// +-q * p as a BF16, for |q| <= 256 and p a power of two, with the sign of
// q flipped when sv is 1: |q| becomes an FP32 by the 2^23 magic add and the
// product is exact with at most eight significant bits, so its BF16 is the
// FP32's upper half (no conversion instruction).
__device__ __forceinline__ __nv_bfloat16 bf16_of_digit(int q, float p, unsigned sv) {
  const unsigned aq = (unsigned)(q < 0 ? -q : q);
  const float f = (__uint_as_float(0x4B000000u | aq) - 8388608.0f) * p;
  const unsigned sign = (sv ^ (unsigned)(q < 0)) << 15;
  return __ushort_as_bfloat16((unsigned short)((__float_as_uint(f) >> 16) | sign));
}

// The same three parts of x = v / 2^k (|x| <= 1) for an FP64 v, in integer
// arithmetic on v's bits, without the FP64 pipe: x is rounded once to the
// nearest multiple of 2^-26 (ties to even), q = x * 2^26 (|q| <= 2^26), and
// |q| is cut into signed 9-bit digits rounded to nearest, q = q1 2^18 + q2 2^9
// + q3 with |q1|, |q2|, |q3| <= 256.  The parts q1 2^-8, q2 2^-17, q3 2^-26
// are exact in BF16 and carry x to within 2^-27.
__device__ __forceinline__ void fx_split_bits(double v, int k, __nv_bfloat16& hi, __nv_bfloat16& mid,
                                              __nv_bfloat16& lo) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(v);
  const int e = (int)((b >> 52) & 0x7ff);
  long long a = 0;  // |q|
  if (e != 0) {     // zeros and subnormals (below 2^-1022) give q = 0
    const unsigned long long m = (b & ((1ull << 52) - 1)) | (1ull << 52);
    const int sh = 1049 + k - e;  // x * 2^26 = m * 2^-sh
    if (sh <= 0) {
      a = 1ll << 26;  // |x| > 1 does not occur for the tables (S_phi >= max |phi|): saturate
    } else if (sh < 64) {
      const unsigned long long half = 1ull << (sh - 1);
      const unsigned long long rem = m & ((half << 1) - 1);
      unsigned long long q = m >> sh;
      if (rem > half || (rem == half && (q & 1))) ++q;  // round to nearest, ties to even
      a = (long long)q;
    }
  }
  const int q1 = (int)((a + (1ll << 17)) >> 18);  // nearest multiple of 2^18 (ties up)
  const int r = (int)(a - ((long long)q1 << 18));   // [-2^17, 2^17)
  const int q2 = (r + 256) >> 9;                    // floor((r + 256) / 512)
  const int q3 = r - (q2 << 9);                     // [-256, 256)
  const unsigned sv = (unsigned)(b >> 63);
  hi = bf16_of_digit(q1, 0.00390625f, sv);          // 2^-8
  mid = bf16_of_digit(q2, 7.62939453125e-06f, sv);  // 2^-17
  lo = bf16_of_digit(q3, 1.4901161193847656e-08f, sv);  // 2^-26
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

// Exponent e of the smallest power of two >= |x| (x given by its bits with the
// sign cleared; 0 for x = 0, as pow2_ceil), by integer operations only.
__device__ __forceinline__ int pow2_ceil_exp(unsigned long long absbits) {
  if (absbits == 0) return 0;
  const int be = (int)(absbits >> 52);                  // biased exponent (0: subnormal)
  const unsigned long long man = absbits & ((1ull << 52) - 1);
  if (be == 0) return -1022;                            // subnormal: 2^-1022 bounds it
  return (be - 1023) + (man != 0 ? 1 : 0);
}
__device__ __forceinline__ double pow2_from_exp(int e) {  // 2^e for |e| <= 1022, exact
  return __longlong_as_double((long long)(e + 1023) << 52);
}

__device__ __forceinline__ void cp_async16(void* sdst, const void* gsrc) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(tc::smem_u32(sdst)), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// Maximum of v over the block (blockDim.x a multiple of 32, at most 1024),
// valid in thread 0.
__device__ __forceinline__ unsigned long long block_max_u64(unsigned long long v) {
  __shared__ unsigned long long s_max[32];
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long y = __shfl_xor_sync(0xffffffffu, v, o);
    v = y > v ? y : v;
  }
  const int warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if ((threadIdx.x & 31) == 0) s_max[warp] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    v = threadIdx.x < nw ? s_max[threadIdx.x] : 0ull;
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long y = __shfl_xor_sync(0xffffffffu, v, o);
      v = y > v ? y : v;
    }
  }
  return v;
}

// max |x| over n doubles (non-negative doubles order like their bit patterns)
__global__ void absmax_kernel(const double* __restrict__ x, int64_t n, unsigned long long* out) {
  // on the bits with the sign cleared (integer operations only)
  unsigned long long m = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x[i]) & 0x7fffffffffffffffull;
    m = b > m ? b : m;
  }
  // one atomic per block: thousands of warps' atomics on one address
  // serialise in L2 and cost more than the loads
  m = block_max_u64(m);
  if (threadIdx.x == 0 && m > 0) atomicMax(out, m);
}

// scale[0] = power of two >= factor * max, scale[1] = its inverse
__global__ void pow2_scale_kernel(const unsigned long long* mx, double factor, double* scale) {
  pdl_trigger();
  pdl_wait();
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    const double s = pow2_ceil(__longlong_as_double((long long)*mx) * factor);
    scale[0] = s;
    scale[1] = 1.0 / s;
  }
}

// Batched: max |D| per cell over tiles of kAbsTile entries (block g: a tile
// of the cell c with start[c] <= g < start[c+1]) into tmp[c].
constexpr int kAbsTile = 4096;
__global__ void absmax_batch_kernel(int32_t ncells, const DsymCell* __restrict__ cells,
                                    const int64_t* __restrict__ start, unsigned long long* tmp) {
  const int64_t g = blockIdx.x;
  int lo = 0, hi = ncells;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (start[mid] <= g) lo = mid;
    else hi = mid;
  }
  const DsymCell& c = cells[lo];
  const int64_t x0 = (g - start[lo]) * kAbsTile, x1 = min(c.hsize, x0 + kAbsTile);
  unsigned long long m = 0;
  for (int64_t i = x0 + threadIdx.x; i < x1; i += blockDim.x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(c.dm[i]) & 0x7fffffffffffffffull;
    m = b > m ? b : m;
  }
  m = block_max_u64(m);
  if (threadIdx.x == 0 && m > 0) atomicMax(tmp + lo, m);
}

__global__ void pow2_scale_batch_kernel(int32_t ncells, const unsigned long long* __restrict__ mx, double factor,
                                        double* scale) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < ncells) {
    const double s = pow2_ceil(__longlong_as_double((long long)mx[c]) * factor);
    scale[2 * c] = s;
    scale[2 * c + 1] = 1.0 / s;
  }
}

// Sphere point of every (first block, slot) of the table: code = block * 128
// + slot of each sphere point k (one thread per point).
__global__ void brick_slot_kernel(const int32_t* __restrict__ point_code, int64_t npoints, int32_t* __restrict__ slot_point) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < npoints; k += (int64_t)gridDim.x * blockDim.x)
    slot_point[point_code[k]] = (int32_t)k;
}

// The split-BF16 tables, one atom image per block of 256 threads: for each
// of its 16-orbital chunks, thread (h, g, r) -- orbital half h, point group
// g, point r of the group -- reads eight orbitals of its point's FP64 row and
// writes the three parts as one 16-byte store each, so every part of a table
// block is written as 4 KB of consecutive stores.  Empty slots and orbitals
// past the atom's are zeros.  phi / S_phi is split from phi's FP64 bits in
// integer arithmetic (fx_split_bits): no FP64 instruction per entry.
__global__ void __launch_bounds__(256) brick_table_kernel(const double* __restrict__ phi,
                                                          const int64_t* __restrict__ phi_off,
                                                          const int32_t* __restrict__ numorbs,
                                                          const int64_t* __restrict__ sph_off,
                                                          const int32_t* __restrict__ block_atom,
                                                          const int32_t* __restrict__ first_block, int64_t nimg,
                                                          const int32_t* __restrict__ slot_point,
                                                          const double* __restrict__ scale,
                                                          __nv_bfloat16* __restrict__ tab, int64_t nblocks) {
  const int t = threadIdx.x, r = t & 7, g = (t >> 3) & 15, h = t >> 7;
  const int slot = g * 8 + r;
  for (int64_t im = blockIdx.x; im < nimg; im += gridDim.x) {
    const int64_t b0 = first_block[im];
    const int atom = block_atom[b0];
    const int no = numorbs[atom];
    const int k = slot_point[b0 * 128 + slot];
    const double* src = k >= 0 ? phi + phi_off[atom] + (k - sph_off[atom]) * (int64_t)no : nullptr;
    // the scale is a power of two: phi / S_phi is phi with its exponent lowered by ks
    const int ks = (int)(((unsigned long long)__double_as_longlong(scale[0]) >> 52) & 0x7ff) - 1023;
    for (int c = 0; c * 16 < no; ++c) {
      uint4 part[3];
      __nv_bfloat16* ph = reinterpret_cast<__nv_bfloat16*>(&part[0]);
      __nv_bfloat16* pm = reinterpret_cast<__nv_bfloat16*>(&part[1]);
      __nv_bfloat16* pl = reinterpret_cast<__nv_bfloat16*>(&part[2]);
#pragma unroll
      for (int e = 0; e < 8; ++e) {
        const int o = c * 16 + h * 8 + e;
        fx_split_bits((src && o < no) ? src[o] : 0.0, ks, ph[e], pm[e], pl[e]);
      }
      const int64_t off = (b0 + c) * kPart + (int64_t)((h * 16 + g) * 64 + r * 8);
#pragma unroll
      for (int q = 0; q < 3; ++q) *reinterpret_cast<uint4*>(tab + q * nblocks * kPart + off) = part[q];
    }
  }
}

// Dsym blocks in the K-major B layout [kh][nh][8 n][8 k], one per sub-pair
// (pair, chunk ca, chunk cb): n = orbital 16 ca + a' of the pair's atom,
// k = orbital 16 cb + b' of its jatom; fixed-point with scale[0].  Dsym adds
// the partner's transposed block, except on the diagonal chunks of a self
// pair (which is its own partner).  Entry nsub is a zero block.
__device__ __forceinline__ void dsym_entry(int64_t sp, int w, int64_t nsub, const int32_t* __restrict__ sub_pair,
                                           const int32_t* __restrict__ sub_chunks,
                                           const int32_t* __restrict__ pair_atom,
                                           const int32_t* __restrict__ pair_jatom, const int64_t* __restrict__ boff,
                                           const int32_t* __restrict__ partner, const int32_t* __restrict__ numorbs,
                                           const double* __restrict__ dm, double inv, __nv_bfloat16* __restrict__ out) {
  const int kh = w >> 7, nh = (w >> 6) & 1, rr = (w >> 3) & 7, cc = w & 7;
  double v = 0.0;
  if (sp < nsub) {
    const int p = sub_pair[sp], ch = sub_chunks[sp];
    const int ca = ch >> 8, cb = ch & 255;
    const int a = ca * 16 + nh * 8 + rr, b = cb * 16 + kh * 8 + cc;
    const int i = pair_atom[p], j = pair_jatom[p];
    const int noi = numorbs[i], noj = numorbs[j];
    if (a < noi && b < noj) {
      v = dm[boff[p] + (int64_t)a * noj + b];
      const int q = partner[p];
      if (q != p || ca != cb) v += dm[boff[q] + (int64_t)b * noi + a];
    }
  }
  __nv_bfloat16 h, mm, l;
  const double x = v * inv;
  const float xf = (float)x;
  fx_split_f(xf, (float)(x - (double)xf), h, mm, l);
  out[sp * kDsymElems + w] = h;
  out[sp * kDsymElems + 256 + w] = mm;
  out[sp * kDsymElems + 512 + w] = l;
}

__global__ void dsym_kernel(int64_t nsub, const int32_t* __restrict__ sub_pair, const int32_t* __restrict__ sub_chunks,
                            const int32_t* __restrict__ pair_atom, const int32_t* __restrict__ pair_jatom,
                            const int64_t* __restrict__ boff, const int32_t* __restrict__ partner,
                            const int32_t* __restrict__ numorbs, const double* __restrict__ dm,
                            const double* __restrict__ scale, __nv_bfloat16* __restrict__ out) {
  pdl_trigger();
  pdl_wait();
  const double inv = scale[1];
  const int64_t total = (nsub + 1) * 256;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x)
    dsym_entry(e >> 8, (int)(e & 255), nsub, sub_pair, sub_chunks, pair_atom, pair_jatom, boff, partner, numorbs, dm,
               inv, out);
}

// Batched: the split D blocks of several cells (each with its zero block),
// cell c's entries at start[c] .. start[c+1] (in blocks) of the launch.
__global__ void dsym_batch_kernel(int32_t ncells, const DsymCell* __restrict__ cells,
                                  const int64_t* __restrict__ start) {
  const int64_t total = start[ncells] * 256;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t g = e >> 8;
    int lo = 0, hi = ncells;  // cell with start[lo] <= g < start[lo+1]
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (start[mid] <= g) lo = mid;
      else hi = mid;
    }
    const DsymCell& c = cells[lo];
    dsym_entry(g - start[lo], (int)(e & 255), c.nsub, c.sub_pair, c.sub_chunks, c.pair_atom, c.pair_jatom, c.boff,
               c.partner, c.numorbs, c.dm, c.scale[1], c.out);
  }
}

// Grid index of slot p of home brick hb, or -1 for a slot of a ragged brick
// that lies past the grid.
__device__ __forceinline__ int64_t brick_point_index(int64_t hb, int p, const int32_t* bdim, const int32_t* nb,
                                                     const int32_t* ngrid) {
  const int l2 = p % bdim[2], l1 = (p / bdim[2]) % bdim[1], l0 = p / (bdim[1] * bdim[2]);
  const int64_t h2 = hb % nb[2], h1 = (hb / nb[2]) % nb[1], h0 = hb / ((int64_t)nb[1] * nb[2]);
  const int64_t x = h0 * bdim[0] + l0, y = h1 * bdim[1] + l1, z = h2 * bdim[2] + l2;
  if (x >= ngrid[0] || y >= ngrid[1] || z >= ngrid[2]) return -1;
  return (x * ngrid[1] + y) * ngrid[2] + z;
}

// The 16 fixed-point values of point p of a table block staged in shared
// memory ([part][h][g][8 pt][8 orb]); hi + mid + lo is a multiple of 2^-23 of
// magnitude <= 1, so the FP32 sum is exact.
__device__ __forceinline__ void smem_point_row(const uint8_t* blk, int p, float* u) {
  const int g = p >> 3, r = p & 7;
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const uint8_t* c = blk + (h * 16 + g) * 128 + r * 16;
    const uint4 vh = *reinterpret_cast<const uint4*>(c);
    const uint4 vm = *reinterpret_cast<const uint4*>(c + 4096);
    const uint4 vl = *reinterpret_cast<const uint4*>(c + 8192);
    const __nv_bfloat16* bh = reinterpret_cast<const __nv_bfloat16*>(&vh);
    const __nv_bfloat16* bm = reinterpret_cast<const __nv_bfloat16*>(&vm);
    const __nv_bfloat16* bl = reinterpret_cast<const __nv_bfloat16*>(&vl);
#pragma unroll
    for (int k = 0; k < 8; ++k)
      u[h * 8 + k] = (__bfloat162float(bh[k]) + __bfloat162float(bm[k])) + __bfloat162float(bl[k]);
  }
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
// with Y in TMEM, 16 columns per image of a window of up to 8 images s.  K
// steps run t = m-1 ... c0 so the first step writes every column of the
// window.  The epilogue (one thread per point) sums in float-float; every
// grid point lies in one brick, so rho is written once, without atomics.
// ==========================================================================

struct TcDensArgs {
  TcCell cell0;          // the cell of a single-cell launch
  TcBatch batch;         // or the cells of a batch
  int* status;
  uint32_t poll;         // polls of every bounded wait before it gives up
  int32_t stall;         // failure-path tests only: 1 = epilogue warp 2 never releases its stages
};

// Cell and cell-local brick index of brick k of a launch.
__device__ __forceinline__ const TcCell* tc_cell(const TcCell* c0, const TcBatch& b, int64_t k, int64_t& hb) {
  if (!b.cells) {
    hb = k;
    return c0;
  }
  hb = b.brick_local[k];
  return b.cells + b.brick_cell[k];
}


// Brick of round j for this CTA of a persistent launch: the brick list is
// sorted heaviest first and cut into rounds of gridDim.x consecutive bricks,
// taken in alternating directions so that no CTA gets the heavier brick of
// every round.  -1 past the end (the last round may be partial).  Every role
// of a CTA walks the same sequence.
__device__ __forceinline__ int64_t round_brick(int64_t j, int64_t ntotal) {
  const int64_t g = gridDim.x, k = j * g + ((j & 1) ? g - 1 - (int64_t)blockIdx.x : (int64_t)blockIdx.x);
  return k < ntotal ? k : -1;
}

// Density kernel roles (448 threads, one CTA per SM, persistent over bricks):
//   warp 0     table producer: per K step (brick, window, image t) three 4 KB
//              bulk copies of t's table block (operand A), completing as
//              transactions on full[stage] of a ring of kDStages stages;
//   warps 6-13 D gatherers: the Dsym(s, t) pieces of the window (operand B)
//              as 16-byte cp.async copies (one warp's cp.async issue costs
//              ~35 cycles, a small bulk copy ~70, whatever its size), each
//              warp publishing its share on full[stage] kDLag steps later,
//              once landed and fenced for the tensor core;
//   warp 1     MMA issuer (one elected lane): eight tcgen05 MMAs per K step
//              into one of two TMEM window buffers.  After step t of a
//              window, column block t is final: the commit goes to
//              mdone[stage]; other steps commit empty[stage] (4 arrivals);
//   warps 2-5  epilogue: one thread per point (its TMEM lane).  On
//              mdone[stage] it contracts column block t with phi_t(p), read
//              from the stage's A operand, then frees the stage; after a
//              window it frees the TMEM buffer, after a brick it writes rho.
// Every wait is bounded; a timeout sets *status and stops all roles.
constexpr int kDWin = 8;                          // images s per window (N <= 128)
constexpr int kDStages = 8;
constexpr uint32_t kDBLbo = kDWin * 2 * 128;      // B: [part][kh][n-group][8 n][8 k]
constexpr int kDStageA = 3 * 4096;                // table block: hi, mid, lo
constexpr int kDStageB = 3 * 2 * kDBLbo;          // Dsym pieces: (part, kh) x LBO
constexpr int kDStageBytes = kDStageA + kDStageB;  // 24 KB
constexpr size_t kDSmemStages = (size_t)kDStages * kDStageBytes;
constexpr int kDLag = 2;                          // K steps whose D pieces may still be in flight
constexpr int kDGatherWarps = 8;                  // warps gathering D pieces (cp.async)
constexpr int kDPieces = (kDWin * 96 + kDGatherWarps * 32 - 1) / (kDGatherWarps * 32);  // per thread and step
constexpr size_t kDSmem = kDSmemStages;            // 192 KB
constexpr uint32_t kDBufCols = 256;               // TMEM columns per window buffer
constexpr uint32_t kDCross = 128;                 // cross accumulator within a buffer

__global__ void __launch_bounds__(192 + 32 * kDGatherWarps, 1) density_tc_kernel(const __grid_constant__ TcDensArgs args) {
  extern __shared__ __align__(1024) uint8_t smem[];
  __shared__ uint64_t full_bar[kDStages], empty_bar[kDStages], mdone_bar[kDStages], tempty_bar[2], drain_bar;
  __shared__ uint32_t tslot;
  __shared__ volatile int abort_flag;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (warp == 0) tc::tmem_alloc(&tslot, 512);
  if (tid == 32) {
    for (int s = 0; s < kDStages; ++s) {
      tc::mbar_init(&full_bar[s], 1 + kDGatherWarps);  // A transactions + each gatherer's D pieces
      tc::mbar_init(&empty_bar[s], 4);
      tc::mbar_init(&mdone_bar[s], 1);
    }
    for (int b = 0; b < 2; ++b) tc::mbar_init(&tempty_bar[b], 4);
    tc::mbar_init(&drain_bar, 1);
    tc::fence_mbar_init();
    abort_flag = 0;
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  // launched as a dependent of the D-block (or V-weight) kernel: its setup
  // above overlaps that kernel's tail; its outputs are read only from here on
  pdl_wait();
  const uint32_t tmem = tslot;
  const int64_t ntotal = args.batch.cells ? args.batch.nbricks : args.cell0.nbricks;
  auto give_up = [&]() {
    if (!abort_flag) atomicExch(args.status, LCP_ETIMEDOUT);
    abort_flag = 1;
  };

  if (warp == 0) {
    // ------------------------------------------------------------ table producer
    uint32_t it = 0;
    for (int64_t j = 0; j * gridDim.x < ntotal && !abort_flag; ++j) {
      const int64_t k = round_brick(j, ntotal);
      if (k < 0) continue;
      int64_t hb;
      const TcCell& cl = *tc_cell(&args.cell0, args.batch, k, hb);
      const int64_t i0 = cl.img_off[hb];
      const int m = (int)(cl.img_off[hb + 1] - i0);
      for (int c0 = 0; c0 < m && !abort_flag; c0 += kDWin) {
        for (int k = 0; k < m - c0; ++k, ++it) {
          const int t = m - 1 - k;
          const int stage = (int)(it % kDStages);
          const uint32_t use = it / kDStages;
          if (use > 0 && !tc::mbar_wait_abortable(&empty_bar[stage], (use - 1) & 1, &abort_flag, args.poll)) {
            give_up();
            break;
          }
          if (lane == 0) {
            uint8_t* sA = smem + stage * kDStageBytes;
            tc::mbar_arrive_expect_tx(&full_bar[stage], kDStageA);
            // check build: a block outside the tables is replaced by block 0 (the
            // copy keeps the stage's transaction count) and recorded
            const int64_t blk = bounds_ok(i0 + t, cl.nblocks, 9) ? i0 + t : 0;
            for (int part = 0; part < 3; ++part)
              tc::bulk_g2s(sA + part * 4096, cl.tab + ((int64_t)part * cl.nblocks + blk) * kPart, 4096,
                           &full_bar[stage]);
          }
          __syncwarp();
        }
      }
    }
    // wait for the copies still in flight before the CTA's shared memory goes away
    for (int s = 0; s < kDStages; ++s) {
      const uint32_t uses = it / kDStages + ((uint32_t)s < it % kDStages ? 1u : 0u);
      if (uses > 0 && !tc::mbar_wait(&full_bar[s], (uses - 1) & 1, args.poll)) give_up();
    }
  } else if (warp >= 6) {
    // ------------------------------------------------------------ D gatherers
    const int gw = warp - 6;
    uint32_t it = 0;
    for (int64_t j = 0; j * gridDim.x < ntotal && !abort_flag; ++j) {
      const int64_t k = round_brick(j, ntotal);
      if (k < 0) continue;
      int64_t hb;
      const TcCell& cl = *tc_cell(&args.cell0, args.batch, k, hb);
      const int64_t i0 = cl.img_off[hb];
      const int m = (int)(cl.img_off[hb + 1] - i0);
      if (m == 0) continue;
      const int32_t* ptab = cl.tab_pair + cl.tab_off[hb];
      const uint8_t* dsym = reinterpret_cast<const uint8_t*>(cl.dsym);
      const int32_t* prow = ptab;  // the brick's m x m pair table, read through L1
      for (int c0 = 0; c0 < m && !abort_flag; c0 += kDWin) {
        const int c1 = min(c0 + kDWin, m);
        for (int k = 0; k < m - c0; ++k, ++it) {
          const int t = m - 1 - k;
          const int nimg = min(t, c1 - 1) - c0 + 1;
          const int stage = (int)(it % kDStages);
          const uint32_t use = it / kDStages;
          if (use > 0 && !tc::mbar_wait_abortable(&empty_bar[stage], (use - 1) & 1, &abort_flag, args.poll)) {
            give_up();
            break;
          }
          uint8_t* sB = smem + stage * kDStageBytes + kDStageA;
          // 16-byte pieces (image, part, kh, 16 x 16 B), at most kDPieces per
          // thread: every pair index first, then the copies (a load between
          // two copies would wait for the copy, as both touch shared memory)
          int pr[kDPieces];
#pragma unroll
          for (int r = 0; r < kDPieces; ++r) {
            const int c = gw * 32 + lane + r * kDGatherWarps * 32;
            pr[r] = c < nimg * 96 ? prow[(c0 + c / 96) * m + t] : 0;
          }
#pragma unroll
          for (int r = 0; r < kDPieces; ++r) {
            const int c = gw * 32 + lane + r * kDGatherWarps * 32;
            if (c < nimg * 96) {
              const int si = c / 96, w = c - si * 96, part = w >> 5, kh = (w >> 4) & 1, q = w & 15;
              int64_t pp = pr[r] < 0 ? cl.zero_pair : pr[r];
              if (!bounds_ok(pp, cl.zero_pair + 1, 8)) pp = cl.zero_pair;  // check build
              cp_async16(sB + part * (2 * kDBLbo) + kh * kDBLbo + si * 256 + q * 16,
                         dsym + pp * (kDsymElems * 2) + part * 512 + kh * 256 + q * 16);
            }
          }
          cp_async_commit();
          if (it >= (uint32_t)kDLag) {
            // this warp's pieces of step it - kDLag have landed: make them
            // visible to the tensor core and publish them
            cp_async_wait<kDLag>();
            tc::fence_proxy_async_smem();
            __syncwarp();
            if (lane == 0) tc::mbar_arrive(&full_bar[(it - kDLag) % kDStages]);
          }
          __syncwarp();
        }
      }
    }
    cp_async_wait<0>();
    tc::fence_proxy_async_smem();
    __syncwarp();
    if (lane == 0)
      for (uint32_t j = it >= (uint32_t)kDLag ? it - kDLag : 0; j < it; ++j) tc::mbar_arrive(&full_bar[j % kDStages]);
    __syncwarp();
  } else if (warp == 1) {
    // ------------------------------------------------------------ MMA issuer
    uint32_t it = 0, win = 0;
    for (int64_t j = 0; j * gridDim.x < ntotal && !abort_flag; ++j) {
      const int64_t k = round_brick(j, ntotal);
      if (k < 0) continue;
      int64_t hb;
      const TcCell& cl = *tc_cell(&args.cell0, args.batch, k, hb);
      const int64_t i0 = cl.img_off[hb];
      const int m = (int)(cl.img_off[hb + 1] - i0);
      for (int c0 = 0; c0 < m && !abort_flag; c0 += kDWin, ++win) {
        const int c1 = min(c0 + kDWin, m);
        const uint32_t buf = win & 1, wuse = win >> 1;
        if (wuse > 0 && !tc::mbar_wait_warp(&tempty_bar[buf], (wuse - 1) & 1, &abort_flag, args.poll)) {
          give_up();
          break;
        }
        tc::fence_after_sync();
        const uint32_t d0 = tmem + buf * kDBufCols, d1 = d0 + kDCross;
        for (int k = 0; k < m - c0; ++k, ++it) {
          const int t = m - 1 - k;
          const int nimg = min(t, c1 - 1) - c0 + 1;
          const int stage = (int)(it % kDStages);
          if (!tc::mbar_wait_warp(&full_bar[stage], (it / kDStages) & 1, &abort_flag, args.poll)) {
            give_up();
            break;
          }
          tc::fence_after_sync();
          // Descriptors are formed by the whole warp (warp-uniform values)
          // and the lane elected by elect.sync issues: with the MMAs inside a
          // lane-0 branch instead, each issue cost ~115 cycles whatever its N
          // (measured), about twice the tensor core's own time.  elect.sync
          // elects the same lane every time, so the commits below track
          // every MMA of this warp.
          const uint32_t idesc = tc::idesc_bf16_f32(128, 16 * nimg, 0, 0);
          const uint32_t a0 = tc::smem_u32(smem + stage * kDStageBytes), b0 = a0 + kDStageA;
          const uint64_t dah = tc::smem_desc(a0, kALbo, kASbo), dam = tc::smem_desc(a0 + 4096, kALbo, kASbo),
                         dal = tc::smem_desc(a0 + 8192, kALbo, kASbo);
          const uint64_t dbh = tc::smem_desc(b0, kDBLbo, 128), dbm = tc::smem_desc(b0 + 2 * kDBLbo, kDBLbo, 128),
                         dbl = tc::smem_desc(b0 + 4 * kDBLbo, kDBLbo, 128);
          const uint32_t acc = k > 0 ? 1u : 0u;
          if (tc::elect_one()) {
            tc::mma_bf16(d0, dah, dbh, idesc, acc);
            tc::mma_bf16(d1, dah, dbm, idesc, acc);
            tc::mma_bf16(d1, dam, dbh, idesc, 1u);
            tc::mma_bf16(d1, dah, dbl, idesc, 1u);
            tc::mma_bf16(d1, dal, dbh, idesc, 1u);
            tc::mma_bf16(d1, dam, dbm, idesc, 1u);
            tc::mma_bf16(d1, dam, dbl, idesc, 1u);
            tc::mma_bf16(d1, dal, dbm, idesc, 1u);
            if (t < c1) {
              // column block t is final once these MMAs finish; the epilogue
              // reads it with phi_t from this stage and then frees the stage
              tc::mma_commit(&mdone_bar[stage]);
            } else {
              for (int r = 0; r < 4; ++r) tc::mma_commit(&empty_bar[stage]);
            }
          }
          __syncwarp();
        }
      }
    }
    // every MMA issued by the elected thread has finished before TMEM is released
    if (tc::elect_one()) {
      tc::mma_commit(&drain_bar);
      if (!tc::mbar_wait(&drain_bar, 0, args.poll)) give_up();
    }
    __syncwarp();
  } else {
    // ------------------------------------------------------------ epilogue
    const uint32_t quarter = warp & 3;  // TMEM lanes [32 * quarter, 32 * quarter + 32)
    const int p = (int)quarter * 32 + lane;
    // failure-path tests: this warp withholds its releases, so the producers'
    // bounded waits for those stages run out and every role unwinds
    const bool withhold = args.stall == 1 && warp == 2;
    uint32_t it = 0, win = 0, mpar = 0;  // mpar: phase bit of mdone_bar per stage
    for (int64_t j = 0; j * gridDim.x < ntotal && !abort_flag; ++j) {
      const int64_t k = round_brick(j, ntotal);
      if (k < 0) continue;
      int64_t hb;
      const TcCell& cl = *tc_cell(&args.cell0, args.batch, k, hb);
      const int64_t i0 = cl.img_off[hb];
      const int m = (int)(cl.img_off[hb + 1] - i0);
      float acc_hi = 0.0f, acc_lo = 0.0f;
      for (int c0 = 0; c0 < m && !abort_flag; c0 += kDWin, ++win) {
        const int c1 = min(c0 + kDWin, m);
        const uint32_t buf = win & 1;
        it += (uint32_t)(m - c1);  // steps t >= c1 touch no final column
        for (int t = c1 - 1; t >= c0; --t, ++it) {
          const int stage = (int)(it % kDStages);
          if (!tc::mbar_wait_abortable(&mdone_bar[stage], (mpar >> stage) & 1u, &abort_flag, args.poll)) {
            give_up();
            break;
          }
          mpar ^= 1u << stage;
          tc::fence_after_sync();
          float ym[16], yc[16], u[16];
          const uint32_t col = buf * kDBufCols + 16 * (t - c0);
          tc::tmem_ld16(tc::tmem_addr(tmem, quarter * 32, col), ym);
          tc::tmem_ld16(tc::tmem_addr(tmem, quarter * 32, col + kDCross), yc);
          smem_point_row(smem + stage * kDStageBytes, p, u);
          float d = 0.0f;
#pragma unroll
          for (int c = 0; c < 16; ++c) d = fmaf(u[c], ym[c] + yc[c], d);
          ff_add(acc_hi, acc_lo, d);
          tc::fence_before_sync();
          __syncwarp();
          if (lane == 0 && !withhold) tc::mbar_arrive(&empty_bar[stage]);
        }
        if (abort_flag) break;
        __syncwarp();
        if (lane == 0 && !withhold) tc::mbar_arrive(&tempty_bar[buf]);
      }
      if (abort_flag) break;
      const int64_t gi = p < cl.npts ? brick_point_index(hb, p, cl.bdim, cl.nb, cl.ngrid) : -1;
      if (gi >= 0 && bounds_ok(gi, (int64_t)cl.ngrid[0] * cl.ngrid[1] * cl.ngrid[2], 10))
        cl.rho[gi] = ((double)acc_hi + (double)acc_lo) * (cl.phi_scale * cl.phi_scale * cl.dscale[0]);
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
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
// orbitals of 8 images s (the brick tables as stored), N the orbitals of a
// window of up to 4 images t (V-weighted in shared memory with a per-brick
// scale of V), K the brick's 128 point slots.  Both operands are
// MN-major: the table block [h][g][8 pt][8 orb] is that layout with
// LBO = 128 B (point groups) and SBO = 2048 B (orbital halves; images 4096 B
// apart).  Partial blocks go to a scratch array (FP32); h_reduce_kernel sums
// them per folded pair in a fixed order and writes both orientations of H --
// no atomics.
// ==========================================================================

// Roles (448 threads, one CTA per SM, persistent over bricks).  A tile is
// (brick, s-group of kHGroup images, t-window of kHWin images t >= the
// group's first image); V weights the t side:
//   warp 0     producer: per s-group the plain tables of its images into the
//              A region (after a_free) -- one bulk copy per part, the images
//              of a brick being consecutive blocks;
//   warps 6-13 per tile the raw t window from the tables into registers,
//              then (after b_empty) its V-weighted fixed-point split into one
//              of kHStages B stages (b_ready), with the brick's V / S_V
//              prepared by vweight_kernel;
//   warp 1     MMA issuer: 8 K steps x 4 MMAs per tile into one of two TMEM
//              tile buffers (4 accumulators x 64 columns each); after the
//              group's last tile it commits a_free;
//   warps 2-5  epilogue: per tile the FP32 partial blocks, TMEM read four
//              loads per wait, then the buffer is freed.
// Every wait is bounded; a timeout sets *status and stops all roles.
constexpr int kHGroup = 8;                 // s images per M tile (M = 128)
constexpr int kHWin = 4;                   // t images per N tile (N <= 64)
constexpr int kHStages = 2;
constexpr int kHXformWarps = 8;            // warps V-weighting the B stages
constexpr int kImgBytes = 4096;            // one part of an image block
constexpr int kHABytes = kHGroup * kImgBytes;   // one part of the A operand
constexpr int kHBBytes = kHWin * kImgBytes;     // one part of a B stage
constexpr size_t kHSmem = 3 * (size_t)kHABytes + (size_t)kHStages * 3 * kHBBytes;  // 192 KB
// TMEM: two tile buffers of 256 columns; inside one, the four accumulators
// (W = 16 x the tile's t images columns each, at most 64), one per quantum
// of the products: hi*hi (2^-16), hi*mid + mid*hi (2^-25),
// hi*lo + lo*hi + mid*mid (2^-34), mid*lo + lo*mid (2^-43).  Over the 128
// points of a brick the first two sums stay within 2^24 of their quanta (128
// terms of at most 1, 256 of at most 2^-9), so they are exact in FP32; the
// third could exceed it only if all of its 384 terms were near their bound
// with one sign.  lo*lo (at most 2^-36 of the scales' product, 2^-9 of the
// inputs' own quantisation bound 2^-27) is not formed.  Three MMAs per K
// step fill them (B parts stacked along N, N = 3W, 3W, 2W): per-clock
// tcgen05 traces showed the tile's MMAs set the kernel's pace (~93 cycles
// per MMA, ~21 of them fixed cost), so fewer and wider MMAs, and N sized to
// the images present, are what shorten a tile.
constexpr uint32_t kHBufCols = 256;

struct TcHamArgs {
  TcCell cell0;
  TcBatch batch;
  int* status;
};

// Per brick: S_V = power of two >= max|V| over the brick's points, and V / S_V
// (exact) as an FP32 pair hi + lo, for the V-weighting inside the matrix
// element kernel; S_V * S_phi^2 per brick for its epilogue.  One block of 128
// threads (point slots) per brick.
__global__ void __launch_bounds__(128) vweight_kernel(const __grid_constant__ TcHamArgs args) {
  pdl_trigger();
  pdl_wait();
  __shared__ unsigned long long smax[4];
  const int p = threadIdx.x, warp = p >> 5, lane = p & 31;
  const int64_t ntotal = args.batch.cells ? args.batch.nbricks : args.cell0.nbricks;
  for (int64_t k = blockIdx.x; k < ntotal; k += gridDim.x) {
    int64_t hb;
    const TcCell& cl = *tc_cell(&args.cell0, args.batch, k, hb);
    const int64_t gi = p < cl.npts ? brick_point_index(hb, p, cl.bdim, cl.nb, cl.ngrid) : -1;
    const double v = gi >= 0 ? cl.vpot[gi] : 0.0;
    // |v| as bits: non-negative doubles order like their bit patterns
    unsigned long long m = (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffull;
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long x = __shfl_xor_sync(0xffffffffu, m, o);
      m = x > m ? x : m;
    }
    if (lane == 0) smax[warp] = m;
    __syncthreads();
    unsigned long long mx = smax[0];
    for (int w = 1; w < 4; ++w) mx = smax[w] > mx ? smax[w] : mx;
    const int e = pow2_ceil_exp(mx);
    const double sv = pow2_from_exp(e);
    const double vs = v * pow2_from_exp(-e);  // exact: a power-of-two scaling
    const float vh = (float)vs;
    cl.vw[hb * 128 + p] = make_float2(vh, (float)(vs - (double)vh));
    if (p == 0) cl.vscale[hb] = (float)(sv * cl.phi_scale * cl.phi_scale);
    __syncthreads();
  }
}

__global__ void __launch_bounds__(192 + 32 * kHXformWarps, 1) hamiltonian_tc_kernel(const __grid_constant__ TcHamArgs args) {
  extern __shared__ __align__(1024) uint8_t smem[];
  __shared__ uint64_t bready_bar[kHStages], bempty_bar[kHStages], tfull_bar[2], tempty_bar[2];
  __shared__ uint64_t afull_bar, afree_bar, drain_bar;
  __shared__ uint32_t tslot;
  __shared__ volatile int abort_flag;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  uint8_t* sA = smem;                  // [part][s image][4096 B], plain tables
  uint8_t* sB0 = smem + 3 * kHABytes;  // stages of [part][t image][4096 B], V-weighted
  if (warp == 0) tc::tmem_alloc(&tslot, 512);
  if (tid == 32) {
    for (int s = 0; s < kHStages; ++s) {
      tc::mbar_init(&bready_bar[s], 32 * kHXformWarps);
      tc::mbar_init(&bempty_bar[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      tc::mbar_init(&tfull_bar[b], 1);
      tc::mbar_init(&tempty_bar[b], 4);
    }
    tc::mbar_init(&afull_bar, 1);
    tc::mbar_init(&afree_bar, 1);
    tc::mbar_init(&drain_bar, 1);
    tc::fence_mbar_init();
    abort_flag = 0;
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  // launched as a dependent of the D-block (or V-weight) kernel: its setup
  // above overlaps that kernel's tail; its outputs are read only from here on
  pdl_wait();
  const uint32_t tmem = tslot;
  const int64_t ntotal = args.batch.cells ? args.batch.nbricks : args.cell0.nbricks;
  auto give_up = [&]() {
    if (!abort_flag) atomicExch(args.status, LCP_ETIMEDOUT);
    abort_flag = 1;
  };

  if (warp == 0) {
    // ------------------------------------------------------------ producer: the A operand
    uint32_t grp = 0;
    for (int64_t j = 0; j * gridDim.x < ntotal && !abort_flag; ++j) {
      const int64_t k = round_brick(j, ntotal);
      if (k < 0) continue;
      int64_t hb;
      const TcCell& cl = *tc_cell(&args.cell0, args.batch, k, hb);
      const int64_t i0 = cl.img_off[hb];
      const int m = (int)(cl.img_off[hb + 1] - i0);
      for (int s0 = 0; s0 < m && !abort_flag; s0 += kHGroup, ++grp) {
        // the refill waits for the previous group's MMAs
        if (grp > 0 && !tc::mbar_wait_abortable(&afree_bar, (grp - 1) & 1, &abort_flag)) {
          give_up();
          break;
        }
        const int na = min(kHGroup, m - s0);
        if (lane == 0) {
          tc::mbar_arrive_expect_tx(&afull_bar, na * 3 * kImgBytes);
          // check build: a group outside the tables is replaced by blocks 0.. (same bytes)
          const int64_t blk = bounds_ok(i0 + s0 + na - 1, cl.nblocks, 11) ? i0 + s0 : 0;
          for (int part = 0; part < 3; ++part)
            tc::bulk_g2s(sA + part * kHABytes, cl.tab + ((int64_t)part * cl.nblocks + blk) * kPart,
                         na * kImgBytes, &afull_bar);
        }
        __syncwarp();
      }
    }
    if (grp > 0 && !tc::mbar_wait(&afull_bar, (grp - 1) & 1, 1u << 24)) give_up();
  } else if (warp == 1) {
    // ------------------------------------------------------------ MMA issuer
    uint32_t it = 0, grp = 0;
    for (int64_t j = 0; j * gridDim.x < ntotal && !abort_flag; ++j) {
      const int64_t k = round_brick(j, ntotal);
      if (k < 0) continue;
      int64_t hb;
      const TcCell& cl = *tc_cell(&args.cell0, args.batch, k, hb);
      const int64_t i0 = cl.img_off[hb];
      const int m = (int)(cl.img_off[hb + 1] - i0);
      for (int s0 = 0; s0 < m && !abort_flag; s0 += kHGroup, ++grp) {
        if (!tc::mbar_wait_warp(&afull_bar, grp & 1, &abort_flag)) {
          give_up();
          break;
        }
        for (int t0 = s0; t0 < m; t0 += kHWin, ++it) {
          const int stage = (int)(it % kHStages);
          const uint32_t buf = it & 1, tuse = it >> 1;
          if (tuse > 0 && !tc::mbar_wait_warp(&tempty_bar[buf], (tuse - 1) & 1, &abort_flag)) {
            give_up();
            break;
          }
          if (!tc::mbar_wait_warp(&bready_bar[stage], (it / kHStages) & 1, &abort_flag)) {
            give_up();
            break;
          }
          tc::fence_after_sync();
          // B parts stacked along N: the stage is [hi | mid | lo] x nt images,
          // one MN-major operand of N = 3W (W = 16 nt) with uniform SBO.
          // Descriptors are warp-uniform; the lane elected by elect.sync (the
          // same lane every time) issues and commits.
          const int nt = min(kHWin, m - t0);
          const uint32_t W = 16u * (uint32_t)nt;
          const uint32_t idesc3 = tc::idesc_bf16_f32(128, 3 * W, 1, 1);
          const uint32_t idesc2 = tc::idesc_bf16_f32(128, 2 * W, 1, 1);
          const uint32_t idesc1 = tc::idesc_bf16_f32(128, W, 1, 1);
          const uint32_t a0 = tc::smem_u32(sA), b0 = tc::smem_u32(sB0 + stage * 3 * kHBBytes);
          const uint32_t bl = b0 + 2u * (uint32_t)nt * kImgBytes;  // the lo part of the stage
          const uint32_t d0 = tmem + buf * kHBufCols;
#pragma unroll
          for (int ks = 0; ks < 8; ++ks) {
            const uint32_t ko = ks * 256;
            const uint64_t dah = tc::smem_desc(a0 + ko, 128, 2048),
                           dam = tc::smem_desc(a0 + kHABytes + ko, 128, 2048),
                           dal = tc::smem_desc(a0 + 2 * kHABytes + ko, 128, 2048);
            const uint64_t dbh = tc::smem_desc(b0 + ko, 128, 2048),  // [hi | mid | lo] from here
                           dbl = tc::smem_desc(bl + ko, 128, 2048);
            // Accumulator k (quantum 2^-(16+9k)) at columns d0 + kW: a product
            // of parts (i, j) lands in accumulator i + j when the MMA with
            // A part i starts at column d0 + iW.  K step 0 writes every
            // accumulator first (lo * [hi, mid] the last two, hi * [hi, mid]
            // the first two) and adds hi * lo on its own; later steps take
            // hi * [hi, mid, lo] and lo * [hi, mid] whole.
            if (tc::elect_one()) {
              if (ks == 0) {
                tc::mma_bf16(d0 + 2 * W, dal, dbh, idesc2, 0u);  // lo * [hi, mid] -> acc 2, 3 (first write)
                tc::mma_bf16(d0, dah, dbh, idesc2, 0u);          // hi * [hi, mid] -> acc 0, 1 (first write)
                tc::mma_bf16(d0 + 2 * W, dah, dbl, idesc1, 1u);  // hi * lo -> acc 2
              } else {
                tc::mma_bf16(d0, dah, dbh, idesc3, 1u);          // hi * [hi, mid, lo] -> acc 0, 1, 2
                tc::mma_bf16(d0 + 2 * W, dal, dbh, idesc2, 1u);  // lo * [hi, mid] -> acc 2, 3
              }
              tc::mma_bf16(d0 + W, dam, dbh, idesc3, 1u);        // mid * [hi, mid, lo] -> acc 1, 2, 3
            }
          }
          if (tc::elect_one()) {
            tc::mma_commit(&bempty_bar[stage]);
            tc::mma_commit(&tfull_bar[buf]);
          }
          __syncwarp();
        }
        if (abort_flag) break;
        if (tc::elect_one()) tc::mma_commit(&afree_bar);  // the A region may be refilled
        __syncwarp();
      }
    }
    if (tc::elect_one()) {
      tc::mma_commit(&drain_bar);
      if (!tc::mbar_wait(&drain_bar, 0, 1u << 24)) give_up();
    }
    __syncwarp();
  } else if (warp >= 6) {
    // ------------------------------------------------------------ B tiles: load and V-weight
    // Each thread owns chunk q = tt of every image of a tile: 8 orbitals of
    // one point slot, all three parts.  It loads the tile's raw parts from
    // the tables into registers (coalesced 16-byte loads, before waiting for
    // the stage, so their latency overlaps the MMAs still reading it), then
    // writes the V-weighted split into the stage.  Staging the raw tile in
    // shared memory first made load, weighting and MMAs three chained phases
    // over two stages; a third stage does not fit beside the A operand.
    const int tt = tid - 192;
    static_assert(32 * kHXformWarps == 256, "one B thread per chunk of an image");
    const int pt = ((tt >> 3) & 15) * 8 + (tt & 7);  // its point slot
    uint32_t it = 0;
    for (int64_t j = 0; j * gridDim.x < ntotal && !abort_flag; ++j) {
      const int64_t k = round_brick(j, ntotal);
      if (k < 0) continue;
      int64_t hb;
      const TcCell& cl = *tc_cell(&args.cell0, args.batch, k, hb);
      const int64_t i0 = cl.img_off[hb];
      const int m = (int)(cl.img_off[hb + 1] - i0);
      if (m == 0) continue;
      const float2 w = cl.vw[hb * 128 + pt];
      const float vh = w.x, vl = w.y;
      const uint4* tab4 = reinterpret_cast<const uint4*>(cl.tab) + tt;  // 16-byte chunk tt of block 0, part 0
      const int64_t pstride = cl.nblocks * (kPart / 8);                 // one part, in 16-byte chunks
      for (int s0 = 0; s0 < m && !abort_flag; s0 += kHGroup) {
        for (int t0 = s0; t0 < m && !abort_flag; t0 += kHWin, ++it) {
          const int nt = min(kHWin, m - t0);
          const int stage = (int)(it % kHStages);
          const uint32_t use = it / kHStages;
          uint4 raw[kHWin][3];
          const uint4* src = tab4 + (i0 + t0) * (kPart / 8);
#pragma unroll
          for (int j = 0; j < kHWin; ++j) {
            if (j < nt) {
#pragma unroll
              for (int part = 0; part < 3; ++part) raw[j][part] = __ldg(src + part * pstride + j * (kPart / 8));
            }
          }
          if (use > 0 && !tc::mbar_wait_abortable(&bempty_bar[stage], (use - 1) & 1, &abort_flag)) {
            give_up();
            break;
          }
          uint8_t* sB = sB0 + stage * 3 * kHBBytes + tt * 16;
          const int pbytes = nt * kImgBytes;  // one part of this tile's stage: [hi | mid | lo] x nt images
#pragma unroll
          for (int j = 0; j < kHWin; ++j) {
            if (j < nt) {
              const __nv_bfloat16* xb_h = reinterpret_cast<const __nv_bfloat16*>(&raw[j][0]);
              const __nv_bfloat16* xb_m = reinterpret_cast<const __nv_bfloat16*>(&raw[j][1]);
              const __nv_bfloat16* xb_l = reinterpret_cast<const __nv_bfloat16*>(&raw[j][2]);
              uint4 oh, om, ol;
              __nv_bfloat16* xh = reinterpret_cast<__nv_bfloat16*>(&oh);
              __nv_bfloat16* xm = reinterpret_cast<__nv_bfloat16*>(&om);
              __nv_bfloat16* xl = reinterpret_cast<__nv_bfloat16*>(&ol);
#pragma unroll
              for (int e = 0; e < 8; ++e) {
                const float u = (__bfloat162float(xb_h[e]) + __bfloat162float(xb_m[e])) + __bfloat162float(xb_l[e]);
                // u * (vh + vl) = pr + er exactly up to u*vl's rounding (~2^-48)
                const float pr = u * vh;
                const float er = fmaf(u, vh, -pr) + u * vl;
                fx_split_f(pr, er, xh[e], xm[e], xl[e]);
              }
              *reinterpret_cast<uint4*>(sB + j * kImgBytes) = oh;
              *reinterpret_cast<uint4*>(sB + pbytes + j * kImgBytes) = om;
              *reinterpret_cast<uint4*>(sB + 2 * pbytes + j * kImgBytes) = ol;
            }
          }
          tc::fence_proxy_async_smem();
          tc::mbar_arrive(&bready_bar[stage]);
        }
      }
    }
  } else {
    // ------------------------------------------------------------ epilogue (warps 2-5)
    const uint32_t quarter = warp & 3;
    const int row = (int)quarter * 32 + lane;  // TMEM lane = M row = (s image, orbital)
    uint32_t it = 0;
    for (int64_t j = 0; j * gridDim.x < ntotal && !abort_flag; ++j) {
      const int64_t k = round_brick(j, ntotal);
      if (k < 0) continue;
      int64_t hb;
      const TcCell& cl = *tc_cell(&args.cell0, args.batch, k, hb);
      const int64_t i0 = cl.img_off[hb];
      const int m = (int)(cl.img_off[hb + 1] - i0);
      if (m == 0) continue;
      const int64_t tb = cl.tab_off[hb];
      const int64_t sbase = cl.slot_base[hb];
      const float out_scale = cl.vscale[hb];  // S_V * S_phi^2, a power of two
      for (int s0 = 0; s0 < m && !abort_flag; s0 += kHGroup) {
        const int s = s0 + (row >> 4), a = row & 15;
        for (int t0 = s0; t0 < m && !abort_flag; t0 += kHWin, ++it) {
          const int nt = min(kHWin, m - t0);
          const uint32_t W = 16u * (uint32_t)nt;  // accumulator k at columns kW of the buffer
          const uint32_t buf = it & 1;
          int slot[kHWin];
#pragma unroll
          for (int j = 0; j < kHWin; ++j)
            slot[j] = (j < nt && s < m && s <= t0 + j) ? cl.tab_slot[tb + s * m + t0 + j] : -1;
          if (!tc::mbar_wait_abortable(&tfull_bar[buf], (it >> 1) & 1, &abort_flag)) {
            give_up();
            break;
          }
          tc::fence_after_sync();
#pragma unroll
          for (int j = 0; j < kHWin; ++j) {
            if (j < nt) {
              uint32_t y[4][16];
              const uint32_t col = buf * kHBufCols + 16 * j;
#pragma unroll
              for (int k = 0; k < 4; ++k) tc::tmem_ld16_nowait(tc::tmem_addr(tmem, quarter * 32, col + k * W), y[k]);
              tc::tmem_wait_ld();
#pragma unroll
              for (int k = 0; k < 4; ++k) tc::tmem_regs_ready(y[k]);
              if (slot[j] >= 0 && bounds_ok(sbase + slot[j], cl.slot_base[cl.nbricks], 12)) {
                float o[16];
#pragma unroll
                for (int c = 0; c < 16; ++c)
                  o[c] = (__uint_as_float(y[0][c]) +
                          (__uint_as_float(y[1][c]) + (__uint_as_float(y[2][c]) + __uint_as_float(y[3][c])))) *
                         out_scale;
                float4* dst = reinterpret_cast<float4*>(cl.scratch + (sbase + slot[j]) * 256 + a * 16);
                dst[0] = make_float4(o[0], o[1], o[2], o[3]);
                dst[1] = make_float4(o[4], o[5], o[6], o[7]);
                dst[2] = make_float4(o[8], o[9], o[10], o[11]);
                dst[3] = make_float4(o[12], o[13], o[14], o[15]);
              }
            }
          }
          tc::fence_before_sync();
          __syncwarp();
          if (lane == 0) tc::mbar_arrive(&tempty_bar[buf]);
        }
      }
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (warp == 0) tc::tmem_dealloc(tmem, 512);
}

// Float-float sum of the partial blocks of each 16 x 16 sub-block of a folded
// pair's H block in a fixed order, written (x dV, as FP64) to both blocks.  One
// block of 256 threads per sub-block; warp w sums every 8th slot with
// coalesced float4 loads
// (lane l holds entries 8l .. 8l+7 of the 16 x 16 partial), keeping direct
// and transposed partials apart.  The
// eight warps' sums are then combined in warp order through shared memory,
// the partner ones transposed -- the same order on every run.
__device__ __forceinline__ void ff_add8(float* hi, float* lo, float4 a, float4 b) {
  ff_add(hi[0], lo[0], a.x); ff_add(hi[1], lo[1], a.y); ff_add(hi[2], lo[2], a.z); ff_add(hi[3], lo[3], a.w);
  ff_add(hi[4], lo[4], b.x); ff_add(hi[5], lo[5], b.y); ff_add(hi[6], lo[6], b.z); ff_add(hi[7], lo[7], b.w);
}

constexpr int kRedRing = 8;        // partial blocks in flight per warp
constexpr int kRedCodes = 1024;    // slot codes staged per pass
// ring [warp][buffer][256 floats] (lane l owns floats 8l .. 8l+7 of each
// buffer), then the staged slot codes; the ring is reused for the warps' sums
constexpr size_t kRedRingBytes = (size_t)8 * kRedRing * 1024;
constexpr size_t kRedSmem = kRedRingBytes + kRedCodes * sizeof(int64_t);  // 72 KB
static_assert(kRedRingBytes >= 4 * 8 * 256 * sizeof(float), "the ring holds the warps' partial sums");

__device__ __forceinline__ void h_reduce_block(int64_t u, const int64_t* __restrict__ red_off,
                                               const int64_t* __restrict__ red_slot,
                                               const int32_t* __restrict__ sb_fold,
                                               const int32_t* __restrict__ sb_chunks,
                                               const float* __restrict__ scratch, const DevPairs& pr,
                                               const int32_t* __restrict__ numorbs, double dv, double* H,
                                               uint8_t* smem) {
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  int64_t* s_code = reinterpret_cast<int64_t*>(smem + kRedRingBytes);
  float (*s_part)[8][256] = reinterpret_cast<float (*)[8][256]>(smem);
  float* my = reinterpret_cast<float*>(smem) + (warp * kRedRing) * 256 + lane * 8;
  float dh[8], dl[8], th[8], tl[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) dh[i] = dl[i] = th[i] = tl[i] = 0.0f;
  const int fq = sb_fold[u], ch = sb_chunks[u];
  const int ia = pr.atom[fq], ja = pr.jatom[fq];
  const int noi = numorbs[ia], noj = numorbs[ja];
  // rows of a partial past its atom's orbitals are padding: lane pair
  // (2r, 2r+1) holds row r, which a direct partial indexes by the i chunk's
  // orbitals and a transposed one by the j chunk's
  const int row = lane >> 1;
  const bool row_d = row < noi - (ch >> 8) * 16, row_t = row < noj - (ch & 255) * 16;
  const int64_t k0 = red_off[u], k1 = red_off[u + 1];
  for (int64_t kb = k0; kb < k1; kb += kRedCodes) {
    const int n = (int)min((int64_t)kRedCodes, k1 - kb);
    __syncthreads();  // the previous pass's (or sub-block's) readers are done
    for (int i = tid; i < n; i += blockDim.x) s_code[i] = red_slot[kb + i];
    __syncthreads();
    // warp w adds slots w, w + 8, w + 16, ... in that order.  Each lane
    // copies its own 32 bytes of a partial into the warp's ring (cp.async,
    // kRedRing partials ahead) and reads back only those, so its own
    // wait_group is all the synchronisation it needs.
    const int cnt = warp < n ? (n - warp + 7) / 8 : 0;
    auto code_of = [&](int i) -> int64_t {
      const int64_t c = s_code[warp + 8 * i];
      return ((c & 1) ? row_t : row_d) ? c : -1;  // padding row: nothing to add
    };
    auto issue = [&](int i) {
      const int64_t c = code_of(i);
      if (c >= 0) {
        const float* src = scratch + (c >> 1) * 256 + lane * 8;
        float* dst = my + (i % kRedRing) * 256;
        cp_async16(dst, src);
        cp_async16(dst + 4, src + 4);
      }
    };
#pragma unroll 1
    for (int i = 0; i < kRedRing; ++i) {
      if (i < cnt) issue(i);
      cp_async_commit();
    }
#pragma unroll 1
    for (int i = 0; i < cnt; ++i) {
      cp_async_wait<kRedRing - 1>();  // this lane's copies of slot i have landed
      const int64_t c = code_of(i);
      if (c >= 0) {
        const float* b = my + (i % kRedRing) * 256;
        const float4 x = *reinterpret_cast<const float4*>(b), y = *reinterpret_cast<const float4*>(b + 4);
        if (c & 1) ff_add8(th, tl, x, y);
        else ff_add8(dh, dl, x, y);
      }
      if (i + kRedRing < cnt) issue(i + kRedRing);
      cp_async_commit();
    }
    cp_async_wait<0>();
  }
  __syncthreads();  // every ring is drained and read: it now holds the warps' sums
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    s_part[0][warp][lane * 8 + i] = dh[i];
    s_part[1][warp][lane * 8 + i] = dl[i];
    s_part[2][warp][lane * 8 + i] = th[i];
    s_part[3][warp][lane * 8 + i] = tl[i];
  }
  __syncthreads();
  const int a = tid >> 4, b = tid & 15, et = b * 16 + a;
  float hi = 0.0f, lo = 0.0f;
  for (int w = 0; w < 8; ++w) {
    ff_add(hi, lo, s_part[0][w][tid]);
    lo += s_part[1][w][tid];
    ff_add(hi, lo, s_part[2][w][et]);
    lo += s_part[3][w][et];
  }
  const double acc = (double)hi + (double)lo;
  const int ra = (ch >> 8) * 16 + a, rb = (ch & 255) * 16 + b;  // entry of the pair's block
  if (ra < noi && rb < noj) {
    const double v = acc * dv;
    H[pr.boff_p[fq] + (int64_t)ra * noj + rb] = v;
    if (!pr.self[fq]) H[pr.boff_q[fq] + (int64_t)rb * noi + ra] = v;
  }
}

__global__ void __launch_bounds__(256) h_reduce_kernel(int64_t nsb, const int64_t* __restrict__ red_off,
                                                       const int64_t* __restrict__ red_slot,
                                                       const int32_t* __restrict__ sb_fold,
                                                       const int32_t* __restrict__ sb_chunks,
                                                       const float* __restrict__ scratch, DevPairs pr,
                                                       const int32_t* __restrict__ numorbs, double dv, double* H) {
  pdl_trigger();
  pdl_wait();
  extern __shared__ __align__(16) uint8_t hsm[];
  for (int64_t u = blockIdx.x; u < nsb; u += gridDim.x)
    h_reduce_block(u, red_off, red_slot, sb_fold, sb_chunks, scratch, pr, numorbs, dv, H, hsm);
}

// Batched: the sub-blocks of several cells, cell c's at start[c] .. start[c+1].
__global__ void __launch_bounds__(256) h_reduce_batch_kernel(int32_t ncells, const RedCell* __restrict__ cells,
                                                             const int64_t* __restrict__ start,
                                                             const int64_t* __restrict__ order) {
  extern __shared__ __align__(16) uint8_t hsm[];
  for (int64_t i = blockIdx.x; i < start[ncells]; i += gridDim.x) {
    const int64_t g = order ? order[i] : i;  // visiting order (longest first), or as stored
    int lo = 0, hi = ncells;
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (start[mid] <= g) lo = mid;
      else hi = mid;
    }
    const RedCell& c = cells[lo];
    h_reduce_block(g - start[lo], c.red_off, c.red_slot, c.sb_fold, c.sb_chunks, c.scratch, c.pr, c.numorbs, c.dv,
                   c.H, hsm);
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
  return launch_pdl(pow2_scale_kernel, dim3(1), dim3(32), 0, st, (const unsigned long long*)tmp, factor, scale);
}

cudaError_t launch_brick_table(const double* phi, const int64_t* phi_off, const int32_t* numorbs,
                               const int64_t* sph_off, const int32_t* point_code, int64_t npoints,
                               const int32_t* block_atom, const int32_t* first_block, int64_t nimg,
                               int32_t* slot_point, const double* scale, __nv_bfloat16* tab, int64_t nblocks,
                               cudaStream_t st) {
  if (nimg == 0) return cudaSuccess;
  LCP_CUDA_TRY(cudaMemsetAsync(slot_point, 0xff, (size_t)nblocks * 128 * sizeof(int32_t), st));
  if (npoints > 0) {
    const int blocks = (int)std::min<int64_t>((npoints + 255) / 256, (int64_t)sm_count() * 16);
    brick_slot_kernel<<<blocks, 256, 0, st>>>(point_code, npoints, slot_point);
    LCP_CUDA_TRY(cudaGetLastError());
  }
  const int blocks = (int)std::min<int64_t>(nimg, (int64_t)sm_count() * 8);
  brick_table_kernel<<<blocks, 256, 0, st>>>(phi, phi_off, numorbs, sph_off, block_atom, first_block, nimg, slot_point,
                                              scale, tab, nblocks);
  return cudaGetLastError();
}

cudaError_t launch_dsym(int64_t nsub, const int32_t* sub_pair, const int32_t* sub_chunks, const int32_t* pair_atom,
                        const int32_t* pair_jatom, const int64_t* boff, const int32_t* partner, const int32_t* numorbs,
                        const double* dm, const double* scale, __nv_bfloat16* out, cudaStream_t st) {
  int64_t total = (nsub + 1) * 256;
  int blocks = (int)std::min<int64_t>((total + 255) / 256, (int64_t)sm_count() * 16);
  return launch_pdl(dsym_kernel, dim3(blocks), dim3(256), 0, st, nsub, sub_pair, sub_chunks, pair_atom, pair_jatom, boff,
                    partner, numorbs, dm, scale, out);
}

cudaError_t launch_dsym_batch(int32_t ncells, const DsymCell* cells, const int64_t* start, int64_t total_blocks,
                              cudaStream_t st) {
  const int64_t total = total_blocks * 256;
  if (total == 0) return cudaSuccess;
  const int blocks = (int)std::min<int64_t>((total + 255) / 256, (int64_t)sm_count() * 16);
  dsym_batch_kernel<<<blocks, 256, 0, st>>>(ncells, cells, start);
  return cudaGetLastError();
}

int64_t abs_tiles(int64_t n) { return (n + kAbsTile - 1) / kAbsTile; }

cudaError_t launch_absmax_scale_batch(int32_t ncells, const DsymCell* cells, const int64_t* start, int64_t total_tiles,
                                      double factor, unsigned long long* tmp, double* scale, cudaStream_t st) {
  LCP_CUDA_TRY(cudaMemsetAsync(tmp, 0, (size_t)ncells * sizeof(unsigned long long), st));
  if (total_tiles > 0) {
    absmax_batch_kernel<<<(unsigned)total_tiles, 256, 0, st>>>(ncells, cells, start, tmp);
    LCP_CUDA_TRY(cudaGetLastError());
  }
  pow2_scale_batch_kernel<<<(ncells + 127) / 128, 128, 0, st>>>(ncells, tmp, factor, scale);
  return cudaGetLastError();
}

cudaError_t launch_h_reduce_batch(int32_t ncells, const RedCell* cells, const int64_t* start, const int64_t* order,
                                  int64_t total, cudaStream_t st) {
  if (total == 0) return cudaSuccess;
  const int grid = (int)std::min<int64_t>(total, (int64_t)sm_count() * 8);
  LCP_CUDA_TRY(cudaFuncSetAttribute(h_reduce_batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kRedSmem));
  h_reduce_batch_kernel<<<grid, 256, kRedSmem, st>>>(ncells, cells, start, order);
  return cudaGetLastError();
}

TcCell tc_cell_of(const TcBrickGeom& bg, const __nv_bfloat16* tab) {
  TcCell c{};
  c.nbricks = bg.nbricks;
  c.nblocks = bg.nblocks;
  for (int d = 0; d < 3; ++d) {
    c.bdim[d] = bg.bdim[d];
    c.nb[d] = bg.nb[d];
    c.ngrid[d] = bg.ngrid[d];
  }
  c.npts = bg.npts;
  c.tab = tab;
  c.img_off = bg.img_off;
  c.tab_off = bg.tab_off;
  c.tab_pair = bg.tab_pair;
  return c;
}

static int tc_grid(const TcCell& cell0, const TcBatch& batch) {
  const int64_t n = batch.cells ? batch.nbricks : cell0.nbricks;
  return (int)std::max<int64_t>(1, std::min<int64_t>(n, sm_count()));
}

cudaError_t launch_density_tc_batch(const TcCell& cell0, const TcBatch& batch, int* status, cudaStream_t st,
                                    uint32_t poll, int32_t stall) {
  TcDensArgs a{};
  a.cell0 = cell0;
  a.batch = batch;
  a.status = status;
  a.poll = poll ? poll : (1u << 24);
  a.stall = stall;
  // 512 TMEM columns per CTA: the shared-memory ring (> half an SM) keeps one CTA per SM
  static_assert(kDSmem > 120 * 1024, "one CTA per SM");
  LCP_CUDA_TRY(cudaFuncSetAttribute(density_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kDSmem));
  return launch_pdl(density_tc_kernel, tc_grid(cell0, batch), dim3(192 + 32 * kDGatherWarps), kDSmem, st, a);
}

cudaError_t launch_density_tc(const TcBrickGeom& bg, const __nv_bfloat16* tab, double phi_scale,
                              const __nv_bfloat16* dsym, const double* dscale, int zero_pair, double* rho,
                              int* status, cudaStream_t st, uint32_t poll, int32_t stall) {
  TcCell c = tc_cell_of(bg, tab);
  c.phi_scale = phi_scale;
  c.dsym = dsym;
  c.zero_pair = zero_pair;
  c.dscale = dscale;
  c.rho = rho;
  return launch_density_tc_batch(c, TcBatch{}, status, st, poll, stall);
}

cudaError_t launch_hamiltonian_tc_batch(const TcCell& cell0, const TcBatch& batch, int* status, cudaStream_t st,
                                        cudaEvent_t ev_begin, cudaEvent_t ev_end) {
  TcHamArgs a{};
  a.cell0 = cell0;
  a.batch = batch;
  a.status = status;
  const int64_t n = batch.cells ? batch.nbricks : cell0.nbricks;
  if (n > 0) {
    const int vgrid = (int)std::min<int64_t>(n, (int64_t)sm_count() * 16);
    LCP_CUDA_TRY(launch_pdl(vweight_kernel, dim3(vgrid), dim3(128), 0, st, a));
  }
  LCP_CUDA_TRY(cudaFuncSetAttribute(hamiltonian_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kHSmem));
  static_assert(kHSmem > 120 * 1024, "one CTA per SM");
  if (ev_begin) LCP_CUDA_TRY(cudaEventRecord(ev_begin, st));
  LCP_CUDA_TRY(launch_pdl(hamiltonian_tc_kernel, tc_grid(cell0, batch), dim3(192 + 32 * kHXformWarps), kHSmem, st, a));
  if (ev_end) LCP_CUDA_TRY(cudaEventRecord(ev_end, st));
  return cudaSuccess;
}

cudaError_t launch_hamiltonian_tc(const TcBrickGeom& bg, const int32_t* tab_slot, const int64_t* slot_base,
                                  const __nv_bfloat16* tab, double phi_scale, const double* vpot, float2* vw,
                                  float* vscale, float* scratch, int* status, cudaStream_t st, cudaEvent_t ev_begin,
                                  cudaEvent_t ev_end) {
  TcCell c = tc_cell_of(bg, tab);
  c.tab_slot = tab_slot;
  c.slot_base = slot_base;
  c.phi_scale = phi_scale;
  c.vpot = vpot;
  c.vw = vw;
  c.vscale = vscale;
  c.scratch = scratch;
  return launch_hamiltonian_tc_batch(c, TcBatch{}, status, st, ev_begin, ev_end);
}

cudaError_t launch_h_reduce(int64_t nsb, const int64_t* red_off, const int64_t* red_slot, const int32_t* sb_fold,
                            const int32_t* sb_chunks, const float* scratch, const DevPairs& pr,
                            const int32_t* numorbs, double dv, double* H, cudaStream_t st) {
  if (nsb == 0) return cudaSuccess;
  const int grid = (int)std::min<int64_t>(nsb, (int64_t)sm_count() * 8);
  LCP_CUDA_TRY(cudaFuncSetAttribute(h_reduce_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kRedSmem));
  return launch_pdl(h_reduce_kernel, dim3(grid), dim3(256), kRedSmem, st, nsb, red_off, red_slot, sb_fold, sb_chunks,
                    scratch, pr, numorbs, dv, H);
}

cudaError_t bounds_take_tc(unsigned long long* word) {
#ifdef LCP_BOUNDS_CHECK
  return bounds_take(word);
#else
  *word = 0;
  return cudaErrorNotSupported;
#endif
}

}  // namespace lcp
