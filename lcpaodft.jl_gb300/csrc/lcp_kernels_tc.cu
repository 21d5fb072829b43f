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
                                                          int* __restrict__ status) {
  extern __shared__ __align__(1024) uint8_t smem[];
  __shared__ uint64_t mbar;
  __shared__ uint32_t tslot;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  uint8_t* sa = smem;
  uint8_t* sb = smem + kSelfM * K * 2;
  // layouts: [k-group][mn-group][128 B core matrix]; SBO = 128 B, LBO = rows/8 * 128 B
  const uint32_t lbo_a = (kSelfM / 8) * 128, lbo_b = (N / 8) * 128, sbo = 128;
  for (int idx = tid; idx < kSelfM * K; idx += blockDim.x) {
    const int m = idx / K, k = idx - m * K;
    const uint32_t off = a_mn ? tc::mnmajor_off(m, k, lbo_a, sbo) : tc::kmajor_off(m, k, lbo_a, sbo);
    *reinterpret_cast<__nv_bfloat16*>(sa + off) = __float2bfloat16_rn(A[idx]);
  }
  for (int idx = tid; idx < N * K; idx += blockDim.x) {
    const int n = idx / K, k = idx - n * K;
    const uint32_t off = b_mn ? tc::mnmajor_off(n, k, lbo_b, sbo) : tc::kmajor_off(n, k, lbo_b, sbo);
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
      const uint64_t da = tc::smem_desc(tc::smem_u32(sa + 2 * ks * lbo_a), lbo_a, sbo);
      const uint64_t db = tc::smem_desc(tc::smem_u32(sb + 2 * ks * lbo_b), lbo_b, sbo);
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
                               int* status, cudaStream_t st) {
  const size_t smem = (size_t)(kSelfM + N) * K * 2;
  LCP_CUDA_TRY(cudaFuncSetAttribute(tc_selftest_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  tc_selftest_kernel<<<1, 128, smem, st>>>(A, B, D, N, K, a_mn, b_mn, status);
  return cudaGetLastError();
}

}  // namespace lcp
