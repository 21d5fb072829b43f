// Bounds checks of gathered indices, compiled in by LCP_BOUNDS_CHECK (the
// check build, liblcpgrid_check.so).  A failed check records the first
// violation of the translation unit in a device word -- (site << 56) | (index
// + 1), low 56 bits -- and the caller skips the access; nothing traps.  In the
// normal build every check is the constant true.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

namespace lcp {
namespace {

#ifdef LCP_BOUNDS_CHECK
__device__ unsigned long long g_bounds_word;

__device__ __forceinline__ bool bounds_ok(int64_t i, int64_t n, int site) {
  if (i >= 0 && i < n) return true;
  const unsigned long long code =
      ((unsigned long long)site << 56) | ((unsigned long long)(i + 1) & ((1ull << 56) - 1));
  atomicCAS(&g_bounds_word, 0ull, code);
  return false;
}

// Reads and clears this translation unit's word (host side).
cudaError_t bounds_take(unsigned long long* word) {
  cudaError_t e = cudaMemcpyFromSymbol(word, g_bounds_word, sizeof(*word));
  if (e != cudaSuccess) return e;
  const unsigned long long zero = 0;
  return cudaMemcpyToSymbol(g_bounds_word, &zero, sizeof(zero));
}
#else
__device__ __forceinline__ constexpr bool bounds_ok(int64_t, int64_t, int) { return true; }
#endif

}  // namespace
}  // namespace lcp
