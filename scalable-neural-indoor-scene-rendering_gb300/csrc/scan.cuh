// Exclusive scan of m uint32 values in place, in three launches: per-tile
// sums (4096 values per 1024-thread block, 4 consecutive values per thread
// so that a warp reads 512 contiguous bytes), one block scanning the tile
// sums, and a per-tile scan that adds the tile's offset.  `sums` holds
// scan_tiles(m) words.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace snisr {
namespace scan {
namespace {  // one copy per translation unit (kernels in a header)

constexpr int kThreads = 1024, kPer = 4, kTile = kThreads * kPer;

// Exclusive scan of one value per thread over a 1024-thread block; `total`
// receives the block sum.  warp_tot: 33 words of shared memory.
__device__ __forceinline__ uint32_t block_exclusive(uint32_t x, uint32_t* warp_tot, uint32_t& total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t v = x;
#pragma unroll
  for (int s = 1; s < 32; s <<= 1) {
    const uint32_t u = __shfl_up_sync(0xFFFFFFFFu, v, s);
    if (lane >= s) v += u;
  }
  if (lane == 31) warp_tot[warp] = v;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = warp_tot[lane];
#pragma unroll
    for (int s = 1; s < 32; s <<= 1) {
      const uint32_t u = __shfl_up_sync(0xFFFFFFFFu, w, s);
      if (lane >= s) w += u;
    }
    warp_tot[lane] = w;  // inclusive
    if (lane == 31) warp_tot[32] = w;
  }
  __syncthreads();
  const uint32_t before = (warp > 0 ? warp_tot[warp - 1] : 0u) + v - x;
  total = warp_tot[32];
  __syncthreads();
  return before;
}

__global__ void __launch_bounds__(kThreads) reduce_kernel(const uint32_t* __restrict__ v, int64_t m, uint32_t* sums) {
  __shared__ uint32_t wt[33];
  const int64_t b = (int64_t)blockIdx.x * kTile + (int64_t)threadIdx.x * kPer;
  uint32_t s = 0;
#pragma unroll
  for (int j = 0; j < kPer; ++j) s += b + j < m ? v[b + j] : 0u;
  uint32_t total;
  block_exclusive(s, wt, total);
  if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

__global__ void __launch_bounds__(kThreads) sums_kernel(uint32_t* sums, int nb) {
  __shared__ uint32_t wt[33];
  uint32_t carry = 0;
  for (int base = 0; base < nb; base += kThreads) {
    const int i = base + threadIdx.x;
    const uint32_t x = i < nb ? sums[i] : 0u;
    uint32_t total;
    const uint32_t before = block_exclusive(x, wt, total);
    if (i < nb) sums[i] = carry + before;
    carry += total;
  }
}

__global__ void __launch_bounds__(kThreads) apply_kernel(uint32_t* v, int64_t m, const uint32_t* __restrict__ sums) {
  __shared__ uint32_t wt[33];
  const int64_t b = (int64_t)blockIdx.x * kTile + (int64_t)threadIdx.x * kPer;
  uint32_t x[kPer], s = 0;
#pragma unroll
  for (int j = 0; j < kPer; ++j) {
    x[j] = b + j < m ? v[b + j] : 0u;
    s += x[j];
  }
  uint32_t total;
  uint32_t run = sums[blockIdx.x] + block_exclusive(s, wt, total);
#pragma unroll
  for (int j = 0; j < kPer; ++j) {
    if (b + j < m) v[b + j] = run;
    run += x[j];
  }
}

inline int tiles(int64_t m) { return (int)((m + kTile - 1) / kTile); }

inline cudaError_t exclusive(uint32_t* v, int64_t m, uint32_t* sums, cudaStream_t st) {
  const int nb = tiles(m);
  if (nb <= 0) return cudaSuccess;
  reduce_kernel<<<nb, kThreads, 0, st>>>(v, m, sums);
  sums_kernel<<<1, kThreads, 0, st>>>(sums, nb);
  apply_kernel<<<nb, kThreads, 0, st>>>(v, m, sums);
  return cudaGetLastError();
}

}  // namespace
}  // namespace scan
}  // namespace snisr
