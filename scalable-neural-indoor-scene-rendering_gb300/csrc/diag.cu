// Diagnostics of the tcgen05 operand layouts (used by the GPU tests).
//
// mode 0: A [128][64], B [N][64] K-major (the MLP's forward layout),
//         D = A B^T (K = 64).
// mode 3: as mode 0 with A taken from tensor memory: every thread stores its
//         row of A into columns [64, 96) of the CTA's allocation
//         (tcgen05.st 32x32b), the MMA reads it as the TMEM A operand.
// mode 1/2: At [128][64], Bt [128][64] stored sample-major (row = K index,
//         the layout the epilogues write), consumed as MN-major operands,
//         D[m][n] = sum_k At[k][m] Bt[k][n] for m < 64 (K = 128), the second
//         64-row atom of A pointing at a zero tile.  Mode 1: leading byte
//         offset = MN atom stride, stride byte offset = 8-row K group stride;
//         mode 2: the two swapped.
// diag_wait_kernel: a wait on an mbarrier that nothing completes, with a
// given time limit: the bounded-wait error path of the tensor-core kernels
// (the wait runs out, the kernel reports it and returns, the context stays
// usable), exercised without a fault.
// march_math_kernel: the render march's single-precision e^x, log1p and
// softplus on an array, so that tests can compare their bits with the host
// restatement.
#include <cuda_runtime.h>

#include <string>

#include "device_common.cuh"
#include "kernels.h"
#include "snisr.h"
#include "snisr_internal.h"
#include "tc_ptx.cuh"

namespace snisr {
namespace {

__device__ __forceinline__ uint64_t sdesc_sw128_mn(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | ((uint64_t)1u << 46) | ((uint64_t)2u << 61);
}

__global__ void __launch_bounds__(128) diag_mma_kernel(const uint16_t* A, const uint16_t* B, float* D, int N,
                                                       int bf16, int mode, int* status) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* base = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint8_t* As = base;               // 16 KB
  uint8_t* Zs = base + 16384;       // 16 KB zeros
  uint8_t* Bs = base + 32768;       // 16 KB (+16 KB slack)
  uint64_t* bar = reinterpret_cast<uint64_t*>(base + 65536);
  uint32_t* slot = reinterpret_cast<uint32_t*>(bar + 1);
  const int tid = threadIdx.x, warp = tid >> 5;
  // zero [Zs, base + 64 KB): the zero tile, the B tile and its slack
  for (int k = tid; k < (65536 - 16384) / 16; k += 128) reinterpret_cast<uint4*>(Zs)[k] = make_uint4(0, 0, 0, 0);
  __syncthreads();
  const int brows = (mode == 0 || mode == 3) ? N : 128;
  for (int c = 0; c < 8; ++c) {
    *reinterpret_cast<uint4*>(As + tc::sw128_offset(tid, c)) = *reinterpret_cast<const uint4*>(A + tid * 64 + 8 * c);
    if (tid < brows)
      *reinterpret_cast<uint4*>(Bs + tc::sw128_offset(tid, c)) = *reinterpret_cast<const uint4*>(B + tid * 64 + 8 * c);
  }
  if (tid == 0) {
    tc::mbar_init(tc::smem_addr(bar), 1);
    tc::fence_mbar_init();
  }
  if (warp == 0) {
    tc::tmem_alloc(tc::smem_addr(slot), 128);
    tc::tmem_relinquish();
  }
  tc::fence_proxy_async();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *slot;
  if (mode == 3) {
    // row tid of A (64 16-bit values = 32 columns) into lane tid, columns 64..95
    const uint32_t* row = reinterpret_cast<const uint32_t*>(A + tid * 64);
    uint32_t v[32];
#pragma unroll
    for (int c = 0; c < 32; ++c) v[c] = row[c];
    const uint32_t lane_base = tmem + ((uint32_t)(warp * 32) << 16);
    tc::tmem_st16(lane_base + 64, v);
    tc::tmem_st16(lane_base + 80, v + 16);
    tc::tmem_wait_st();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
  }
  if (tid == 0) {
    if (mode == 3) {
      const uint32_t idesc = tc::idesc_f16(N, bf16);
      for (int kk = 0; kk < 4; ++kk)
        tc::mma_f16_ta(tmem, tmem + 64 + 8 * kk, tc::sdesc_sw128(tc::smem_addr(Bs) + 32 * kk), idesc, kk > 0);
    } else if (mode == 0) {
      const uint32_t idesc = tc::idesc_f16(N, bf16);
      for (int kk = 0; kk < 4; ++kk)
        tc::mma_f16(tmem, tc::sdesc_sw128(tc::smem_addr(As) + 32 * kk), tc::sdesc_sw128(tc::smem_addr(Bs) + 32 * kk),
                    idesc, kk > 0);
    } else {
      const uint32_t idesc = tc::idesc_f16(64, bf16) | (1u << 15) | (1u << 16);  // A, B MN-major
      const uint32_t lbo = mode == 1 ? 16384u : 1024u, sbo = mode == 1 ? 1024u : 16384u;
      for (int kk = 0; kk < 8; ++kk)
        tc::mma_f16(tmem, sdesc_sw128_mn(tc::smem_addr(As) + 2048 * kk, lbo, sbo),
                    sdesc_sw128_mn(tc::smem_addr(Bs) + 2048 * kk, lbo, sbo), idesc, kk > 0);
    }
    tc::mma_commit(tc::smem_addr(bar));
  }
  bool ok = tid == 0 ? tc::mbar_wait(tc::smem_addr(bar), 0) : true;
  tc::fence_after_sync();
  bool drained = true;
  if (__syncthreads_or(!ok)) {
    if (tid == 0) {
      // once more, bounded: the MMAs must be done before TMEM is freed
      drained = tc::mbar_wait(tc::smem_addr(bar), 0);
      *status = drained ? 1 : 2;
    }
  } else {
    const int nc = (mode == 0 || mode == 3) ? N : 64;
    float v[64];
    const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16);
    for (int cc = 0; cc < nc; cc += 16) tc::tmem_ld16(taddr + cc, v + cc);
    tc::tmem_wait_ld();
    for (int j = 0; j < nc; ++j) D[tid * nc + j] = v[j];
    if (tid == 0) *status = 0;
  }
  tc::fence_before_sync();
  // tensor memory stays allocated when the MMAs did not drain (status 2)
  if (__syncthreads_or(!drained) == 0 && warp == 0) tc::tmem_dealloc(tmem, 128);
}

__global__ void diag_wait_kernel(uint64_t limit_ns, long long* out) {
  __shared__ uint64_t bar;
  const uint32_t b = tc::smem_addr(&bar);
  if (threadIdx.x == 0) {
    tc::mbar_init(b, 1);  // one arrival expected; none comes
    tc::fence_mbar_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const uint64_t t0 = tc::global_ns();
    const bool ok = tc::mbar_wait(b, 0, limit_ns);
    out[0] = ok ? 0 : 1;
    out[1] = (long long)(tc::global_ns() - t0);
  }
}

__global__ void march_math_kernel(int fn, const float* __restrict__ x, int64_t n, float* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float v = x[i];
    out[i] = fn == 0 ? exp_nonpos(v) : fn == 1 ? log1p_unit(v) : softplus_march(v);
  }
}

}  // namespace

cudaError_t launch_diag_wait(int64_t limit_ns, int64_t* waited_ns, bool* ran_out, cudaStream_t st) {
  long long* out = nullptr;
  cudaError_t e = cudaMallocAsync(&out, 2 * sizeof(long long), st);
  if (e != cudaSuccess) return e;
  diag_wait_kernel<<<1, 32, 0, st>>>((uint64_t)limit_ns, out);
  e = cudaGetLastError();
  long long h[2] = {-1, -1};
  if (e == cudaSuccess) e = cudaMemcpyAsync(h, out, sizeof(h), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaFreeAsync(out, st);
  *ran_out = h[0] == 1;
  *waited_ns = h[1];
  return e;
}

cudaError_t launch_diag_mma(const uint16_t* A, const uint16_t* B, float* D, int N, int bf16, int mode,
                            cudaStream_t st) {
  int* status = nullptr;
  cudaError_t e = cudaMallocAsync(&status, sizeof(int), st);
  if (e != cudaSuccess) return e;
  const int smem = 1024 + 65536 + 64;
  e = cudaFuncSetAttribute(diag_mma_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e == cudaSuccess) {
    diag_mma_kernel<<<1, 128, smem, st>>>(A, B, D, N, bf16, mode, status);
    e = cudaGetLastError();
  }
  int h = -1;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&h, status, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaFreeAsync(status, st);
  if (e == cudaSuccess && h != 0) e = cudaErrorLaunchTimeout;
  return e;
}

}  // namespace snisr

extern "C" snisr_status snisr_diag_march_math(int32_t fn, const float* x_dev, int64_t n, float* out_dev,
                                              void* stream) {
  using namespace snisr;
  if (fn < 0 || fn > 2 || n < 0 || (n > 0 && (!x_dev || !out_dev)))
    return set_error(SNISR_INVALID_ARG, "diag_march_math: bad argument (fn 0..2, device arrays of n floats)");
  if (n == 0) return SNISR_OK;
  int64_t blocks = (n + 255) / 256;
  if (blocks > 65536) blocks = 65536;
  march_math_kernel<<<(int)blocks, 256, 0, (cudaStream_t)stream>>>(fn, x_dev, n, out_dev);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_error(SNISR_CUDA_ERROR, std::string("diag_march_math: ") + cudaGetErrorString(e));
  return SNISR_OK;
}
