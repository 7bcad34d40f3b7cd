// Footprint of the last batched frame: the distinct voxels whose samples
// the MLP stage read, and the distinct vertices (trilinear corners) behind
// them.  A profiling aid for the compulsory-bytes roofline; it runs outside
// the render path.
#include <cuda_runtime.h>

#include "kernels.h"

namespace snisr {
namespace {

__global__ void mark_voxels_kernel(const SampleRec* __restrict__ sorted, const int* __restrict__ ctrl, int64_t nvox,
                                   uint32_t* vox_bits) {
  const int n = ctrl[CTRL_SAMPLES];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const uint32_t v = sorted[i].rec;
    if ((int64_t)v < nvox) atomicOr(vox_bits + (v >> 5), 1u << (v & 31));
  }
}

__global__ void mark_vertices_kernel(const uint32_t* __restrict__ vox_bits, int64_t nvox,
                                     const int32_t* __restrict__ corners, int64_t nvert, uint32_t* vert_bits) {
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < nvox; v += (int64_t)gridDim.x * blockDim.x) {
    if (!((vox_bits[v >> 5] >> (v & 31)) & 1u)) continue;
    for (int k = 0; k < 8; ++k) {
      const int32_t c = corners[v * 8 + k];
      if (c >= 0 && c < nvert) atomicOr(vert_bits + (c >> 5), 1u << (c & 31));
    }
  }
}

__global__ void popcount_kernel(const uint32_t* __restrict__ bits, int64_t words, unsigned long long* out) {
  unsigned long long s = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < words; i += (int64_t)gridDim.x * blockDim.x)
    s += __popc(bits[i]);
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xFFFFFFFFu, s, o);
  if ((threadIdx.x & 31) == 0 && s) atomicAdd(out, s);
}

}  // namespace

cudaError_t launch_footprint(const SceneDev& S, const Workspace& ws, int64_t nvox, int64_t nvert, uint32_t* vox_bits,
                             uint32_t* vert_bits, unsigned long long* counts, int num_sms, cudaStream_t st) {
  const int64_t vw = (nvox + 31) / 32, tw = (nvert + 31) / 32;
  cudaError_t e;
  if ((e = cudaMemsetAsync(vox_bits, 0, vw * 4, st)) != cudaSuccess) return e;
  if ((e = cudaMemsetAsync(vert_bits, 0, tw * 4, st)) != cudaSuccess) return e;
  if ((e = cudaMemsetAsync(counts, 0, 2 * sizeof(unsigned long long), st)) != cudaSuccess) return e;
  const int grid = num_sms * 8;
  mark_voxels_kernel<<<grid, 256, 0, st>>>(ws.sorted, ws.ctrl, nvox, vox_bits);
  mark_vertices_kernel<<<grid, 256, 0, st>>>(vox_bits, nvox, S.corners, nvert, vert_bits);
  popcount_kernel<<<grid, 256, 0, st>>>(vox_bits, vw, counts);
  popcount_kernel<<<grid, 256, 0, st>>>(vert_bits, tw, counts + 1);
  return cudaGetLastError();
}

}  // namespace snisr
