// Scene construction kernels: expand per-vertex data into per-voxel
// 8-corner blocks so that one sample reads one contiguous record.
//
//   dens   [NVOX][8]        FP32 density logits per corner
//   feat32 [NVOX][F/4][8]   float4 = 4 channels of one corner
//   feat16 [NVOX][8][F/8]   uint4  = 8 FP16 channels of one corner,
//                           corner-major: the F/8 lanes that interpolate one
//                           sample read one contiguous F*2-byte slice per corner
#include <cuda_fp16.h>

#include "scene_dev.h"

namespace snisr {

namespace {

__device__ __forceinline__ float load_val(const void* p, int64_t i, int f16) {
  return f16 ? __half2float(reinterpret_cast<const __half*>(p)[i]) : reinterpret_cast<const float*>(p)[i];
}

__global__ void expand_kernel(const int32_t* __restrict__ corners, const void* vfeat, const void* vdens, int f16,
                              int F, int64_t nvox, float* dens, float4* feat32, uint4* feat16) {
  const int G4 = F / 4, G8 = F / 8;
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < nvox; v += (int64_t)gridDim.x * blockDim.x) {
    for (int k = 0; k < 8; ++k) {
      int64_t vid = corners[v * 8 + k];
      dens[v * 8 + k] = load_val(vdens, vid, f16);
      for (int g = 0; g < G4; ++g) {
        float4 q;
        q.x = load_val(vfeat, vid * F + 4 * g + 0, f16);
        q.y = load_val(vfeat, vid * F + 4 * g + 1, f16);
        q.z = load_val(vfeat, vid * F + 4 * g + 2, f16);
        q.w = load_val(vfeat, vid * F + 4 * g + 3, f16);
        feat32[(v * G4 + g) * 8 + k] = q;
      }
      for (int g = 0; g < G8; ++g) {
        __align__(16) __half h[8];
        for (int c = 0; c < 8; ++c) h[c] = __float2half_rn(load_val(vfeat, vid * F + 8 * g + c, f16));
        feat16[(v * 8 + k) * G8 + g] = *reinterpret_cast<const uint4*>(h);
      }
    }
  }
}

}  // namespace

cudaError_t launch_expand(const int32_t* corners, const void* vfeat, const void* vdens, int f16, int F, int64_t nvox,
                          float* dens, float4* feat32, uint4* feat16, cudaStream_t st) {
  int64_t blocks = (nvox + 255) / 256;
  if (blocks < 1) blocks = 1;
  if (blocks > 65536) blocks = 65536;
  expand_kernel<<<(int)blocks, 256, 0, st>>>(corners, vfeat, vdens, f16, F, nvox, dens, feat32, feat16);
  return cudaGetLastError();
}

}  // namespace snisr
