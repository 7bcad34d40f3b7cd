// Drop-in for the reference's diffuse renderer on its own scene format
// (FASTRENDERING.rendering_diffuse_octree_fp16,
// rendering/src/raydiffuse_render_octree_fp16.cu:10-235): per pixel the
// visited tiles in order; per tile a DDA over its 4^3 blocks; in a block with
// a node, samples every sample_step from the block entry where the node's
// sample flag is set; FP16 trilinear of the node's half4 RGBA through its
// int16 index map and FP16 compositing; early stop on the FP16
// transmittance; the first sample with transmittance below trans_th records
// 1/(z + tile entry) and the tile's group; with soft_hit a pixel without a
// first hit takes the last examined tile's group and 1/(its exit distance)
// (:223-228).  Every FP16 and FP32 operation rounds on its own (the _rn
// intrinsics keep the compiler from contracting a multiply and an add behind
// our back) except where the reference's nvcc build fuses them, which is
// written out: the FP32 entry point, sample point and dilated block corner,
// every FP16 linear interpolation (fma(v1, 1 - x, v2 * x)) and the colour
// accumulation (fma(weight, rgb, colour)).  The camera origin is a
// kernel argument (the reference keeps it in a __constant__ symbol) and the
// stream is the caller's.  Tile ids outside [0, num_tiles) and reads outside
// a node's dilated grid are skipped.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <string>

#include "device_common.cuh"
#include "kernels.h"
#include "snisr.h"
#include "snisr_internal.h"

namespace snisr {
namespace {

constexpr int kOctBlocks = 4;

// a * (1 - x) + b * x on both FP16 lanes (r, g) or (b, a), with the left
// product fused into the add as in the compiled reference: the same per-lane
// operations and roundings as the scalar form, half the instructions
__device__ __forceinline__ __half2 hlerp2(__half2 a, __half2 b, __half2 one_minus_x, __half2 x) {
  return __hfma2(a, one_minus_x, __hmul2_rn(b, x));
}

__global__ void octree_diffuse_kernel(const float* __restrict__ rays_d, const int32_t* __restrict__ visited,
                                      int64_t npix, int K, const float* __restrict__ origin,
                                      const int32_t* __restrict__ group_map, const uint2* __restrict__ data,
                                      const int32_t* __restrict__ block_map, const int16_t* __restrict__ node_map,
                                      const uint8_t* __restrict__ flags, const int64_t* __restrict__ vstart,
                                      const float* __restrict__ centers, int num_tiles, float tile_size,
                                      float voxel_size, float sample_step, int D, __half trans_th, float early,
                                      bool soft_hit, float* frame, float* inv_near, int16_t* net, RayOrder ord) {
  const int DD = D * D, D3 = D * D * D;
  const float bs = fdiv(tile_size, (float)kOctBlocks);
  // float3 / float multiplies by the reciprocal (cutil_math.h:397-401)
  const float inv_bs = fdiv(1.0f, bs), inv_vs = fdiv(1.0f, voxel_size);
  const __half early_h = __float2half(early);
  const __half one = __float2half(1.0f);
  const float o[3] = {__ldg(origin), __ldg(origin + 1), __ldg(origin + 2)};
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < npix; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p = ray_pixel(i, ord);  // this thread's pixel (warps march 4 x 8 pixel tiles of an image)
    const float d[3] = {rays_d[3 * p], rays_d[3 * p + 1], rays_d[3 * p + 2]};
    __half col[3] = {__float2half(0.f), __float2half(0.f), __float2half(0.f)};
    __half T = one;
    bool first_hit = false;
    int last_group = -1;
    float last_exit = 0.0f;
    const int32_t* vis = visited + p * K;
    for (int i = 0; i < K; ++i) {
      const int tile = vis[i];
      if (tile == -1) break;
      if (__hlt(T, early_h)) break;
      if (tile < 0 || tile >= num_tiles) continue;
      const int group = group_map[tile];
      const float c[3] = {centers[3 * tile], centers[3 * tile + 1], centers[3 * tile + 2]};
      const float hs = fdiv(tile_size, 2.0f);
      const float h3[3] = {hs, hs, hs};
      const float2 b = slab(o, d, c, h3);
      last_group = group;
      last_exit = b.y;
      if (b.x == -1.0f) continue;
      float ro[3];
      int cb[3], st[3];
      float tmax[3], tdel[3];
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        ro[a] = fsub(ffma(b.x, d[a], o[a]), fsub(c[a], hs));
        ro[a] = fminf(fmaxf(ro[a], 0.0f), fsub(tile_size, 0.00001f));
        cb[a] = (int)fmul(ro[a], inv_bs);
        st[a] = d[a] >= 0.0f ? 1 : -1;
        float nb = fmul((float)(cb[a] + st[a]), bs);
        if (st[a] < 0) nb = fadd(nb, bs);
        tmax[a] = safe_div(fsub(nb, ro[a]), d[a]);
        tdel[a] = safe_div(fmul(bs, (float)st[a]), d[a]);
      }
      if (cb[0] < 0 || cb[1] < 0 || cb[2] < 0 || cb[0] >= kOctBlocks || cb[1] >= kOctBlocks || cb[2] >= kOctBlocks)
        continue;  // entry rounded onto the far face (tile sizes where 1e-5 is below FP32 resolution)
      float near_ = 0.0f, far_ = fminf(fminf(tmax[0], tmax[1]), tmax[2]);
      const int32_t* bmap = block_map + (int64_t)tile * kOctBlocks * kOctBlocks * kOctBlocks;
      for (;;) {
        const int nidx = bmap[(cb[0] * kOctBlocks + cb[1]) * kOctBlocks + cb[2]];
        if (nidx != -1) {
          const int16_t* nodes = node_map + (int64_t)nidx * D3;
          const uint8_t* fl = flags + (int64_t)nidx * D3;
          const uint2* vox = data + vstart[nidx];
          float dc[3];
#pragma unroll
          for (int a = 0; a < 3; ++a) dc[a] = ffma((float)cb[a], bs, -voxel_size);
          float z = near_;
          while (z < far_) {
            float rel[3];
            int vl[3];
#pragma unroll
            for (int a = 0; a < 3; ++a) {
              rel[a] = fmul(fsub(ffma(z, d[a], ro[a]), dc[a]), inv_vs);
              vl[a] = (int)rel[a];
            }
            const bool inside = vl[0] >= 0 && vl[1] >= 0 && vl[2] >= 0 && vl[0] < D && vl[1] < D && vl[2] < D;
            if (!inside || !fl[vl[0] * DD + vl[1] * D + vl[2]]) {
              z = march_next(z, sample_step);
              continue;
            }
            if (!first_hit && __hlt(T, trans_th)) {
              first_hit = true;
              inv_near[p] = fdiv(1.0f, fadd(z, b.x));
              net[p] = (int16_t)group;
            }
            float f[3];
            int x0[3];
            bool ok = true;
#pragma unroll
            for (int a = 0; a < 3; ++a) {
              f[a] = fsub(rel[a], 0.5f);  // the product is shared with vl: not fused
              x0[a] = (int)f[a];
              ok = ok && x0[a] >= 0 && x0[a] + 1 < D;
            }
            if (ok) {
              __half2 wx[3], ux[3];  // x and 1 - x in FP16 on both lanes
#pragma unroll
              for (int a = 0; a < 3; ++a) {
                const float w = fmaxf(fsub(f[a], (float)x0[a]), 0.0f);
                wx[a] = __float2half2_rn(w);
                ux[a] = __float2half2_rn(fsub(1.0f, w));
              }
              __half2 rg[8], ba[8];  // corner k = (dx, dy, dz) = (k & 1, (k >> 1) & 1, (k >> 2) & 1)
#pragma unroll
              for (int k = 0; k < 8; ++k) {
                const int xi = x0[0] + (k & 1), yi = x0[1] + ((k >> 1) & 1), zi = x0[2] + ((k >> 2) & 1);
                const uint2 q = __ldg(vox + nodes[xi * DD + yi * D + zi]);
                rg[k] = *reinterpret_cast<const __half2*>(&q.x);
                ba[k] = *reinterpret_cast<const __half2*>(&q.y);
              }
              const __half2 rg0 = hlerp2(hlerp2(rg[0], rg[1], ux[0], wx[0]), hlerp2(rg[2], rg[3], ux[0], wx[0]), ux[1],
                                         wx[1]);
              const __half2 rg1 = hlerp2(hlerp2(rg[4], rg[5], ux[0], wx[0]), hlerp2(rg[6], rg[7], ux[0], wx[0]), ux[1],
                                         wx[1]);
              const __half2 ba0 = hlerp2(hlerp2(ba[0], ba[1], ux[0], wx[0]), hlerp2(ba[2], ba[3], ux[0], wx[0]), ux[1],
                                         wx[1]);
              const __half2 ba1 = hlerp2(hlerp2(ba[4], ba[5], ux[0], wx[0]), hlerp2(ba[6], ba[7], ux[0], wx[0]), ux[1],
                                         wx[1]);
              const __half2 rgm = hlerp2(rg0, rg1, ux[2], wx[2]), bam = hlerp2(ba0, ba1, ux[2], wx[2]);
              const __half rgba[4] = {__low2half(rgm), __high2half(rgm), __low2half(bam), __high2half(bam)};
              const float interval = fminf(sample_step, fsub(far_, z));
              const __half alpha =
                  __hsub_rn(one, hexp(__hmul_rn(__hmul_rn(rgba[3], __float2half(-1.0f)), __float2half(interval))));
              const __half wgt = __hmul_rn(alpha, T);
#pragma unroll
              for (int a = 0; a < 3; ++a) col[a] = __hfma(wgt, rgba[a], col[a]);
              T = __hmul_rn(T, __hsub_rn(one, alpha));
            }
            z = march_next(z, sample_step);
          }
        }
        int a = 2;
        if (tmax[0] < tmax[1]) a = tmax[0] < tmax[2] ? 0 : 2;
        else a = tmax[1] < tmax[2] ? 1 : 2;
        cb[a] += st[a];
        tmax[a] = fadd(tmax[a], tdel[a]);
        near_ = far_;
        far_ = fminf(fminf(tmax[0], tmax[1]), tmax[2]);
        if (cb[a] < 0 || cb[a] >= kOctBlocks) break;
      }
    }
    if (soft_hit && !first_hit && last_group != -1) {
      inv_near[p] = fdiv(1.0f, last_exit);
      net[p] = (int16_t)last_group;
    }
    frame[3 * p] = __half2float(col[0]);
    frame[3 * p + 1] = __half2float(col[1]);
    frame[3 * p + 2] = __half2float(col[2]);
  }
}

}  // namespace
}  // namespace snisr

using namespace snisr;

extern "C" snisr_status snisr_op_rendering_diffuse_octree(
    const float* rays_d, const int32_t* visited, int64_t npix, int32_t K, const float* origin,
    const int32_t* group_map, const uint16_t* data_voxels, const int32_t* block_map, const int16_t* node_map,
    const uint8_t* sample_flags, const int64_t* voxels_start, const float* centers, int32_t num_tiles,
    float tile_size, float voxel_size, float sample_step, int32_t dilated_voxels, float trans_th, float early_stop,
    int32_t soft_hit, float* frame, float* inverse_near, int16_t* net_idx, int32_t image_width, void* stream) {
  if (npix < 0 || K <= 0 || num_tiles <= 0 || dilated_voxels <= 1 || !(tile_size > 0) || !(voxel_size > 0) ||
      !(sample_step > 0))
    return set_error(SNISR_INVALID_ARG, "rendering_diffuse_octree: bad size");
  if (!(sample_step >= voxel_size * kMinStepVox))
    return set_error(SNISR_INVALID_ARG, "rendering_diffuse_octree: sample_step below voxel_size / 1024");
  if (npix == 0) return SNISR_OK;
  if (!rays_d || !visited || !origin || !group_map || !data_voxels || !block_map || !node_map ||
      !sample_flags || !voxels_start || !centers || !frame || !inverse_near || !net_idx)
    return set_error(SNISR_INVALID_ARG, "rendering_diffuse_octree: null argument");
  if (reinterpret_cast<uintptr_t>(data_voxels) % 8 != 0)
    return set_error(SNISR_INVALID_ARG, "rendering_diffuse_octree: data_voxels must be 8-byte aligned");
  if (image_width < 0) return set_error(SNISR_INVALID_ARG, "rendering_diffuse_octree: negative image width");
  // pixels [npix] of an image image_width wide (row-major): warps take 4 x 8
  // pixel tiles when the image divides into them (outputs identical)
  const RayOrder ord =
      image_width > 0 && npix % image_width == 0 ? frame_ray_order(image_width, (int)(npix / image_width), npix)
                                                 : RayOrder{};
  const int64_t blocks = (npix + 127) / 128;
  octree_diffuse_kernel<<<(int)(blocks < (1 << 20) ? blocks : (1 << 20)), 128, 0, (cudaStream_t)stream>>>(
      rays_d, visited, npix, K, origin, group_map,
      reinterpret_cast<const uint2*>(data_voxels), block_map, node_map, sample_flags, voxels_start, centers, num_tiles,
      tile_size, voxel_size, sample_step, dilated_voxels, __float2half(trans_th), early_stop, soft_hit != 0, frame,
      inverse_near, net_idx, ord);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess)
    return set_error(SNISR_CUDA_ERROR, std::string("rendering_diffuse_octree: ") + cudaGetErrorString(e));
  return SNISR_OK;
}
