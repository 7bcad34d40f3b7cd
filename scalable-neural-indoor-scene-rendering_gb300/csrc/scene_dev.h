// Plain-data scene view shared by host and device code (no device functions).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace snisr {

#define SNISR_INF 100000000.0f  // reference INF (rendering/src/include/cuda_utils.h:9)

struct __align__(16) OccWord {
  unsigned long long bits;  // occupancy of 64 consecutive voxels
  uint32_t base;            // global voxel id of the first occupied voxel of this word
  uint32_t pad;
};

struct __align__(16) BvhNodeDev {
  float bmin[3];
  int32_t first;
  float bmax[3];
  int32_t count;
};

constexpr int kBlkDistCap = 15;

// Device view of a scene, passed to kernels by value.
struct SceneDev {
  int gx, gy, gz;
  float smin[3];
  float tile_size, voxel, inv_voxel, step_len;
  float early_stop, start_offset;
  int res, words_per_tile, num_tiles, feat_dim;
  int dir_freqs, mlp_in, mlp_hidden, mlp_layers, params_per_tile;
  const int32_t* tile_index;     // dense -> sparse
  const float* tile_center;      // [NT][3]
  const OccWord* occ;            // [NT][words_per_tile]
  const uint8_t* blk_dist;       // [NT][(N/4)^3] Chebyshev distance, in 4^3 blocks, to the nearest
                                 // occupied block of the tile (0: occupied), at most kBlkDistCap + 1
  const float* dens;             // [NVOX][8] density logits per corner
  const int32_t* corners;        // [NVOX][8] vertex ids (training gathers/scatters)
  const float4* feat32;          // [NVOX][F/4][8] float4 per (channel group, corner)
  const uint4* feat16;           // [NVOX][8][F/8] 8 halves per (corner, channel group)
  const float* mlp_plain;        // [NT][plain stride] padded FP32 weights
  int plain_stride;
  const BvhNodeDev* bvh;
  const float4* tri;             // [ntri][3] v0, v1, v2 (w = 0) in BVH order
  const int32_t* tri_id;         // original triangle id per BVH slot
  int has_mesh;
  uint32_t* err;                 // device error word
};

// ERR_DRAIN: after a wait ran out, the in-flight copy or MMAs did not finish
// either; the CTA kept its tensor memory and the context is unusable.
enum : uint32_t { ERR_OVERFLOW = 1u, ERR_TIMEOUT = 2u, ERR_TMEM = 4u, ERR_DRAIN = 8u };

// One compacted sample of the batched form (16 bytes): the voxel's global
// id (its tile follows from the id: tiles own consecutive id ranges); the
// ray's pixel (24 bits) under the top 8 bits of the 24-bit compositing weight
// w = T_i alpha_i; the weight's low 16 bits under the position inside the
// voxel along x; the positions along y and z.  The weight keeps 16 of FP32's
// 23 mantissa bits (rounded to nearest, relative error <= 2^-17), the
// positions are 16-bit fixed point in [0, 1] (error <= 2^-17 voxel).
struct __align__(16) SampleRec {
  uint32_t rec;   // global voxel id
  uint32_t pix_w;
  uint32_t w_fx;
  uint32_t fy_fz;
};
constexpr int64_t kMaxBatchedRays = 1 << 24;  // the 24-bit pixel field

__host__ __device__ inline SampleRec pack_sample(uint32_t rec, uint32_t pix, float w, const float f[3]) {
  union { float f; uint32_t u; } wb{w};
  const uint32_t w24 = (wb.u + 0x40u) >> 7;  // w >= 0: sign bit 0
  uint32_t q[3];
  for (int a = 0; a < 3; ++a) q[a] = (uint32_t)(f[a] * 65535.0f + 0.5f);
  return SampleRec{rec, pix | ((w24 >> 16) << 24), (w24 & 0xFFFFu) | (q[0] << 16), q[1] | (q[2] << 16)};
}
__host__ __device__ inline uint32_t sample_pix(uint32_t pix_w) { return pix_w & 0xFFFFFFu; }
__host__ __device__ inline float sample_weight(uint32_t pix_w, uint32_t w_fx) {
  union { uint32_t u; float f; } wb{(((pix_w >> 24) << 16) | (w_fx & 0xFFFFu)) << 7};
  return wb.f;
}
__host__ __device__ inline float sample_pos(uint32_t q16) { return (float)q16 * (1.0f / 65535.0f); }

// Control words of one batched frame (zeroed per frame).
enum : int {
  CTRL_RESERVED = 0,   // sample slots handed out
  CTRL_WORK = 1,       // MLP work-queue head
  CTRL_CHUNKS = 2,     // total 128-sample chunks
  CTRL_SAMPLES = 3,    // total valid samples
  CTRL_STEPS = 4,      // u64 (words 4-5): voxel DDA steps of the frame
  CTRL_HEADER = 8,     // per-tile arrays follow: count, offset, chunk offset, cursor
};

}  // namespace snisr
