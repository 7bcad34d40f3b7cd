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

// One compacted sample of the batched form (32 bytes).
struct __align__(16) SampleRec {
  uint32_t rec;   // global voxel id, 0xFFFFFFFF for an unused slot
  uint32_t ray;
  float w;        // compositing weight T_i * alpha_i
  uint32_t tile;
  float f[3];     // position inside the voxel
  uint32_t pad;
};

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
