// Internal declarations shared by the host translation units of libsnisr.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "snisr.h"

namespace snisr {

snisr_status set_error(snisr_status st, const std::string& msg);

// Smallest fixed march step accepted by the entry points, in voxels.  Every
// march position is a tile-local distance below two tile sizes, and a step of
// voxel / 1024 is at least tile_size * 2^-20 for res <= 1024: four float
// spacings at the largest position, so each step advances the march.
constexpr float kMinStepVox = 1.0f / 1024.0f;
float f16_bits_to_f32(uint16_t h);
uint16_t f32_to_f16(float f);

// Flattened BVH node (32 bytes).  Inner node: count == 0, children at
// `first` and `first + 1`.  Leaf: `count` triangles starting at `first` in the
// BVH-ordered triangle arrays.
struct BvhNode {
  float bmin[3];
  int32_t first;
  float bmax[3];
  int32_t count;
};
static_assert(sizeof(BvhNode) == 32, "BvhNode must be 32 bytes");

// Binned-SAH build.  `order` receives the triangle ids in leaf order.
void build_bvh(const float* verts, const int32_t* faces, int64_t ntri, int leaf_max,
               std::vector<BvhNode>& nodes, std::vector<int32_t>& order);

}  // namespace snisr
