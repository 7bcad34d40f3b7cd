// Host check of the camera-frame ray order (csrc/kernels.h: RayOrder,
// ray_pixel): for each image size the order is a permutation of the pixels,
// every warp of 32 rays covers one 4 x 8 pixel tile, and with `grouped` the
// 4 warps of each group cover one 8 x 16 block.  Prints "ok" or the first
// failure; exit status 0 / 1.
#include <cstdio>
#include <vector>

#include "kernels.h"

using snisr::RayOrder;

static bool check(int W, int H) {
  const int64_t n = (int64_t)W * H;
  const RayOrder o = snisr::frame_ray_order(W, H, n);
  const bool tiled = W % snisr::kRayTileW == 0 && H % snisr::kRayTileH == 0;
  if ((o.w != 0) != tiled) {
    std::printf("%dx%d: tiled %d expected %d\n", W, H, o.w != 0, tiled);
    return false;
  }
  std::vector<char> seen((size_t)n, 0);
  for (int64_t i = 0; i < n; ++i) {
    const int64_t p = snisr::ray_pixel(i, o);
    if (p < 0 || p >= n || seen[(size_t)p]) {
      std::printf("%dx%d: ray %lld -> pixel %lld out of range or repeated\n", W, H, (long long)i, (long long)p);
      return false;
    }
    seen[(size_t)p] = 1;
  }
  if (!tiled) return true;
  const int span = o.grouped ? 128 : 32, bw = o.grouped ? 8 : 4, bh = o.grouped ? 16 : 8;
  for (int64_t b = 0; b < n; b += span) {
    const int64_t p0 = snisr::ray_pixel(b, o);
    int x0 = (int)(p0 % W), y0 = (int)(p0 / W);
    for (int64_t i = b; i < b + span; ++i) {
      const int64_t p = snisr::ray_pixel(i, o);
      x0 = std::min(x0, (int)(p % W));
      y0 = std::min(y0, (int)(p / W));
    }
    for (int64_t i = b; i < b + span; ++i) {
      const int64_t p = snisr::ray_pixel(i, o);
      const int x = (int)(p % W) - x0, y = (int)(p / W) - y0;
      if (x < 0 || x >= bw || y < 0 || y >= bh) {
        std::printf("%dx%d: rays %lld.. do not form a %dx%d block\n", W, H, (long long)b, bw, bh);
        return false;
      }
    }
  }
  return true;
}

int main() {
  const int sizes[][2] = {{1280, 720}, {1920, 1080}, {256, 256}, {640, 480}, {1000, 600}, {36, 20}, {4, 8}};
  for (const auto& s : sizes)
    if (!check(s[0], s[1])) return 1;
  // the caller's rays (n != W * H) keep their order
  if (snisr::frame_ray_order(1280, 720, 1000).w != 0) return 1;
  std::printf("ok\n");
  return 0;
}
