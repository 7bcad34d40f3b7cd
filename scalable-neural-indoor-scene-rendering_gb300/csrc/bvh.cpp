// Binned surface-area-heuristic BVH over the proxy triangle mesh.
//
// The reference intersects rays with a per-tile uniform grid of face lists
// (BConFaceNum / BConFaceIdx, training/src/cuda_func.cu:130-282), whose build
// is not part of the reference tree.  A BVH bounds the per-ray work by the
// tree depth instead of the faces per grid block.
#include <algorithm>
#include <cfloat>
#include <cmath>

#include "snisr_internal.h"

namespace snisr {

namespace {

struct Aabb {
  float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX};
  float hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
  void grow(const float* p) {
    for (int a = 0; a < 3; ++a) { lo[a] = std::min(lo[a], p[a]); hi[a] = std::max(hi[a], p[a]); }
  }
  void grow(const Aabb& b) {
    for (int a = 0; a < 3; ++a) { lo[a] = std::min(lo[a], b.lo[a]); hi[a] = std::max(hi[a], b.hi[a]); }
  }
  double area() const {
    double e[3];
    for (int a = 0; a < 3; ++a) e[a] = hi[a] >= lo[a] ? (double)hi[a] - lo[a] : 0.0;
    return 2.0 * (e[0] * e[1] + e[1] * e[2] + e[2] * e[0]);
  }
};

constexpr int kBins = 16;

}  // namespace

void build_bvh(const float* verts, const int32_t* faces, int64_t ntri, int leaf_max,
               std::vector<BvhNode>& nodes, std::vector<int32_t>& order) {
  nodes.clear();
  order.resize((size_t)ntri);
  if (ntri == 0) return;
  std::vector<Aabb> tb((size_t)ntri);
  std::vector<float> cen((size_t)ntri * 3);
  for (int64_t t = 0; t < ntri; ++t) {
    for (int k = 0; k < 3; ++k) tb[(size_t)t].grow(verts + 3 * (int64_t)faces[3 * t + k]);
    for (int a = 0; a < 3; ++a) cen[(size_t)(3 * t + a)] = 0.5f * (tb[(size_t)t].lo[a] + tb[(size_t)t].hi[a]);
    order[(size_t)t] = (int32_t)t;
  }
  nodes.reserve((size_t)(2 * ntri / std::max(1, leaf_max / 2) + 2));
  struct Task { int32_t node, begin, end; };
  std::vector<Task> stack;
  nodes.push_back(BvhNode{});
  stack.push_back({0, 0, (int32_t)ntri});
  while (!stack.empty()) {
    Task tk = stack.back();
    stack.pop_back();
    Aabb box, cbox;
    for (int32_t i = tk.begin; i < tk.end; ++i) {
      box.grow(tb[(size_t)order[(size_t)i]]);
      cbox.grow(&cen[(size_t)order[(size_t)i] * 3]);
    }
    BvhNode& nd = nodes[(size_t)tk.node];
    for (int a = 0; a < 3; ++a) { nd.bmin[a] = box.lo[a]; nd.bmax[a] = box.hi[a]; }
    int32_t n = tk.end - tk.begin;
    auto make_leaf = [&]() {
      nodes[(size_t)tk.node].first = tk.begin;
      nodes[(size_t)tk.node].count = n;
    };
    if (n <= leaf_max) { make_leaf(); continue; }
    // SAH over binned centroids on each axis
    double best_cost = DBL_MAX;
    int best_axis = -1, best_split = -1;
    for (int a = 0; a < 3; ++a) {
      float lo = cbox.lo[a], hi = cbox.hi[a];
      if (!(hi > lo)) continue;
      Aabb bb[kBins];
      int cnt[kBins] = {0};
      float scale = kBins / (hi - lo);
      for (int32_t i = tk.begin; i < tk.end; ++i) {
        int32_t t = order[(size_t)i];
        int b = std::min(kBins - 1, (int)((cen[(size_t)t * 3 + a] - lo) * scale));
        cnt[b]++;
        bb[b].grow(tb[(size_t)t]);
      }
      double right_area[kBins];
      int right_cnt[kBins];
      Aabb acc;
      int c = 0;
      for (int b = kBins - 1; b > 0; --b) {
        acc.grow(bb[b]);
        c += cnt[b];
        right_area[b] = acc.area();
        right_cnt[b] = c;
      }
      Aabb lacc;
      int lc = 0;
      for (int b = 0; b < kBins - 1; ++b) {
        lacc.grow(bb[b]);
        lc += cnt[b];
        if (lc == 0 || right_cnt[b + 1] == 0) continue;
        double cost = lacc.area() * lc + right_area[b + 1] * right_cnt[b + 1];
        if (cost < best_cost) { best_cost = cost; best_axis = a; best_split = b; }
      }
    }
    int32_t mid;
    if (best_axis < 0 || best_cost >= box.area() * n) {
      if (n <= 4 * leaf_max && best_axis < 0) { make_leaf(); continue; }
      // fall back to a median split along the widest centroid axis
      int a = 0;
      for (int k = 1; k < 3; ++k) if (cbox.hi[k] - cbox.lo[k] > cbox.hi[a] - cbox.lo[a]) a = k;
      mid = tk.begin + n / 2;
      std::nth_element(order.begin() + tk.begin, order.begin() + mid, order.begin() + tk.end,
                       [&](int32_t x, int32_t y) {
                         float cx = cen[(size_t)x * 3 + a], cy = cen[(size_t)y * 3 + a];
                         return cx < cy || (cx == cy && x < y);
                       });
    } else {
      float lo = cbox.lo[best_axis], scale = kBins / (cbox.hi[best_axis] - lo);
      auto it = std::partition(order.begin() + tk.begin, order.begin() + tk.end, [&](int32_t t) {
        int b = std::min(kBins - 1, (int)((cen[(size_t)t * 3 + best_axis] - lo) * scale));
        return b <= best_split;
      });
      mid = (int32_t)(it - order.begin());
      if (mid == tk.begin || mid == tk.end) mid = tk.begin + n / 2;
    }
    int32_t left = (int32_t)nodes.size();
    nodes.push_back(BvhNode{});
    nodes.push_back(BvhNode{});
    nodes[(size_t)tk.node].first = left;
    nodes[(size_t)tk.node].count = 0;
    stack.push_back({left + 1, mid, tk.end});
    stack.push_back({left, tk.begin, mid});
  }
}

}  // namespace snisr
