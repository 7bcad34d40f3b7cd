// Host-side launchers of the GB300 kernels (implemented in *.cu).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>
#include <mutex>

#include "scene_dev.h"

namespace snisr {

struct CamDev {
  int W, H;
  float cx, cy, inv_f;
  float c2w[12];
};

// Launch shapes chosen per scene (snisr_scene_set_tuning / autotune).
struct Tuning {
  int traverse_threads = 128;     // traverse_kernel block size (multiple of 32, <= 256)
  int scatter_blocks_per_sm = 16; // scatter_kernel grid = SMs x this
  int mlp_ctas_per_sm = 0;        // persistent mlp_tc_kernel CTAs per SM (0 = resident maximum)
  int train_march_threads = 128;  // tr_march_kernel block size (multiple of 32, <= 256)
  int train_fwd_warps = 8;        // tr_mlp_fwd_tc warps per CTA (4 or 8; one CTA per SM)
};

// Per-scene workspace, sized at creation; nothing is allocated per frame.
struct Workspace {
  float4* ray_o = nullptr;     // [max_rays] origin
  float4* ray_d = nullptr;     // [max_rays] direction, w = start distance
  uint4* enc = nullptr;        // [max_rays][4] FP16 view encoding (32 halves), by pixel
  SampleRec* recs = nullptr;   // [cap] compacted samples
  SampleRec* sorted = nullptr; // [cap] samples grouped by tile
  uint32_t* blk_count = nullptr;  // [cap/256 + 1] valid samples per 256-slot block
  uint32_t cap = 0;
  int* ctrl = nullptr;         // frame control words
  int ctrl_words = 0;
  int64_t max_rays = 0;
  const uint8_t* wimg = nullptr;  // per-tile tensor-core weight images
  int wimg_stride = 0;            // bytes per tile image
  int wimg_bytes = 0;             // bytes copied per tile
  Tuning tune;
};

// Runs `setup` (returning cudaError_t) once per device ordinal (< 64) for
// this flag word, e.g. kernel attribute setup; later calls on that device
// return cudaSuccess without running it, a failed setup is retried.
// Serialised by one process-wide mutex.
std::mutex& setup_mutex();
template <class Fn>
cudaError_t once_per_device(unsigned long long* flags, Fn&& setup) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const unsigned long long bit = dev >= 0 && dev < 64 ? 1ull << dev : 0ull;
  std::lock_guard<std::mutex> lock(setup_mutex());
  if (bit && (*flags & bit)) return cudaSuccess;
  e = setup();
  if (e == cudaSuccess) *flags |= bit;
  return e;
}

// Shape of a supported MLP instantiation.
bool mlp_shape_supported(int F, int H, int L);
// Bytes of one tile's tensor-core weight image (see build in api.cpp).
int tc_image_bytes(int H, int L);

// Order of the rays of a camera frame.  Ray i of the frame (its slot in the
// ray arrays and its lane in the traversal) is pixel ray_pixel(i): each warp
// of 32 rays takes a 4 x 8 pixel tile (tiles row by row; with `grouped`, in
// 2 x 2 groups, so that the 4 warps of a 128-thread block cover 8 x 16
// pixels).  Rays of one warp then start close together and cross the same
// voxels, which cuts the traversal's divergence and scattered loads.  The
// outputs (colour, depth, opacity) and the view encodings are indexed by
// pixel.  w = 0: ray i is pixel i (the caller's own rays, or an image the
// tiles do not divide).
struct RayOrder {
  int w = 0;
  bool grouped = false;
};
constexpr int kRayTileW = 4, kRayTileH = 8;
inline RayOrder frame_ray_order(int W, int H, int64_t n) {
  RayOrder o;
  if (n != (int64_t)W * H || W % kRayTileW != 0 || H % kRayTileH != 0) return o;
  o.w = W;
  o.grouped = W % (2 * kRayTileW) == 0 && H % (2 * kRayTileH) == 0;
  return o;
}
__host__ __device__ inline int64_t ray_pixel(int64_t i, RayOrder o) {
  if (o.w == 0) return i;
  const int64_t t = i >> 5;  // warp tile
  const int k = (int)(i & 31);
  const int tpr = o.w / kRayTileW;  // tiles per row
  int64_t ty;
  int tx;
  if (o.grouped) {
    const int64_t g = t >> 2;
    const int r = (int)(t & 3);
    ty = (g / (tpr / 2)) * 2 + (r >> 1);
    tx = (int)(g % (tpr / 2)) * 2 + (r & 1);
  } else {
    ty = t / tpr;
    tx = (int)(t % tpr);
  }
  return (ty * kRayTileH + k / kRayTileW) * o.w + tx * kRayTileW + k % kRayTileW;
}

cudaError_t launch_raygen(const SceneDev& S, const CamDev* cam, const float* origins, const float* dirs,
                          int64_t n, const Workspace& ws, bool want_enc, cudaStream_t st, RayOrder ord = RayOrder{});
cudaError_t launch_render_plain(const SceneDev& S, const Workspace& ws, int64_t n, float* rgb, float* depth,
                                float* opac, cudaStream_t st, RayOrder ord = RayOrder{});
// ev (optional, 5 events): recorded before traverse, after traverse, scan,
// scatter and the MLP.
cudaError_t launch_render_tc(const SceneDev& S, const Workspace& ws, int64_t n, float* rgb, float* depth,
                             float* opac, int num_sms, cudaStream_t st, cudaEvent_t* ev = nullptr,
                             RayOrder ord = RayOrder{});
cudaError_t launch_trace(const SceneDev& S, const Workspace& ws, int64_t n, int K, int32_t* visited,
                         int32_t* count, cudaStream_t st);
cudaError_t launch_proxy(const SceneDev& S, const float* origins, const float* dirs, int64_t n, float* t,
                         int32_t* tri, cudaStream_t st);
// Two nearest proxy hits per (ray, visited tile) (trainprep.cu).
cudaError_t launch_double_hits(const SceneDev& S, const float* ro, const float* rd, const int32_t* visited,
                               int64_t n, int K, float* hits, cudaStream_t st);
// Tensor-core training MLP (forward colours / backward with recomputation).
struct TrainTcArgs {
  const float* vfeat;
  const float* mlp;
  const float* dirs;
  int64_t n;
  const void* recs;
  const int32_t* tstart;
  int32_t* coff;
  int* work;
  uint4* enc;
  uint8_t* wimg;
  int img_stride;
  float4* cout;
  const float4* dout;
  float* gvfeat;
  float* gmlp;
  float* gstage;  // [NT][4][64 x 64 + 64] weight-gradient staging of the backward kernel
  int num_sms;
  int fwd_warps;
  uint8_t* htiles;  // [128-row chunks][L][16 KB] the forward's hidden activations (hi, swizzled)
};
int train_tc_image_bytes(int H, int L);
int train_tc_bwd_smem_bytes(int H, int L);
// enc: [n][12] uint4 (BF16 hi / mid / lo view encoding); coff: [2][NT + 2]
// chunk offsets per tile (128-row chunks, then 256-row units)
cudaError_t launch_train_tc(const SceneDev& S, const TrainTcArgs& a, bool backward, cudaStream_t st);

// distinct voxels / vertices read by the last batched frame -> counts[0], counts[1]
cudaError_t launch_footprint(const SceneDev& S, const Workspace& ws, int64_t nvox, int64_t nvert, uint32_t* vox_bits,
                             uint32_t* vert_bits, unsigned long long* counts, int num_sms, cudaStream_t st);

// specular pass ops (specular.cu)
cudaError_t launch_sort_by_key(int16_t* keys, int32_t* values, int32_t* starts, int64_t n, int64_t* count_host,
                               cudaStream_t st);
cudaError_t launch_assign_pixels(const int16_t* net, const int32_t* pixel_starts, const int32_t* block_starts,
                                 int64_t num_net, int16_t* new_net, int32_t* new_pixel_starts, cudaStream_t st);
int inference_mlp_param_count();
cudaError_t launch_inference_mlp(int spr, int num_block, float inv_far, float trans_stop, const int16_t* net,
                                 int num_groups, const float* transparency, const int32_t* qpix,
                                 const int32_t* pstarts, const float* centers, const float* samples,
                                 const float* rays_d, const uint16_t* params, float* results, int* work,
                                 uint32_t* err, int num_sms, cudaStream_t st);

cudaError_t launch_diag_wait(int64_t limit_ns, int64_t* waited_ns, bool* ran_out, cudaStream_t st);
cudaError_t launch_diag_mma(const uint16_t* A, const uint16_t* B, float* D, int N, int bf16, int mode,
                            cudaStream_t st);

}  // namespace snisr
