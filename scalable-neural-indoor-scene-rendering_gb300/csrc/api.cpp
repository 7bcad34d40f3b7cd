// C ABI of libsnisr: scene lifetime, render entry points, per-stage ops.
// No exception crosses this boundary; failures become snisr_status codes
// with a thread-local message (snisr_last_error_string).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "kernels.h"
#include "snisr_internal.h"

namespace snisr {

namespace {
thread_local std::string g_last_error;
}

snisr_status set_error(snisr_status st, const std::string& msg) {
  g_last_error = msg;
  return st;
}

struct TrainWS;
TrainWS* train_ws_new();
void train_ws_free(TrainWS* T);
cudaError_t launch_expand(const int32_t* corners, const void* vfeat, const void* vdens, int f16, int F, int64_t nvox,
                          float* dens, float4* feat32, uint4* feat16, cudaStream_t st);
int train_ctrl_words(int NT);

}  // namespace snisr

using namespace snisr;

struct snisr_scene {
  int device = 0;
  int num_sms = 0;
  SceneDev S{};
  Workspace ws{};
  snisr_scene_info info{};
  std::vector<void*> allocs;  // every device allocation of the scene
  // training workspace (allocated lazily at the first training call)
  TrainWS* train = nullptr;
  int max_samples_per_ray = 48;
  // host copies needed for MLP re-layout
  int F = 0, H = 0, L = 0, NT = 0, in = 0, P = 0;
  uint32_t* err_host = nullptr;  // pinned mirror of the device error word
  const int32_t* corners = nullptr;  // [NVOX][8] vertex ids on the device
  bool profiling = false;
  int last_form = -1;
  cudaEvent_t ev[8] = {};
  float* out_bufs = nullptr;          // staging for render_host
  uint32_t* fp_bits = nullptr;        // footprint bitmaps (voxels, vertices) + 2 counters, lazily
  // render_host_async: two device staging slots, a copy stream, per-slot
  // events (render done -> copy may start; copy done -> slot may be reused)
  float* async_bufs = nullptr;
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t render_done[2] = {}, copy_done[2] = {};
  int async_slot = 0;
};

namespace {

#define CUDA_TRY(expr, what)                                                                              \
  do {                                                                                                    \
    cudaError_t e__ = (expr);                                                                             \
    if (e__ != cudaSuccess) {                                                                             \
      return set_error(e__ == cudaErrorMemoryAllocation ? SNISR_OOM : SNISR_CUDA_ERROR,                   \
                       std::string(what) + ": " + cudaGetErrorString(e__));                               \
    }                                                                                                     \
  } while (0)

template <class T>
snisr_status dev_alloc(snisr_scene* sc, T** p, size_t bytes, const char* what) {
  void* q = nullptr;
  if (bytes == 0) bytes = 16;
  cudaError_t e = cudaMalloc(&q, bytes);
  if (e != cudaSuccess) return set_error(SNISR_OOM, std::string("cudaMalloc ") + what + ": " + cudaGetErrorString(e));
  sc->allocs.push_back(q);
  sc->info.device_bytes += (int64_t)bytes;
  *p = static_cast<T*>(q);
  return SNISR_OK;
}

template <class T>
snisr_status upload(snisr_scene* sc, T** p, const void* src, size_t bytes, const char* what) {
  snisr_status st = dev_alloc(sc, p, bytes, what);
  if (st != SNISR_OK) return st;
  if (bytes) CUDA_TRY(cudaMemcpy(*p, src, bytes, cudaMemcpyHostToDevice), what);
  return SNISR_OK;
}

void free_scene(snisr_scene* sc) {
  if (!sc) return;
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(sc->device);
  for (void* p : sc->allocs) cudaFree(p);
  if (sc->train) train_ws_free(sc->train);
  if (sc->err_host) cudaFreeHost(sc->err_host);
  for (cudaEvent_t e : sc->ev)
    if (e) cudaEventDestroy(e);
  for (int k = 0; k < 2; ++k) {
    if (sc->render_done[k]) cudaEventDestroy(sc->render_done[k]);
    if (sc->copy_done[k]) cudaEventDestroy(sc->copy_done[k]);
  }
  if (sc->copy_stream) {
    cudaStreamSynchronize(sc->copy_stream);
    cudaStreamDestroy(sc->copy_stream);
  }
  cudaSetDevice(prev);
  delete sc;
}

// Plain FP32 layout: for each Linear W[out][round4(in)] then b[round4(out)].
std::vector<float> plain_layout(const float* p, int in, int H, int L, int& stride) {
  std::vector<float> out;
  int64_t off = 0;
  for (int l = 0; l <= L; ++l) {
    int fi = l == 0 ? in : H, fo = l == L ? 3 : H;
    int fip = (fi + 3) & ~3, fop = (fo + 3) & ~3;
    for (int o = 0; o < fo; ++o)
      for (int i = 0; i < fip; ++i) out.push_back(i < fi ? p[off + (int64_t)o * fi + i] : 0.0f);
    off += (int64_t)fi * fo;
    for (int o = 0; o < fop; ++o) out.push_back(o < fo ? p[off + o] : 0.0f);
    off += fo;
  }
  stride = (int)out.size();
  return out;
}

// Tensor-core image of one tile (layout in tc_image_bytes): FP16 weights
// and biases in 128-byte swizzled K-major tiles.
void tc_image(const float* p, int in, int H, int L, uint8_t* img) {
  const int bytes = tc_image_bytes(H, L);
  std::memset(img, 0, (size_t)bytes);
  auto put = [&](uint8_t* tile, int row, int k, float v) {
    uint16_t h = f32_to_f16(v);
    uint32_t o = ((uint32_t)row >> 3) * 1024u + ((uint32_t)row & 7u) * 128u +
                 ((((uint32_t)k >> 3) ^ ((uint32_t)row & 7u)) << 4) + (((uint32_t)k & 7u) << 1);
    std::memcpy(tile + o, &h, 2);
  };
  uint8_t* wout = img + L * H * 128;
  uint8_t* bhid = wout + 2048;
  uint8_t* bout = bhid + H * 128;
  int64_t off = 0;
  for (int l = 0; l <= L; ++l) {
    int fi = l == 0 ? in : H, fo = l == L ? 3 : H;
    uint8_t* wt = l < L ? img + l * H * 128 : wout;
    for (int n = 0; n < fo; ++n)
      for (int k = 0; k < fi; ++k) put(wt, n, k, p[off + (int64_t)n * fi + k]);
    off += (int64_t)fi * fo;
    for (int n = 0; n < fo; ++n)
      for (int k = 0; k < 16; ++k) put(l < L ? bhid : bout, n, (l < L ? 16 * l : 0) + k, p[off + n]);
    off += fo;
  }
}

snisr_status upload_mlp(snisr_scene* sc, const float* params_host, bool allocate) {
  const int NT = sc->NT, in = sc->in, H = sc->H, L = sc->L, P = sc->P;
  std::vector<float> plain;
  int stride = 0;
  for (int t = 0; t < NT; ++t) {
    std::vector<float> one = plain_layout(params_host + (int64_t)t * P, in, H, L, stride);
    plain.insert(plain.end(), one.begin(), one.end());
  }
  const int img = tc_image_bytes(H, L);
  const int img_stride = (img + 127) & ~127;
  std::vector<uint8_t> imgs((size_t)NT * img_stride, 0);
  for (int t = 0; t < NT; ++t) tc_image(params_host + (int64_t)t * P, in, H, L, imgs.data() + (size_t)t * img_stride);
  if (allocate) {
    float* dplain = nullptr;
    uint8_t* dimg = nullptr;
    snisr_status st = upload(sc, &dplain, plain.data(), plain.size() * 4, "mlp plain");
    if (st != SNISR_OK) return st;
    st = upload(sc, &dimg, imgs.data(), imgs.size(), "mlp images");
    if (st != SNISR_OK) return st;
    sc->S.mlp_plain = dplain;
    sc->S.plain_stride = stride;
    sc->ws.wimg = dimg;
    sc->ws.wimg_stride = img_stride;
    sc->ws.wimg_bytes = img;
  } else {
    CUDA_TRY(cudaMemcpy(const_cast<float*>(sc->S.mlp_plain), plain.data(), plain.size() * 4, cudaMemcpyHostToDevice), "mlp plain");
    CUDA_TRY(cudaMemcpy(const_cast<uint8_t*>(sc->ws.wimg), imgs.data(), imgs.size(), cudaMemcpyHostToDevice), "mlp images");
  }
  return SNISR_OK;
}

struct DeviceGuard {
  int prev = -1;
  explicit DeviceGuard(int dev) {
    cudaGetDevice(&prev);
    if (prev != dev) cudaSetDevice(dev);
  }
  ~DeviceGuard() {
    int cur = -1;
    cudaGetDevice(&cur);
    if (prev >= 0 && cur != prev) cudaSetDevice(prev);
  }
};

snisr_status validate_desc(const snisr_scene_desc* d) {
  if (!d) return set_error(SNISR_INVALID_ARG, "scene_create: desc is null");
  if (d->grid[0] <= 0 || d->grid[1] <= 0 || d->grid[2] <= 0) return set_error(SNISR_INVALID_ARG, "scene_create: grid must be positive");
  if (!(d->tile_size > 0.0f)) return set_error(SNISR_INVALID_ARG, "scene_create: tile_size must be > 0");
  if (d->res <= 0 || d->res % 4 != 0 || d->res > 1024) return set_error(SNISR_INVALID_ARG, "scene_create: res must be a positive multiple of 4 (<= 1024)");
  if (d->num_tiles < 0 || !d->tile_index) return set_error(SNISR_INVALID_ARG, "scene_create: tile_index missing");
  if (d->num_tiles > 0 && !d->occupancy) return set_error(SNISR_INVALID_ARG, "scene_create: occupancy missing");
  if (d->feat_dim != 16 && d->feat_dim != 32) return set_error(SNISR_INVALID_ARG, "scene_create: feat_dim must be 16 or 32");
  if (d->feat_type != SNISR_F32 && d->feat_type != SNISR_F16) return set_error(SNISR_INVALID_ARG, "scene_create: bad feat_type");
  if (d->dir_freqs != 4) return set_error(SNISR_UNSUPPORTED, "scene_create: dir_freqs must be 4");
  if (!mlp_shape_supported(d->feat_dim, d->mlp_hidden, d->mlp_layers))
    return set_error(SNISR_UNSUPPORTED, "scene_create: supported MLPs are (F,H,L) in {(16,32,2),(32,64,3),(16,64,3),(32,32,2)}");
  if (!d->mlp_params) return set_error(SNISR_INVALID_ARG, "scene_create: mlp_params missing");
  if (d->num_voxels < 0 || d->num_vertices < 0) return set_error(SNISR_INVALID_ARG, "scene_create: negative counts");
  if (d->num_voxels > 0 && (!d->voxel_corners || !d->vertex_feat || !d->vertex_density))
    return set_error(SNISR_INVALID_ARG, "scene_create: voxel data missing");
  if (d->num_voxels >= (int64_t)0xFFFFFFF0) return set_error(SNISR_UNSUPPORTED, "scene_create: more than 2^32-16 voxels");
  if (d->num_triangles < 0 || (d->num_triangles > 0 && (!d->mesh_vertices || !d->mesh_faces)))
    return set_error(SNISR_INVALID_ARG, "scene_create: mesh data missing");
  if (!(d->step_vox > 0.0f) || !(d->early_stop >= 0.0f)) return set_error(SNISR_INVALID_ARG, "scene_create: bad marching parameters (step_vox > 0, early_stop >= 0)");
  // A march position inside a tile stays below 2 tile sizes, whose float
  // spacing is tile_size * 2^-22; steps of at least voxel / 1024 (>= tile_size
  // * 2^-20 for res <= 1024) always advance it.
  if (!(d->step_vox >= kMinStepVox) || !(d->step_vox <= 64.0f))
    return set_error(SNISR_INVALID_ARG, "scene_create: step_vox must lie in [1/1024, 64] voxels");
  if (d->max_pixels < 0 || d->max_samples_per_ray < 0) return set_error(SNISR_INVALID_ARG, "scene_create: negative workspace bound");
  return SNISR_OK;
}

snisr_status check_scene(snisr_scene* sc) {
  if (!sc) return set_error(SNISR_INVALID_ARG, "scene is null");
  return SNISR_OK;
}

snisr_status cam_to_dev(const snisr_camera* c, CamDev& out) {
  if (!c) return set_error(SNISR_INVALID_ARG, "camera is null");
  if (c->width <= 0 || c->height <= 0) return set_error(SNISR_INVALID_ARG, "camera size must be positive");
  out.W = c->width;
  out.H = c->height;
  out.cx = c->cx;
  out.cy = c->cy;
  out.inv_f = c->inv_focal;
  std::memcpy(out.c2w, c->c2w, sizeof(out.c2w));
  return SNISR_OK;
}

}  // namespace

namespace snisr {
snisr_status scene_train_ws(snisr_scene* sc, TrainWS** out, int* num_sms, int* msr, int64_t* nvox) {
  if (!sc) return set_error(SNISR_INVALID_ARG, "scene is null");
  if (!sc->train) sc->train = train_ws_new();
  *out = sc->train;
  *num_sms = sc->num_sms;
  *msr = sc->max_samples_per_ray;
  *nvox = sc->info.num_voxels;
  return SNISR_OK;
}
snisr_status scene_views(snisr_scene* sc, SceneDev* S, Workspace* ws, int* device) {
  if (!sc) return set_error(SNISR_INVALID_ARG, "scene is null");
  *S = sc->S;
  *ws = sc->ws;
  *device = sc->device;
  return SNISR_OK;
}
}  // namespace snisr

namespace {

// Chebyshev distance, in 4^3 blocks, from every block of a tile's nb^3 block
// grid to the nearest occupied block (0 for an occupied block), capped at
// kBlkDistCap + 1: the L-infinity distance transform taken one axis at a
// time (exact: max(|dx|, |dy|, |dz|) separates into three 1-D passes).
void block_distance(const uint32_t* bmask, int nb, uint8_t* out) {
  const int big = kBlkDistCap + 1;
  const size_t n = (size_t)nb * nb * nb;
  auto id = [nb](int x, int y, int z) { return ((size_t)x * nb + y) * nb + z; };
  std::vector<uint8_t> a(n), b(n);
  for (int x = 0; x < nb; ++x)  // z: distance to the nearest occupied block of the row
    for (int y = 0; y < nb; ++y) {
      int last = -1000000;
      for (int z = 0; z < nb; ++z) {
        const size_t k = id(x, y, z);
        if ((bmask[k >> 5] >> (k & 31)) & 1u) last = z;
        a[k] = (uint8_t)std::min(big, z - last);
      }
      int next = 1000000;
      for (int z = nb - 1; z >= 0; --z) {
        const size_t k = id(x, y, z);
        if ((bmask[k >> 5] >> (k & 31)) & 1u) next = z;
        a[k] = (uint8_t)std::min<int>(a[k], std::min(big, next - z));
      }
    }
  auto pass = [&](const std::vector<uint8_t>& src, std::vector<uint8_t>& dst, int axis) {
    for (int x = 0; x < nb; ++x)
      for (int y = 0; y < nb; ++y)
        for (int z = 0; z < nb; ++z) {
          int c[3] = {x, y, z};
          int m = src[id(x, y, z)];
          for (int dd = 1; dd < m; ++dd)
            for (int sgn = -1; sgn <= 1; sgn += 2) {
              int q[3] = {c[0], c[1], c[2]};
              q[axis] += sgn * dd;
              if (q[axis] < 0 || q[axis] >= nb) continue;
              m = std::min(m, std::max<int>(src[id(q[0], q[1], q[2])], dd));
            }
          dst[id(x, y, z)] = (uint8_t)m;
        }
  };
  pass(a, b, 1);
  std::vector<uint8_t> r(n);
  pass(b, r, 0);
  std::copy(r.begin(), r.end(), out);
}

}  // namespace

namespace {

snisr_status render_impl(snisr_scene* sc, const CamDev* cam, const float* origins, const float* dirs, int64_t n,
                         int32_t form, float* rgb, float* depth, float* opac, void* stream) {
  if (check_scene(sc) != SNISR_OK) return SNISR_INVALID_ARG;
  if (n < 0 || n > sc->ws.max_rays) return set_error(SNISR_INVALID_ARG, "render: ray count exceeds the workspace (max_pixels)");
  if (n == 0) return SNISR_OK;
  if (!rgb || !depth || !opac) return set_error(SNISR_INVALID_ARG, "render: output buffer is null");
  if (form != SNISR_FORM_PLAIN_FP32 && form != SNISR_FORM_TC) return set_error(SNISR_INVALID_ARG, "render: bad form");
  if (form == SNISR_FORM_TC && n > kMaxBatchedRays)
    return set_error(SNISR_INVALID_ARG, "render: the tensor-core form takes at most 2^24 rays per call");
  DeviceGuard guard(sc->device);
  cudaStream_t st = (cudaStream_t)stream;
  cudaEvent_t* ev = sc->profiling ? sc->ev : nullptr;
  if (ev) CUDA_TRY(cudaEventRecord(ev[5], st), "render: event");
  // camera frames march in 4 x 8 pixel warp tiles; the caller's rays in their order
  const RayOrder ord = cam ? frame_ray_order(cam->W, cam->H, n) : RayOrder{};
  CUDA_TRY(launch_raygen(sc->S, cam, origins, dirs, n, sc->ws, form == SNISR_FORM_TC, st, ord),
           "render: ray generation");
  if (ev) CUDA_TRY(cudaEventRecord(ev[6], st), "render: event");
  if (form == SNISR_FORM_PLAIN_FP32) {
    CUDA_TRY(launch_render_plain(sc->S, sc->ws, n, rgb, depth, opac, st, ord), "render: plain kernel");
    if (ev) CUDA_TRY(cudaEventRecord(ev[7], st), "render: event");
  } else {
    CUDA_TRY(launch_render_tc(sc->S, sc->ws, n, rgb, depth, opac, sc->num_sms, st, ev, ord), "render: batched kernels");
  }
  sc->last_form = form;
  return SNISR_OK;
}

}  // namespace

extern "C" {

const char* snisr_last_error_string(void) { return g_last_error.c_str(); }
const char* snisr_version(void) { return "snisr 0.1 (sm_103a)"; }
int32_t snisr_abi_version(void) { return SNISR_ABI_VERSION; }

snisr_status snisr_scene_create(const snisr_scene_desc* d, int32_t device, snisr_scene** out) {
  if (!out) return set_error(SNISR_INVALID_ARG, "scene_create: out is null");
  *out = nullptr;
  snisr_status st = validate_desc(d);
  if (st != SNISR_OK) return st;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return set_error(SNISR_CUDA_ERROR, "scene_create: no CUDA device");
  if (device < 0 || device >= ndev) return set_error(SNISR_INVALID_ARG, "scene_create: bad device ordinal");
  DeviceGuard guard(device);
  snisr_scene* sc = new (std::nothrow) snisr_scene();
  if (!sc) return set_error(SNISR_OOM, "scene_create: host allocation failed");
  sc->device = device;
  cudaDeviceGetAttribute(&sc->num_sms, cudaDevAttrMultiProcessorCount, device);
  if (sc->num_sms <= 0) sc->num_sms = 1;
  auto fail = [&](snisr_status s) { free_scene(sc); return s; };

  const int N = d->res, NT = d->num_tiles, F = d->feat_dim;
  const int GX = d->grid[0], GY = d->grid[1], GZ = d->grid[2];
  const int64_t words = (int64_t)N * N * N / 64;
  const int64_t ndense = (int64_t)GX * GY * GZ;
  sc->F = F; sc->H = d->mlp_hidden; sc->L = d->mlp_layers; sc->NT = NT;
  sc->in = F + 3 + 6 * d->dir_freqs;
  sc->P = (int)snisr_mlp_param_count(F, d->dir_freqs, d->mlp_hidden, d->mlp_layers);

  // tile index / centres
  std::vector<float> centers((size_t)NT * 3, 0.0f);
  std::vector<int> seen((size_t)NT, 0);
  for (int x = 0; x < GX; ++x)
    for (int y = 0; y < GY; ++y)
      for (int z = 0; z < GZ; ++z) {
        int32_t id = d->tile_index[((int64_t)x * GY + y) * GZ + z];
        if (id < -1 || id >= NT) return fail(set_error(SNISR_CORRUPT_SCENE, "scene_create: tile_index entry out of range"));
        if (id < 0) continue;
        if (seen[(size_t)id]++) return fail(set_error(SNISR_CORRUPT_SCENE, "scene_create: tile id used twice"));
        const int tcoord[3] = {x, y, z};
        for (int a = 0; a < 3; ++a) {
          // centre = min + (t + 0.5) * S, float arithmetic
          volatile float tf = (float)tcoord[a] + 0.5f;
          volatile float m = tf * d->tile_size;
          centers[(size_t)id * 3 + a] = d->scene_min[a] + m;
        }
      }
  for (int t = 0; t < NT; ++t)
    if (!seen[(size_t)t]) return fail(set_error(SNISR_CORRUPT_SCENE, "scene_create: tile id without a grid cell"));

  // occupancy words with global voxel bases, coarse 4^3 block masks (host only:
  // they give the block distances below)
  std::vector<OccWord> occ((size_t)(NT * words));
  const int nb = N / 4;
  const int64_t bwords = ((int64_t)nb * nb * nb + 31) / 32;
  std::vector<uint32_t> bmask((size_t)(NT * bwords), 0u);
  uint64_t base = 0;
  for (int t = 0; t < NT; ++t)
    for (int64_t w = 0; w < words; ++w) {
      uint64_t bits = d->occupancy[(size_t)(t * words + w)];
      OccWord& o = occ[(size_t)(t * words + w)];
      o.bits = bits;
      o.base = (uint32_t)base;
      o.pad = 0;
      base += (uint64_t)__builtin_popcountll(bits);
      while (bits) {
        int b = __builtin_ctzll(bits);
        bits &= bits - 1;
        int64_t vid = w * 64 + b;
        int x = (int)(vid / ((int64_t)N * N)), y = (int)((vid / N) % N), z = (int)(vid % N);
        int64_t bid = ((int64_t)(x >> 2) * nb + (y >> 2)) * nb + (z >> 2);
        bmask[(size_t)(t * bwords + (bid >> 5))] |= 1u << (bid & 31);
      }
    }
  if ((int64_t)base != d->num_voxels) return fail(set_error(SNISR_CORRUPT_SCENE, "scene_create: num_voxels does not match the occupancy popcount"));
  for (int64_t i = 0; i < d->num_voxels * 8; ++i)
    if (d->voxel_corners[i] < 0 || d->voxel_corners[i] >= d->num_vertices)
      return fail(set_error(SNISR_CORRUPT_SCENE, "scene_create: voxel corner vertex id out of range"));

  SceneDev& S = sc->S;
  S.gx = GX; S.gy = GY; S.gz = GZ;
  for (int a = 0; a < 3; ++a) S.smin[a] = d->scene_min[a];
  S.tile_size = d->tile_size;
  S.voxel = d->tile_size / (float)N;
  S.inv_voxel = (float)N / d->tile_size;
  S.step_len = d->step_vox * S.voxel;
  S.early_stop = d->early_stop;
  S.start_offset = d->start_offset_vox * S.voxel;
  S.res = N;
  S.words_per_tile = (int)words;
  S.num_tiles = NT;
  S.feat_dim = F;
  S.dir_freqs = d->dir_freqs;
  S.mlp_in = sc->in;
  S.mlp_hidden = d->mlp_hidden;
  S.mlp_layers = d->mlp_layers;
  S.params_per_tile = sc->P;

  // per-tile block distances (jumps of the training march over empty space)
  std::vector<uint8_t> bdist((size_t)NT * nb * nb * nb);
  for (int t = 0; t < NT; ++t)
    block_distance(bmask.data() + (size_t)t * bwords, nb, bdist.data() + (size_t)t * nb * nb * nb);

  int32_t* d_tindex = nullptr; float* d_cent = nullptr; OccWord* d_occ = nullptr; uint8_t* d_bdist = nullptr;
  if ((st = upload(sc, &d_tindex, d->tile_index, (size_t)ndense * 4, "tile index")) != SNISR_OK) return fail(st);
  if ((st = upload(sc, &d_cent, centers.data(), centers.size() * 4, "tile centres")) != SNISR_OK) return fail(st);
  if ((st = upload(sc, &d_occ, occ.data(), occ.size() * sizeof(OccWord), "occupancy")) != SNISR_OK) return fail(st);
  if ((st = upload(sc, &d_bdist, bdist.data(), bdist.size(), "block distances")) != SNISR_OK) return fail(st);
  S.tile_index = d_tindex; S.tile_center = d_cent; S.occ = d_occ; S.blk_dist = d_bdist;

  // per-voxel corner caches, expanded on the device
  const int64_t nvox = d->num_voxels, nv = d->num_vertices;
  float* d_dens = nullptr; float4* d_f32 = nullptr; uint4* d_f16 = nullptr;
  if ((st = dev_alloc(sc, &d_dens, (size_t)nvox * 8 * 4, "density cache")) != SNISR_OK) return fail(st);
  if ((st = dev_alloc(sc, &d_f32, (size_t)nvox * F * 8 * 4, "FP32 feature cache")) != SNISR_OK) return fail(st);
  if ((st = dev_alloc(sc, &d_f16, (size_t)nvox * F * 8 * 2, "FP16 feature cache")) != SNISR_OK) return fail(st);
  S.dens = d_dens; S.feat32 = d_f32; S.feat16 = d_f16;
  if (nvox > 0) {
    const int esz = d->feat_type == SNISR_F16 ? 2 : 4;
    void *t_corner = nullptr, *t_feat = nullptr, *t_dens = nullptr;
    cudaError_t e = cudaMalloc(&t_corner, (size_t)nvox * 8 * 4);
    if (e == cudaSuccess) e = cudaMalloc(&t_feat, (size_t)nv * F * esz);
    if (e == cudaSuccess) e = cudaMalloc(&t_dens, (size_t)nv * esz);
    if (e == cudaSuccess) e = cudaMemcpy(t_corner, d->voxel_corners, (size_t)nvox * 8 * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(t_feat, d->vertex_feat, (size_t)nv * F * esz, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(t_dens, d->vertex_density, (size_t)nv * esz, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = launch_expand((const int32_t*)t_corner, t_feat, t_dens, esz == 2, F, nvox, d_dens, d_f32, d_f16, 0);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    cudaFree(t_corner); cudaFree(t_feat); cudaFree(t_dens);
    if (e != cudaSuccess) return fail(set_error(e == cudaErrorMemoryAllocation ? SNISR_OOM : SNISR_CUDA_ERROR, std::string("scene_create: cache expansion: ") + cudaGetErrorString(e)));
  }
  // corner ids stay resident for training (gradient scatter to vertices)
  int32_t* d_corners = nullptr;
  if ((st = upload(sc, &d_corners, d->voxel_corners, (size_t)nvox * 8 * 4, "voxel corners")) != SNISR_OK) return fail(st);
  sc->info.num_vertices = nv;
  // MLPs
  if ((st = upload_mlp(sc, d->mlp_params, true)) != SNISR_OK) return fail(st);

  // proxy mesh BVH
  if (d->num_triangles > 0) {
    for (int64_t i = 0; i < d->num_triangles * 3; ++i)
      if (d->mesh_faces[i] < 0 || d->mesh_faces[i] >= d->num_mesh_vertices)
        return fail(set_error(SNISR_CORRUPT_SCENE, "scene_create: mesh face index out of range"));
    std::vector<BvhNode> nodes;
    std::vector<int32_t> order;
    build_bvh(d->mesh_vertices, d->mesh_faces, d->num_triangles, 4, nodes, order);
    // the traversal packs a node's child index / first triangle and count
    // into one word: first < 2^27, count < 32
    for (const BvhNode& nd : nodes)
      if (nd.first < 0 || nd.first >= (1 << 27) || nd.count < 0 || nd.count > 31)
        return fail(set_error(SNISR_INVALID_ARG, "scene_create: proxy mesh too large for the BVH node format"));
    std::vector<float> tri((size_t)d->num_triangles * 12);
    for (int64_t s = 0; s < d->num_triangles; ++s) {
      int32_t t = order[(size_t)s];
      for (int k = 0; k < 3; ++k) {
        const float* v = d->mesh_vertices + 3 * (int64_t)d->mesh_faces[3 * (int64_t)t + k];
        for (int a = 0; a < 3; ++a) tri[(size_t)(s * 12 + k * 4 + a)] = v[a];
        tri[(size_t)(s * 12 + k * 4 + 3)] = 0.0f;
      }
    }
    BvhNodeDev* d_bvh = nullptr; float4* d_tri = nullptr; int32_t* d_tid = nullptr;
    if ((st = upload(sc, &d_bvh, nodes.data(), nodes.size() * sizeof(BvhNode), "bvh")) != SNISR_OK) return fail(st);
    if ((st = upload(sc, &d_tri, tri.data(), tri.size() * 4, "triangles")) != SNISR_OK) return fail(st);
    if ((st = upload(sc, &d_tid, order.data(), order.size() * 4, "triangle ids")) != SNISR_OK) return fail(st);
    S.bvh = d_bvh; S.tri = d_tri; S.tri_id = d_tid; S.has_mesh = 1;
    sc->info.bvh_nodes = (int64_t)nodes.size();
  }
  uint32_t* d_err = nullptr;
  if ((st = dev_alloc(sc, &d_err, 16, "error word")) != SNISR_OK) return fail(st);
  CUDA_TRY(cudaMemset(d_err, 0, 16), "error word");
  S.err = d_err;
  if (cudaMallocHost(&sc->err_host, 16) != cudaSuccess) return fail(set_error(SNISR_OOM, "scene_create: pinned error word"));

  // workspace for the largest frame
  Workspace& ws = sc->ws;
  const int64_t maxr = std::max<int64_t>(d->max_pixels, 1);
  ws.max_rays = maxr;
  if ((st = dev_alloc(sc, &ws.ray_o, (size_t)maxr * 16, "ray origins")) != SNISR_OK) return fail(st);
  if ((st = dev_alloc(sc, &ws.ray_d, (size_t)maxr * 16, "ray directions")) != SNISR_OK) return fail(st);
  if ((st = dev_alloc(sc, &ws.enc, (size_t)maxr * 64, "ray encodings")) != SNISR_OK) return fail(st);
  int64_t cap = maxr * (int64_t)std::max(d->max_samples_per_ray, 1);
  if (cap > (int64_t)0xFFFFFF00) cap = 0xFFFFFF00;
  ws.cap = (uint32_t)cap;
  if ((st = dev_alloc(sc, &ws.recs, (size_t)cap * sizeof(SampleRec), "sample buffer")) != SNISR_OK) return fail(st);
  if ((st = dev_alloc(sc, &ws.sorted, (size_t)cap * sizeof(SampleRec), "sorted samples")) != SNISR_OK) return fail(st);
  if ((st = dev_alloc(sc, &ws.blk_count, (size_t)(cap / 256 + 2) * 4, "block counts")) != SNISR_OK) return fail(st);
  ws.ctrl_words = std::max(CTRL_HEADER + 4 * NT + 2, train_ctrl_words(NT));
  if ((st = dev_alloc(sc, &ws.ctrl, (size_t)ws.ctrl_words * 4, "control words")) != SNISR_OK) return fail(st);

  snisr_scene_info& I = sc->info;
  I.num_voxels = nvox;
  I.num_triangles = d->num_triangles;
  I.num_tiles = NT;
  I.res = N;
  I.feat_dim = F;
  I.mlp_in = sc->in;
  I.mlp_hidden = sc->H;
  I.mlp_layers = sc->L;
  I.params_per_tile = sc->P;
  I.sample_capacity = cap;
  sc->corners = d_corners;
  sc->S.corners = d_corners;
  sc->max_samples_per_ray = std::max(d->max_samples_per_ray, 1);
  *out = sc;
  return SNISR_OK;
}

snisr_status snisr_scene_destroy(snisr_scene* sc) {
  free_scene(sc);
  return SNISR_OK;
}

snisr_status snisr_scene_get_info(const snisr_scene* sc, snisr_scene_info* info) {
  if (!sc || !info) return set_error(SNISR_INVALID_ARG, "scene_get_info: null argument");
  *info = sc->info;
  return SNISR_OK;
}

snisr_status snisr_scene_check(snisr_scene* sc, void* stream) {
  if (check_scene(sc) != SNISR_OK) return SNISR_INVALID_ARG;
  DeviceGuard guard(sc->device);
  cudaStream_t st = (cudaStream_t)stream;
  CUDA_TRY(cudaMemcpyAsync(sc->err_host, sc->S.err, 4, cudaMemcpyDeviceToHost, st), "scene_check");
  CUDA_TRY(cudaStreamSynchronize(st), "scene_check");
  uint32_t e = sc->err_host[0];
  CUDA_TRY(cudaMemsetAsync(sc->S.err, 0, 4, st), "scene_check");
  CUDA_TRY(cudaStreamSynchronize(st), "scene_check");
  if (e & ERR_DRAIN)
    return set_error(SNISR_DEVICE_TIMEOUT,
                     "a bounded device wait ran out and the tensor-core work in flight did not finish: the CUDA "
                     "context is unusable (destroy the scene and exit the process)");
  if (e & ERR_TIMEOUT) return set_error(SNISR_DEVICE_TIMEOUT, "a bounded device wait ran out");
  if (e & ERR_OVERFLOW) return set_error(SNISR_OVERFLOW, "sample workspace or traversal stack overflowed; raise max_samples_per_ray");
  if (e) return set_error(SNISR_CUDA_ERROR, "device error word set");
  return SNISR_OK;
}

snisr_status snisr_scene_set_mlp(snisr_scene* sc, const float* params_dev, void* stream) {
  if (check_scene(sc) != SNISR_OK || !params_dev) return set_error(SNISR_INVALID_ARG, "scene_set_mlp: null argument");
  DeviceGuard guard(sc->device);
  std::vector<float> host((size_t)sc->NT * sc->P);
  cudaStream_t st = (cudaStream_t)stream;
  CUDA_TRY(cudaMemcpyAsync(host.data(), params_dev, host.size() * 4, cudaMemcpyDeviceToHost, st), "scene_set_mlp");
  CUDA_TRY(cudaStreamSynchronize(st), "scene_set_mlp");
  return upload_mlp(sc, host.data(), false);
}

snisr_status snisr_render_rays(snisr_scene* sc, const float* origins, const float* dirs, int64_t n, int32_t form,
                               float* rgb, float* depth, float* opac, void* stream) {
  if (!dirs || !origins) return set_error(SNISR_INVALID_ARG, "render_rays: origins/directions missing");
  return render_impl(sc, nullptr, origins, dirs, n, form, rgb, depth, opac, stream);
}

snisr_status snisr_render(snisr_scene* sc, const snisr_camera* cam, int32_t form, float* rgb, float* depth,
                          float* opac, void* stream) {
  CamDev c;
  snisr_status st = cam_to_dev(cam, c);
  if (st != SNISR_OK) return st;
  return render_impl(sc, &c, nullptr, nullptr, (int64_t)c.W * c.H, form, rgb, depth, opac, stream);
}

snisr_status snisr_render_host(snisr_scene* sc, const snisr_camera* cam, int32_t form, float* rgb_h, float* depth_h,
                               float* opac_h, void* stream) {
  if (check_scene(sc) != SNISR_OK) return SNISR_INVALID_ARG;
  if (!cam || !rgb_h || !depth_h || !opac_h) return set_error(SNISR_INVALID_ARG, "render_host: null argument");
  const int64_t n = (int64_t)cam->width * cam->height;
  if (n <= 0 || n > sc->ws.max_rays) return set_error(SNISR_INVALID_ARG, "render_host: frame exceeds the workspace");
  DeviceGuard guard(sc->device);
  cudaStream_t st = (cudaStream_t)stream;
  if (!sc->out_bufs) {
    void* p = nullptr;
    CUDA_TRY(cudaMalloc(&p, (size_t)sc->ws.max_rays * 5 * 4), "render_host: output staging");
    sc->out_bufs = static_cast<float*>(p);
    sc->allocs.push_back(p);
    sc->info.device_bytes += (int64_t)sc->ws.max_rays * 20;
  }
  float* drgb = sc->out_bufs;
  float* ddep = drgb + 3 * sc->ws.max_rays;
  float* dop = ddep + sc->ws.max_rays;
  snisr_status s = snisr_render(sc, cam, form, drgb, ddep, dop, stream);
  if (s != SNISR_OK) return s;
  CUDA_TRY(cudaMemcpyAsync(rgb_h, drgb, (size_t)n * 12, cudaMemcpyDeviceToHost, st), "render_host: copy rgb");
  CUDA_TRY(cudaMemcpyAsync(depth_h, ddep, (size_t)n * 4, cudaMemcpyDeviceToHost, st), "render_host: copy depth");
  CUDA_TRY(cudaMemcpyAsync(opac_h, dop, (size_t)n * 4, cudaMemcpyDeviceToHost, st), "render_host: copy opacity");
  CUDA_TRY(cudaStreamSynchronize(st), "render_host: synchronise");
  return SNISR_OK;
}

snisr_status snisr_render_host_async(snisr_scene* sc, const snisr_camera* cam, int32_t form, float* rgb_h,
                                     float* depth_h, float* opac_h, void* stream) {
  if (check_scene(sc) != SNISR_OK) return SNISR_INVALID_ARG;
  if (!cam || !rgb_h || !depth_h || !opac_h) return set_error(SNISR_INVALID_ARG, "render_host_async: null argument");
  const int64_t n = (int64_t)cam->width * cam->height;
  if (n <= 0 || n > sc->ws.max_rays)
    return set_error(SNISR_INVALID_ARG, "render_host_async: frame exceeds the workspace");
  DeviceGuard guard(sc->device);
  cudaStream_t st = (cudaStream_t)stream;
  const int64_t cap = sc->ws.max_rays;
  if (!sc->async_bufs) {
    // Build the copy stream, the events and the staging into locals and
    // publish them together, so that a failure part-way leaves the scene as
    // it was (the next call sets everything up again).
    cudaStream_t cs = nullptr;
    cudaEvent_t rd[2] = {}, cd[2] = {};
    void* p = nullptr;
    auto undo = [&]() {
      for (int k = 0; k < 2; ++k) {
        if (rd[k]) cudaEventDestroy(rd[k]);
        if (cd[k]) cudaEventDestroy(cd[k]);
      }
      if (cs) cudaStreamDestroy(cs);
      if (p) cudaFree(p);
    };
    cudaError_t e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
    for (int k = 0; k < 2 && e == cudaSuccess; ++k) {
      e = cudaEventCreateWithFlags(&rd[k], cudaEventDisableTiming);
      if (e == cudaSuccess) e = cudaEventCreateWithFlags(&cd[k], cudaEventDisableTiming);
      if (e == cudaSuccess) e = cudaEventRecord(cd[k], cs);
    }
    if (e == cudaSuccess) e = cudaMalloc(&p, (size_t)cap * 5 * 4 * 2);
    if (e != cudaSuccess) {
      undo();
      return set_error(e == cudaErrorMemoryAllocation ? SNISR_OOM : SNISR_CUDA_ERROR,
                       std::string("render_host_async: set-up: ") + cudaGetErrorString(e));
    }
    sc->copy_stream = cs;
    for (int k = 0; k < 2; ++k) {
      sc->render_done[k] = rd[k];
      sc->copy_done[k] = cd[k];
    }
    sc->allocs.push_back(p);
    sc->info.device_bytes += cap * 40;
    sc->async_bufs = static_cast<float*>(p);
  }
  const int k = sc->async_slot;
  sc->async_slot ^= 1;
  float* drgb = sc->async_bufs + (size_t)k * cap * 5;
  float* ddep = drgb + 3 * cap;
  float* dop = ddep + cap;
  // the slot's previous copy must be done before this frame overwrites it
  CUDA_TRY(cudaStreamWaitEvent(st, sc->copy_done[k], 0), "render_host_async: order");
  snisr_status s = snisr_render(sc, cam, form, drgb, ddep, dop, stream);
  if (s != SNISR_OK) return s;
  CUDA_TRY(cudaEventRecord(sc->render_done[k], st), "render_host_async: order");
  CUDA_TRY(cudaStreamWaitEvent(sc->copy_stream, sc->render_done[k], 0), "render_host_async: order");
  CUDA_TRY(cudaMemcpyAsync(rgb_h, drgb, (size_t)n * 12, cudaMemcpyDeviceToHost, sc->copy_stream),
           "render_host_async: copy rgb");
  CUDA_TRY(cudaMemcpyAsync(depth_h, ddep, (size_t)n * 4, cudaMemcpyDeviceToHost, sc->copy_stream),
           "render_host_async: copy depth");
  CUDA_TRY(cudaMemcpyAsync(opac_h, dop, (size_t)n * 4, cudaMemcpyDeviceToHost, sc->copy_stream),
           "render_host_async: copy opacity");
  CUDA_TRY(cudaEventRecord(sc->copy_done[k], sc->copy_stream), "render_host_async: order");
  return SNISR_OK;
}

snisr_status snisr_render_host_wait(snisr_scene* sc) {
  if (check_scene(sc) != SNISR_OK) return SNISR_INVALID_ARG;
  if (!sc->copy_stream) return SNISR_OK;
  DeviceGuard guard(sc->device);
  CUDA_TRY(cudaStreamSynchronize(sc->copy_stream), "render_host_wait");
  return SNISR_OK;
}

snisr_status snisr_camera_rays(const snisr_camera* cam, float* dirs_dev, void* stream);

snisr_status snisr_proxy_hit(snisr_scene* sc, const float* origins, const float* dirs, int64_t n, float* t,
                             int32_t* tri, void* stream) {
  if (check_scene(sc) != SNISR_OK) return SNISR_INVALID_ARG;
  if (n < 0 || (n > 0 && (!origins || !dirs || !t || !tri))) return set_error(SNISR_INVALID_ARG, "proxy_hit: bad argument");
  if (n == 0) return SNISR_OK;
  DeviceGuard guard(sc->device);
  CUDA_TRY(launch_proxy(sc->S, origins, dirs, n, t, tri, (cudaStream_t)stream), "proxy_hit");
  return SNISR_OK;
}

snisr_status snisr_scene_double_hits(snisr_scene* sc, const float* rays_o, const float* rays_d,
                                    const int32_t* visited, int64_t n, int32_t K, float* double_hits, void* stream) {
  if (check_scene(sc) != SNISR_OK) return SNISR_INVALID_ARG;
  if (n < 0 || K <= 0) return set_error(SNISR_INVALID_ARG, "double_hits: bad size");
  if (n == 0) return SNISR_OK;
  if (!rays_o || !rays_d || !visited || !double_hits) return set_error(SNISR_INVALID_ARG, "double_hits: null argument");
  if (!sc->S.has_mesh) return set_error(SNISR_INVALID_ARG, "double_hits: the scene has no proxy mesh");
  DeviceGuard guard(sc->device);
  CUDA_TRY(launch_double_hits(sc->S, rays_o, rays_d, visited, n, K, double_hits, (cudaStream_t)stream), "double_hits");
  return SNISR_OK;
}

snisr_status snisr_trace_voxels(snisr_scene* sc, const float* origins, const float* dirs, int64_t n, int32_t K,
                                int32_t* visited, int32_t* count, void* stream) {
  if (check_scene(sc) != SNISR_OK) return SNISR_INVALID_ARG;
  if (n < 0 || K < 0 || n > sc->ws.max_rays) return set_error(SNISR_INVALID_ARG, "trace_voxels: bad size");
  if (n == 0) return SNISR_OK;
  if (!origins || !dirs || !count || (K > 0 && !visited)) return set_error(SNISR_INVALID_ARG, "trace_voxels: null argument");
  DeviceGuard guard(sc->device);
  cudaStream_t st = (cudaStream_t)stream;
  CUDA_TRY(launch_raygen(sc->S, nullptr, origins, dirs, n, sc->ws, false, st), "trace_voxels: ray setup");
  CUDA_TRY(launch_trace(sc->S, sc->ws, n, K, visited, count, st), "trace_voxels");
  return SNISR_OK;
}

snisr_status snisr_scene_set_profiling(snisr_scene* sc, int32_t enable) {
  if (check_scene(sc) != SNISR_OK) return SNISR_INVALID_ARG;
  DeviceGuard guard(sc->device);
  if (enable && !sc->ev[0])
    for (cudaEvent_t& e : sc->ev) CUDA_TRY(cudaEventCreate(&e), "set_profiling: event");
  sc->profiling = enable != 0;
  return SNISR_OK;
}

snisr_status snisr_scene_stage_times(snisr_scene* sc, float* ms, int32_t cap, int32_t* n_out) {
  if (check_scene(sc) != SNISR_OK || !ms || !n_out) return set_error(SNISR_INVALID_ARG, "stage_times: null argument");
  if (!sc->profiling || sc->last_form < 0) return set_error(SNISR_INVALID_ARG, "stage_times: profiling is off or nothing rendered");
  DeviceGuard guard(sc->device);
  float v[6] = {0, 0, 0, 0, 0, 0};
  int n = 0;
  auto el = [&](int a, int b) -> snisr_status {
    float t = 0;
    CUDA_TRY(cudaEventElapsedTime(&t, sc->ev[a], sc->ev[b]), "stage_times");
    v[n++] = t;
    return SNISR_OK;
  };
  if (sc->last_form == SNISR_FORM_TC) {
    CUDA_TRY(cudaEventSynchronize(sc->ev[4]), "stage_times");
    snisr_status s;
    if ((s = el(5, 6)) || (s = el(0, 1)) || (s = el(1, 2)) || (s = el(2, 3)) || (s = el(3, 4)) || (s = el(5, 4))) return s;
  } else {
    CUDA_TRY(cudaEventSynchronize(sc->ev[7]), "stage_times");
    snisr_status s;
    if ((s = el(5, 6)) || (s = el(6, 7)) || (s = el(5, 7))) return s;
  }
  for (int i = 0; i < n && i < cap; ++i) ms[i] = v[i];
  *n_out = n;
  return SNISR_OK;
}

snisr_status snisr_scene_frame_stats(snisr_scene* sc, int64_t* out, void* stream) {
  if (check_scene(sc) != SNISR_OK || !out) return set_error(SNISR_INVALID_ARG, "frame_stats: null argument");
  DeviceGuard guard(sc->device);
  int32_t w[6];
  cudaStream_t st = (cudaStream_t)stream;
  CUDA_TRY(cudaMemcpyAsync(w, sc->ws.ctrl, sizeof(w), cudaMemcpyDeviceToHost, st), "frame_stats");
  CUDA_TRY(cudaStreamSynchronize(st), "frame_stats");
  uint64_t steps;
  std::memcpy(&steps, w + CTRL_STEPS, 8);
  out[0] = w[CTRL_SAMPLES];
  out[1] = (int64_t)steps;
  out[2] = w[CTRL_RESERVED];
  out[3] = w[CTRL_CHUNKS];
  return SNISR_OK;
}

snisr_status snisr_scene_frame_footprint(snisr_scene* sc, int64_t* out, void* stream) {
  if (check_scene(sc) != SNISR_OK || !out) return set_error(SNISR_INVALID_ARG, "frame_footprint: null argument");
  if (sc->last_form != SNISR_FORM_TC) return set_error(SNISR_INVALID_ARG, "frame_footprint: no tensor-core frame rendered");
  DeviceGuard guard(sc->device);
  const int64_t nvox = sc->info.num_voxels, nvert = sc->info.num_vertices;
  const int64_t vw = (nvox + 31) / 32, tw = (nvert + 31) / 32;
  if (!sc->fp_bits) {
    snisr_status s = dev_alloc(sc, &sc->fp_bits, (size_t)(vw + tw + 6) * 4, "frame_footprint");
    if (s != SNISR_OK) return s;
  }
  cudaStream_t st = (cudaStream_t)stream;
  unsigned long long* counts = reinterpret_cast<unsigned long long*>(sc->fp_bits + ((vw + tw + 1) & ~int64_t(1)));
  CUDA_TRY(launch_footprint(sc->S, sc->ws, nvox, nvert, sc->fp_bits, sc->fp_bits + vw, counts, sc->num_sms, st),
           "frame_footprint");
  unsigned long long h[2];
  CUDA_TRY(cudaMemcpyAsync(h, counts, sizeof(h), cudaMemcpyDeviceToHost, st), "frame_footprint");
  CUDA_TRY(cudaStreamSynchronize(st), "frame_footprint");
  out[0] = (int64_t)h[0];
  out[1] = (int64_t)h[1];
  return SNISR_OK;
}

snisr_status snisr_diag_block_distance(const uint32_t* mask, int32_t nb, uint8_t* out) {
  if (!mask || !out || nb <= 0 || nb > 1024) return set_error(SNISR_INVALID_ARG, "diag_block_distance: bad argument");
  block_distance(mask, nb, out);
  return SNISR_OK;
}

snisr_status snisr_scene_get_tuning(const snisr_scene* sc, snisr_tuning* out) {
  if (check_scene(const_cast<snisr_scene*>(sc)) != SNISR_OK || !out)
    return set_error(SNISR_INVALID_ARG, "get_tuning: null argument");
  const Tuning& t = sc->ws.tune;
  *out = snisr_tuning{t.traverse_threads, t.scatter_blocks_per_sm, t.mlp_ctas_per_sm, t.train_march_threads,
                      t.train_fwd_warps};
  return SNISR_OK;
}

snisr_status snisr_scene_set_tuning(snisr_scene* sc, const snisr_tuning* t) {
  if (check_scene(sc) != SNISR_OK || !t) return set_error(SNISR_INVALID_ARG, "set_tuning: null argument");
  auto warps_ok = [](int v) { return v >= 32 && v <= 256 && v % 32 == 0; };
  if (!warps_ok(t->traverse_threads) || !warps_ok(t->train_march_threads) || t->scatter_blocks_per_sm < 1 ||
      t->scatter_blocks_per_sm > 64 || t->mlp_ctas_per_sm < 0 || t->mlp_ctas_per_sm > 8 ||
      (t->train_fwd_warps != 4 && t->train_fwd_warps != 8))
    return set_error(SNISR_INVALID_ARG, "set_tuning: value out of range");
  sc->ws.tune = Tuning{t->traverse_threads, t->scatter_blocks_per_sm, t->mlp_ctas_per_sm, t->train_march_threads,
                       t->train_fwd_warps};
  return SNISR_OK;
}

}  // extern "C"

namespace {

// coordinate descent over the knobs: `eval` times the current sc->ws.tune
template <class Eval>
snisr_status tune_descent(snisr_scene* sc, const std::vector<std::pair<int Tuning::*, std::vector<int>>>& knobs,
                          Eval&& eval, float* best_ms) {
  float best = 0.f;
  snisr_status s = eval(&best);
  if (s != SNISR_OK) return s;
  for (const auto& kv : knobs) {
    Tuning keep = sc->ws.tune;
    for (int v : kv.second) {
      if (v == keep.*(kv.first)) continue;
      sc->ws.tune = keep;
      sc->ws.tune.*(kv.first) = v;
      float ms = 0.f;
      if ((s = eval(&ms)) != SNISR_OK) {
        sc->ws.tune = keep;
        return s;
      }
      if (ms < best) {
        best = ms;
        keep = sc->ws.tune;
      }
    }
    sc->ws.tune = keep;
  }
  *best_ms = best;
  return SNISR_OK;
}

struct DevBuf {
  void* p = nullptr;
  ~DevBuf() { if (p) cudaFree(p); }
};

}  // namespace

extern "C" {

snisr_status snisr_scene_autotune_render(snisr_scene* sc, const snisr_camera* cam, int32_t reps, void* stream,
                                         snisr_tuning* out, float* best_ms) {
  if (check_scene(sc) != SNISR_OK || !cam || !out || !best_ms || reps < 1)
    return set_error(SNISR_INVALID_ARG, "autotune_render: bad argument");
  const int64_t n = (int64_t)cam->width * cam->height;
  if (n <= 0 || n > sc->ws.max_rays) return set_error(SNISR_INVALID_ARG, "autotune_render: camera exceeds max_pixels");
  DeviceGuard guard(sc->device);
  cudaStream_t st = (cudaStream_t)stream;
  DevBuf buf;
  CUDA_TRY(cudaMalloc(&buf.p, (size_t)n * 5 * sizeof(float)), "autotune_render: buffers");
  float* rgb = static_cast<float*>(buf.p);
  cudaEvent_t e0, e1;
  CUDA_TRY(cudaEventCreate(&e0), "autotune_render: event");
  CUDA_TRY(cudaEventCreate(&e1), "autotune_render: event");
  const bool prof = sc->profiling;
  sc->profiling = false;
  auto eval = [&](float* ms) -> snisr_status {
    snisr_status s = snisr_render(sc, cam, SNISR_FORM_TC, rgb, rgb + 3 * n, rgb + 4 * n, stream);
    if (s != SNISR_OK) return s;
    CUDA_TRY(cudaEventRecord(e0, st), "autotune_render");
    for (int r = 0; r < reps; ++r)
      if ((s = snisr_render(sc, cam, SNISR_FORM_TC, rgb, rgb + 3 * n, rgb + 4 * n, stream)) != SNISR_OK) return s;
    CUDA_TRY(cudaEventRecord(e1, st), "autotune_render");
    CUDA_TRY(cudaEventSynchronize(e1), "autotune_render");
    float t = 0.f;
    CUDA_TRY(cudaEventElapsedTime(&t, e0, e1), "autotune_render");
    *ms = t / (float)reps;
    return snisr_scene_check(sc, stream);
  };
  const std::vector<std::pair<int Tuning::*, std::vector<int>>> knobs = {
      {&Tuning::traverse_threads, {64, 128, 256}},
      {&Tuning::scatter_blocks_per_sm, {8, 16, 32}},
      {&Tuning::mlp_ctas_per_sm, {2, 3, 0}},
  };
  snisr_status s = tune_descent(sc, knobs, eval, best_ms);
  sc->profiling = prof;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (s != SNISR_OK) return s;
  return snisr_scene_get_tuning(sc, out);
}

snisr_status snisr_scene_autotune_train(snisr_scene* sc, const float* vfeat, const float* vdens, const float* mlp,
                                        const float* origins, const float* dirs, const int32_t* ray_tile, int64_t n,
                                        int32_t reps, void* stream, snisr_tuning* out, float* best_ms) {
  if (check_scene(sc) != SNISR_OK || !vfeat || !vdens || !mlp || !origins || !dirs || !ray_tile || n <= 0 ||
      reps < 1 || !out || !best_ms)
    return set_error(SNISR_INVALID_ARG, "autotune_train: bad argument");
  DeviceGuard guard(sc->device);
  cudaStream_t st = (cudaStream_t)stream;
  const int64_t nv = sc->info.num_vertices, F = sc->F, NT = sc->NT, P = sc->P;
  const size_t grads = (size_t)(nv * F + nv + NT * P), bytes = (grads + (size_t)n * 6) * sizeof(float);
  DevBuf buf;
  CUDA_TRY(cudaMalloc(&buf.p, bytes), "autotune_train: buffers");
  float* gF = static_cast<float*>(buf.p);
  float* gG = gF + nv * F;
  float* gW = gG + nv;
  float* rgb = gW + NT * P;
  float* grad = rgb + 3 * n;
  std::vector<float> ones((size_t)n * 3, 1.0f);
  CUDA_TRY(cudaMemcpyAsync(grad, ones.data(), ones.size() * sizeof(float), cudaMemcpyHostToDevice, st),
           "autotune_train: gradient");
  cudaEvent_t e0, e1;
  CUDA_TRY(cudaEventCreate(&e0), "autotune_train: event");
  CUDA_TRY(cudaEventCreate(&e1), "autotune_train: event");
  auto step = [&]() -> snisr_status {
    uint64_t gen = 0;
    snisr_status s =
        snisr_train_forward(sc, vfeat, vdens, mlp, origins, dirs, ray_tile, n, SNISR_FORM_TC, rgb, &gen, stream);
    if (s != SNISR_OK) return s;
    return snisr_train_backward(sc, vfeat, vdens, mlp, origins, dirs, ray_tile, n, SNISR_FORM_TC, gen, rgb, grad, gF,
                                gG, gW, stream);
  };
  auto eval = [&](float* ms) -> snisr_status {
    snisr_status s = step();
    if (s != SNISR_OK) return s;
    CUDA_TRY(cudaEventRecord(e0, st), "autotune_train");
    for (int r = 0; r < reps; ++r)
      if ((s = step()) != SNISR_OK) return s;
    CUDA_TRY(cudaEventRecord(e1, st), "autotune_train");
    CUDA_TRY(cudaEventSynchronize(e1), "autotune_train");
    float t = 0.f;
    CUDA_TRY(cudaEventElapsedTime(&t, e0, e1), "autotune_train");
    *ms = t / (float)reps;
    return snisr_scene_check(sc, stream);
  };
  const std::vector<std::pair<int Tuning::*, std::vector<int>>> knobs = {
      {&Tuning::train_march_threads, {64, 128, 256}},
      {&Tuning::train_fwd_warps, {4, 8}},
  };
  snisr_status s = tune_descent(sc, knobs, eval, best_ms);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (s != SNISR_OK) return s;
  return snisr_scene_get_tuning(sc, out);
}

snisr_status snisr_diag_wait_timeout(int64_t limit_ns, int64_t* waited_ns, void* stream) {
  if (limit_ns <= 0 || limit_ns > 10000000000ll || !waited_ns)
    return set_error(SNISR_INVALID_ARG, "diag_wait_timeout: bad argument (limit in (0, 10 s])");
  bool ran_out = false;
  CUDA_TRY(launch_diag_wait(limit_ns, waited_ns, &ran_out, (cudaStream_t)stream), "diag_wait_timeout");
  if (ran_out) return set_error(SNISR_DEVICE_TIMEOUT, "diag_wait_timeout: the wait ran out (expected)");
  return SNISR_OK;
}

snisr_status snisr_diag_mma(const uint16_t* A_dev, const uint16_t* B_dev, float* D_dev, int32_t N, int32_t bf16,
                            int32_t mode, void* stream) {
  if (!A_dev || !B_dev || !D_dev || (N != 32 && N != 64) || (bf16 != 0 && bf16 != 1) || mode < 0 || mode > 3 ||
      ((mode == 1 || mode == 2) && N != 64))
    return set_error(SNISR_INVALID_ARG, "diag_mma: bad argument");
  cudaError_t e = launch_diag_mma(A_dev, B_dev, D_dev, N, bf16, mode, (cudaStream_t)stream);
  if (e == cudaErrorLaunchTimeout) return set_error(SNISR_DEVICE_TIMEOUT, "diag_mma: MMA completion wait ran out");
  CUDA_TRY(e, "diag_mma");
  return SNISR_OK;
}

}  // extern "C"
