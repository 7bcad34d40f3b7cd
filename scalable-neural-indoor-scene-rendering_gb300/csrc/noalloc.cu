// Render entry point that allocates no device memory.
//
// Who needs it: callers that may not call cudaMalloc (or any allocating
// routine) when they render -- hosts that hand out all device memory from a
// pool of their own and forbid allocation by plugins, and real-time frame
// loops that must never block on the device allocator.  They create the
// scene once at start-up and then render through this entry point.
//
// The per-call scratch (ray origin/direction staging, 32 bytes per ray) is a
// file-scope __device__ array of kNoAllocMaxRays rays (2 MiB) that every GPU
// loading the library holds until the process exits.  In host code the
// array's name is only a host-side stand-in, so its device address is
// looked up with cudaGetSymbolAddress once per device (with that device
// current) and cached; the first call on a device performs this set-up, so
// make that first call before any stream capture on that device.  The cache
// remembers the id of the CUDA context the address belongs to: after a
// cudaDeviceReset (a new context, the array loaded again, possibly at another
// address) the next call sees a different id and looks the address up again,
// so that first call after a reset also belongs before any stream capture.
#include <cuda.h>
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "kernels.h"
#include "snisr.h"
#include "snisr_internal.h"

namespace snisr {

namespace {

constexpr int64_t kNoAllocMaxRays = 32768;
constexpr int kMaxDevices = 64;

// [0, kNoAllocMaxRays): origins, [kNoAllocMaxRays, 2*kNoAllocMaxRays): directions
__device__ __align__(256) float4 g_noalloc_rays[2 * kNoAllocMaxRays];

std::mutex g_symbol_mutex;
float4* g_symbol_ptr[kMaxDevices] = {};
unsigned long long g_symbol_ctx[kMaxDevices] = {};  // id of the context the cached address belongs to

using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);

// Unique id of the calling thread's current CUDA context (cuCtxGetId, through
// the runtime's driver entry points, so the library needs no link to the
// driver library); 0 when there is none or it cannot be read.
unsigned long long current_context_id() {
  static CtxGetCurrentFn get_current = nullptr;
  static CtxGetIdFn get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<CtxGetCurrentFn>(f);
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<CtxGetIdFn>(f);
  });
  CUcontext c = nullptr;
  unsigned long long id = 0;
  if (!get_current || !get_id || get_current(&c) != CUDA_SUCCESS || !c || get_id(c, &id) != CUDA_SUCCESS) return 0;
  return id;
}

// Device address of g_noalloc_rays on the current device: looked up on the
// first use and again whenever the device's context has changed.
snisr_status noalloc_scratch(int device, float4** out) {
  if (device < 0 || device >= kMaxDevices) return set_error(SNISR_UNSUPPORTED, "render_rays_noalloc: device ordinal too large");
  std::lock_guard<std::mutex> lock(g_symbol_mutex);
  const unsigned long long ctx = current_context_id();
  if (!g_symbol_ptr[device] || ctx == 0 || ctx != g_symbol_ctx[device]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_rays);  // also brings up the device's context
    if (e != cudaSuccess || !p)
      return set_error(SNISR_CUDA_ERROR, std::string("render_rays_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    g_symbol_ptr[device] = static_cast<float4*>(p);
    g_symbol_ctx[device] = current_context_id();
  }
  *out = g_symbol_ptr[device];
  return SNISR_OK;
}

}  // namespace

// Implemented in api.cpp: scene view, workspace and device of a scene.
snisr_status scene_views(snisr_scene* scene, SceneDev* S, Workspace* ws, int* device);

}  // namespace snisr

using namespace snisr;

extern "C" snisr_status snisr_render_rays_noalloc(snisr_scene* scene, const float* origins_dev, const float* dirs_dev,
                                                  int64_t n, float* rgb_dev, float* depth_dev, float* opacity_dev,
                                                  void* stream) {
  if (!scene) return set_error(SNISR_INVALID_ARG, "render_rays_noalloc: scene is null");
  if (n < 0 || n > kNoAllocMaxRays)
    return set_error(SNISR_INVALID_ARG, "render_rays_noalloc: at most 32768 rays per call (static scratch size)");
  if (n == 0) return SNISR_OK;
  if (!origins_dev || !dirs_dev || !rgb_dev || !depth_dev || !opacity_dev)
    return set_error(SNISR_INVALID_ARG, "render_rays_noalloc: null pointer argument");
  SceneDev S;
  Workspace ws;
  int device = 0;
  snisr_status st = scene_views(scene, &S, &ws, &device);
  if (st != SNISR_OK) return st;
  int prev = -1;
  cudaGetDevice(&prev);
  if (prev != device) cudaSetDevice(device);
  float4* scratch = nullptr;
  st = noalloc_scratch(device, &scratch);
  if (st == SNISR_OK) {
    // the static array replaces the scene workspace's ray staging; every ray
    // slot [0, n) is written before it is read, so nothing needs clearing
    Workspace w2 = ws;
    w2.ray_o = scratch;
    w2.ray_d = scratch + kNoAllocMaxRays;
    w2.enc = nullptr;
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = launch_raygen(S, nullptr, origins_dev, dirs_dev, n, w2, false, s);
    if (e == cudaSuccess) e = launch_render_plain(S, w2, n, rgb_dev, depth_dev, opacity_dev, s);
    if (e != cudaSuccess) st = set_error(SNISR_CUDA_ERROR, std::string("render_rays_noalloc: ") + cudaGetErrorString(e));
  }
  if (prev >= 0 && prev != device) cudaSetDevice(prev);
  return st;
}
