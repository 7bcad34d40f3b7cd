// Training-ray preparation of one tile from posed views (get_trainData_v3,
// training/src/cuda_func.cu:1341-1686), as device ops:
//   train_rays        computing_rays_kernel / get_rays (cuda_func.cu:15-50,
//                     training/src/include/cuda_utils.h:143-155): pixel
//                     (x, y) -> direction C2W[:3,:3] (x - cx)/fx, (y - cy)/fy, 1
//                     (not normalised), origin C2W[:, 3];
//   train_tracing     tracingTile_kernel (cuda_func.cu:52-128): tile DDA of
//                     the normalised direction from the origin (or its scene
//                     entry), clamped into the scene;
//   double_hits       ray_doubleHit_inTile_kernel (cuda_func.cu:284-444): per
//                     (ray, visited tile) the two nearest proxy-mesh hits whose
//                     points lie in the tile (+-1e-5), from this library's BVH;
//   train_bgdepth     get_trainData_kernel (cuda_func.cu:587-663): rays whose
//                     first hit lies in the training tile or behind it are
//                     valid; the background depth is the next hit;
//   gen_diffuse       gen_diffuse_in_tile_kernel (cuda_func.cu:1197-1339): the
//                     hit point projected into every selected view with a depth
//                     test, bilinear colours weighted by (1 - cos)^2 of the view
//                     angle; background depths no view sees become -1;
//   sample_bg         Sample_bg_cuda_kernel (training/src/Sample_kernel.cu:481-542);
//   patch_rows        the host patch loop of get_trainData_v3 (:1545-1600):
//                     patches with a valid pixel, as rows of 14 floats.
// Positions and projections use non-contracting FP32 arithmetic; the depth
// lookup rounds (int)(p + 0.5) in double, as the reference's 0.5 literal does.  Where the
// reference normalises with rsqrtf this uses the correctly rounded reciprocal
// square root (FP64 sqrt and divide, then one rounding).
#include <cuda_runtime.h>

#include <string>

#include "device_common.cuh"
#include "kernels.h"
#include "proxy.cuh"
#include "snisr.h"
#include "snisr_internal.h"

namespace snisr {
namespace {

constexpr float kThresh = 0.00001f;  // THRESH (training/src/include/cuda_utils.h:9)

inline int grid_n(int64_t n, int threads) {
  int64_t b = (n + threads - 1) / threads;
  return (int)(b < (1 << 20) ? b : (1 << 20));
}

__device__ __forceinline__ float rinv_sqrt(float x) {
  return (float)__ddiv_rn(1.0, __dsqrt_rn((double)x));
}
__device__ __forceinline__ void normalize3(const float v[3], float out[3]) {
  const float inv = rinv_sqrt(fadd(fadd(fmul(v[0], v[0]), fmul(v[1], v[1])), fmul(v[2], v[2])));
#pragma unroll
  for (int a = 0; a < 3; ++a) out[a] = fmul(v[a], inv);
}

__global__ void train_rays_kernel(const float* __restrict__ Km, const float* __restrict__ C, int H, int W,
                                  float* ro, float* rd) {
  const int64_t n = (int64_t)H * W;
  const float fx = Km[0], cx = Km[2], fy = Km[4], cy = Km[5];
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int y = (int)(i / W), x = (int)(i % W);
    const float u = fdiv(fsub((float)x, cx), fx);
    const float v = fdiv(fsub((float)y, cy), fy);
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      // C0 u + C1 v + C2 with the reference build's contraction: fma(C0, u, C1 v) + C2
      rd[3 * i + a] = fadd(ffma(C[4 * a], u, fmul(C[4 * a + 1], v)), C[4 * a + 2]);
      ro[3 * i + a] = C[4 * a + 3];
    }
  }
}

template <bool kStaged>
__global__ void train_tracing_kernel(const float* __restrict__ ro, const float* __restrict__ rd, int64_t n,
                                     const int32_t* __restrict__ imap, int3 shape, float3 smin, float tile, int K,
                                     int32_t* visited) {
  extern __shared__ int32_t rows[];  // kStaged: blockDim.x lists of K
  const int M[3] = {shape.x, shape.y, shape.z};
  const float sm[3] = {smin.x, smin.y, smin.z};
  float size[3], c[3], h[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    size[a] = fmul((float)M[a], tile);
    h[a] = fmul(size[a], 0.5f);
    c[a] = fadd(sm[a], h[a]);
  }
  for (int64_t base = blockIdx.x * (int64_t)blockDim.x; base < n; base += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = base + threadIdx.x;
    int32_t* vis = kStaged ? rows + threadIdx.x * K : visited + i * K;
    if (kStaged || i < n)
      for (int j = 0; j < K; ++j) vis[j] = -1;
    if (i < n) {
      const float o[3] = {ro[3 * i], ro[3 * i + 1], ro[3 * i + 2]};
      const float d0[3] = {rd[3 * i], rd[3 * i + 1], rd[3 * i + 2]};
      float d[3];
      normalize3(d0, d);
      float p[3];
#pragma unroll
      for (int a = 0; a < 3; ++a) p[a] = fsub(o[a], sm[a]);
      if (p[0] < 0 || p[0] >= size[0] || p[1] < 0 || p[1] >= size[1] || p[2] < 0 || p[2] >= size[2]) {
        const float2 b = slab(o, d, c, h);
#pragma unroll
        for (int a = 0; a < 3; ++a) p[a] = ffma(b.x, d[a], p[a]);
      }
#pragma unroll
      for (int a = 0; a < 3; ++a) p[a] = fmaxf(0.0f, fminf(p[a], fsub(size[a], 0.000001f)));
      tile_grid_walk(p, d, imap, M, tile, K, vis);
    }
    if (kStaged) trace_rows_flush(rows, visited, base, n, K);
  }
}

// Two nearest hits (with multiplicity) of the ray with the proxy mesh whose
// points lie in the box c +- (h + kThresh).  BVH nodes are clipped to that
// box before the slab test, so only the tile's part of the mesh is visited.
// A node is tested when pushed and goes on the stack with its entry distance
// and child index / triangle range (first << 5 | count), the nearer child on
// top; popped, only that distance is compared with the current second hit
// (the same test as re-testing the clipped box).  The result -- the two
// smallest in-box hit distances -- does not depend on the visiting order.
__device__ float2 bvh_two_nearest_in_box(const SceneDev& S, const float o[3], const float d[3], const float c[3],
                                         float h) {
  float inv[3], lo[3], hi[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    inv[a] = fdiv(1.0f, d[a]);
    lo[a] = fsub(fsub(c[a], h), 2.0f * kThresh);
    hi[a] = fadd(fadd(c[a], h), 2.0f * kThresh);
  }
  float near1 = SNISR_INF, near2 = SNISR_INF;
  // the node's box clipped to the tile box, against [0, near2]
  auto clipped_hit = [&](const BvhNodeDev& nd, float& tn) {
    float bmin[3], bmax[3];
    bool empty = false;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      bmin[a] = fmaxf(nd.bmin[a], lo[a]);
      bmax[a] = fminf(nd.bmax[a], hi[a]);
      empty = empty || bmin[a] > bmax[a];
    }
    return !empty && box_hit(o, inv, bmin, bmax, near2, tn);
  };
  uint32_t stack[64];
  float snear[64];
  int sp = 0;
  {
    const BvhNodeDev r = S.bvh[0];
    float tn;
    if (clipped_hit(r, tn)) {
      stack[0] = ((uint32_t)r.first << 5) | (uint32_t)r.count;
      snear[0] = tn;
      sp = 1;
    }
  }
  while (sp > 0) {
    --sp;
    if (!(snear[sp] <= fmul(near2, 1.0000005f))) continue;
    const int first = (int)(stack[sp] >> 5), count = (int)(stack[sp] & 31u);
    if (count > 0) {
      for (int k = 0; k < count; ++k) {
        const int slot = first + k;
        const float4 a4 = __ldg(S.tri + 3 * slot), b4 = __ldg(S.tri + 3 * slot + 1), c4 = __ldg(S.tri + 3 * slot + 2);
        const float A[3] = {a4.x, a4.y, a4.z}, B[3] = {b4.x, b4.y, b4.z}, Cc[3] = {c4.x, c4.y, c4.z};
        float t;
        if (!tri_hit(o, d, A, B, Cc, t) || !(t < near2)) continue;
        bool in = true;
#pragma unroll
        for (int a = 0; a < 3; ++a) in = in && fsub(fabsf(fsub(fadd(o[a], fmul(t, d[a])), c[a])), h) <= kThresh;
        if (!in) continue;
        if (t < near1) {
          near2 = near1;
          near1 = t;
        } else {
          near2 = t;
        }
      }
    } else {
      const BvhNodeDev l = S.bvh[first], r = S.bvh[first + 1];
      float tl, tr;
      const bool hl = clipped_hit(l, tl), hr = clipped_hit(r, tr);
      if (sp + 2 > 64) {
        atomicOr(S.err, ERR_OVERFLOW);
        break;
      }
      const uint32_t el = ((uint32_t)l.first << 5) | (uint32_t)l.count, er = ((uint32_t)r.first << 5) | (uint32_t)r.count;
      if (hl && hr) {
        if (tl <= tr) { stack[sp] = er; snear[sp++] = tr; stack[sp] = el; snear[sp++] = tl; }
        else { stack[sp] = el; snear[sp++] = tl; stack[sp] = er; snear[sp++] = tr; }
      } else if (hl) {
        stack[sp] = el; snear[sp++] = tl;
      } else if (hr) {
        stack[sp] = er; snear[sp++] = tr;
      }
    }
  }
  return make_float2(near1, near2);
}

// One thread per ray, looping over its visited tiles (a ray visits a few of
// its K slots; one thread per slot would leave most lanes of a warp idle).
__global__ void double_hits_kernel(SceneDev S, const float* __restrict__ ro, const float* __restrict__ rd,
                                   const int32_t* __restrict__ visited, int64_t n, int K, float2* hits) {
  const float hs = fdiv(S.tile_size, 2.0f);
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    const float o[3] = {ro[3 * r], ro[3 * r + 1], ro[3 * r + 2]};
    const float d[3] = {rd[3 * r], rd[3 * r + 1], rd[3 * r + 2]};
    for (int j = 0; j < K; ++j) {
      float2 out = make_float2(-1.0f, -1.0f);
      const int tile = visited[r * K + j];
      if (tile >= 0 && tile < S.num_tiles && S.has_mesh) {
        const float c[3] = {S.tile_center[3 * tile], S.tile_center[3 * tile + 1], S.tile_center[3 * tile + 2]};
        const float2 t = bvh_two_nearest_in_box(S, o, d, c, hs);
        if (t.x != SNISR_INF) {
          out.x = t.x;
          if (t.y != SNISR_INF) out.y = t.y;
        }
      }
      hits[r * K + j] = out;
    }
  }
}

__global__ void train_bgdepth_kernel(int train_tile, const int32_t* __restrict__ visited,
                                     const float2* __restrict__ hits, int64_t n, int K, float* bgdepth,
                                     int32_t* valid) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float2* h = hits + i * K;
    const int32_t* vis = visited + i * K;
    float first = -1.0f, second = -1.0f;
    int flag_first = -1;
    for (int j = 0; j < K; ++j) {
      if (h[j].x != -1.0f) {
        if (flag_first == -1) {
          flag_first = j;
          first = h[j].x;
        } else {
          second = h[j].x;
          break;
        }
      }
    }
    float bg = -1.0f;
    int ok = 0;
    for (int j = 0; j <= flag_first; ++j) {
      if (vis[j] == train_tile) {
        bg = j == flag_first ? second : first;
        ok = 1;
        break;
      }
    }
    bgdepth[i] = bg;
    valid[i] = ok;
  }
}

// The diffuse estimate's arithmetic as the reference's compiled kernel does
// it (gen_diffuse_in_tile_kernel, training/src/cuda_func.cu:1197-1339, built
// by nvcc with its default contraction): every `a*b + c*d + ...` chain fuses
// the left product of the first add and then each further product into a
// multiply-add, and normalize() multiplies by CUDA's rsqrtf of the squared
// length (training/src/include/cutil_math.h).  rsqrtf matters here: for the
// training view itself the view-angle weight (1 - cos)^2 is a rounding
// residue, non-zero for most pixels, so a hit seen by no other view takes its
// own pixel colour.
__device__ __forceinline__ float dot3_fused(const float a[3], const float b[3]) {
  return ffma(a[2], b[2], ffma(a[0], b[0], fmul(a[1], b[1])));
}
__device__ __forceinline__ void normalize3_rsqrt(const float v[3], float out[3]) {
  const float inv = rsqrtf(dot3_fused(v, v));
#pragma unroll
  for (int a = 0; a < 3; ++a) out[a] = fmul(v[a], inv);
}
__device__ __forceinline__ bool project(const float* m, const float p[3], int H, int W, float& z, float& px,
                                        float& py) {
  const float x = fadd(ffma(m[2], p[2], ffma(m[0], p[0], fmul(m[1], p[1]))), m[3]);
  const float y = fadd(ffma(m[6], p[2], ffma(m[4], p[0], fmul(m[5], p[1]))), m[7]);
  z = fadd(ffma(m[10], p[2], ffma(m[8], p[0], fmul(m[9], p[1]))), m[11]);
  if (z <= 0.0f) return false;
  px = fdiv(x, z);
  py = fdiv(y, z);
  return !(px < 0.0f || px >= (float)(W - 1) || py < 0.0f || py >= (float)(H - 1));
}

__global__ void gen_diffuse_kernel(const float* __restrict__ origins, int train_tile, const float* __restrict__ ro,
                                   const float* __restrict__ rd, const float2* __restrict__ hits,
                                   const int32_t* __restrict__ visited, const float* __restrict__ images,
                                   const float* __restrict__ depths, const float* __restrict__ ms, int K, int nimg,
                                   int H, int W, float* diffuse, float* bgdepth) {
  const int64_t npix = (int64_t)H * W;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < npix; i += (int64_t)gridDim.x * blockDim.x) {
    const float2* h = hits + i * K;
    const int32_t* vis = visited + i * K;
    const float o[3] = {ro[3 * i], ro[3 * i + 1], ro[3 * i + 2]};
    const float d[3] = {rd[3 * i], rd[3 * i + 1], rd[3 * i + 2]};
    diffuse[3 * i] = diffuse[3 * i + 1] = diffuse[3 * i + 2] = 0.0f;
    float first = -1.0f;
    for (int j = 0; j < K; ++j)
      if (h[j].x != -1.0f && vis[j] == train_tile) {
        first = h[j].x;
        break;
      }
    if (first == -1.0f) continue;
    const float bg = bgdepth[i];
    if (bg != -1.0f) {
      float p[3];
#pragma unroll
      for (int a = 0; a < 3; ++a) p[a] = ffma(bg, d[a], o[a]);
      bool visible = false;
      for (int j = 0; j < nimg && !visible; ++j) {
        float z, px, py;
        if (!project(ms + 12 * j, p, H, W, z, px, py)) continue;
        const float dep = __ldg(depths + (int64_t)j * npix + (int64_t)(int)__dadd_rn((double)py, 0.5) * W +
                                (int)__dadd_rn((double)px, 0.5));
        if (fabsf(fsub(z, dep)) > 0.01f) continue;
        visible = true;
      }
      if (!visible) bgdepth[i] = -1.0f;
    }
    float hp[3], dn[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) hp[a] = ffma(first, d[a], o[a]);
    normalize3_rsqrt(d, dn);
    float sum[3] = {0.0f, 0.0f, 0.0f}, weight = 0.0f;
    for (int j = 0; j < nimg; ++j) {
      float z, px, py;
      if (!project(ms + 12 * j, hp, H, W, z, px, py)) continue;
      const float* dj = depths + (int64_t)j * npix;
      const float dep = __ldg(dj + (int64_t)(int)__dadd_rn((double)py, 0.5) * W + (int)__dadd_rn((double)px, 0.5));
      if (fabsf(fsub(z, dep)) > 0.01f) continue;
      float v[3], vp[3];
#pragma unroll
      for (int a = 0; a < 3; ++a) v[a] = fsub(hp[a], __ldg(origins + 3 * j + a));
      normalize3_rsqrt(v, vp);
      const int x0 = (int)px, y0 = (int)py;
      const float fx = fsub(px, (float)x0), fy = fsub(py, (float)y0);
      const float w00 = fmul(fsub(1.0f, fx), fsub(1.0f, fy));
      const float w11 = fmul(fx, fy);
      const float w01 = fmul(fsub(1.0f, fx), fy);
      const float w10 = fmul(fx, fsub(1.0f, fy));
      const int64_t i00 = (int64_t)j * npix + (int64_t)y0 * W + x0;
      const int64_t i10 = i00 + 1, i01 = i00 + W, i11 = i01 + 1;
      float wc = fsub(1.0f, dot3_fused(dn, vp));
      wc = fmul(wc, wc);
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        const float c00 = __ldg(images + 3 * i00 + a), c01 = __ldg(images + 3 * i01 + a);
        const float c10 = __ldg(images + 3 * i10 + a), c11 = __ldg(images + 3 * i11 + a);
        const float c = ffma(c11, w11, ffma(c10, w10, ffma(c00, w00, fmul(c01, w01))));
        sum[a] = ffma(wc, c, sum[a]);
      }
      weight = fadd(weight, wc);
    }
    if (weight != 0.0f) {
      const float inv = fdiv(1.0f, weight);  // float3 / float multiplies by the reciprocal
#pragma unroll
      for (int a = 0; a < 3; ++a) diffuse[3 * i + a] = fmul(sum[a], inv);
    }
  }
}

__global__ void sample_bg_kernel(const float* __restrict__ ro, const float* __restrict__ rd,
                                 const float* __restrict__ bgz, int64_t n, int ns, float range,
                                 const float* __restrict__ center, float tile, float* z) {
  const float c[3] = {center[0], center[1], center[2]};
  const float hs = fdiv(tile, 2.0f);
  const float h3[3] = {hs, hs, hs};
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float bg = bgz[i];
    if (bg == -1.0f) continue;
    const float half = fdiv(range, 2.0f);
    const float o[3] = {ro[3 * i], ro[3 * i + 1], ro[3 * i + 2]};
    const float d[3] = {rd[3 * i], rd[3 * i + 1], rd[3 * i + 2]};
    const float2 b = slab(o, d, c, h3);
    float near_ = fsub(bg, half), far_ = fadd(bg, half);
    if (near_ <= b.y) {
      near_ = fadd(b.y, 0.00001f);
      far_ = fadd(near_, range);
    }
    const float interval = fdiv(fsub(far_, near_), (float)(ns - 1));
    for (int k = 0; k < ns; ++k) z[i * ns + k] = ffma((float)k, interval, near_);
  }
}

// Patch grid of get_trainData_v3: centres y = half, half + P, ... < H - P.
__host__ __device__ inline int patch_count(int L, int P) {
  const int half = P / 2;
  return L - P > half ? (L - P - half + P - 1) / P : 0;
}

__global__ void patch_flags_kernel(const int32_t* __restrict__ valid, int H, int W, int P, int32_t* flags) {
  const int ny = patch_count(H, P), nx = patch_count(W, P), half = P / 2;
  const int64_t np = (int64_t)ny * nx;
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < np; q += (int64_t)gridDim.x * blockDim.x) {
    const int y = half + (int)(q / nx) * P, x = half + (int)(q % nx) * P;
    int f = 0;
    for (int dy = -half; dy <= half && !f; ++dy)
      for (int dx = -half; dx <= half; ++dx)
        if (valid[(int64_t)(y + dy) * W + (x + dx)] != 0) {
          f = 1;
          break;
        }
    flags[q] = f;
  }
}

// One block: exclusive scan of the patch flags into offsets, total in *count.
__global__ void patch_scan_kernel(const int32_t* __restrict__ flags, int64_t np, int32_t* offsets, int64_t* count) {
  __shared__ int32_t warp_sums[32];
  __shared__ int32_t carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int64_t base = 0; base < np; base += blockDim.x) {
    const int64_t q = base + threadIdx.x;
    const int32_t f = q < np ? flags[q] : 0;
    int32_t v = f;
#pragma unroll
    for (int s = 1; s < 32; s <<= 1) {
      const int32_t u = __shfl_up_sync(0xFFFFFFFFu, v, s);
      if (lane >= s) v += u;
    }
    if (lane == 31) warp_sums[warp] = v;
    __syncthreads();
    if (warp == 0) {
      int32_t w = lane < nw ? warp_sums[lane] : 0;
#pragma unroll
      for (int s = 1; s < 32; s <<= 1) {
        const int32_t u = __shfl_up_sync(0xFFFFFFFFu, w, s);
        if (lane >= s) w += u;
      }
      if (lane < nw) warp_sums[lane] = w;
    }
    __syncthreads();
    const int32_t before = carry + (warp > 0 ? warp_sums[warp - 1] : 0) + v - f;
    if (q < np) offsets[q] = before;
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry = before + f;
    __syncthreads();
  }
  if (threadIdx.x == 0) *count = carry;
}

__global__ void patch_rows_kernel(const int32_t* __restrict__ flags, const int32_t* __restrict__ offsets, int H,
                                  int W, int P, const float* __restrict__ ro, const float* __restrict__ rd,
                                  const float* __restrict__ bgdepth, const float* __restrict__ gt,
                                  const float* __restrict__ diffuse, const int32_t* __restrict__ valid, float* rows) {
  const int ny = patch_count(H, P), nx = patch_count(W, P), half = P / 2, PP = P * P;
  const int64_t total = (int64_t)ny * nx * PP;
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < total; k += (int64_t)gridDim.x * blockDim.x) {
    const int64_t q = k / PP;
    if (!flags[q]) continue;
    const int e = (int)(k % PP);
    const int y = half + (int)(q / nx) * P + e / P - half, x = half + (int)(q % nx) * P + e % P - half;
    const int64_t idx = (int64_t)y * W + x;
    float* r = rows + ((int64_t)offsets[q] * PP + e) * 14;
    for (int a = 0; a < 3; ++a) {
      r[a] = ro[3 * idx + a];
      r[3 + a] = rd[3 * idx + a];
      r[7 + a] = gt[3 * idx + a];
      r[10 + a] = diffuse[3 * idx + a];
    }
    r[6] = bgdepth[idx];
    r[13] = (float)valid[idx];
  }
}

}  // namespace

cudaError_t launch_double_hits(const SceneDev& S, const float* ro, const float* rd, const int32_t* visited,
                               int64_t n, int K, float* hits, cudaStream_t st) {
  double_hits_kernel<<<grid_n(n, 128), 128, 0, st>>>(S, ro, rd, visited, n, K, reinterpret_cast<float2*>(hits));
  return cudaGetLastError();
}

}  // namespace snisr

using namespace snisr;

#define PREP_CHECK(name)                                                                                     \
  do {                                                                                                       \
    cudaError_t e = cudaGetLastError();                                                                      \
    if (e != cudaSuccess) return set_error(SNISR_CUDA_ERROR, std::string(name ": ") + cudaGetErrorString(e)); \
  } while (0)

extern "C" {

snisr_status snisr_op_train_rays(const float* K_dev, const float* c2w_dev, int32_t height, int32_t width,
                                 float* rays_o, float* rays_d, void* stream) {
  if (height <= 0 || width <= 0) return set_error(SNISR_INVALID_ARG, "train_rays: bad size");
  if (!K_dev || !c2w_dev || !rays_o || !rays_d) return set_error(SNISR_INVALID_ARG, "train_rays: null argument");
  train_rays_kernel<<<grid_n((int64_t)height * width, 256), 256, 0, (cudaStream_t)stream>>>(K_dev, c2w_dev, height,
                                                                                         width, rays_o, rays_d);
  PREP_CHECK("train_rays");
  return SNISR_OK;
}

snisr_status snisr_op_train_tracing_tiles(const float* rays_o, const float* rays_d, int64_t n, const int32_t* index_map,
                                          const int32_t tile_shape[3], const float scene_min_corner[3],
                                          float tile_size, int32_t K, int32_t* visited, void* stream) {
  if (n < 0 || K <= 0 || !(tile_size > 0) || !tile_shape || !scene_min_corner || tile_shape[0] <= 0 ||
      tile_shape[1] <= 0 || tile_shape[2] <= 0)
    return set_error(SNISR_INVALID_ARG, "train_tracing_tiles: bad size");
  if (n == 0) return SNISR_OK;
  if (!rays_o || !rays_d || !index_map || !visited)
    return set_error(SNISR_INVALID_ARG, "train_tracing_tiles: null argument");
  const int3 shp = make_int3(tile_shape[0], tile_shape[1], tile_shape[2]);
  const float3 smn = make_float3(scene_min_corner[0], scene_min_corner[1], scene_min_corner[2]);
  if (trace_rows_staged(K))
    train_tracing_kernel<true><<<grid_n(n, kTraceRowsThreads), kTraceRowsThreads, (size_t)kTraceRowsThreads * K * 4,
                                 (cudaStream_t)stream>>>(rays_o, rays_d, n, index_map, shp, smn, tile_size, K, visited);
  else
    train_tracing_kernel<false><<<grid_n(n, 128), 128, 0, (cudaStream_t)stream>>>(rays_o, rays_d, n, index_map, shp,
                                                                                  smn, tile_size, K, visited);
  PREP_CHECK("train_tracing_tiles");
  return SNISR_OK;
}

snisr_status snisr_op_train_bgdepth(int32_t train_tile, const int32_t* visited, const float* double_hits, int64_t n,
                                    int32_t K, float* bgdepth, int32_t* valid, void* stream) {
  if (n < 0 || K <= 0) return set_error(SNISR_INVALID_ARG, "train_bgdepth: bad size");
  if (n == 0) return SNISR_OK;
  if (!visited || !double_hits || !bgdepth || !valid) return set_error(SNISR_INVALID_ARG, "train_bgdepth: null argument");
  train_bgdepth_kernel<<<grid_n(n, 256), 256, 0, (cudaStream_t)stream>>>(
      train_tile, visited, reinterpret_cast<const float2*>(double_hits), n, K, bgdepth, valid);
  PREP_CHECK("train_bgdepth");
  return SNISR_OK;
}

snisr_status snisr_op_gen_diffuse(const float* origins, int32_t train_tile, const float* rays_o, const float* rays_d,
                                  const float* double_hits, const int32_t* visited, const float* images,
                                  const float* depths, const float* proj, int32_t K, int32_t num_images,
                                  int32_t height, int32_t width, float* diffuse, float* bgdepth, void* stream) {
  if (K <= 0 || num_images < 0 || height < 2 || width < 2) return set_error(SNISR_INVALID_ARG, "gen_diffuse: bad size");
  if (!rays_o || !rays_d || !double_hits || !visited || !diffuse || !bgdepth ||
      (num_images > 0 && (!origins || !images || !depths || !proj)))
    return set_error(SNISR_INVALID_ARG, "gen_diffuse: null argument");
  gen_diffuse_kernel<<<grid_n((int64_t)height * width, 128), 128, 0, (cudaStream_t)stream>>>(
      origins, train_tile, rays_o, rays_d, reinterpret_cast<const float2*>(double_hits), visited, images, depths,
      proj, K, num_images, height, width, diffuse, bgdepth);
  PREP_CHECK("gen_diffuse");
  return SNISR_OK;
}

snisr_status snisr_op_sample_bg(const float* rays_o, const float* rays_d, const float* bg_zval, int64_t n,
                                int32_t nsamples, float sample_range, const float* tile_center, float tile_size,
                                float* z_vals, void* stream) {
  if (n < 0 || nsamples < 2 || !(tile_size > 0)) return set_error(SNISR_INVALID_ARG, "sample_bg: bad size");
  if (n == 0) return SNISR_OK;
  if (!rays_o || !rays_d || !bg_zval || !tile_center || !z_vals)
    return set_error(SNISR_INVALID_ARG, "sample_bg: null argument");
  sample_bg_kernel<<<grid_n(n, 256), 256, 0, (cudaStream_t)stream>>>(rays_o, rays_d, bg_zval, n, nsamples,
                                                                      sample_range, tile_center, tile_size, z_vals);
  PREP_CHECK("sample_bg");
  return SNISR_OK;
}

int64_t snisr_op_patch_capacity(int32_t height, int32_t width, int32_t patch_size) {
  if (height <= 0 || width <= 0 || patch_size <= 0 || patch_size % 2 == 0) return -1;
  return (int64_t)patch_count(height, patch_size) * patch_count(width, patch_size);
}

snisr_status snisr_op_patch_rows(const int32_t* valid, int32_t height, int32_t width, int32_t patch_size,
                                 const float* rays_o, const float* rays_d, const float* bgdepth, const float* gt_rgb,
                                 const float* diffuse, int32_t* scratch, float* rows, int64_t* num_patches,
                                 void* stream) {
  const int64_t np = snisr_op_patch_capacity(height, width, patch_size);
  if (np < 0) return set_error(SNISR_INVALID_ARG, "patch_rows: bad size (odd patch_size)");
  if (!valid || !rays_o || !rays_d || !bgdepth || !gt_rgb || !diffuse || !scratch || !rows || !num_patches)
    return set_error(SNISR_INVALID_ARG, "patch_rows: null argument");
  cudaStream_t st = (cudaStream_t)stream;
  if (np == 0) {
    cudaError_t e = cudaMemsetAsync(num_patches, 0, sizeof(int64_t), st);
    if (e != cudaSuccess) return set_error(SNISR_CUDA_ERROR, std::string("patch_rows: ") + cudaGetErrorString(e));
    return SNISR_OK;
  }
  int32_t* flags = scratch;
  int32_t* offsets = scratch + np;
  patch_flags_kernel<<<grid_n(np, 256), 256, 0, st>>>(valid, height, width, patch_size, flags);
  PREP_CHECK("patch_rows");
  patch_scan_kernel<<<1, 1024, 0, st>>>(flags, np, offsets, num_patches);
  PREP_CHECK("patch_rows");
  patch_rows_kernel<<<grid_n(np * patch_size * patch_size, 256), 256, 0, st>>>(
      flags, offsets, height, width, patch_size, rays_o, rays_d, bgdepth, gt_rgb, diffuse, valid, rows);
  PREP_CHECK("patch_rows");
  return SNISR_OK;
}

}  // extern "C"
