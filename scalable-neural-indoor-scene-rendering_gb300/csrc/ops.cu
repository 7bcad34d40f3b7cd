// Drop-in re-implementations of the reference's per-stage ops, with the
// reference's argument meaning.  Inputs that the reference passes through
// __constant__ symbols (cudaMemcpyToSymbol per call) are read from device
// pointers here, so the ops are re-entrant and stream-ordered.
//
// Arithmetic uses explicit round-to-nearest intrinsics, with ffma() exactly
// where the reference's nvcc build fuses a multiply into the following add
// (compute_rays, tracing_tiles, Sample_sparse, inverse_z_sampling,
// integrate_points), so that the outputs equal the compiled reference
// kernels' bit for bit; the host oracle states the same fused operations.
#include <cuda_fp16.h>

#include "device_common.cuh"
#include "snisr.h"
#include "snisr_internal.h"

namespace snisr {

namespace {

inline int blocks_for(int64_t n, int threads) {
  int64_t b = (n + threads - 1) / threads;
  if (b < 1) b = 1;
  if (b > (1 << 20)) b = 1 << 20;
  return (int)b;
}

// compute_rays_kernel (rendering/src/compute_rays.cu:18-44)
__global__ void op_compute_rays_kernel(const float* __restrict__ intr, const float* __restrict__ rot, int H, int W,
                                       float* rays_d) {
  const int64_t n = (int64_t)H * W;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    int py = (int)(i / W), px = (int)(i - (int64_t)py * W);
    float x = fmul(fsub((float)px, intr[0]), intr[2]);
    float y = fmul(fsub((float)py, intr[1]), intr[2]);
    // c0*x + c1*y + c2 compiles to fma(c0, x, c1*y) + c2
    for (int a = 0; a < 3; ++a) rays_d[3 * i + a] = fadd(ffma(rot[3 * a], x, fmul(rot[3 * a + 1], y)), rot[3 * a + 2]);
  }
}

// tracing_tiles_kernel + voxel_traversal (rendering/src/raytile_tracing.cu:9-60,
// rendering/src/include/cuda_utils.h:158-238).  A ray whose origin lies
// outside the scene is moved to its entry point; as in the reference, a
// missed scene box leaves t = -1 and the clamped point is traversed anyway.
template <bool kStaged>
__global__ void op_tracing_tiles_kernel(const float* __restrict__ rays_d, int64_t npix, const int32_t* __restrict__ imap,
                                        const float* __restrict__ origin, const int32_t* __restrict__ shape,
                                        const float* __restrict__ smin, const float* __restrict__ ssize, float tile,
                                        int K, int32_t* visited) {
  extern __shared__ int32_t rows[];  // kStaged: blockDim.x lists of K
  for (int64_t base = blockIdx.x * (int64_t)blockDim.x; base < npix; base += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = base + threadIdx.x;
    int32_t* vis = kStaged ? rows + threadIdx.x * K : visited + i * K;
    if (kStaged || i < npix)
      for (int j = 0; j < K; ++j) vis[j] = -1;
    if (i < npix) {
      float d[3] = {rays_d[3 * i], rays_d[3 * i + 1], rays_d[3 * i + 2]};
      float o[3] = {origin[0], origin[1], origin[2]};
      float p[3], size[3] = {ssize[0], ssize[1], ssize[2]};
      for (int a = 0; a < 3; ++a) p[a] = fsub(o[a], smin[a]);
      if (p[0] < 0 || p[0] >= size[0] || p[1] < 0 || p[1] >= size[1] || p[2] < 0 || p[2] >= size[2]) {
        float c[3], h[3];
        for (int a = 0; a < 3; ++a) { h[a] = fdiv(size[a], 2.0f); c[a] = fadd(smin[a], h[a]); }
        float2 b = slab(o, d, c, h);
        for (int a = 0; a < 3; ++a) {
          p[a] = ffma(b.x, d[a], p[a]);
          p[a] = fminf(fmaxf(p[a], 0.0f), fsub(size[a], 0.000001f));
        }
      }
      const int M[3] = {shape[0], shape[1], shape[2]};
      tile_grid_walk(p, d, imap, M, tile, K, vis);
    }
    if (kStaged) trace_rows_flush(rows, visited, base, npix, K);
  }
}

__device__ __forceinline__ float2 slab_scalar(const float o[3], const float d[3], const float c[3], float h) {
  const float hh[3] = {h, h, h};
  return slab(o, d, c, hh);
}

// uniform_sample_bound_v3 (rendering/src/include/cuda_utils.h:104-115)
__device__ __forceinline__ void uniform_v3(float* z, float* dist, float near, float far, int n) {
  float interval = fdiv(fsub(far, near), (float)n);
  for (int i = 0; i < n; ++i) {
    z[i] = ffma((float)i, interval, near);
    dist[i] = interval;
  }
}

// Sample_sparse_cuda_kernel (training/src/Sample_kernel.cu:181-394).
__global__ void op_sample_sparse_kernel(const float* __restrict__ ro, const float* __restrict__ rd, int64_t B,
                                        const int16_t* __restrict__ flags, float cx, float cy, float cz, float tile,
                                        int N, int ns, float* zv, float* dv) {
  const float half = fmul(tile, 0.5f);
  const float vs = fdiv(tile, (float)N);
  const float inv_vs = fdiv(1.0f, vs);  // float3 / float is a multiply by the reciprocal (cutil_math.h:396-400)
  const float center[3] = {cx, cy, cz};
  float minc[3];
  for (int a = 0; a < 3; ++a) minc[a] = fsub(center[a], half);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < B; i += (int64_t)gridDim.x * blockDim.x) {
    float* z = zv + i * ns;
    float* dd = dv + i * ns;
    float o[3] = {ro[3 * i], ro[3 * i + 1], ro[3 * i + 2]};
    float d[3] = {rd[3 * i], rd[3 * i + 1], rd[3 * i + 2]};
    float2 nf = slab_scalar(o, d, center, half);
    if (nf.x == -1.0f && nf.y == -1.0f) continue;
    // every per-voxel slab test of the ray divides by the same direction
    const float inv_d[3] = {safe_div(1.0f, d[0]), safe_div(1.0f, d[1]), safe_div(1.0f, d[2])};
    float near = nf.x, far = nf.y;
    float total = 0.0f;
    float loc[3], nb[3], tmax[3], tdel[3];
    int cur[3], st[3];
    for (int a = 0; a < 3; ++a) {
      loc[a] = fsub(ffma(near, d[a], o[a]), minc[a]);
      loc[a] = fminf(fmaxf(loc[a], 0.0f), fsub(tile, 0.000001f));
      cur[a] = min(max((int)fmul(loc[a], inv_vs), 0), N - 1);
      st[a] = d[a] >= 0 ? 1 : -1;
      nb[a] = fmul((float)(cur[a] + st[a]), vs);
      if (st[a] < 0) nb[a] = fadd(nb[a], vs);
      tmax[a] = safe_div(fsub(nb[a], loc[a]), d[a]);
      tdel[a] = safe_div(fmul((float)st[a], vs), d[a]);
    }
    auto voxel_bound = [&](const int* c) {
      float vc[3];
      for (int a = 0; a < 3; ++a) vc[a] = fadd(ffma((float)c[a], vs, minc[a]), fmul(0.5f, vs));
      return slab_inv(o, inv_d, vc, fmul(0.5f, vs));
    };
    auto step = [&]() {
      int a = (tmax[0] < tmax[1]) ? ((tmax[0] < tmax[2]) ? 0 : 2) : ((tmax[1] < tmax[2]) ? 1 : 2);
      cur[a] += st[a];
      tmax[a] = fadd(tmax[a], tdel[a]);
      return !(cur[a] < 0 || cur[a] >= N);
    };
    for (;;) {
      if (flags[(cur[0] * N + cur[1]) * N + cur[2]] == 1) {
        float2 b = voxel_bound(cur);
        total = fadd(total, fsub(b.y, b.x));
      }
      if (!step()) break;
    }
    if (total == 0.0f) continue;
    for (int a = 0; a < 3; ++a) {
      cur[a] = min(max((int)fmul(loc[a], inv_vs), 0), N - 1);
      tmax[a] = safe_div(fsub(nb[a], loc[a]), d[a]);
    }
    int count = 0;
    bool acc = false, first = false;
    int bsm = 4;
    const int ins = ns - 2 * bsm;
    for (;;) {
      if (flags[(cur[0] * N + cur[1]) * N + cur[2]] == 1) {
        float2 b = voxel_bound(cur);
        if (b.x != -1.0f && b.y != -1.0f) {
          if (acc) {
            far = b.y;
          } else {
            near = b.x;
            far = b.y;
            acc = true;
            if (!first) {
              first = true;
              uniform_v3(z + count, dd + count, fsub(near, vs), fsub(near, 0.000001f), bsm);
              count += bsm;
            }
          }
        }
      } else if (acc) {
        int num = (int)ceilf(fdiv(fmul((float)ins, fsub(far, near)), total));
        num = min(ns - count, num);
        uniform_v3(z + count, dd + count, near, far, num);
        count += num;
        acc = false;
      }
      if (!step()) break;
    }
    if (acc) {
      int num = (int)ceilf(fdiv(fmul((float)ins, fsub(far, near)), total));
      num = min(ns - count, num);
      uniform_v3(z + count, dd + count, near, far, num);
      count += num;
    }
    bsm = min(ns - count, bsm);
    uniform_v3(z + count, dd + count, fadd(far, 0.000001f), fadd(far, vs), bsm);
  }
}

// inverse_z_sampling_kernel (rendering/src/sampling.cu:5-45)
__global__ void op_inverse_z_kernel(const float* __restrict__ rays_d, const float* __restrict__ origin,
                                    const float* __restrict__ inv_near, const float* __restrict__ inv_bound,
                                    int64_t npix, int offset, int spr, float* pts, float* steps) {
  const int64_t n = npix * spr;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
    int64_t p = t / spr;
    int j = (int)(t - p * spr);
    float z = fdiv(1.0f, ffma((float)(offset + j), inv_bound[p], inv_near[p]));
    float zn = fdiv(1.0f, ffma((float)(offset + j + 1), inv_bound[p], inv_near[p]));
    steps[t] = fmaxf(fsub(zn, z), 0.0f);
    for (int a = 0; a < 3; ++a) pts[3 * t + a] = ffma(z, rays_d[3 * p + a], origin[a]);
  }
}

// integrate_points_kernel (rendering/src/volume_rendering.cu:5-58), 16 samples
// per call, transmittance carried across calls; the reference's exponential
// is the __expf intrinsic.  A block stages its pixels' samples in shared
// memory with coalesced loads (one thread per pixel reading its own 256-byte
// row makes every load instruction touch 32 scattered sectors), rows padded
// to 17 entries so that the per-pixel reads are free of bank conflicts; each
// pixel is then composited in the reference's order.
constexpr int kIntPix = 128;  // pixels (and threads) per block
__global__ void __launch_bounds__(kIntPix) op_integrate_kernel(const float4* __restrict__ rgba,
                                                              const float* __restrict__ dz, int64_t npix,
                                                              float early, float* frame, float* trans) {
  __shared__ float4 s_rgba[kIntPix * 17];
  __shared__ float s_dz[kIntPix * 17];
  for (int64_t base = (int64_t)blockIdx.x * kIntPix; base < npix; base += (int64_t)gridDim.x * kIntPix) {
    const int cnt = (int)(npix - base < kIntPix ? npix - base : kIntPix);
    for (int j = threadIdx.x; j < cnt * 16; j += kIntPix) {
      const int p = j >> 4, q = j & 15;
      s_rgba[p * 17 + q] = rgba[base * 16 + j];
      s_dz[p * 17 + q] = dz[base * 16 + j];
    }
    __syncthreads();
    if ((int)threadIdx.x < cnt) {
      const int64_t i = base + threadIdx.x;
      float T = trans[i];
      if (!(T < early)) {  // the reference skips a pixel when T < early
        const float4* v4 = s_rgba + threadIdx.x * 17;
        const float* d1 = s_dz + threadIdx.x * 17;
        float c[3] = {0.f, 0.f, 0.f};
        for (int q = 0; q < 16; ++q) {
          const float4 v = v4[q];
          float alpha = fsub(1.0f, __expf(fmul(fmul(-1.0f, v.w), d1[q])));
          float w = fmul(alpha, T);
          c[0] = ffma(w, v.x, c[0]);
          c[1] = ffma(w, v.y, c[1]);
          c[2] = ffma(w, v.z, c[2]);
          T = fmul(T, fsub(1.0f, alpha));
        }
        trans[i] = T;
        for (int a = 0; a < 3; ++a) frame[3 * i + a] = fadd(frame[3 * i + a], c[a]);
      }
    }
    __syncthreads();
  }
}

__global__ void camera_rays_kernel(int W, int H, float cx, float cy, float inv_f, snisr_camera cam, float* dirs) {
  const int64_t n = (int64_t)W * H;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    int py = (int)(i / W), px = (int)(i - (int64_t)py * W);
    float d[3];
    camera_dir(cam.c2w, cx, cy, inv_f, px, py, d);
    for (int a = 0; a < 3; ++a) dirs[3 * i + a] = d[a];
  }
}

#define OP_CHECK(what)                                                                           \
  do {                                                                                           \
    cudaError_t e__ = cudaGetLastError();                                                        \
    if (e__ != cudaSuccess) return set_error(SNISR_CUDA_ERROR, std::string(what) + ": " + cudaGetErrorString(e__)); \
  } while (0)

}  // namespace
}  // namespace snisr

using namespace snisr;

extern "C" {

snisr_status snisr_camera_rays(const snisr_camera* cam, float* dirs, void* stream) {
  if (!cam || !dirs || cam->width <= 0 || cam->height <= 0) return set_error(SNISR_INVALID_ARG, "camera_rays: bad argument");
  int64_t n = (int64_t)cam->width * cam->height;
  camera_rays_kernel<<<blocks_for(n, 256), 256, 0, (cudaStream_t)stream>>>(cam->width, cam->height, cam->cx, cam->cy,
                                                                           cam->inv_focal, *cam, dirs);
  OP_CHECK("camera_rays");
  return SNISR_OK;
}

snisr_status snisr_op_compute_rays(const float* intr, const float* rot, int32_t H, int32_t W, float* rays_d,
                                   void* stream) {
  if (!intr || !rot || !rays_d || H <= 0 || W <= 0) return set_error(SNISR_INVALID_ARG, "compute_rays: bad argument");
  int64_t n = (int64_t)H * W;
  op_compute_rays_kernel<<<blocks_for(n, 256), 256, 0, (cudaStream_t)stream>>>(intr, rot, H, W, rays_d);
  OP_CHECK("compute_rays");
  return SNISR_OK;
}

snisr_status snisr_op_tracing_tiles(const float* rays_d, int64_t npix, const int32_t* imap, const float* origin,
                                    const int32_t* shape, const float* smin, const float* ssize, float tile_size,
                                    int32_t K, int32_t* visited, void* stream) {
  if (npix < 0 || K <= 0 || !(tile_size > 0)) return set_error(SNISR_INVALID_ARG, "tracing_tiles: bad size");
  if (npix == 0) return SNISR_OK;
  if (!rays_d || !imap || !origin || !shape || !smin || !ssize || !visited)
    return set_error(SNISR_INVALID_ARG, "tracing_tiles: null argument");
  if (trace_rows_staged(K))
    op_tracing_tiles_kernel<true><<<blocks_for(npix, kTraceRowsThreads), kTraceRowsThreads,
                                    (size_t)kTraceRowsThreads * K * 4, (cudaStream_t)stream>>>(
        rays_d, npix, imap, origin, shape, smin, ssize, tile_size, K, visited);
  else
    op_tracing_tiles_kernel<false><<<blocks_for(npix, 256), 256, 0, (cudaStream_t)stream>>>(
        rays_d, npix, imap, origin, shape, smin, ssize, tile_size, K, visited);
  OP_CHECK("tracing_tiles");
  return SNISR_OK;
}

snisr_status snisr_op_sample_sparse(const float* ro, const float* rd, int64_t B, const int16_t* flags, float cx,
                                    float cy, float cz, float tile_size, int32_t N, int32_t ns, float* z, float* d,
                                    void* stream) {
  if (B < 0 || N <= 0 || ns < 8 || !(tile_size > 0)) return set_error(SNISR_INVALID_ARG, "sample_sparse: bad size (nsamples >= 8)");
  if (B == 0) return SNISR_OK;
  if (!ro || !rd || !flags || !z || !d) return set_error(SNISR_INVALID_ARG, "sample_sparse: null argument");
  op_sample_sparse_kernel<<<blocks_for(B, 128), 128, 0, (cudaStream_t)stream>>>(ro, rd, B, flags, cx, cy, cz, tile_size,
                                                                                N, ns, z, d);
  OP_CHECK("sample_sparse");
  return SNISR_OK;
}

snisr_status snisr_op_inverse_z_sampling(const float* rays_d, const float* origin, const float* inv_near,
                                         const float* inv_bound, int64_t npix, int32_t offset, int32_t spr,
                                         float* pts, float* steps, void* stream) {
  if (npix < 0 || spr <= 0) return set_error(SNISR_INVALID_ARG, "inverse_z_sampling: bad size");
  if (npix == 0) return SNISR_OK;
  if (!rays_d || !origin || !inv_near || !inv_bound || !pts || !steps)
    return set_error(SNISR_INVALID_ARG, "inverse_z_sampling: null argument");
  op_inverse_z_kernel<<<blocks_for(npix * spr, 256), 256, 0, (cudaStream_t)stream>>>(rays_d, origin, inv_near,
                                                                                     inv_bound, npix, offset, spr,
                                                                                     pts, steps);
  OP_CHECK("inverse_z_sampling");
  return SNISR_OK;
}

snisr_status snisr_op_integrate_points(const float* rgba, const float* dz, int64_t npix, float early, float* frame,
                                       float* trans, void* stream) {
  if (npix < 0) return set_error(SNISR_INVALID_ARG, "integrate_points: bad size");
  if (npix == 0) return SNISR_OK;
  if (!rgba || !dz || !frame || !trans) return set_error(SNISR_INVALID_ARG, "integrate_points: null argument");
  op_integrate_kernel<<<blocks_for(npix, kIntPix), kIntPix, 0, (cudaStream_t)stream>>>(
      reinterpret_cast<const float4*>(rgba), dz, npix, early, frame, trans);
  OP_CHECK("integrate_points");
  return SNISR_OK;
}

}  // extern "C"
