// Device-side scene view and ray traversal shared by the GB300 kernels.
//
// Traversal arithmetic is written with explicit round-to-nearest intrinsics
// (__fadd_rn, __fmul_rn, __fdiv_rn) so that no multiply-add is contracted
// behind our back: the visited voxel sequence is then bit-identical to an
// IEEE single precision evaluation of the same expressions on the host.
//
// The drop-ins of the reference's own CUDA ops (ops.cu, prune.cu, octree.cu)
// also reproduce the fused multiply-adds that the reference's nvcc build
// forms (its default contraction: a product feeding an add becomes one fma,
// the left product when both operands are products, e.g. a*b + c*d + e ->
// fma(a, b, c*d) + e; a product that has a second use stays unfused).  They
// write those with ffma() at exactly the places where the compiled reference
// kernels have them, as measured by running those kernels bit-for-bit
// against these drop-ins.
#pragma once

#include <cstdint>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "scene_dev.h"

namespace snisr {


// Four FP32 atomic adds at a 16-byte aligned address in one reduction
// (red.global.add.v4.f32, sm_90 and later): a quarter of the instructions
// and one L2 operation for four consecutive gradient entries.
__device__ __forceinline__ void red_add_v4(float* addr, float a, float b, float c, float d) {
  asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(addr), "f"(a), "f"(b), "f"(c), "f"(d)
               : "memory");
}

// Packed pair of floats in one 64-bit register, and the FP32x2 fused
// multiply-add of sm_100 and later (two independent round-to-nearest FMAs per
// instruction: the same results as two scalar FMAs, half the instructions).
__device__ __forceinline__ uint64_t f32x2(float lo, float hi) {
  uint64_t d;
  asm("mov.b64 %0, {%1, %2};" : "=l"(d) : "f"(lo), "f"(hi));
  return d;
}
__device__ __forceinline__ void split_f32x2(uint64_t v, float& lo, float& hi) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
__device__ __forceinline__ uint64_t ffma2(uint64_t a, uint64_t b, uint64_t c) {
  uint64_t d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}

__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fdiv(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ float ffma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
// reference safe_divide (rendering/src/include/cutil_math.h:867-869)
__device__ __forceinline__ float safe_div(float a, float b) { return b != 0.0f ? __fdiv_rn(a, b) : SNISR_INF; }

// One step of a fixed-step march.  When the step is too small to change z
// (below half the float spacing at z) the march would repeat the same sample
// forever; the step then returns +inf, which ends every `while (z < far)`
// loop.  For any step that does advance z the result is z + step, so outputs
// are unchanged.
__device__ __forceinline__ float march_next(float z, float step) {
  const float zn = __fadd_rn(z, step);
  return zn > z ? zn : SNISR_INF;
}

// Slab test with the reference's conventions (RayAABBIntersection,
// rendering/src/include/cuda_utils.h:506-598): t_low starts at 0, t_high at
// 1e5, a miss returns (-1, -1).
__device__ __forceinline__ float2 slab(const float o[3], const float d[3], const float c[3], const float h[3]) {
  float lo = 0.0f, hi = 100000.0f;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    float inv = safe_div(1.0f, d[a]);
    float l = fmul(fsub(fsub(c[a], h[a]), o[a]), inv);
    float u = fmul(fsub(fadd(c[a], h[a]), o[a]), inv);
    if (u < l) { float t = l; l = u; u = t; }
    if (u < lo) return make_float2(-1.0f, -1.0f);
    if (l > hi) return make_float2(-1.0f, -1.0f);
    lo = (l > lo) ? l : lo;
    hi = (u < hi) ? u : hi;
    if (lo > hi) return make_float2(-1.0f, -1.0f);
  }
  return make_float2(lo, hi);
}

// The same slab test with the reciprocals of the direction computed once per
// ray (safe_div(1, d[a]), as slab() computes them on every call).
__device__ __forceinline__ float2 slab_inv(const float o[3], const float inv[3], const float c[3], float h) {
  float lo = 0.0f, hi = 100000.0f;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    float l = fmul(fsub(fsub(c[a], h), o[a]), inv[a]);
    float u = fmul(fsub(fadd(c[a], h), o[a]), inv[a]);
    if (u < l) { float t = l; l = u; u = t; }
    if (u < lo) return make_float2(-1.0f, -1.0f);
    if (l > hi) return make_float2(-1.0f, -1.0f);
    lo = (l > lo) ? l : lo;
    hi = (u < hi) ? u : hi;
    if (lo > hi) return make_float2(-1.0f, -1.0f);
  }
  return make_float2(lo, hi);
}

// voxel_traversal (rendering/src/include/cuda_utils.h:158-238) over the tile
// grid: p is the start in scene-local coordinates, the visited sparse ids
// (dense cells mapping to -1 are skipped) go to vis[0..K).
__device__ __forceinline__ void tile_grid_walk(const float p[3], const float d[3], const int32_t* imap,
                                               const int M[3], float tile, int K, int32_t* vis) {
  int cur[3], st[3];
  float tmax[3], tdel[3];
  for (int a = 0; a < 3; ++a) {
    cur[a] = (int)floorf(fdiv(p[a], tile));
    cur[a] = min(max(cur[a], 0), M[a] - 1);
    st[a] = d[a] >= 0 ? 1 : -1;
    float nb = fmul((float)(cur[a] + st[a]), tile);
    if (st[a] < 0) nb = fadd(nb, tile);
    tmax[a] = d[a] != 0 ? fdiv(fsub(nb, p[a]), d[a]) : SNISR_INF;
    tdel[a] = d[a] != 0 ? fmul(fdiv(tile, d[a]), (float)st[a]) : SNISR_INF;
  }
  int idx = 0;
  int id = imap[(cur[0] * M[1] + cur[1]) * M[2] + cur[2]];
  if (id != -1) vis[idx++] = id;
  while (idx < K) {
    int a = (tmax[0] < tmax[1]) ? ((tmax[0] < tmax[2]) ? 0 : 2) : ((tmax[1] < tmax[2]) ? 1 : 2);
    cur[a] += st[a];
    tmax[a] = fadd(tmax[a], tdel[a]);
    if (cur[a] < 0 || cur[a] >= M[a]) break;
    id = imap[(cur[0] * M[1] + cur[1]) * M[2] + cur[2]];
    if (id != -1) vis[idx++] = id;
  }
}

// Visited-tile lists (K ints per pixel) are built per block in shared memory
// and written out as the block's one contiguous range with coalesced stores
// (a thread writing its own row alone makes every store a scattered 4-byte
// write, 32 cache lines per warp instruction).  kTraceRowsThreads pixels per
// block; lists longer than fit in 48 KB are written directly.
constexpr int kTraceRowsThreads = 128;
inline bool trace_rows_staged(int K) { return (size_t)kTraceRowsThreads * K * 4 <= 48 * 1024; }

__device__ __forceinline__ void trace_rows_flush(const int32_t* rows, int32_t* visited, int64_t base, int64_t n,
                                                 int K) {
  __syncthreads();
  const int64_t count = (n - base < (int64_t)blockDim.x ? n - base : (int64_t)blockDim.x) * K;
  int32_t* dst = visited + base * K;
  for (int64_t j = threadIdx.x; j < count; j += blockDim.x) dst[j] = rows[j];
  __syncthreads();
}

__device__ __forceinline__ bool occupied(const SceneDev& S, int tile, int vid, uint32_t& rec) {
  const OccWord* w = S.occ + (size_t)tile * S.words_per_tile + (vid >> 6);
  uint4 raw = __ldg(reinterpret_cast<const uint4*>(w));
  unsigned long long bits = ((unsigned long long)raw.y << 32) | raw.x;
  int b = vid & 63;
  if (!((bits >> b) & 1ull)) return false;
  rec = raw.z + (uint32_t)__popcll(bits & ((1ull << b) - 1ull));
  return true;
}

// Ray state machine: tile DDA over the scene grid, voxel DDA inside each
// visited tile, fixed-step samples inside each occupied voxel.
//
// Follows, in order: the scene clip + tile DDA of tracing_tiles_kernel /
// voxel_traversal (rendering/src/raytile_tracing.cu:32-56,
// rendering/src/include/cuda_utils.h:158-238), the per-tile AABB clip of
// rendering_diffuse_octree_fp16_kernel (raydiffuse_render_octree_fp16.cu:
// 202-214), the voxel DDA of Sample_sparse_cuda_kernel
// (training/src/Sample_kernel.cu:228-283) and the fixed-step march of
// block_traversal_rendering (raydiffuse_render_octree_fp16.cu:67-106),
// applied per occupied voxel instead of per 4^3 block.
struct RayState {
  float o[3], d[3];
  float t_start;
  // tile DDA (relative to the scene entry point)
  int tc[3], tstep[3];
  float tmax[3], tdelta[3];
  bool tile_live;     // tile DDA still inside the grid
  bool pending_tile;  // current tile-DDA cell not yet opened
  bool entry_pending; // tile opened, its entry voxel not yet examined
  // voxel DDA inside the current tile
  int tile;        // sparse id, -1 when no tile is open
  float t_in, q[3];
  int vc[3], vstep[3];
  float vmax[3], vdelta[3];
  float near_, far_;
  // current occupied voxel
  uint32_t rec;
  float z;         // next sample position (relative to t_in)
  bool in_voxel;
  uint32_t steps;  // voxel cells examined (for traffic accounting)

  __device__ bool init(const SceneDev& S, const float* oo, const float* dd, float ts) {
    for (int a = 0; a < 3; ++a) { o[a] = oo[a]; d[a] = dd[a]; }
    t_start = ts;
    tile = -1;
    in_voxel = false;
    tile_live = false;
    entry_pending = false;
    steps = 0;
    const int g[3] = {S.gx, S.gy, S.gz};
    float size[3], half[3], cen[3];
    for (int a = 0; a < 3; ++a) {
      size[a] = fmul((float)g[a], S.tile_size);
      half[a] = fmul(size[a], 0.5f);
      cen[a] = fadd(S.smin[a], half[a]);
    }
    float2 b = slab(o, d, cen, half);
    if (b.x == -1.0f) return false;
    float t0 = fmaxf(b.x, t_start);
    if (!(t0 < b.y)) return false;
    float p[3];
    for (int a = 0; a < 3; ++a) {
      p[a] = fsub(fadd(o[a], fmul(t0, d[a])), S.smin[a]);
      p[a] = fminf(fmaxf(p[a], 0.0f), fsub(size[a], 0.000001f));
      int c = (int)floorf(fdiv(p[a], S.tile_size));
      tc[a] = min(max(c, 0), g[a] - 1);
      tstep[a] = d[a] >= 0.0f ? 1 : -1;
      float nb = fmul((float)(tc[a] + tstep[a]), S.tile_size);
      if (tstep[a] < 0) nb = fadd(nb, S.tile_size);
      tmax[a] = d[a] != 0.0f ? fdiv(fsub(nb, p[a]), d[a]) : SNISR_INF;
      tdelta[a] = d[a] != 0.0f ? fmul(fdiv(S.tile_size, d[a]), (float)tstep[a]) : SNISR_INF;
    }
    tile_live = true;
    pending_tile = true;
    return true;
  }

  // Opens the current tile of the tile DDA if it is non-empty and the ray
  // overlaps it; returns false if nothing to march in it.
  __device__ bool open_tile(const SceneDev& S) {
    int dense = (tc[0] * S.gy + tc[1]) * S.gz + tc[2];
    int id = __ldg(S.tile_index + dense);
    if (id < 0) return false;
    return open_tile_id(S, id);
  }

  // Per-tile AABB clip and voxel-DDA set-up for sparse tile `id`.
  __device__ bool open_tile_id(const SceneDev& S, int id) {
    float c[3], h[3];
    for (int a = 0; a < 3; ++a) { c[a] = __ldg(S.tile_center + 3 * id + a); h[a] = fmul(S.tile_size, 0.5f); }
    float2 b = slab(o, d, c, h);
    if (b.x == -1.0f) return false;
    float ti = fmaxf(b.x, t_start);
    if (!(ti < b.y)) return false;
    t_in = ti;
    const int N = S.res;
    for (int a = 0; a < 3; ++a) {
      float corner = fsub(c[a], h[a]);
      q[a] = fsub(fadd(o[a], fmul(ti, d[a])), corner);
      q[a] = fminf(fmaxf(q[a], 0.0f), fsub(S.tile_size, 0.00001f));
      int v = (int)fdiv(q[a], S.voxel);
      vc[a] = min(max(v, 0), N - 1);
      vstep[a] = d[a] >= 0.0f ? 1 : -1;
      float nb = fmul((float)(vc[a] + vstep[a]), S.voxel);
      if (vstep[a] < 0) nb = fadd(nb, S.voxel);
      vmax[a] = safe_div(fsub(nb, q[a]), d[a]);
      vdelta[a] = safe_div(fmul((float)vstep[a], S.voxel), d[a]);
    }
    near_ = 0.0f;
    tile = id;
    entry_pending = true;
    return true;
  }

  // Ray segment restricted to sparse tile `id` (training rays split at tile
  // faces): no tile DDA, the segment ends where the ray leaves the tile.
  __device__ bool init_segment(const SceneDev& S, const float* oo, const float* dd, int id) {
    for (int a = 0; a < 3; ++a) { o[a] = oo[a]; d[a] = dd[a]; }
    t_start = 0.0f;
    tile = -1;
    in_voxel = false;
    tile_live = false;
    pending_tile = false;
    entry_pending = false;
    steps = 0;
    return open_tile_id(S, id);
  }

  // One Amanatides-Woo step with the reference tie rule: x only when strictly
  // smallest, then y only when strictly smaller than z, otherwise z.
  __device__ __forceinline__ int dda_axis(const float* m) const {
    if (m[0] < m[1]) return (m[0] < m[2]) ? 0 : 2;
    return (m[1] < m[2]) ? 1 : 2;
  }

  template <int A>
  __device__ __forceinline__ bool tile_axis_step(int g) {
    tc[A] += tstep[A];
    tmax[A] = fadd(tmax[A], tdelta[A]);
    return tc[A] >= 0 && tc[A] < g;
  }
  // Advances the tile DDA to the next tile; false when it leaves the grid.
  // Same axis choice as dda_axis(), written with compile-time indices so the
  // state stays in registers.
  __device__ bool step_tile(const SceneDev& S) {
    bool in;
    if (tmax[0] < tmax[1]) in = (tmax[0] < tmax[2]) ? tile_axis_step<0>(S.gx) : tile_axis_step<2>(S.gz);
    else in = (tmax[1] < tmax[2]) ? tile_axis_step<1>(S.gy) : tile_axis_step<2>(S.gz);
    if (!in) tile_live = false;
    return in;
  }
  template <int A>
  __device__ __forceinline__ bool voxel_axis_step(int N) {
    vc[A] += vstep[A];
    vmax[A] = fadd(vmax[A], vdelta[A]);
    return vc[A] >= 0 && vc[A] < N;
  }

  // Moves to the next occupied voxel along the ray, crossing tiles as
  // needed.  Sets rec, near_, far_.  Returns false when the ray has left the
  // scene.  Every step moves one DDA coordinate by one cell, so the loop ends
  // after at most (grid + tile) extent steps.  Empty space: when the current
  // voxel's 4^3 block is empty, with block distance D, every block within
  // Chebyshev distance D - 1 of it is empty too, and the DDA steps on through
  // that box in a tight loop without occupancy loads -- the same steps (the
  // same additions and comparisons) as examining the cells one by one, so the
  // voxels met and their entry and exit distances are unchanged.
  __device__ bool next_voxel(const SceneDev& S) {
    const int N = S.res, nb = N >> 2;
    for (;;) {
      if (tile < 0) {
        if (!tile_live) return false;
        if (!pending_tile && !step_tile(S)) return false;
        pending_tile = false;
        if (!open_tile(S)) continue;
      }
      if (entry_pending) {
        entry_pending = false;  // the entry voxel of a tile, or the first voxel past an empty box
      } else {
        bool in;
        if (vmax[0] < vmax[1]) in = (vmax[0] < vmax[2]) ? voxel_axis_step<0>(N) : voxel_axis_step<2>(N);
        else in = (vmax[1] < vmax[2]) ? voxel_axis_step<1>(N) : voxel_axis_step<2>(N);
        near_ = far_;
        if (!in) { tile = -1; continue; }
      }
      ++steps;
      far_ = fminf(fminf(vmax[0], vmax[1]), vmax[2]);
      const int bx = vc[0] >> 2, by = vc[1] >> 2, bz = vc[2] >> 2;
      const int D = __ldg(S.blk_dist + (size_t)tile * nb * nb * nb + (size_t)((bx * nb + by) * nb + bz));
      if (D == 0) {
        int vid = (vc[0] * N + vc[1]) * N + vc[2];
        uint32_t r;
        if (occupied(S, tile, vid, r)) { rec = r; return true; }
        continue;
      }
      // the empty box [lo, hi) in voxels: step through it without loads
      const int r = 4 * (D - 1);
      const int lo0 = 4 * bx - r, lo1 = 4 * by - r, lo2 = 4 * bz - r;
      const int hi0 = 4 * bx + 4 + r, hi1 = 4 * by + 4 + r, hi2 = 4 * bz + 4 + r;
      bool in = true;
      for (;;) {
        if (vmax[0] < vmax[1]) in = (vmax[0] < vmax[2]) ? voxel_axis_step<0>(N) : voxel_axis_step<2>(N);
        else in = (vmax[1] < vmax[2]) ? voxel_axis_step<1>(N) : voxel_axis_step<2>(N);
        near_ = far_;
        if (!in) break;
        ++steps;
        far_ = fminf(fminf(vmax[0], vmax[1]), vmax[2]);
        if (vc[0] < lo0 || vc[0] >= hi0 || vc[1] < lo1 || vc[1] >= hi1 || vc[2] < lo2 || vc[2] >= hi2) break;
      }
      if (!in) { tile = -1; continue; }
      --steps;             // counted again when the voxel past the box is examined
      entry_pending = true;  // examine the voxel past the box without stepping
    }
  }
};

// One sample inside an occupied voxel.
struct Sample {
  uint32_t rec;
  int tile;
  float f[3];      // position inside the voxel, clamped to [0,1]
  float interval;  // world length represented by the sample
  float t;         // world distance from the ray origin
};

// Produces the next sample of the ray; false when the ray left the scene.
__device__ __forceinline__ bool next_sample(const SceneDev& S, RayState& R, Sample& s) {
  for (;;) {
    if (R.in_voxel && R.z < R.far_) {
      s.rec = R.rec;
      s.tile = R.tile;
      for (int a = 0; a < 3; ++a) {
        float pos = fadd(R.q[a], fmul(R.z, R.d[a]));
        float f = fsub(fmul(pos, S.inv_voxel), (float)R.vc[a]);
        s.f[a] = fminf(fmaxf(f, 0.0f), 1.0f);
      }
      s.interval = fminf(S.step_len, fsub(R.far_, R.z));
      s.t = fadd(R.t_in, R.z);
      R.z = march_next(R.z, S.step_len);
      return true;
    }
    if (!R.next_voxel(S)) return false;
    R.in_voxel = true;
    R.z = R.near_;
  }
}

__device__ __forceinline__ void trilinear_weights(const float f[3], float w[8]) {
  float wx[2] = {1.0f - f[0], f[0]}, wy[2] = {1.0f - f[1], f[1]}, wz[2] = {1.0f - f[2], f[2]};
#pragma unroll
  for (int k = 0; k < 8; ++k) w[k] = wx[(k >> 2) & 1] * wy[(k >> 1) & 1] * wz[k & 1];
}

__device__ __forceinline__ float softplusf(float x) { return fmaxf(x, 0.0f) + log1pf(expf(-fabsf(x))); }
__device__ __forceinline__ float sigmoidf_(float x) { return 1.0f / (1.0f + expf(-x)); }

// Transmittance arithmetic of the render march.  Its exponential and log1p
// are this library's own single-precision functions, evaluated with explicit
// round-to-nearest operations and fused multiply-adds only where written, so
// that the host restatement (the same operations in the same order) gives
// the same bits: transmittance, and with it the early-stop decision, is then
// identical on both sides.
//
// e^x for x <= 0: Cody-Waite reduction x = k ln2 + r with ln2 split into a
// 16-bit head and a tail, |r| <= ln2/2; the degree-7 Taylor polynomial of e^r
// (truncation error below 2^-26 on that interval) by Horner's rule in fused
// multiply-adds; scaling by 2^k through the exponent field.  Below -80 the
// result is 0 (e^-80 < 2^-115); NaN propagates.  Error below 1 ulp.
__device__ __forceinline__ float exp_nonpos(float x) {
  if (!(x >= -80.0f)) return x != x ? x : 0.0f;
  const float k = rintf(__fmul_rn(x, 1.44269504088896341f));
  float r = __fmaf_rn(-k, 0.693145751953125f, x);   // ln2 head (exact product)
  r = __fmaf_rn(-k, 1.42860682030941723212e-6f, r);  // ln2 tail
  float p = 1.98412698412698413e-4f;                 // 1/7!
  p = __fmaf_rn(p, r, 1.38888888888888889e-3f);      // 1/6!
  p = __fmaf_rn(p, r, 8.33333333333333333e-3f);      // 1/5!
  p = __fmaf_rn(p, r, 4.16666666666666667e-2f);      // 1/4!
  p = __fmaf_rn(p, r, 1.66666666666666667e-1f);      // 1/3!
  p = __fmaf_rn(p, r, 0.5f);
  p = __fmaf_rn(p, r, 1.0f);
  p = __fmaf_rn(p, r, 1.0f);
  return __fmul_rn(p, __int_as_float(((int)k + 127) << 23));  // k in [-116, 0]: an exact power of two
}

// log(1 + y) for y in [0, 1]: 2 atanh(s) with s = y / (2 + y) in [0, 1/3],
// atanh(s) = s (1 + s^2/3 + s^4/5 + ... + s^18/19) (next term below 2^-35).
// Error below 3 ulp (the roundings of 2 + y, the quotient and the product).
__device__ __forceinline__ float log1p_unit(float y) {
  const float s = __fdiv_rn(y, __fadd_rn(2.0f, y));
  const float s2 = __fmul_rn(s, s);
  float q = 5.26315789473684211e-2f;             // 1/19
  q = __fmaf_rn(q, s2, 5.88235294117647059e-2f);  // 1/17
  q = __fmaf_rn(q, s2, 6.66666666666666667e-2f);  // 1/15
  q = __fmaf_rn(q, s2, 7.69230769230769231e-2f);  // 1/13
  q = __fmaf_rn(q, s2, 9.09090909090909091e-2f);  // 1/11
  q = __fmaf_rn(q, s2, 1.11111111111111111e-1f);  // 1/9
  q = __fmaf_rn(q, s2, 1.42857142857142857e-1f);  // 1/7
  q = __fmaf_rn(q, s2, 2.0e-1f);                  // 1/5
  q = __fmaf_rn(q, s2, 3.33333333333333333e-1f);  // 1/3
  q = __fmaf_rn(q, s2, 1.0f);
  const float t = __fmul_rn(s, q);
  return __fadd_rn(t, t);
}

// softplus(x) = max(x, 0) + log(1 + e^-|x|)
__device__ __forceinline__ float softplus_march(float x) {
  return __fadd_rn(fmaxf(x, 0.0f), log1p_unit(exp_nonpos(-fabsf(x))));
}

// Opacity of a sample: 1 - e^(-sigma * interval / voxel).
__device__ __forceinline__ float alpha_march(float sigma, float dv) {
  return __fsub_rn(1.0f, exp_nonpos(__fmul_rn(-sigma, dv)));
}

// Density of a sample: softplus of the trilinear density logit, per voxel
// length; the logit summed corner by corner in order, unfused.
__device__ __forceinline__ float sample_sigma(const SceneDev& S, const Sample& s, float w[8]) {
  trilinear_weights(s.f, w);
  const float4* dp = reinterpret_cast<const float4*>(S.dens + (size_t)s.rec * 8);
  float4 a = __ldg(dp), b = __ldg(dp + 1);
  const float v[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
  float g = __fmul_rn(w[0], v[0]);
#pragma unroll
  for (int k = 1; k < 8; ++k) g = __fadd_rn(g, __fmul_rn(w[k], v[k]));
  return softplus_march(g);
}

// View-direction encoding: [d, sin(2^0 d), cos(2^0 d), ..., sin(2^{L-1} d), cos(2^{L-1} d)]
// (reference Positional_Encoding, training/scripts/networks.py:4-15).
__device__ __forceinline__ void dir_encoding(const float d[3], int L, float* out) {
  out[0] = d[0]; out[1] = d[1]; out[2] = d[2];
  float scale = 1.0f;
  for (int i = 0; i < L; ++i) {
    for (int a = 0; a < 3; ++a) {
      float s, c;
      sincosf(scale * d[a], &s, &c);
      out[3 + 6 * i + a] = s;
      out[3 + 6 * i + 3 + a] = c;
    }
    scale *= 2.0f;
  }
}

// Ray direction of a pixel (reference get_direction, rendering/src/compute_rays.cu:7-17),
// normalised.
__device__ __forceinline__ void camera_dir(const float* c2w, float cx, float cy, float inv_f, int px, int py, float d[3]) {
  float x = fmul(fsub((float)px, cx), inv_f);
  float y = fmul(fsub((float)py, cy), inv_f);
  float r[3];
  for (int a = 0; a < 3; ++a) r[a] = fadd(fadd(fmul(c2w[4 * a + 0], x), fmul(c2w[4 * a + 1], y)), c2w[4 * a + 2]);
  float n = __fsqrt_rn(fadd(fadd(fmul(r[0], r[0]), fmul(r[1], r[1])), fmul(r[2], r[2])));
  for (int a = 0; a < 3; ++a) d[a] = fdiv(r[a], n);
}

}  // namespace snisr
