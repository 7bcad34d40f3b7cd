// Render kernels: ray generation with the proxy-mesh start, the plain FP32
// form (one thread per ray, CUDA-core MLP) and the batched tensor-core form
// (warp-compacted traversal -> per-tile bucketing -> tcgen05 MLP).
#include <cuda_fp16.h>

#include "device_common.cuh"
#include "kernels.h"
#include "proxy.cuh"
#include "tc_ptx.cuh"

namespace snisr {

namespace {

constexpr unsigned kFull = 0xFFFFFFFFu;
constexpr uint32_t kInvalid = 0xFFFFFFFFu;

// {lo, hi} -> packed FP16 pair (round to nearest)
__device__ __forceinline__ uint32_t pack_h2(float lo, float hi) {
  uint32_t d;
  asm("cvt.rn.f16x2.f32 %0, %1, %2;" : "=r"(d) : "f"(hi), "f"(lo));
  return d;
}
// {max(lo,0), max(hi,0)} -> packed FP16 pair
__device__ __forceinline__ uint32_t pack_relu_h2(float lo, float hi) {
  uint32_t d;
  asm("cvt.rn.relu.f16x2.f32 %0, %1, %2;" : "=r"(d) : "f"(hi), "f"(lo));
  return d;
}

__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// ---------------------------------------------------------------------------
// Ray generation: direction, proxy-mesh start distance, FP16 view encoding.
// ---------------------------------------------------------------------------
__global__ void raygen_kernel(SceneDev S, CamDev cam, const float* __restrict__ origins,
                              const float* __restrict__ dirs, int64_t n, float4* ray_o, float4* ray_d,
                              uint4* enc, int want_enc, RayOrder ord) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    float o[3], d[3];
    const int64_t pix = ray_pixel(i, ord);
    if (dirs) {
      for (int a = 0; a < 3; ++a) { o[a] = origins[3 * i + a]; d[a] = dirs[3 * i + a]; }
    } else {
      int py = (int)(pix / cam.W), px = (int)(pix - (int64_t)py * cam.W);
      camera_dir(cam.c2w, cam.cx, cam.cy, cam.inv_f, px, py, d);
      o[0] = cam.c2w[3]; o[1] = cam.c2w[7]; o[2] = cam.c2w[11];
    }
    float ts = 0.0f;
    if (S.has_mesh) {
      int tri;
      float th = bvh_nearest(S, o, d, tri);
      if (th >= 0.0f) ts = fmaxf(fsub(th, S.start_offset), 0.0f);
    }
    ray_o[i] = make_float4(o[0], o[1], o[2], 0.0f);
    ray_d[i] = make_float4(d[0], d[1], d[2], ts);
    if (want_enc) {
      // the FP16 view encoding of the tensor-core form: [d, sin(2^i d),
      // cos(2^i d)] for i < 4 from one sincosf per axis and double-angle steps
      // (a few FP32 ulps at 2^3, far below the encoding's FP16 rounding)
      float e[27], sn[3], cs[3];
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        e[a] = d[a];
        sincosf(d[a], &sn[a], &cs[a]);
      }
#pragma unroll
      for (int f = 0; f < 4; ++f) {
#pragma unroll
        for (int a = 0; a < 3; ++a) {
          e[3 + 6 * f + a] = sn[a];
          e[6 + 6 * f + a] = cs[a];
          const float s2 = 2.f * sn[a] * cs[a], c2 = (cs[a] - sn[a]) * (cs[a] + sn[a]);
          sn[a] = s2;
          cs[a] = c2;
        }
      }
      __align__(16) __half h[32];
      for (int k = 0; k < 32; ++k) h[k] = __float2half_rn(k < 27 ? e[k] : 0.0f);
      const uint4* src = reinterpret_cast<const uint4*>(h);
      for (int k = 0; k < 4; ++k) enc[4 * pix + k] = src[k];
    }
  }
}

__global__ void proxy_kernel(SceneDev S, const float* __restrict__ origins, const float* __restrict__ dirs,
                             int64_t n, float* t_out, int32_t* tri_out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    float o[3] = {origins[3 * i], origins[3 * i + 1], origins[3 * i + 2]};
    float d[3] = {dirs[3 * i], dirs[3 * i + 1], dirs[3 * i + 2]};
    int tri = -1;
    float t = S.has_mesh ? bvh_nearest(S, o, d, tri) : -1.0f;
    t_out[i] = t;
    tri_out[i] = tri;
  }
}

// ---------------------------------------------------------------------------
// Occupied-voxel sequences (no transmittance), for parity checks.
// ---------------------------------------------------------------------------
__global__ void trace_kernel(SceneDev S, const float4* __restrict__ ray_o, const float4* __restrict__ ray_d,
                             int64_t n, int K, int32_t* visited, int32_t* count) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    float4 o4 = ray_o[i], d4 = ray_d[i];
    float o[3] = {o4.x, o4.y, o4.z}, d[3] = {d4.x, d4.y, d4.z};
    RayState R;
    int c = 0;
    if (R.init(S, o, d, d4.w)) {
      while (R.next_voxel(S)) {
        if (c < K) visited[i * K + c] = (int32_t)R.rec;
        ++c;
      }
    }
    for (int k = c; k < K; ++k) visited[i * K + k] = -1;
    count[i] = c;
  }
}

// ---------------------------------------------------------------------------
// Plain FP32 form: one thread per ray, FP32 features/weights, CUDA-core MLP.
// Weight layout per tile: for each Linear, W[out][round4(in)] then b[round4(out)].
// ---------------------------------------------------------------------------
template <int KIN, int H, int L>
__device__ __forceinline__ void mlp_plain(const float* __restrict__ P, const float* x, float out[3]) {
  constexpr int KP = (KIN + 3) & ~3;
  float h[H];
  {
    const float4* W = reinterpret_cast<const float4*>(P);
#pragma unroll
    for (int j = 0; j < H; ++j) {
      float acc = 0.0f;
#pragma unroll
      for (int i = 0; i < KP / 4; ++i) {
        float4 w = __ldg(W + j * (KP / 4) + i);
        acc = fmaf(w.x, x[4 * i], acc);
        acc = fmaf(w.y, x[4 * i + 1], acc);
        acc = fmaf(w.z, x[4 * i + 2], acc);
        acc = fmaf(w.w, x[4 * i + 3], acc);
      }
      h[j] = acc;
    }
    P += H * KP;
#pragma unroll
    for (int j = 0; j < H; ++j) h[j] = fmaxf(h[j] + __ldg(P + j), 0.0f);
    P += H;
  }
#pragma unroll
  for (int l = 1; l < L; ++l) {
    float g[H];
    const float4* W = reinterpret_cast<const float4*>(P);
#pragma unroll
    for (int j = 0; j < H; ++j) {
      float acc = 0.0f;
#pragma unroll
      for (int i = 0; i < H / 4; ++i) {
        float4 w = __ldg(W + j * (H / 4) + i);
        acc = fmaf(w.x, h[4 * i], acc);
        acc = fmaf(w.y, h[4 * i + 1], acc);
        acc = fmaf(w.z, h[4 * i + 2], acc);
        acc = fmaf(w.w, h[4 * i + 3], acc);
      }
      g[j] = acc;
    }
    P += H * H;
#pragma unroll
    for (int j = 0; j < H; ++j) h[j] = fmaxf(g[j] + __ldg(P + j), 0.0f);
    P += H;
  }
  const float4* W = reinterpret_cast<const float4*>(P);
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    float acc = 0.0f;
#pragma unroll
    for (int i = 0; i < H / 4; ++i) {
      float4 w = __ldg(W + c * (H / 4) + i);
      acc = fmaf(w.x, h[4 * i], acc);
      acc = fmaf(w.y, h[4 * i + 1], acc);
      acc = fmaf(w.z, h[4 * i + 2], acc);
      acc = fmaf(w.w, h[4 * i + 3], acc);
    }
    out[c] = acc;
  }
  P += 3 * H;
  for (int c = 0; c < 3; ++c) out[c] += __ldg(P + c);
}

template <int F, int H, int L>
__global__ void __launch_bounds__(128) render_plain_kernel(SceneDev S, const float4* __restrict__ ray_o,
                                                           const float4* __restrict__ ray_d, int64_t n,
                                                           float* rgb, float* depth, float* opac, RayOrder ord) {
  constexpr int KIN = F + 27;
  constexpr int KP = (KIN + 3) & ~3;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    float4 o4 = ray_o[i], d4 = ray_d[i];
    float o[3] = {o4.x, o4.y, o4.z}, d[3] = {d4.x, d4.y, d4.z};
    float x[KP];
#pragma unroll
    for (int k = 0; k < KP; ++k) x[k] = 0.0f;
    dir_encoding(d, 4, x + F);
    float C[3] = {0.f, 0.f, 0.f}, D = 0.f, T = 1.f;
    RayState R;
    if (R.init(S, o, d, d4.w)) {
      Sample s;
      while (next_sample(S, R, s)) {
        float w[8];
        float sig = sample_sigma(S, s, w);
        float alpha = alpha_march(sig, fmul(s.interval, S.inv_voxel));
        float wt = T * alpha;
        const float4* fp = S.feat32 + (size_t)s.rec * (F / 4) * 8;
#pragma unroll
        for (int g = 0; g < F / 4; ++g) {
          float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
          for (int k = 0; k < 8; ++k) {
            float4 v = __ldg(fp + g * 8 + k);
            acc.x = fmaf(w[k], v.x, acc.x); acc.y = fmaf(w[k], v.y, acc.y);
            acc.z = fmaf(w[k], v.z, acc.z); acc.w = fmaf(w[k], v.w, acc.w);
          }
          x[4 * g] = acc.x; x[4 * g + 1] = acc.y; x[4 * g + 2] = acc.z; x[4 * g + 3] = acc.w;
        }
        float out[3];
        mlp_plain<KIN, H, L>(S.mlp_plain + (size_t)s.tile * S.plain_stride, x, out);
        for (int c = 0; c < 3; ++c) C[c] += wt * sigmoidf_(out[c]);
        D = fadd(D, fmul(wt, s.t));
        T *= (1.0f - alpha);
        if (T < S.early_stop) break;
      }
    }
    const int64_t p = ray_pixel(i, ord);
    rgb[3 * p] = C[0]; rgb[3 * p + 1] = C[1]; rgb[3 * p + 2] = C[2];
    depth[p] = D;
    opac[p] = 1.0f - T;
  }
}

// ---------------------------------------------------------------------------
// Batched tensor-core form, stage 1: traversal with per-warp compaction.
// Each lane marches one ray (camera frames: a warp marches a 4 x 8 pixel
// tile, RayOrder); every round the warp converges, ballots the
// lanes that produced a sample and writes them to consecutive slots of a
// per-warp block of the sample buffer (one global atomic per 256 samples).
// Records and outputs carry the ray's pixel.
// Depth and opacity are final here: density comes from the voxel data, so
// transmittance and early stop do not wait for the MLP.
// ---------------------------------------------------------------------------
constexpr int kTravMaxThreads = 256;  // block size is a tuning knob (multiple of 32)
// traverse_kernel is issue-bound and latency-sensitive: 4 resident 256-thread
// blocks' worth of registers (64 per thread, with some spilling) measured
// 5 % faster than 3 (80 registers) on the 1920x1080 frame and the same on the
// 1280x720 one; 2 (95 registers, no spills) was slower on both.
constexpr uint32_t kBlk = 256;

__global__ void __launch_bounds__(kTravMaxThreads, 4) traverse_kernel(SceneDev S, const float4* __restrict__ ray_o,
                                                                const float4* __restrict__ ray_d, int64_t n,
                                                                SampleRec* recs, uint32_t cap, uint32_t* blk_count,
                                                                int* ctrl, float* depth, float* opac, RayOrder ord) {
  // per-warp tile histogram (no CTA-wide barrier: warps finish independently)
  extern __shared__ uint32_t hist_all[];
  const int lane = threadIdx.x & 31;
  uint32_t* hist = hist_all + (threadIdx.x >> 5) * S.num_tiles;
  for (int t = lane; t < S.num_tiles; t += 32) hist[t] = 0;
  __syncwarp();
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  RayState R;
  bool live = false;
  float T = 1.0f, D = 0.0f;
  if (i < n) {
    float4 o4 = ray_o[i], d4 = ray_d[i];
    float o[3] = {o4.x, o4.y, o4.z}, d[3] = {d4.x, d4.y, d4.z};
    live = R.init(S, o, d, d4.w);
  }
  const int64_t pix = ray_pixel(i, ord);
  const uint32_t ray_id = (uint32_t)pix;
  uint32_t cur = 0, end = 0;  // warp-uniform block cursor
  // Each round a live lane emits the samples of one voxel (up to kVoxSamples:
  // a voxel holds at most 4 samples at 0.5-voxel steps), so that a voxel's
  // samples are consecutive records and later share their corner loads.
  constexpr int kVoxSamples = 4;
  for (;;) {
    uint32_t vrec = 0, vtile = 0;
    float vf[kVoxSamples][3], vw[kVoxSamples];
    int ns = 0;
    if (live) {
      Sample s;
#pragma unroll
      for (int j = 0; j < kVoxSamples; ++j) {
        if (j > 0 && !(live && R.in_voxel && R.z < R.far_)) break;
        if (!next_sample(S, R, s)) {
          live = false;
          break;
        }
        float w[8];
        const float sig = sample_sigma(S, s, w);
        const float alpha = alpha_march(sig, fmul(s.interval, S.inv_voxel));
        const float wt = T * alpha;
        D = fadd(D, fmul(wt, s.t));
        T *= (1.0f - alpha);
        vrec = s.rec;
        vtile = (uint32_t)s.tile;
        vf[j][0] = s.f[0]; vf[j][1] = s.f[1]; vf[j][2] = s.f[2];
        vw[j] = wt;
        ns = j + 1;
        if (T < S.early_stop) {
          live = false;
          break;
        }
      }
    }
    // warp prefix sum of the per-lane sample counts
    uint32_t pre = (uint32_t)ns;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(kFull, pre, o);
      if (lane >= o) pre += y;
    }
    const uint32_t cnt = __shfl_sync(kFull, pre, 31);
    if (cnt == 0) break;
    pre -= (uint32_t)ns;  // exclusive
    const uint32_t base_old = cur;
    uint32_t rem, nb = 0;
    if (cur + cnt > end) {
      // the open block (if any) is filled to the end by this round
      if (lane == 0 && end != 0 && (end - kBlk) / kBlk < (cap + kBlk - 1) / kBlk) blk_count[(end - kBlk) / kBlk] = kBlk;
      if (lane == 0) nb = (uint32_t)atomicAdd(ctrl + CTRL_RESERVED, (int)kBlk);
      nb = __shfl_sync(kFull, nb, 0);
      rem = end - cur;
      cur = nb + (cnt - rem);
      end = nb + kBlk;
    } else {
      rem = cnt;  // everything fits in the open block
      cur += cnt;
    }
    bool dropped = false;
#pragma unroll
    for (int j = 0; j < kVoxSamples; ++j) {
      if (j < ns) {
        const uint32_t k = pre + (uint32_t)j;
        const uint32_t slot = k < rem ? base_old + k : nb + (k - rem);
        if (slot < cap) {
          recs[slot] = pack_sample(vrec, ray_id, vw[j], vf[j]);
        } else {
          dropped = true;
        }
      }
    }
    if (dropped) atomicOr(S.err, ERR_OVERFLOW);
    // tile histogram: one add per group of lanes that emitted samples of the same tile
    const unsigned mh = __ballot_sync(kFull, ns > 0);
    if (ns > 0) {
      const unsigned g = __match_any_sync(mh, vtile);
      const unsigned tot = __reduce_add_sync(g, (unsigned)ns);
      if (lane == __ffs(g) - 1) atomicAdd(hist + vtile, tot);
    }
  }
  if (lane == 0 && end != 0 && (end - kBlk) / kBlk < (cap + kBlk - 1) / kBlk)
    blk_count[(end - kBlk) / kBlk] = cur - (end - kBlk);
  if (i < n) {
    depth[pix] = D;
    opac[pix] = 1.0f - T;
  }
  unsigned long long st = (i < n) ? R.steps : 0u;
#pragma unroll
  for (int sh = 16; sh > 0; sh >>= 1) st += __shfl_xor_sync(kFull, st, sh);
  if (lane == 0 && st) atomicAdd(reinterpret_cast<unsigned long long*>(ctrl + CTRL_STEPS), st);
  __syncwarp();
  for (int t = lane; t < S.num_tiles; t += 32)
    if (hist[t]) atomicAdd(ctrl + CTRL_HEADER + t, (int)hist[t]);
}

// Stage 2: per-tile offsets and 128-sample chunk offsets (one thread; the
// tile count is small).  Layout after the header: count[NT], off[NT+1],
// coff[NT+1], cursor[NT].  When the frame produced more samples than the
// buffer holds (the traversal has flagged the overflow), every offset and
// the chunk count are zero: the scatter stays inside the buffer and the MLP
// does no work for the invalid frame.
__global__ void scan_kernel(int* ctrl, int NT, uint32_t cap) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  int* cnt = ctrl + CTRL_HEADER;
  int* off = cnt + NT;
  int* coff = off + NT + 1;
  int* cursor = coff + NT + 1;
  int o = 0, c = 0;
  for (int t = 0; t < NT; ++t) {
    off[t] = o;
    coff[t] = c;
    o += cnt[t];
    c += (cnt[t] + 127) / 128;
    cursor[t] = 0;
  }
  off[NT] = o;
  coff[NT] = c;
  ctrl[CTRL_CHUNKS] = c;
  ctrl[CTRL_SAMPLES] = o;
  if ((uint32_t)o > cap) {
    for (int t = 0; t <= NT; ++t) off[t] = coff[t] = 0;
    ctrl[CTRL_CHUNKS] = ctrl[CTRL_SAMPLES] = 0;
  }
}

// Stage 3: move samples into per-tile order.  A CTA takes a slab of
// kScatU * 256 consecutive record slots, ranks its records per tile with
// warp-aggregated shared-memory counters, reserves one range per tile with a
// single global atomic, and writes.  Slot s is valid iff s % 256 <
// blk_count[s / 256] (per-warp blocks are filled in order; only each warp's
// last block is partial).  Consecutive records of one tile keep their order
// within a warp (samples of one voxel stay adjacent).  A record's tile is the
// last tile whose first voxel id does not exceed the record's (binary search
// over the tiles' first ids in shared memory).
constexpr int kScatThreads = 256, kScatU = 4;
__global__ void __launch_bounds__(kScatThreads) scatter_kernel(SceneDev S, const SampleRec* __restrict__ recs,
                                                               uint32_t cap, const uint32_t* __restrict__ blk_count,
                                                               int* ctrl, int NT, SampleRec* sorted) {
  extern __shared__ uint32_t sh_scat[];  // count[NT], base[NT], first voxel id[NT]
  uint32_t* scount = sh_scat;
  uint32_t* sbase = sh_scat + NT;
  uint32_t* sfirst = sh_scat + 2 * NT;
  const int tid = threadIdx.x, lane = tid & 31;
  for (int t = tid; t < NT; t += kScatThreads) sfirst[t] = S.occ[(size_t)t * S.words_per_tile].base;
  auto tile_of = [&](uint32_t rec) {
    int lo = 0, hi = NT;  // largest t with sfirst[t] <= rec
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (sfirst[mid] <= rec) lo = mid; else hi = mid;
    }
    return (uint32_t)lo;
  };
  const uint32_t total = min((uint32_t)ctrl[CTRL_RESERVED], cap);
  const int* off = ctrl + CTRL_HEADER + NT;
  int* cursor = ctrl + CTRL_HEADER + NT + (NT + 1) + (NT + 1);
  constexpr uint32_t kSlab = kScatU * kScatThreads;
  for (uint32_t slab = blockIdx.x * kSlab; slab < total; slab += gridDim.x * kSlab) {
    for (int t = tid; t < NT; t += kScatThreads) scount[t] = 0;
    __syncthreads();
    uint4 a[kScatU];
    uint32_t rank[kScatU], tl[kScatU];
    bool valid[kScatU];
#pragma unroll
    for (int u = 0; u < kScatU; ++u) {
      const uint32_t sidx = slab + u * kScatThreads + tid;
      valid[u] = sidx < total && (sidx % kBlk) < __ldg(blk_count + sidx / kBlk);
      if (valid[u]) a[u] = __ldg(reinterpret_cast<const uint4*>(recs + sidx));
    }
#pragma unroll
    for (int u = 0; u < kScatU; ++u) {
      const unsigned m = __ballot_sync(kFull, valid[u]);
      if (valid[u]) {
        tl[u] = tile_of(a[u].x);
        const unsigned g = __match_any_sync(m, tl[u]);
        const int leader = __ffs(g) - 1;
        uint32_t r0 = 0;
        if (lane == leader) r0 = atomicAdd(scount + tl[u], (uint32_t)__popc(g));
        r0 = __shfl_sync(g, r0, leader);
        rank[u] = r0 + __popc(g & lanemask_lt());
      }
    }
    __syncthreads();
    for (int t = tid; t < NT; t += kScatThreads)
      if (scount[t]) sbase[t] = (uint32_t)atomicAdd(cursor + t, (int)scount[t]);
    __syncthreads();
#pragma unroll
    for (int u = 0; u < kScatU; ++u) {
      if (valid[u]) {
        const uint32_t t = tl[u];
        *reinterpret_cast<uint4*>(sorted + off[t] + sbase[t] + rank[u]) = a[u];
      }
    }
    __syncthreads();  // counts are reset for the next slab
  }
}

// Tensor-memory columns of one MLP CTA: the H-column accumulator and the
// H/2-column A operand of the hidden layers (two FP16 values per column),
// rounded up to the allocation granularity (a power of two >= 32).
constexpr int mlp_tmem_cols(int H) { return H + H / 2 <= 64 ? 64 : 128; }

// Stage 4: per-tile MLP on tcgen05.  One CTA = 4 warps; each chunk is 128
// samples of one tile.  The first layer's A operand (gathered trilinear
// features + view encoding) is written by the threads into shared memory in
// the 128-byte swizzled K-major layout; the hidden activations stay in tensor
// memory: each thread reads its row of the accumulator, applies ReLU, packs
// FP16 pairs and stores them into its own lane of the A-operand columns
// (tcgen05.st), which the next layer's MMA reads as a TMEM A operand -- no
// shared-memory traffic for them.  Weights arrive by bulk copy (TMA) once per
// tile change; accumulators live in tensor memory (H columns x 128 lanes).
// Every Linear, the output one included (N = 16, 3 used), is FP16 x FP16 ->
// FP32 on tcgen05; biases enter as one extra K = 16 step (A = 1/16
// everywhere, B slice = 16 copies of the bias).  The epilogue applies ReLU
// (hidden) or sigmoid + compositing weight (output).  Persistent CTAs (four
// per SM) pull chunks from a device work queue and run a software pipeline:
// the next chunk's A rows are gathered into registers during the current
// chunk's MMA chain.
template <int F, int H, int L>
__global__ void __launch_bounds__(128, 4) mlp_tc_kernel(SceneDev S, const SampleRec* __restrict__ sorted, int* ctrl,
                                                     int NT, const uint4* __restrict__ enc,
                                                     const uint8_t* __restrict__ wimg, int img_stride, int img_bytes,
                                                     float* rgb) {
  constexpr int G = F / 8;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* base = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  // shared memory: A tile (16 KB) | weight image of the current tile | ones atom | barriers
  uint8_t* A0 = base;            // layer input: features+encoding, then hidden activations
  uint8_t* Wsm = base + 16384;   // tc_image layout (see tc_image_bytes)
  uint8_t* ones = Wsm + ((img_bytes + 1023) & ~1023);  // 1 KB atom of 1/16 (8 rows x 128 B)
  uint64_t* bars = reinterpret_cast<uint64_t*>(ones + 1024);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2);
  int* chunk_slot = reinterpret_cast<int*>(tmem_slot + 1);
  const uint32_t wbar = tc::smem_addr(bars), mbar = tc::smem_addr(bars + 1);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  if (tid == 0) {
    tc::mbar_init(wbar, 1);
    tc::mbar_init(mbar, 1);
    tc::fence_mbar_init();
  }
  if (warp == 0) {
    tc::tmem_alloc(tc::smem_addr(tmem_slot), mlp_tmem_cols(H));
    tc::tmem_relinquish();
  }
  // every fp16 of the atom is 1/16: D += (1/16) * sum_{k<16} bias = bias (exact)
  for (int k = tid; k < 1024 / 16; k += blockDim.x)
    reinterpret_cast<uint4*>(ones)[k] = make_uint4(0x2C002C00u, 0x2C002C00u, 0x2C002C00u, 0x2C002C00u);
  tc::fence_proxy_async();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *tmem_slot;
  const uint32_t idesc = tc::idesc_f16(H, 0);
  const uint32_t idesc_out = tc::idesc_f16(16, 0);
  // A operand of the bias step: the 1 KB atom for all 16 row groups (stride 0)
  const uint64_t ones_desc = tc::sdesc_sw128_sbo(tc::smem_addr(ones), 0);
  const int* off = ctrl + CTRL_HEADER + NT;
  const int* coff = off + NT + 1;
  const int total_chunks = ctrl[CTRL_CHUNKS];
  int cur_tile = -1;
  uint32_t wphase = 0, mphase = 0;
  bool failed = false;
  tc::Drain drain;

  // A chunk: its tile and its rows [row0, row0 + cnt) of the tile-sorted
  // sample records (locate: binary search of the per-tile chunk offsets).
  // load_row: thread tid's row record of a chunk (32 rows per warp).
  struct ChunkRows {
    int c, tile, row0, cnt;
  };
  auto locate = [&](int c) {
    ChunkRows r{c, 0, 0, 0};
    if (c >= total_chunks) return r;
    int lo = 0, hi = NT;  // largest t with coff[t] <= c
    while (hi - lo > 1) {
      int mid = (lo + hi) >> 1;
      if (__ldg(coff + mid) <= c) lo = mid; else hi = mid;
    }
    r.tile = lo;
    r.row0 = __ldg(off + lo) + (c - __ldg(coff + lo)) * 128;
    r.cnt = min(128, __ldg(off + lo + 1) - r.row0);
    return r;
  };
  auto load_row = [&](const ChunkRows& r, uint4& ra) {
    ra = make_uint4(kInvalid, 0, 0, 0);
    if (r.c < total_chunks && tid < r.cnt) ra = __ldg(reinterpret_cast<const uint4*>(sorted + r.row0 + tid));
  };
  // Software pipeline: while chunk c runs its MMA chain, the threads gather
  // chunk c + 1's A rows into registers, a share of the row groups during
  // each layer's MMA, and write them into the A tile once chunk c's last
  // MMA has read it.  Chunks are claimed two ahead (slots rotate by three),
  // so the next chunk is known before its gather starts; thread tid holds
  // row tid's record of the current and of the next chunk.
  //
  // Gather of one row group: RPI = 32/G rows per warp; lane (g = lane / RPI,
  // row = lane % RPI) owns channel group g of one row.  The FP16 cache is
  // corner-major ([voxel][corner][group] x 16 B), so for each corner the G
  // lanes of a row read one contiguous G*16-byte slice: a load instruction
  // touches RPI cache lines, not 32.  Each lane interpolates its 8 channels
  // over the 8 corners in FP32; its row's view encoding chunks come along.
  // A row holds chunks [0,G) features, [G,G+4) view encoding, the rest 0.
  constexpr int RPI = 32 / G, NENC = 4 / G;
  const int my_g = lane / RPI, my_row = lane % RPI;
  // A row group in flight: the corner and encoding loads of one group are
  // issued one layer before they are interpolated (gather_issue at layer l,
  // gather_finish at layer l + 1), so their latency hides behind a whole
  // layer's MMA and epilogue instead of stalling the issuing warp.
  struct Pending {
    bool valid;
    float fx, fy, fz;
    uint4 cv[8];
    uint4 e[NENC];
  };
  auto gather_issue = [&](int it, const uint4& ra, Pending& p) {
    const int src = it * RPI + my_row;
    const uint32_t rec = __shfl_sync(kFull, ra.x, src);
    const uint32_t ray = sample_pix(__shfl_sync(kFull, ra.y, src));
    const uint32_t w_fx = __shfl_sync(kFull, ra.z, src), fy_fz = __shfl_sync(kFull, ra.w, src);
    p.fx = sample_pos(w_fx >> 16);
    p.fy = sample_pos(fy_fz & 0xFFFFu);
    p.fz = sample_pos(fy_fz >> 16);
    p.valid = rec != kInvalid;
    if (p.valid) {
      const uint4* fp = S.feat16 + (size_t)rec * 8 * G + my_g;
#pragma unroll
      for (int k = 0; k < 8; ++k) p.cv[k] = __ldg(fp + k * G);
#pragma unroll
      for (int j = 0; j < NENC; ++j) p.e[j] = __ldg(enc + (size_t)ray * 4 + my_g + j * G);
    }
  };
  // interpolates a group in flight and stores it into rows it*RPI.. of this
  // warp's slice of the A tile (8 consecutive rows per 8-lane phase:
  // conflict-free); chunks [0,G) features, [G,G+4) view encoding, the rest 0
  auto gather_finish = [&](int it, const Pending& p) {
    uint4 f = make_uint4(0, 0, 0, 0);
    uint4 e[NENC];
#pragma unroll
    for (int j = 0; j < NENC; ++j) e[j] = make_uint4(0, 0, 0, 0);
    if (p.valid) {
#pragma unroll
      for (int j = 0; j < NENC; ++j) e[j] = p.e[j];
      // channel pairs accumulate with packed FP32x2 fused multiply-adds (two
      // round-to-nearest FMAs per instruction: the same results as scalar FMAs)
      uint64_t acc2[4] = {0, 0, 0, 0};
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        const float wk = ((k & 4) ? p.fx : 1.0f - p.fx) * ((k & 2) ? p.fy : 1.0f - p.fy) *
                         ((k & 1) ? p.fz : 1.0f - p.fz);
        const uint64_t w2 = f32x2(wk, wk);
        const __half2* hv = reinterpret_cast<const __half2*>(&p.cv[k]);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const float2 pp = __half22float2(hv[q]);
          acc2[q] = ffma2(w2, f32x2(pp.x, pp.y), acc2[q]);
        }
      }
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        float lo, hi;
        split_f32x2(acc2[q], lo, hi);
        (&f.x)[q] = pack_h2(lo, hi);
      }
    }
    const int r = warp * 32 + it * RPI + my_row;
    *reinterpret_cast<uint4*>(A0 + tc::sw128_offset(r, my_g)) = f;
#pragma unroll
    for (int j = 0; j < NENC; ++j) *reinterpret_cast<uint4*>(A0 + tc::sw128_offset(r, G + my_g + j * G)) = e[j];
#pragma unroll
    for (int ch = G + 4 + my_g; ch < 8; ch += G)
      *reinterpret_cast<uint4*>(A0 + tc::sw128_offset(r, ch)) = make_uint4(0, 0, 0, 0);
  };
  Pending pend;

  if (tid == 0) {
    chunk_slot[0] = atomicAdd(ctrl + CTRL_WORK, 1);
    chunk_slot[1] = atomicAdd(ctrl + CTRL_WORK, 1);
  }
  __syncthreads();
  ChunkRows cr = locate(chunk_slot[0]);
  uint4 my_ra;
  load_row(cr, my_ra);
  bool w_pending = false;  // a weight image copy is in flight (block-uniform)
  if (cr.c < total_chunks) {
    // prologue: the first chunk's weights and rows
    if (tid == 0) {
      tc::mbar_arrive_expect_tx(wbar, (uint32_t)img_bytes);
      tc::bulk_g2s(tc::smem_addr(Wsm), wimg + (size_t)cr.tile * img_stride, (uint32_t)img_bytes, wbar);
    }
    cur_tile = cr.tile;
    w_pending = true;
#pragma unroll
    for (int it = 0; it < G; ++it) {
      gather_issue(it, my_ra, pend);
      gather_finish(it, pend);
    }
    tc::fence_proxy_async();
  }
  for (int iter = 0;; ++iter) {
    if (cr.c >= total_chunks) break;
    if (tid == 0) chunk_slot[(iter + 2) % 3] = atomicAdd(ctrl + CTRL_WORK, 1);  // read two iterations later
    const ChunkRows nx = locate(chunk_slot[(iter + 1) % 3]);
    const int cnt = cr.cnt;
    // this thread's output row (ray id, compositing weight)
    const uint32_t my_ray = sample_pix(my_ra.y);
    const float my_wt = sample_weight(my_ra.y, my_ra.z);
    if (w_pending) {
      // one thread polls the barrier; the others wait at bar.sync, which
      // keeps the shared-memory pipe free for the gathers of other CTAs
      bool ok = tid == 0 ? tc::mbar_wait(wbar, wphase) : true;
      wphase ^= 1u;
      w_pending = false;
      if (__syncthreads_or(!ok)) { failed = true; drain.set(wbar, wphase ^ 1u); break; }
    } else {
      __syncthreads();  // the A rows written above are visible to the MMA issuer
    }

    // L hidden Linear layers and the output Linear (N = 16, 3 used), all on
    // the tensor core; each layer's bias enters as one extra K = 16 step.
    // The next chunk's row groups are gathered alongside: group l's loads
    // are issued during layer l and interpolated during layer l + 1, when
    // the A tile (read only by layer 0) is free to take them.
    uint4 nra;
    load_row(nx, nra);
    float out3[3] = {0.f, 0.f, 0.f};
#pragma unroll
    for (int l = 0; l <= L; ++l) {
      if (tid == 0) {
        tc::fence_after_sync();
        const uint32_t a_base = tc::smem_addr(A0);
        const bool last = l == L;
        const uint32_t b_base = tc::smem_addr(Wsm + (last ? L * H * 128 : l * H * 128));
        const uint32_t id = last ? idesc_out : idesc;
        if (l == 0) {  // K = 64 (padded input) from the shared-memory A tile
          for (int kk = 0; kk < 4; ++kk)
            tc::mma_f16(tmem, tc::sdesc_sw128(a_base + 32 * kk), tc::sdesc_sw128(b_base + 32 * kk), id, kk > 0);
        } else {  // K = H from the activations in tensor memory (8 columns per K = 16 step)
          for (int kk = 0; kk < H / 16; ++kk)
            tc::mma_f16_ta(tmem, tmem + H + 8 * kk, tc::sdesc_sw128(b_base + 32 * kk), id, kk > 0);
        }
        const uint32_t bias_tile = tc::smem_addr(Wsm + (last ? L * H * 128 + 2048 + H * 128 : L * H * 128 + 2048));
        tc::mma_f16(tmem, ones_desc, tc::sdesc_sw128(bias_tile + (last ? 0 : 32 * l)), id, 1);
        tc::mma_commit(mbar);
      }
      if (l >= 1 && l - 1 < G) gather_finish(l - 1, pend);  // layer 0 has read the A tile
      if (l < G) gather_issue(l, nra, pend);
      bool ok = tid == 0 ? tc::mbar_wait(mbar, mphase) : true;
      mphase ^= 1u;
      if (__syncthreads_or(!ok)) { failed = true; drain.set(mbar, mphase ^ 1u); break; }
      tc::fence_after_sync();
      const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16);
      if (l < L) {
        // ReLU + FP16 pack of 16 columns at a time into this row's lane of
        // the A-operand columns [H, H + H/2) (16 at a time keeps the
        // registers of the row group in flight free)
#pragma unroll
        for (int part = 0; part < H / 16; ++part) {
          float v[16];
          tc::tmem_ld16(taddr + 16 * part, v);
          tc::tmem_wait_ld();
          uint32_t packed[8];
#pragma unroll
          for (int q = 0; q < 8; ++q) packed[q] = pack_relu_h2(v[2 * q], v[2 * q + 1]);
          tc::tmem_st8(taddr + H + 8 * part, packed);
        }
        tc::tmem_wait_st();
        tc::fence_before_sync();
        __syncthreads();
      } else {
        float v[4];
        tc::tmem_ld4(taddr, v);
        tc::tmem_wait_ld();
        out3[0] = v[0]; out3[1] = v[1]; out3[2] = v[2];
      }
    }
    if (failed) break;
    // chunk c's MMAs are done: the next tile's weights may replace these, and
    // the A tile takes the next chunk's rows
    if (nx.c < total_chunks && nx.tile != cur_tile) {
      if (tid == 0) {
        tc::mbar_arrive_expect_tx(wbar, (uint32_t)img_bytes);
        tc::bulk_g2s(tc::smem_addr(Wsm), wimg + (size_t)nx.tile * img_stride, (uint32_t)img_bytes, wbar);
      }
      cur_tile = nx.tile;
      w_pending = true;
    }
    tc::fence_before_sync();  // output columns read before the next chunk's MMA (barrier at the loop top)
    // the groups not yet interpolated (the one issued during the last layer,
    // and any beyond one per layer)
#pragma unroll
    for (int it = L; it < G; ++it) {
      if (it > L) gather_issue(it, nra, pend);
      gather_finish(it, pend);
    }
    tc::fence_proxy_async();
    if (tid < cnt) {
#pragma unroll
      for (int c3 = 0; c3 < 3; ++c3) atomicAdd(rgb + 3 * (size_t)my_ray + c3, my_wt * sigmoidf_(out3[c3]));
    }
    cr = nx;
    my_ra = nra;
  }
  bool drained = true;
  if (failed && tid == 0) {
    atomicOr(S.err, ERR_TIMEOUT);
    drained = drain.run();
    if (!drained) atomicOr(S.err, ERR_DRAIN);
  }
  tc::fence_before_sync();
  // tensor memory stays allocated when in-flight work did not drain
  if (__syncthreads_or(!drained) == 0 && warp == 0) tc::tmem_dealloc(tmem, mlp_tmem_cols(H));
}

inline int grid_for(int64_t n, int threads, int cap_blocks) {
  int64_t b = (n + threads - 1) / threads;
  if (b < 1) b = 1;
  if (b > cap_blocks) b = cap_blocks;
  return (int)b;
}

template <int F, int H, int L>
cudaError_t render_plain_t(const SceneDev& S, const Workspace& ws, int64_t n, float* rgb, float* depth, float* opac,
                           cudaStream_t st, RayOrder ord) {
  render_plain_kernel<F, H, L><<<grid_for(n, 128, 1 << 20), 128, 0, st>>>(S, ws.ray_o, ws.ray_d, n, rgb, depth, opac,
                                                                        ord);
  return cudaGetLastError();
}

template <int F, int H, int L>
cudaError_t mlp_tc_t(const SceneDev& S, const Workspace& ws, float* rgb, int num_sms, cudaStream_t st) {
  // persistent CTAs per SM: the resident maximum, or fewer when tuned so
  const int smem = 1024 + 16384 + ((ws.wimg_bytes + 1023) & ~1023) + 1024 + 64;
  static int per_sm = 1;  // resident CTAs per SM (same GB300 on every device)
  static unsigned long long done = 0;
  cudaError_t e = once_per_device(&done, [&]() -> cudaError_t {
    cudaError_t r = cudaFuncSetAttribute(mlp_tc_kernel<F, H, L>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (r != cudaSuccess) return r;
    r = cudaFuncSetAttribute(mlp_tc_kernel<F, H, L>, cudaFuncAttributePreferredSharedMemoryCarveout,
                             (int)cudaSharedmemCarveoutMaxShared);
    if (r != cudaSuccess) return r;
    int dev = 0, smem_sm = 0, reserved = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
    cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev);
    cudaFuncAttributes fa{};
    r = cudaFuncGetAttributes(&fa, mlp_tc_kernel<F, H, L>);
    if (r != cudaSuccess) return r;
    const int regs_cta = ((fa.numRegs + 7) & ~7) * 128;
    int n = smem_sm / (smem + reserved);
    n = min(n, 65536 / max(regs_cta, 1));
    n = min(n, 512 / mlp_tmem_cols(H));  // tensor-memory columns per SM
    per_sm = max(1, min(n, 8));
    return cudaSuccess;
  });
  if (e != cudaSuccess) return e;
  const int ctas = ws.tune.mlp_ctas_per_sm > 0 ? min(ws.tune.mlp_ctas_per_sm, per_sm) : per_sm;
  mlp_tc_kernel<F, H, L><<<num_sms * ctas, 128, smem, st>>>(S, ws.sorted, ws.ctrl, S.num_tiles, ws.enc, ws.wimg,
                                                             ws.wimg_stride, ws.wimg_bytes, rgb);
  return cudaGetLastError();
}

}  // namespace

std::mutex& setup_mutex() {
  static std::mutex m;
  return m;
}

bool mlp_shape_supported(int F, int H, int L) {
  return (F == 16 && H == 32 && L == 2) || (F == 32 && H == 64 && L == 3) || (F == 16 && H == 64 && L == 3) ||
         (F == 32 && H == 32 && L == 2);
}

// Per-tile tensor-core image (all tiles 128-byte swizzled, K-major, FP16):
//   [0, L*H*128)               hidden-layer weights W_l [H rows][K <= 64]
//   [+0, +2048)                output weights [16 rows (3 used)][H]
//   [+2048, +2048 + H*128)     hidden biases: row n, K-slice l = 16 x b_l[n]
//   [.., +2048)                output bias: row c, K-slice 0 = 16 x b_out[c]
int tc_image_bytes(int H, int L) { return L * H * 128 + 2048 + H * 128 + 2048; }

cudaError_t launch_raygen(const SceneDev& S, const CamDev* cam, const float* origins, const float* dirs, int64_t n,
                          const Workspace& ws, bool want_enc, cudaStream_t st, RayOrder ord) {
  CamDev c{};
  if (cam) c = *cam;
  if (!cam) ord = RayOrder{};  // the caller's rays keep their order
  raygen_kernel<<<grid_for(n, 128, 1 << 20), 128, 0, st>>>(S, c, origins, dirs, n, ws.ray_o, ws.ray_d, ws.enc,
                                                           want_enc ? 1 : 0, ord);
  return cudaGetLastError();
}

cudaError_t launch_proxy(const SceneDev& S, const float* origins, const float* dirs, int64_t n, float* t, int32_t* tri,
                         cudaStream_t st) {
  proxy_kernel<<<grid_for(n, 128, 1 << 20), 128, 0, st>>>(S, origins, dirs, n, t, tri);
  return cudaGetLastError();
}

cudaError_t launch_trace(const SceneDev& S, const Workspace& ws, int64_t n, int K, int32_t* visited, int32_t* count,
                         cudaStream_t st) {
  trace_kernel<<<grid_for(n, 128, 1 << 20), 128, 0, st>>>(S, ws.ray_o, ws.ray_d, n, K, visited, count);
  return cudaGetLastError();
}

cudaError_t launch_render_plain(const SceneDev& S, const Workspace& ws, int64_t n, float* rgb, float* depth,
                                float* opac, cudaStream_t st, RayOrder ord) {
  const int F = S.feat_dim, H = S.mlp_hidden, L = S.mlp_layers;
  if (F == 16 && H == 32 && L == 2) return render_plain_t<16, 32, 2>(S, ws, n, rgb, depth, opac, st, ord);
  if (F == 32 && H == 64 && L == 3) return render_plain_t<32, 64, 3>(S, ws, n, rgb, depth, opac, st, ord);
  if (F == 16 && H == 64 && L == 3) return render_plain_t<16, 64, 3>(S, ws, n, rgb, depth, opac, st, ord);
  if (F == 32 && H == 32 && L == 2) return render_plain_t<32, 32, 2>(S, ws, n, rgb, depth, opac, st, ord);
  return cudaErrorInvalidValue;
}

cudaError_t launch_render_tc(const SceneDev& S, const Workspace& ws, int64_t n, float* rgb, float* depth, float* opac,
                             int num_sms, cudaStream_t st, cudaEvent_t* ev, RayOrder ord) {
  cudaError_t e = cudaMemsetAsync(ws.ctrl, 0, sizeof(int) * ws.ctrl_words, st);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(rgb, 0, sizeof(float) * 3 * n, st);
  if (e != cudaSuccess) return e;
  if (ev && (e = cudaEventRecord(ev[0], st)) != cudaSuccess) return e;
  const int tt = ws.tune.traverse_threads;
  const int hist_bytes = (int)sizeof(uint32_t) * S.num_tiles * (tt / 32);
  traverse_kernel<<<grid_for(n, tt, 1 << 24), tt, hist_bytes, st>>>(S, ws.ray_o, ws.ray_d, n, ws.recs, ws.cap,
                                                                     ws.blk_count, ws.ctrl, depth, opac, ord);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if (ev && (e = cudaEventRecord(ev[1], st)) != cudaSuccess) return e;
  scan_kernel<<<1, 32, 0, st>>>(ws.ctrl, S.num_tiles, ws.cap);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if (ev && (e = cudaEventRecord(ev[2], st)) != cudaSuccess) return e;
  scatter_kernel<<<num_sms * ws.tune.scatter_blocks_per_sm, kScatThreads, 3 * S.num_tiles * (int)sizeof(uint32_t),
                   st>>>(S, ws.recs, ws.cap, ws.blk_count, ws.ctrl, S.num_tiles, ws.sorted);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if (ev && (e = cudaEventRecord(ev[3], st)) != cudaSuccess) return e;
  const int F = S.feat_dim, H = S.mlp_hidden, L = S.mlp_layers;
  if (F == 16 && H == 32 && L == 2) e = mlp_tc_t<16, 32, 2>(S, ws, rgb, num_sms, st);
  else if (F == 32 && H == 64 && L == 3) e = mlp_tc_t<32, 64, 3>(S, ws, rgb, num_sms, st);
  else if (F == 16 && H == 64 && L == 3) e = mlp_tc_t<16, 64, 3>(S, ws, rgb, num_sms, st);
  else if (F == 32 && H == 32 && L == 2) e = mlp_tc_t<32, 32, 2>(S, ws, rgb, num_sms, st);
  else e = cudaErrorInvalidValue;
  if (e != cudaSuccess) return e;
  if (ev && (e = cudaEventRecord(ev[4], st)) != cudaSuccess) return e;
  return cudaSuccess;
}

}  // namespace snisr
