// Training forward / hand-written adjoint for ray segments inside one tile.
//
// Replaces the autograd graph of the reference's per-tile training step
// (training/scripts/tile/tile.py:667-704: sparse sampling, query_voxel,
// volume_rendering of training/scripts/utils.py:823-837) for the per-corner
// feature model.  Pipeline (all stream-ordered, no host synchronisation):
//
//   count   march each segment (density from the caller's vertex logits)
//   scan    per-ray sample offsets
//   write   march again, one record per sample, ray-contiguous
//   mlp     per-sample colour c_i = sigmoid(MLP(x_i))
//   fwd     per ray  C = sum_i T_i a_i c_i
// backward (reuses the records of the preceding forward call):
//   comp    per ray, reverse walk with suffix sums S_i = sum_{j>i} w_j c_j:
//           dL/dsigma_i = (delta_i/v) [(1-a_i) T_i g.c_i - g.S_i]  -> logit grads (scatter)
//           dL/do_i = g (T_i a_i) c_i (1-c_i)
//   mlp     recompute x_i and the activations, back-propagate -> feature grads (scatter)
//   dW      dW_l = sum_i delta_l,i h_{l-1},i  (split over sample blocks)
#include <cuda_runtime.h>

#include <cstring>
#include <string>

#include "device_common.cuh"
#include "kernels.h"
#include "snisr.h"
#include "snisr_internal.h"

namespace snisr {

int train_ctrl_words(int NT) { return CTRL_HEADER + 4 * NT + 2; }

namespace {

struct __align__(16) TrainRec {
  uint32_t rec, ray, tile, pad0;
  float f[3], dv;  // dv = interval / voxel
  float T, alpha, s, pad1;
};
static_assert(sizeof(TrainRec) == 48, "TrainRec layout");

constexpr int kActStride = 256;  // x (64, input padded) | h1 | h2 | h3
constexpr int kDltStride = 196;  // delta1 | delta2 | delta3 | delta_out (3 + pad)

// Per-voxel corner density logits gathered from the caller's vertex logits
// (32 bytes per voxel), rebuilt at every forward call: the march then reads
// one contiguous block per sample instead of 8 scattered vertex values.
__global__ void tr_dens_cache_kernel(const int32_t* __restrict__ corners, const float* __restrict__ vdens, int64_t nvox,
                                     float4* dc) {
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < nvox; v += (int64_t)gridDim.x * blockDim.x) {
    const int4* cn = reinterpret_cast<const int4*>(corners + v * 8);
    const int4 a = __ldg(cn), b = __ldg(cn + 1);
    dc[2 * v] = make_float4(__ldg(vdens + a.x), __ldg(vdens + a.y), __ldg(vdens + a.z), __ldg(vdens + a.w));
    dc[2 * v + 1] = make_float4(__ldg(vdens + b.x), __ldg(vdens + b.y), __ldg(vdens + b.z), __ldg(vdens + b.w));
  }
}

// trilinear density logit (corner order k = 0..7, the oracle's summation order)
__device__ __forceinline__ float seg_logit(const float4* __restrict__ dc, uint32_t rec, const float f[3], float w[8]) {
  trilinear_weights(f, w);
  const float4 a = __ldg(dc + 2 * (size_t)rec), b = __ldg(dc + 2 * (size_t)rec + 1);
  float g = 0.0f;
  g = fmaf(w[0], a.x, g); g = fmaf(w[1], a.y, g); g = fmaf(w[2], a.z, g); g = fmaf(w[3], a.w, g);
  g = fmaf(w[4], b.x, g); g = fmaf(w[5], b.y, g); g = fmaf(w[6], b.z, g); g = fmaf(w[7], b.w, g);
  return g;
}

constexpr int kStage = 32;  // records per ray in the single-pass staging area

// March of each ray segment.  mode 0 (single pass): count every sample and
// write the first kStage records of ray i to stage[i * kStage + c].
// mode 1 (rays with more than kStage samples only, after the scan): march
// again and write records c >= kStage straight to recs[off[i] + c].
__global__ void tr_march_kernel(SceneDev S, const float4* __restrict__ dc, const float* __restrict__ orig,
                                const float* __restrict__ dirs, const int32_t* __restrict__ ray_tile, int64_t n,
                                int32_t* cnt, const int32_t* __restrict__ off, TrainRec* stage, TrainRec* recs,
                                int64_t cap, int mode) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    if (mode == 1 && cnt[i] <= kStage) continue;
    const int tile = ray_tile[i];
    int c = 0;
    if (tile >= 0 && tile < S.num_tiles) {
      float o[3] = {orig[3 * i], orig[3 * i + 1], orig[3 * i + 2]};
      float d[3] = {dirs[3 * i], dirs[3 * i + 1], dirs[3 * i + 2]};
      RayState R;
      if (R.init_segment(S, o, d, tile)) {
        float T = 1.0f;
        Sample s;
        const int64_t base = mode == 1 ? off[i] : 0;
        while (next_sample(S, R, s)) {
          float w[8];
          const float g = seg_logit(dc, s.rec, s.f, w);
          const float sig = softplusf(g);
          const float dv = fmul(s.interval, S.inv_voxel);
          const float alpha = 1.0f - expf(-sig * dv);
          TrainRec* dst = nullptr;
          if (mode == 0) {
            if (c < kStage) dst = stage + i * kStage + c;
          } else if (c >= kStage) {
            if (base + c < cap) dst = recs + base + c;
            else atomicOr(S.err, ERR_OVERFLOW);
          }
          if (dst) {
            TrainRec r;
            r.rec = s.rec; r.ray = (uint32_t)i; r.tile = (uint32_t)tile; r.pad0 = 0;
            r.f[0] = s.f[0]; r.f[1] = s.f[1]; r.f[2] = s.f[2]; r.dv = dv;
            r.T = T; r.alpha = alpha; r.s = g; r.pad1 = 0.f;
            *dst = r;
          }
          ++c;
          T *= (1.0f - alpha);
          if (T < S.early_stop) break;
        }
      }
    }
    if (mode == 0) cnt[i] = c;
  }
}

// staged records -> ray-contiguous positions off[i] + c (c < kStage)
__global__ void tr_compact_kernel(const TrainRec* __restrict__ stage, const int32_t* __restrict__ cnt,
                                  const int32_t* __restrict__ off, int64_t n, TrainRec* recs, int64_t cap,
                                  uint32_t* err) {
  const int64_t total = n * kStage;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = t / kStage;
    const int c = (int)(t % kStage);
    if (c >= __ldg(cnt + i)) continue;
    const int64_t dst = (int64_t)__ldg(off + i) + c;
    if (dst < cap) {
      const uint4* s4 = reinterpret_cast<const uint4*>(stage + t);
      uint4* d4 = reinterpret_cast<uint4*>(recs + dst);
      d4[0] = s4[0]; d4[1] = s4[1]; d4[2] = s4[2];
    } else {
      atomicOr(err, ERR_OVERFLOW);
    }
  }
}

// ---- exclusive scan of n int32 counts (3 passes, 1024 per block) ----------
__device__ __forceinline__ int block_scan_excl(int v, int* sh, int& total) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(0xFFFFFFFFu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) sh[wid] = x;
  __syncthreads();
  if (wid == 0) {
    int t = lane < (int)(blockDim.x >> 5) ? sh[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xFFFFFFFFu, t, o);
      if (lane >= o) t += y;
    }
    sh[lane] = t;
  }
  __syncthreads();
  total = sh[(blockDim.x >> 5) - 1];
  int pre = wid > 0 ? sh[wid - 1] : 0;
  __syncthreads();
  return pre + x - v;
}

__global__ void scan_pass1(const int32_t* cnt, int64_t n, int32_t* bsum) {
  __shared__ int sh[32];
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  int v = i < n ? cnt[i] : 0, tot;
  block_scan_excl(v, sh, tot);
  if (threadIdx.x == 0) bsum[blockIdx.x] = tot;
}
__global__ void scan_pass2(int32_t* bsum, int nb, int32_t* total_out) {
  __shared__ int sh[32];
  int carry = 0;
  for (int b0 = 0; b0 < nb; b0 += blockDim.x) {
    int idx = b0 + threadIdx.x;
    int v = idx < nb ? bsum[idx] : 0, tot;
    int e = block_scan_excl(v, sh, tot);
    if (idx < nb) bsum[idx] = carry + e;
    carry += tot;
  }
  if (threadIdx.x == 0) *total_out = carry;
}
__global__ void scan_pass3(const int32_t* cnt, int64_t n, const int32_t* bsum, int32_t* off) {
  __shared__ int sh[32];
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  int v = i < n ? cnt[i] : 0, tot;
  int e = block_scan_excl(v, sh, tot);
  if (i < n) off[i] = bsum[blockIdx.x] + e;
}

// per-tile sample ranges (rays sorted by tile): start[t] = off[first ray
// with tile >= t], by the first block; every block checks its share of the
// tile-order precondition
__global__ void tile_ranges_kernel(const int32_t* __restrict__ ray_tile, const int32_t* __restrict__ off, int64_t n,
                                   const int32_t* total, int NT, int64_t cap, int32_t* start, uint32_t* err) {
  for (int t = threadIdx.x; blockIdx.x == 0 && t <= NT; t += blockDim.x) {
    int64_t lo = 0, hi = n;  // first index with ray_tile >= t
    while (lo < hi) {
      int64_t mid = (lo + hi) >> 1;
      if (ray_tile[mid] < t) lo = mid + 1; else hi = mid;
    }
    const int64_t v = lo < n ? off[lo] : *total;
    start[t] = (int32_t)(v < cap ? v : cap);  // records beyond the capacity were not written
  }
  // rays must be grouped by tile (non-decreasing ids)
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x + 1; i < n; i += (int64_t)gridDim.x * blockDim.x)
    if (ray_tile[i] < ray_tile[i - 1]) atomicOr(err, ERR_OVERFLOW);
}

// ---- plain FP32 MLP (weights read from the caller's FP32 parameters) -------
template <int F, int H, int L>
struct PlainMLP {
  static constexpr int IN = F + 27;
  // input x (IN values) and per-layer outputs
  __device__ static void gather_x(const SceneDev& S, const float* __restrict__ vfeat, const TrainRec& r,
                                  const float* __restrict__ dirs, float* x, float w[8], int c[8]) {
    trilinear_weights(r.f, w);
    const int4* cn = reinterpret_cast<const int4*>(S.corners + (size_t)r.rec * 8);
    int4 a = __ldg(cn), b = __ldg(cn + 1);
    c[0] = a.x; c[1] = a.y; c[2] = a.z; c[3] = a.w; c[4] = b.x; c[5] = b.y; c[6] = b.z; c[7] = b.w;
#pragma unroll
    for (int q = 0; q < F; q += 4) {
      float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        float4 v = __ldg(reinterpret_cast<const float4*>(vfeat + (size_t)c[k] * F + q));
        acc.x = fmaf(w[k], v.x, acc.x); acc.y = fmaf(w[k], v.y, acc.y);
        acc.z = fmaf(w[k], v.z, acc.z); acc.w = fmaf(w[k], v.w, acc.w);
      }
      x[q] = acc.x; x[q + 1] = acc.y; x[q + 2] = acc.z; x[q + 3] = acc.w;
    }
    float d[3] = {dirs[3 * r.ray], dirs[3 * r.ray + 1], dirs[3 * r.ray + 2]};
    dir_encoding(d, 4, x + F);
  }
  // y[fo] = W x + b, W [fo][fi] row-major at p
  template <int FI, int FO>
  __device__ static void linear(const float* __restrict__ p, const float* x, float* y) {
#pragma unroll 4
    for (int o = 0; o < FO; ++o) {
      float acc = __ldg(p + FI * FO + o);
      const float* w = p + o * FI;
#pragma unroll 8
      for (int i = 0; i < FI; ++i) acc = fmaf(__ldg(w + i), x[i], acc);
      y[o] = acc;
    }
  }
};

template <int F, int H, int L>
__global__ void __launch_bounds__(128) tr_mlp_fwd_plain(SceneDev S, const float* __restrict__ vfeat,
                                                        const float* __restrict__ mlp, const TrainRec* __restrict__ recs,
                                                        const int32_t* __restrict__ total, int64_t cap,
                                                        const float* __restrict__ dirs, float4* cout) {
  using M = PlainMLP<F, H, L>;
  const int64_t ns = min((int64_t)*total, cap);
  for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < ns; s += (int64_t)gridDim.x * blockDim.x) {
    const TrainRec r = recs[s];
    float x[M::IN], a[H], b[H], w[8];
    int c[8];
    M::gather_x(S, vfeat, r, dirs, x, w, c);
    const float* p = mlp + (size_t)r.tile * S.params_per_tile;
    M::template linear<M::IN, H>(p, x, a);
    p += M::IN * H + H;
#pragma unroll
    for (int j = 0; j < H; ++j) a[j] = fmaxf(a[j], 0.f);
#pragma unroll
    for (int l = 1; l < L; ++l) {
      M::template linear<H, H>(p, a, b);
      p += H * H + H;
#pragma unroll
      for (int j = 0; j < H; ++j) a[j] = fmaxf(b[j], 0.f);
    }
    float o[3];
    M::template linear<H, 3>(p, a, o);
    cout[s] = make_float4(sigmoidf_(o[0]), sigmoidf_(o[1]), sigmoidf_(o[2]), 0.f);
  }
}

__global__ void tr_composite_fwd(const TrainRec* __restrict__ recs, const float4* __restrict__ cin,
                                 const int32_t* __restrict__ cnt, const int32_t* __restrict__ off, int64_t n,
                                 int64_t cap, float* rgb) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    float C[3] = {0.f, 0.f, 0.f};
    const int64_t b = off[i], e = min(b + cnt[i], cap);
    for (int64_t s = b; s < e; ++s) {
      const float w = recs[s].T * recs[s].alpha;
      const float4 c = cin[s];
      C[0] = fmaf(w, c.x, C[0]); C[1] = fmaf(w, c.y, C[1]); C[2] = fmaf(w, c.z, C[2]);
    }
    rgb[3 * i] = C[0]; rgb[3 * i + 1] = C[1]; rgb[3 * i + 2] = C[2];
  }
}

__global__ void tr_composite_bwd(SceneDev S, const TrainRec* __restrict__ recs, const float4* __restrict__ cin,
                                 const int32_t* __restrict__ cnt, const int32_t* __restrict__ off, int64_t n,
                                 int64_t cap, const float* __restrict__ grad_rgb, float4* dout, float* gvdens) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float g[3] = {grad_rgb[3 * i], grad_rgb[3 * i + 1], grad_rgb[3 * i + 2]};
    const int64_t b = off[i], e = min(b + cnt[i], cap);
    float Sx = 0.f, Sy = 0.f, Sz = 0.f;  // suffix sum of w_j c_j over j > current
    for (int64_t s = e - 1; s >= b; --s) {
      const TrainRec r = recs[s];
      const float4 c = cin[s];
      const float wt = r.T * r.alpha;
      const float gc = g[0] * c.x + g[1] * c.y + g[2] * c.z;
      const float gs = g[0] * Sx + g[1] * Sy + g[2] * Sz;
      const float dsig = r.dv * ((1.0f - r.alpha) * r.T * gc - gs);
      const float ds = sigmoidf_(r.s) * dsig;
      float w[8];
      trilinear_weights(r.f, w);
      const int32_t* cn = S.corners + (size_t)r.rec * 8;
#pragma unroll
      for (int k = 0; k < 8; ++k) atomicAdd(gvdens + cn[k], w[k] * ds);
      dout[s] = make_float4(g[0] * wt * c.x * (1.f - c.x), g[1] * wt * c.y * (1.f - c.y), g[2] * wt * c.z * (1.f - c.z), 0.f);
      Sx = fmaf(wt, c.x, Sx); Sy = fmaf(wt, c.y, Sy); Sz = fmaf(wt, c.z, Sz);
    }
  }
}

// Per-sample backward through the MLP (FP32, CUDA cores): recomputes x and the
// activations (stored to `act` for the weight-gradient pass), back-propagates
// the output gradient (deltas stored to `dlt`) and scatters the feature
// gradient to the 8 corner vertices.
template <int F, int H, int L>
__global__ void __launch_bounds__(128) tr_mlp_bwd_plain(SceneDev S, const float* __restrict__ vfeat,
                                                        const float* __restrict__ mlp, const TrainRec* __restrict__ recs,
                                                        const int32_t* __restrict__ total, int64_t cap,
                                                        const float* __restrict__ dirs, const float4* __restrict__ dout,
                                                        float* act, float* dlt, float* gvfeat) {
  using M = PlainMLP<F, H, L>;
  const int64_t ns = min((int64_t)*total, cap);
  for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < ns; s += (int64_t)gridDim.x * blockDim.x) {
    const TrainRec r = recs[s];
    float* A = act + (size_t)s * kActStride;
    float* Dl = dlt + (size_t)s * kDltStride;
    float x[M::IN], h[H], w[8];
    int c[8];
    M::gather_x(S, vfeat, r, dirs, x, w, c);
    for (int i = 0; i < 64; ++i) A[i] = i < M::IN ? x[i] : 0.f;
    const float* P = mlp + (size_t)r.tile * S.params_per_tile;
    // forward, storing post-ReLU activations
    {
      float y[H];
      M::template linear<M::IN, H>(P, x, y);
#pragma unroll
      for (int j = 0; j < H; ++j) { h[j] = fmaxf(y[j], 0.f); A[64 + j] = h[j]; }
      const float* p = P + M::IN * H + H;
      for (int l = 1; l < L; ++l) {
        M::template linear<H, H>(p, h, y);
        p += H * H + H;
#pragma unroll
        for (int j = 0; j < H; ++j) { h[j] = fmaxf(y[j], 0.f); A[64 + 64 * l + j] = h[j]; }
      }
    }
    // backward
    int64_t offs[4];
    offs[0] = 0;
    offs[1] = (int64_t)M::IN * H + H;
    for (int l = 2; l <= L; ++l) offs[l] = offs[l - 1] + H * H + H;
    const float4 d4 = dout[s];
    float dcur[H];
    {
      const float dl[3] = {d4.x, d4.y, d4.z};
      Dl[64 * L] = dl[0]; Dl[64 * L + 1] = dl[1]; Dl[64 * L + 2] = dl[2];
      const float* Wo = P + offs[L];
#pragma unroll
      for (int j = 0; j < H; ++j) {
        float acc = __ldg(Wo + j) * dl[0] + __ldg(Wo + H + j) * dl[1] + __ldg(Wo + 2 * H + j) * dl[2];
        dcur[j] = A[64 + 64 * (L - 1) + j] > 0.f ? acc : 0.f;
        Dl[64 * (L - 1) + j] = dcur[j];
      }
    }
    for (int l = L - 1; l >= 1; --l) {
      const float* Wl = P + offs[l];
      float dprev[H];
#pragma unroll
      for (int i = 0; i < H; ++i) dprev[i] = 0.f;
      for (int o = 0; o < H; ++o) {
        const float dv = dcur[o];
#pragma unroll
        for (int i = 0; i < H; ++i) dprev[i] = fmaf(__ldg(Wl + o * H + i), dv, dprev[i]);
      }
#pragma unroll
      for (int i = 0; i < H; ++i) {
        dcur[i] = A[64 + 64 * (l - 1) + i] > 0.f ? dprev[i] : 0.f;
        Dl[64 * (l - 1) + i] = dcur[i];
      }
    }
    // feature gradient dx = W0^T delta1 (first F inputs)
    float dx[F];
#pragma unroll
    for (int q = 0; q < F; ++q) dx[q] = 0.f;
    for (int o = 0; o < H; ++o) {
      const float dv = dcur[o];
#pragma unroll
      for (int q = 0; q < F; ++q) dx[q] = fmaf(__ldg(P + o * M::IN + q), dv, dx[q]);
    }
#pragma unroll
    for (int k = 0; k < 8; ++k)
#pragma unroll
      for (int q = 0; q < F; q += 4)
        red_add_v4(gvfeat + (size_t)c[k] * F + q, w[k] * dx[q], w[k] * dx[q + 1], w[k] * dx[q + 2], w[k] * dx[q + 3]);
  }
}

// Weight gradients: for tile t, layer l: dW[o][i] += sum_s delta_l[s][o] h_{l-1}[s][i],
// db[o] += sum_s delta_l[s][o].  Block = (sample block of kDwBlock, layer, tile);
// 256 threads each own outputs (o, i) strided over fo x (fi + 1): kPerThread
// of them, enough for the largest layer (H x (max(IN, H) + 1) outputs).
constexpr int kDwBlock = 512;

template <int F, int H, int L>
__global__ void __launch_bounds__(256) tr_dw_kernel(const float* __restrict__ act, const float* __restrict__ dlt,
                                                    const int32_t* __restrict__ tstart, int P, float* gmlp) {
  constexpr int IN = F + 27;
  constexpr int kMaxOut = H * ((IN > H ? IN : H) + 1);
  constexpr int kPerThread = (kMaxOut + 255) / 256;
  const int tile = blockIdx.z, l = blockIdx.y;
  const int fi = l == 0 ? IN : H, fo = l == L ? 3 : H;
  const int a_off = 64 * l;  // input of Linear l: x (l = 0) or h_l
  const int d_off = 64 * l;  // delta of Linear l's output
  int64_t poff = 0;
  for (int j = 0; j < l; ++j) poff += (int64_t)(j == 0 ? IN : H) * H + H;
  float* G = gmlp + (size_t)tile * P + poff;
  __shared__ float sh_a[32][65], sh_d[32][65];
  const int nout = fo * (fi + 1);
  static_assert(kPerThread * 256 >= kMaxOut, "every output of the largest layer has a thread");
  float acc[kPerThread];
#pragma unroll
  for (int k = 0; k < kPerThread; ++k) acc[k] = 0.f;
  const int64_t t0 = tstart[tile], t1 = tstart[tile + 1];
  for (int64_t s0 = t0 + (int64_t)blockIdx.x * kDwBlock; s0 < t1; s0 += (int64_t)gridDim.x * kDwBlock) {
    const int64_t s1 = min(s0 + kDwBlock, t1);
    for (int64_t b = s0; b < s1; b += 32) {
      const int nb = (int)min((int64_t)32, s1 - b);
      for (int e = threadIdx.x; e < 32 * 64; e += 256) {
        const int r = e >> 6, col = e & 63;
        sh_a[r][col] = (r < nb && col < fi) ? act[(size_t)(b + r) * kActStride + a_off + col] : 0.f;
        sh_d[r][col] = (r < nb && col < fo) ? dlt[(size_t)(b + r) * kDltStride + d_off + col] : 0.f;
      }
      __syncthreads();
#pragma unroll
      for (int k = 0; k < kPerThread; ++k) {
        const int idx = threadIdx.x + 256 * k;
        if (idx < nout) {
          const int o = idx / (fi + 1), i = idx % (fi + 1);
          float sacc = 0.f;
          for (int r = 0; r < nb; ++r) sacc = fmaf(sh_d[r][o], i < fi ? sh_a[r][i] : 1.0f, sacc);
          acc[k] += sacc;
        }
      }
      __syncthreads();
    }
  }
#pragma unroll
  for (int k = 0; k < kPerThread; ++k) {
    const int idx = threadIdx.x + 256 * k;
    if (idx < nout && acc[k] != 0.f) {
      const int o = idx / (fi + 1), i = idx % (fi + 1);
      atomicAdd(G + (i < fi ? (int64_t)o * fi + i : (int64_t)fo * fi + o), acc[k]);
    }
  }
}

inline int gridn(int64_t n, int t, int cap = 1 << 20) {
  int64_t b = (n + t - 1) / t;
  return (int)(b < 1 ? 1 : (b > cap ? cap : b));
}

template <int F, int H, int L>
cudaError_t train_plain_mlp_fwd(const SceneDev& S, const float* vfeat, const float* mlp, const TrainRec* recs,
                                const int32_t* total, int64_t cap, const float* dirs, float4* cout, int num_sms,
                                cudaStream_t st) {
  tr_mlp_fwd_plain<F, H, L><<<num_sms * 16, 128, 0, st>>>(S, vfeat, mlp, recs, total, cap, dirs, cout);
  return cudaGetLastError();
}
template <int F, int H, int L>
cudaError_t train_plain_mlp_bwd(const SceneDev& S, const float* vfeat, const float* mlp, const TrainRec* recs,
                                const int32_t* total, int64_t cap, const float* dirs, const float4* dout, float* act,
                                float* dlt, float* gvfeat, const int32_t* tstart, int64_t max_tile_samples,
                                float* gmlp, int num_sms, cudaStream_t st) {
  tr_mlp_bwd_plain<F, H, L><<<num_sms * 16, 128, 0, st>>>(S, vfeat, mlp, recs, total, cap, dirs, dout, act, dlt,
                                                         gvfeat);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  int64_t gx = (max_tile_samples + kDwBlock - 1) / kDwBlock;
  if (gx > num_sms * 2) gx = num_sms * 2;
  if (gx < 1) gx = 1;
  dim3 grid((unsigned)gx, L + 1, S.num_tiles);
  tr_dw_kernel<F, H, L><<<grid, 256, 0, st>>>(act, dlt, tstart, S.params_per_tile, gmlp);
  return cudaGetLastError();
}

}  // namespace

// ---------------------------------------------------------------------------
// Training workspace (per scene; grown on demand at the first call of a
// larger batch, then reused) and the entry points.
// ---------------------------------------------------------------------------
struct TrainWS {
  int64_t rays = 0, cap = 0;
  int32_t* coff = nullptr;
  int* work = nullptr;
  uint4* enc = nullptr;
  uint8_t* wimg = nullptr;
  int img_stride = 0;
  int32_t *cnt = nullptr, *off = nullptr, *bsum = nullptr, *total = nullptr, *tstart = nullptr;
  TrainRec* recs = nullptr;
  TrainRec* stage = nullptr;   // [rays][kStage] single-pass march output
  float4* dcache = nullptr;    // [nvox][2] corner density logits of the current call
  int64_t nvox = 0;
  float4 *c = nullptr, *dout = nullptr;
  float *act = nullptr, *dlt = nullptr;
  float* gstage = nullptr;     // [NT][4][64 x 64 + 64] staged weight gradients (TC backward)
  void* block = nullptr;
  size_t bytes = 0;
  int64_t last_n = -1;
  int last_form = -1;
  // Generation of the forward whose records the workspace holds (0: none).
  // Every forward takes a new one from the counter; a backward must name the
  // generation its forward returned.
  uint64_t last_gen = 0, gen_counter = 0;
};

snisr_status scene_views(snisr_scene* scene, SceneDev* S, Workspace* ws, int* device);
snisr_status scene_train_ws(snisr_scene* scene, TrainWS** out, int* num_sms, int* max_samples_per_ray, int64_t* nvox);

snisr_status train_ws_reserve(TrainWS* T, int64_t n, int msr, int NT, int64_t nvox) {
  if (T->block && n <= T->rays && nvox == T->nvox) return SNISR_OK;
  if (T->block) cudaFree(T->block);
  T->block = nullptr;
  const int64_t rays = n, cap = n * (int64_t)msr, nb = (rays + 1023) / 1024 + 2;
  auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
  const int img_stride = (train_tc_image_bytes(64, 3) + 127) & ~127;
  // T->act holds the plain form's per-sample activations or the TC form's
  // activation tiles (3 hidden layers x 16 KB per 128-row chunk; at most
  // cap / 128 + NT chunks): the larger of the two
  const size_t act_bytes = std::max((size_t)cap * kActStride * 4, ((size_t)cap / 128 + NT + 1) * 3 * 16384);
  size_t sz = al(rays * 4) * 2 + al(nb * 4) + al(16) + al((NT + 2) * 4) + al(cap * sizeof(TrainRec)) +
              al(cap * 16) * 2 + al(act_bytes) + al(cap * kDltStride * 4) + al(2 * (NT + 2) * 4) + al(16) +
              al(rays * 192) + al((size_t)img_stride * NT) + al((size_t)rays * kStage * sizeof(TrainRec)) +
              al((size_t)nvox * 32) + al((size_t)NT * 4 * (64 * 64 + 64) * 4);
  void* p = nullptr;
  cudaError_t e = cudaMalloc(&p, sz);
  if (e != cudaSuccess) return set_error(SNISR_OOM, std::string("train workspace: ") + cudaGetErrorString(e));
  uint8_t* q = static_cast<uint8_t*>(p);
  auto take = [&](size_t b) { uint8_t* r = q; q += al(b); return r; };
  T->cnt = (int32_t*)take(rays * 4);
  T->off = (int32_t*)take(rays * 4);
  T->bsum = (int32_t*)take(nb * 4);
  T->total = (int32_t*)take(16);
  T->tstart = (int32_t*)take((NT + 2) * 4);
  T->recs = (TrainRec*)take(cap * sizeof(TrainRec));
  T->c = (float4*)take(cap * 16);
  T->dout = (float4*)take(cap * 16);
  T->act = (float*)take(act_bytes);  // plain form: activations per sample; TC form: activation tiles
  T->dlt = (float*)take(cap * kDltStride * 4);
  T->coff = (int32_t*)take(2 * (NT + 2) * 4);  // chunk offsets per tile: 128-row chunks, then 256-row units
  T->work = (int*)take(16);
  T->enc = (uint4*)take(rays * 192);  // 12 uint4 per ray: BF16 hi, mid, lo of the view encoding
  T->wimg = (uint8_t*)take((size_t)img_stride * NT);
  T->stage = (TrainRec*)take((size_t)rays * kStage * sizeof(TrainRec));
  T->dcache = (float4*)take((size_t)nvox * 32);
  T->gstage = (float*)take((size_t)NT * 4 * (64 * 64 + 64) * 4);
  T->nvox = nvox;
  T->img_stride = img_stride;
  T->block = p;
  T->bytes = sz;
  T->rays = rays;
  T->cap = cap;
  return SNISR_OK;
}

void train_ws_free(TrainWS* T) {
  if (T && T->block) cudaFree(T->block);
  delete T;
}
TrainWS* train_ws_new() { return new TrainWS(); }

}  // namespace snisr

using namespace snisr;

#define TR_TRY(expr, what)                                                                                    \
  do {                                                                                                        \
    cudaError_t e__ = (expr);                                                                                 \
    if (e__ != cudaSuccess) return set_error(SNISR_CUDA_ERROR, std::string(what) + ": " + cudaGetErrorString(e__)); \
  } while (0)

namespace {

snisr_status train_common(snisr_scene* sc, const float* vdens, const float* orig, const float* dirs,
                          const int32_t* ray_tile, int64_t n, SceneDev& S, TrainWS*& T, int& num_sms, cudaStream_t st,
                          bool march, Workspace& ws) {
  int device = 0, msr = 0;
  int64_t nvox = 0;
  snisr_status s = scene_views(sc, &S, &ws, &device);
  if (s != SNISR_OK) return s;
  if ((s = scene_train_ws(sc, &T, &num_sms, &msr, &nvox)) != SNISR_OK) return s;
  if (march) {  // a forward overwrites the records: the previous generation is gone from here on
    T->last_gen = 0;
    T->last_n = -1;
  }
  if ((s = train_ws_reserve(T, n, msr, S.num_tiles, nvox)) != SNISR_OK) return s;
  if (!march) return SNISR_OK;
  tr_dens_cache_kernel<<<gridn(nvox, 256), 256, 0, st>>>(S.corners, vdens, nvox, T->dcache);
  TR_TRY(cudaGetLastError(), "train: density cache");
  const int mt = ws.tune.train_march_threads;
  tr_march_kernel<<<gridn(n, mt), mt, 0, st>>>(S, T->dcache, orig, dirs, ray_tile, n, T->cnt, nullptr, T->stage,
                                               nullptr, 0, 0);
  TR_TRY(cudaGetLastError(), "train: march");
  const int nb = (int)((n + 1023) / 1024);
  scan_pass1<<<nb, 1024, 0, st>>>(T->cnt, n, T->bsum);
  scan_pass2<<<1, 1024, 0, st>>>(T->bsum, nb, T->total);
  scan_pass3<<<nb, 1024, 0, st>>>(T->cnt, n, T->bsum, T->off);
  TR_TRY(cudaGetLastError(), "train: scan");
  tr_compact_kernel<<<gridn(n * kStage, 256), 256, 0, st>>>(T->stage, T->cnt, T->off, n, T->recs, T->cap, S.err);
  tr_march_kernel<<<gridn(n, mt), mt, 0, st>>>(S, T->dcache, orig, dirs, ray_tile, n, T->cnt, T->off, nullptr,
                                               T->recs, T->cap, 1);
  TR_TRY(cudaGetLastError(), "train: compact");
  tile_ranges_kernel<<<gridn(n, 256), 256, 0, st>>>(ray_tile, T->off, n, T->total, S.num_tiles, T->cap, T->tstart,
                                                     S.err);
  TR_TRY(cudaGetLastError(), "train: tile ranges");
  return SNISR_OK;
}

}  // namespace

extern "C" snisr_status snisr_train_forward(snisr_scene* sc, const float* vfeat, const float* vdens, const float* mlp,
                                            const float* orig, const float* dirs, const int32_t* ray_tile, int64_t n,
                                            int32_t form, float* rgb, uint64_t* generation, void* stream) {
  if (generation) *generation = 0;
  if (!sc) return set_error(SNISR_INVALID_ARG, "train_forward: scene is null");
  if (n < 0) return set_error(SNISR_INVALID_ARG, "train_forward: negative ray count");
  if (n == 0) return SNISR_OK;
  if (!vfeat || !vdens || !mlp || !orig || !dirs || !ray_tile || !rgb)
    return set_error(SNISR_INVALID_ARG, "train_forward: null pointer argument");
  if (form != SNISR_FORM_PLAIN_FP32 && form != SNISR_FORM_TC) return set_error(SNISR_INVALID_ARG, "train_forward: bad form");
  cudaStream_t st = (cudaStream_t)stream;
  SceneDev S;
  TrainWS* T = nullptr;
  int num_sms = 0;
  Workspace ws;
  snisr_status s = train_common(sc, vdens, orig, dirs, ray_tile, n, S, T, num_sms, st, true, ws);
  if (s != SNISR_OK) return s;
  const int F = S.feat_dim, H = S.mlp_hidden, L = S.mlp_layers;
  cudaError_t e;
  if (form != SNISR_FORM_PLAIN_FP32) {
    TrainTcArgs a{vfeat, mlp, dirs, n, T->recs, T->tstart, T->coff, T->work, T->enc, T->wimg, T->img_stride,
                  T->c, T->dout, nullptr, nullptr, nullptr, num_sms, ws.tune.train_fwd_warps,
                  reinterpret_cast<uint8_t*>(T->act)};
    e = launch_train_tc(S, a, false, st);
    if (e == cudaErrorInvalidValue) return set_error(SNISR_UNSUPPORTED, "train_forward: MLP shape not built for training");
  } else if (F == 32 && H == 64 && L == 3) e = train_plain_mlp_fwd<32, 64, 3>(S, vfeat, mlp, T->recs, T->total, T->cap, dirs, T->c, num_sms, st);
  else if (F == 16 && H == 32 && L == 2) e = train_plain_mlp_fwd<16, 32, 2>(S, vfeat, mlp, T->recs, T->total, T->cap, dirs, T->c, num_sms, st);
  else return set_error(SNISR_UNSUPPORTED, "train_forward: MLP shape not built for training");
  TR_TRY(e, "train_forward: mlp");
  tr_composite_fwd<<<gridn(n, 128), 128, 0, st>>>(T->recs, T->c, T->cnt, T->off, n, T->cap, rgb);
  TR_TRY(cudaGetLastError(), "train_forward: composite");
  T->last_n = n;
  T->last_form = form;
  T->last_gen = ++T->gen_counter;
  if (generation) *generation = T->last_gen;
  return SNISR_OK;
}

extern "C" snisr_status snisr_train_backward(snisr_scene* sc, const float* vfeat, const float* vdens, const float* mlp,
                                             const float* orig, const float* dirs, const int32_t* ray_tile, int64_t n,
                                             int32_t form, uint64_t generation, const float* rgb,
                                             const float* grad_rgb, float* gvfeat, float* gvdens, float* gmlp,
                                             void* stream) {
  (void)rgb;
  (void)vdens;
  (void)orig;
  (void)ray_tile;
  if (!sc) return set_error(SNISR_INVALID_ARG, "train_backward: scene is null");
  if (n < 0) return set_error(SNISR_INVALID_ARG, "train_backward: negative ray count");
  if (n == 0) return SNISR_OK;
  if (!vfeat || !mlp || !dirs || !grad_rgb || !gvfeat || !gvdens || !gmlp)
    return set_error(SNISR_INVALID_ARG, "train_backward: null pointer argument");
  if (form != SNISR_FORM_PLAIN_FP32 && form != SNISR_FORM_TC) return set_error(SNISR_INVALID_ARG, "train_backward: bad form");
  if (reinterpret_cast<uintptr_t>(gvfeat) % 16 != 0)
    return set_error(SNISR_INVALID_ARG, "train_backward: gvfeat must be 16-byte aligned (vector reductions)");
  cudaStream_t st = (cudaStream_t)stream;
  SceneDev S;
  TrainWS* T = nullptr;
  int num_sms = 0;
  Workspace ws;
  snisr_status s = train_common(sc, vdens, orig, dirs, ray_tile, n, S, T, num_sms, st, false, ws);
  if (s != SNISR_OK) return s;
  if (generation == 0 || generation != T->last_gen)
    return set_error(SNISR_INVALID_ARG,
                     "train_backward: generation " + std::to_string(generation) +
                         " is not the latest train_forward on this scene (latest: " + std::to_string(T->last_gen) +
                         "); another forward ran in between and replaced its sample records");
  if (T->last_n != n) return set_error(SNISR_INVALID_ARG, "train_backward: must follow train_forward on the same rays");
  tr_composite_bwd<<<gridn(n, 128), 128, 0, st>>>(S, T->recs, T->c, T->cnt, T->off, n, T->cap, grad_rgb, T->dout,
                                                  gvdens);
  TR_TRY(cudaGetLastError(), "train_backward: composite");
  const int F = S.feat_dim, H = S.mlp_hidden, L = S.mlp_layers;
  const int64_t max_tile = T->cap;  // upper bound; empty blocks exit at once
  cudaError_t e;
  if (T->last_form != form) return set_error(SNISR_INVALID_ARG, "train_backward: the forward call used another form");
  if (form != SNISR_FORM_PLAIN_FP32) {
    TrainTcArgs a{vfeat, mlp, dirs, n, T->recs, T->tstart, T->coff, T->work, T->enc, T->wimg, T->img_stride,
                  T->c, T->dout, gvfeat, gmlp, T->gstage, num_sms, ws.tune.train_fwd_warps,
                  reinterpret_cast<uint8_t*>(T->act)};
    e = launch_train_tc(S, a, true, st);
  } else if (F == 32 && H == 64 && L == 3)
    e = train_plain_mlp_bwd<32, 64, 3>(S, vfeat, mlp, T->recs, T->total, T->cap, dirs, T->dout, T->act, T->dlt, gvfeat,
                                        T->tstart, max_tile, gmlp, num_sms, st);
  else if (F == 16 && H == 32 && L == 2)
    e = train_plain_mlp_bwd<16, 32, 2>(S, vfeat, mlp, T->recs, T->total, T->cap, dirs, T->dout, T->act, T->dlt, gvfeat,
                                        T->tstart, max_tile, gmlp, num_sms, st);
  else
    return set_error(SNISR_UNSUPPORTED, "train_backward: MLP shape not built for training");
  TR_TRY(e, "train_backward: mlp");
  return SNISR_OK;
}
