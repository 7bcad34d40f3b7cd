// The reference's specular pass ops, rebuilt for sm_103a:
//   sort_by_key / assign_pixels (rendering/src/reorder.cu:10-94): batching of
//     the reflection pixels by network;
//   inference_mlp (rendering/src/rayreflection_render.cu:111-301): the
//     per-group MLP 63 -> 64 x 5 (LeakyReLU 0.01) -> 28 on position encodings,
//     SH degree 2 of the view direction, sigmoid, density = max(out[27], 0).
// The reference evaluates the MLP with scalar FP16 FMA chains (FP16
// accumulation); here it runs on tcgen05 (FP16 operands, FP32 accumulation
// in tensor memory), which is closer to exact arithmetic.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <string>

#include "kernels.h"
#include "scan.cuh"
#include "snisr.h"
#include "snisr_internal.h"
#include "tc_ptx.cuh"

namespace snisr {
namespace {

constexpr unsigned kFull = 0xFFFFFFFFu;

__device__ __forceinline__ unsigned lanemask_lt_() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// ---------------------------------------------------------------------------
// Stable LSD radix sort of (int16 key, int32 value), 2 passes of 8 bits on
// the key with its sign bit flipped (signed order).  Block = 256 threads x 4
// rounds = 1024 consecutive elements.
// ---------------------------------------------------------------------------
constexpr int kSortThreads = 256, kSortPer = 4, kSortBlock = kSortThreads * kSortPer;

__device__ __forceinline__ uint32_t digit_of(int16_t k, int pass) {
  return ((uint32_t)(uint16_t)(k ^ (int16_t)0x8000) >> (8 * pass)) & 0xFFu;
}

__global__ void sort_hist_kernel(const int16_t* __restrict__ keys, int64_t n, int pass, uint32_t* hist, int nblocks) {
  __shared__ uint32_t h[256];
  h[threadIdx.x] = 0;
  __syncthreads();
  const int64_t base = (int64_t)blockIdx.x * kSortBlock;
  for (int r = 0; r < kSortPer; ++r) {
    const int64_t i = base + r * kSortThreads + threadIdx.x;
    if (i < n) atomicAdd(h + digit_of(keys[i], pass), 1u);
  }
  __syncthreads();
  hist[(size_t)threadIdx.x * nblocks + blockIdx.x] = h[threadIdx.x];  // digit-major
}


__global__ void sort_scatter_kernel(const int16_t* __restrict__ kin, const int32_t* __restrict__ vin, int64_t n,
                                    int pass, const uint32_t* __restrict__ offs, int nblocks, int16_t* kout,
                                    int32_t* vout) {
  __shared__ uint32_t wcnt[kSortThreads / 32][256];
  __shared__ uint32_t run[256];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  run[tid] = 0;
  const int64_t base = (int64_t)blockIdx.x * kSortBlock;
  for (int r = 0; r < kSortPer; ++r) {
    for (int w = 0; w < kSortThreads / 32; ++w) wcnt[w][tid] = 0;
    __syncthreads();
    const int64_t i = base + r * kSortThreads + tid;
    const bool valid = i < n;
    int16_t k = 0;
    int32_t v = 0;
    uint32_t d = 0, rank = 0;
    if (valid) {
      k = kin[i];
      v = vin[i];
      d = digit_of(k, pass);
    }
    const unsigned m = __ballot_sync(kFull, valid);
    if (valid) {
      const unsigned g = __match_any_sync(m, d);
      rank = __popc(g & lanemask_lt_());
      if (rank == 0) wcnt[warp][d] = __popc(g);
    }
    __syncthreads();
    // per digit: prefix over the warps of this round (thread tid owns digit tid)
    {
      uint32_t acc = run[tid];
      for (int w = 0; w < kSortThreads / 32; ++w) {
        const uint32_t c = wcnt[w][tid];
        wcnt[w][tid] = acc;
        acc += c;
      }
      run[tid] = acc;
    }
    __syncthreads();
    if (valid) {
      const uint32_t pos = offs[(size_t)d * nblocks + blockIdx.x] + wcnt[warp][d] + rank;
      kout[pos] = k;
      vout[pos] = v;
    }
    __syncthreads();
  }
}

// unique_by_key: flag[i] = first element of a run of equal keys
__global__ void run_flags_kernel(const int16_t* __restrict__ k, int64_t n, uint32_t* flag) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    flag[i] = (i == 0 || k[i] != k[i - 1]) ? 1u : 0u;
}

__global__ void run_compact_kernel(const int16_t* __restrict__ ksorted, const int32_t* __restrict__ starts_in,
                                   const uint32_t* __restrict__ pos, int64_t n, int16_t* keys, int32_t* starts) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    keys[i] = ksorted[i];  // positions past the run count keep the sorted keys
    if (i == 0 || ksorted[i] != ksorted[i - 1]) starts[pos[i]] = starts_in[i];
  }
}

__global__ void run_keys_kernel(const int16_t* __restrict__ ksorted, const uint32_t* __restrict__ pos, int64_t n,
                                int16_t* keys, int64_t* count) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    if (i == 0 || ksorted[i] != ksorted[i - 1]) keys[pos[i]] = ksorted[i];
    if (i == n - 1) *count = (int64_t)pos[i] + ((i == 0 || ksorted[i] != ksorted[i - 1]) ? 1 : 0);
  }
}

// ---------------------------------------------------------------------------
// assign_pixels: network k's pixels over blocks [bs[k], bs[k+1]), the first
// (count mod blocks) blocks taking one pixel more.
// ---------------------------------------------------------------------------
__global__ void assign_pixels_kernel(const int16_t* __restrict__ net, const int32_t* __restrict__ ps,
                                     const int32_t* __restrict__ bs, int64_t num_net, int16_t* new_net,
                                     int32_t* new_ps) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < num_net; k += (int64_t)gridDim.x * blockDim.x) {
    int32_t p = ps[k];
    const int32_t num = ps[k + 1] - ps[k], nb = bs[k + 1] - bs[k];
    if (nb <= 0) continue;
    const int32_t base = num / nb, add = num - base * nb;
    for (int32_t i = 0; i < nb; ++i) {
      new_net[bs[k] + i] = net[k];
      new_ps[bs[k] + i] = p;
      p += i < add ? base + 1 : base;
    }
  }
}

// ---------------------------------------------------------------------------
// inference_mlp on tcgen05
// ---------------------------------------------------------------------------
constexpr int kSpIn = 63, kSpH = 64, kSpHidden = 5, kSpOut = 28, kSpParams = 22556;
constexpr uint32_t kErrTimeout = 2u;
constexpr uint32_t kErrDrain = 8u;  // in-flight MMAs did not finish after a timeout: context unusable

// reference parameter offsets: per layer bias[fo] then W[fi][fo]
__host__ __device__ constexpr int sp_layer_off(int l) {
  return l == 0 ? 0 : (kSpH + kSpIn * kSpH) + (l - 1) * (kSpH + kSpH * kSpH);
}

__device__ __forceinline__ uint32_t swz(int row, int k) {  // byte offset of element (row, k) in a K-major SW128 tile
  return (uint32_t)(row >> 3) * 1024u + (uint32_t)(row & 7) * 128u + ((uint32_t)((k >> 3) ^ (row & 7)) << 4) +
         (uint32_t)((k & 7) << 1);
}

__device__ __forceinline__ uint32_t pack_h2(float lo, float hi) {
  uint32_t d;
  asm("cvt.rn.f16x2.f32 %0, %1, %2;" : "=r"(d) : "f"(hi), "f"(lo));
  return d;
}

// One CTA = two groups of 4 warps sharing one copy of the network.  Shared
// memory: W0..W4 (5 x 8 KB) | Wout (32 rows, 4 KB) | FP32 biases [6][64]
// (1.5 KB, added by the epilogues) | per group an A tile (16 KB, the
// position encodings: layer 0's operand) | per group and row the current
// chunk's output slot, live flag and view direction (24 B) | barriers,
// slots: ~86 KB, two CTAs per SM.  Tensor memory: per group 128 columns at 128 g, the
// accumulator [0, 64) and the hidden activations [64, 96) (FP16 pairs), the
// A operand of layers 1..5.
constexpr int kSpGroups = 2;
constexpr int kSpW = 0, kSpWout = kSpW + 5 * 8192, kSpBias = kSpWout + 4096,
              kSpA = (kSpBias + 6 * 64 * 4 + 1023) & ~1023, kSpRows = kSpA + kSpGroups * 16384,
              kSpBars = kSpRows + kSpGroups * 128 * 24, kSpSmem = kSpBars + 64;
struct __align__(8) SpRowOut {  // a row's sample: output slot (-1: not live), view direction
  int64_t ori;
  float d[3];
  float pad;
};
static_assert(sizeof(SpRowOut) == 24, "24-byte row slots");

// pack network g's parameters (reference layout, FP16) into the swizzled
// tiles; threads tid of nth
__device__ void pack_net(const __half* __restrict__ P, uint8_t* sm, int tid, int nth) {
  // hidden layers: row = output j, K = input i
  for (int e = tid; e < kSpHidden * kSpH * (kSpH / 8); e += nth) {
    const int l = e / (kSpH * 8), j = (e / 8) % kSpH, c = e % 8;
    const int fi = l == 0 ? kSpIn : kSpH, off = sp_layer_off(l) + kSpH;
    uint32_t w[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int i0 = 8 * c + 2 * q, i1 = i0 + 1;
      const float a = i0 < fi ? __half2float(P[off + i0 * kSpH + j]) : 0.f;
      const float b = i1 < fi ? __half2float(P[off + i1 * kSpH + j]) : 0.f;
      w[q] = pack_h2(a, b);
    }
    *reinterpret_cast<uint4*>(sm + kSpW + l * 8192 + swz(j, 8 * c)) = make_uint4(w[0], w[1], w[2], w[3]);
  }
  // output layer: 32 rows (28 used)
  for (int e = tid; e < 32 * 8; e += nth) {
    const int j = e / 8, c = e % 8, off = sp_layer_off(kSpHidden) + kSpOut;
    uint32_t w[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int i0 = 8 * c + 2 * q;
      const float a = j < kSpOut ? __half2float(P[off + i0 * kSpOut + j]) : 0.f;
      const float b = j < kSpOut ? __half2float(P[off + (i0 + 1) * kSpOut + j]) : 0.f;
      w[q] = pack_h2(a, b);
    }
    *reinterpret_cast<uint4*>(sm + kSpWout + swz(j, 8 * c)) = make_uint4(w[0], w[1], w[2], w[3]);
  }
  // biases (FP32), layer l at [l][64]; output layer: 28 used
  float* bias = reinterpret_cast<float*>(sm + kSpBias);
  for (int e = tid; e < 6 * 64; e += nth) {
    const int l = e / 64, j = e % 64;
    float b = 0.f;
    if (l < kSpHidden) b = __half2float(P[sp_layer_off(l) + j]);
    else if (j < kSpOut) b = __half2float(P[sp_layer_off(kSpHidden) + j]);
    bias[e] = b;
  }
}

// One CTA: chunks of 128 samples of one network's pixel block; group g of
// the two takes chunks g, g + 2, g + 4, ... of the block, with its own A tile,
// tensor memory, MMA issuer (its first thread), mbarrier and named barrier,
// so that the groups' chains overlap.  Layer 0 reads the position encodings
// from shared memory; each hidden layer's epilogue (bias, LeakyReLU, FP16
// pack) writes its row of activations into tensor memory with tcgen05.st,
// where the next layer's MMA reads its A operand.  Software pipeline: the
// group's next chunk's tasks are fetched during layer 0's MMA, and its
// encodings computed and stored into the (then free) A tile during layer
// 1's.
__global__ void __launch_bounds__(128 * kSpGroups, 2)
    inference_mlp_kernel(int spr, int num_block, float inv_far, float trans_stop, const int16_t* __restrict__ net,
                         int num_groups, const float* __restrict__ transparency, const int32_t* __restrict__ qpix,
                         const int32_t* __restrict__ pstarts, const float* __restrict__ centers,
                         const float* __restrict__ samples, const float* __restrict__ rays_d,
                         const __half* __restrict__ params, float4* results, int* work, uint32_t* err) {
  constexpr int NTH = 128 * kSpGroups;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* sm = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint64_t* bars = reinterpret_cast<uint64_t*>(sm + kSpBars);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + kSpGroups);
  int* blk_slot = reinterpret_cast<int*>(tmem_slot + 1);
  const int tid = threadIdx.x, warp = tid >> 5, grp = warp >> 2, row = tid & 127;
  const int leader = 128 * grp;
  const uint32_t gbar = 1u + (uint32_t)grp;
  const uint32_t mbar = tc::smem_addr(bars + grp);
  uint8_t* A = sm + kSpA + grp * 16384;  // this group's A tile
  SpRowOut* my_out = reinterpret_cast<SpRowOut*>(sm + kSpRows) + grp * 128 + row;  // this row's current sample
  if (tid == 0) {
    for (int g = 0; g < kSpGroups; ++g) tc::mbar_init(tc::smem_addr(bars + g), 1);
    tc::fence_mbar_init();
  }
  if (warp == 0) {
    tc::tmem_alloc(tc::smem_addr(tmem_slot), 128 * kSpGroups);
    tc::tmem_relinquish();
  }
  tc::fence_proxy_async();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *tmem_slot;
  const uint32_t gacc = tmem + 128u * (uint32_t)grp;  // the group's accumulator
  const uint32_t tact = gacc + kSpH;                   // its activation columns (A operand of layers 1..5)
  const uint32_t taddr = gacc + ((uint32_t)((warp & 3) * 32) << 16);
  const float* bias = reinterpret_cast<const float*>(sm + kSpBias);
  const uint32_t a_base = tc::smem_addr(A);
  const uint32_t id_h = tc::idesc_f16(kSpH, 0), id_o = tc::idesc_f16(32, 0);
  uint32_t mphase = 0;
  int cur_net = -1;
  bool failed = false;
  tc::Drain drain;  // on the group leaders: MMAs in flight at a timeout
  // The task of this thread's A row: its pixel, whether it is live, the
  // encoded position and the view direction.
  struct Task {
    bool live;
    int64_t ori;
    float p[3], d[3];
  };
  // this thread's row of the group's A tile: the position encoding of task k
  // (zeros when it is not live), [p, sin(2^i p), cos(2^i p)] for i = 0..9.
  // sin/cos of 2^i p: one accurate sincos per coordinate, then double-angle
  // steps (error ~2^9 x FP32 rounding at i = 9, below half an FP16 ulp).  The
  // 64 values are produced in order and stored 8 at a time (16-byte chunks).
  auto encode_row = [&](const Task& k) {
    float buf[8];
    int nb = 0, chunk = 0;
    auto emit = [&](float v) {
      buf[nb++] = v;
      if (nb == 8) {
        *reinterpret_cast<uint4*>(A + tc::sw128_offset(row, chunk)) =
            make_uint4(pack_h2(buf[0], buf[1]), pack_h2(buf[2], buf[3]), pack_h2(buf[4], buf[5]),
                       pack_h2(buf[6], buf[7]));
        ++chunk;
        nb = 0;
      }
    };
    const bool live = k.live;
    float sn[3], cs[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      emit(live ? k.p[a] : 0.f);
      sincosf(live ? k.p[a] : 0.f, &sn[a], &cs[a]);
    }
#pragma unroll
    for (int i = 0; i < 10; ++i) {
#pragma unroll
      for (int a = 0; a < 3; ++a) emit(live ? sn[a] : 0.f);
#pragma unroll
      for (int a = 0; a < 3; ++a) emit(live ? cs[a] : 0.f);
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        const float s2 = 2.f * sn[a] * cs[a], c2 = (cs[a] - sn[a]) * (cs[a] + sn[a]);
        sn[a] = s2;
        cs[a] = c2;
      }
    }
    emit(0.f);
  };
  for (;;) {
    __syncthreads();  // every thread has read the previous slot value; the network copy is free
    if (tid == 0) *blk_slot = atomicAdd(work, 1);
    __syncthreads();
    const int b = *blk_slot;
    if (b >= num_block) break;
    const int g = net[b];
    if (g < 0 || g >= num_groups) continue;  // -1: no network (the reference returns); bad ids are skipped
    if (g != cur_net) {
      pack_net(params + (size_t)g * kSpParams, sm, tid, NTH);
      tc::fence_proxy_async();
      __syncthreads();
      cur_net = g;
    }
    const float cx = centers[3 * g], cy = centers[3 * g + 1], cz = centers[3 * g + 2];
    const int64_t t0 = (int64_t)pstarts[b] * spr, t1 = (int64_t)pstarts[b + 1] * spr;
    auto fetch = [&](int64_t c) {
      Task k;
      const int64_t t = c + row;
      k.live = t < t1;
      k.ori = 0;
      if (k.live) {
        const int64_t pix = qpix[t / spr];
        k.live = transparency[pix] >= trans_stop;
        k.ori = pix * spr + t % spr;
        if (k.live) {
          k.p[0] = (samples[3 * k.ori] - cx) * inv_far;
          k.p[1] = (samples[3 * k.ori + 1] - cy) * inv_far;
          k.p[2] = (samples[3 * k.ori + 2] - cz) * inv_far;
          k.d[0] = rays_d[3 * pix];
          k.d[1] = rays_d[3 * pix + 1];
          k.d[2] = rays_d[3 * pix + 2];
        }
      }
      return k;
    };
    // this group's chunks of the block: t0 + 128 grp, then every 128 x 2 rows
    const int64_t gstart = t0 + 128 * grp, gstep = 128 * kSpGroups;
    bool gfail = false;
    // the row's sample of the current chunk, kept in shared memory for the
    // output step (registers hold only the next chunk's task)
    auto keep = [&](const Task& k) { *my_out = SpRowOut{k.live ? k.ori : -1, {k.d[0], k.d[1], k.d[2]}, 0.f}; };
    if (gstart < t1) {
      {
        const Task first = fetch(gstart);
        encode_row(first);
        keep(first);
      }
      tc::fence_proxy_async();
      for (int64_t c0 = gstart; c0 < t1; c0 += gstep) {
        const bool more = c0 + gstep < t1;
        tc::fence_before_sync();
        tc::bar_sync(gbar, 128);  // this chunk's A rows are visible to the group's MMA issuer
        Task nxt;
        nxt.live = false;
        float out[32];
        for (int l = 0; l <= kSpHidden; ++l) {
          if (tid == leader) {
            tc::fence_after_sync();
            const bool last = l == kSpHidden;
            const uint32_t wb = tc::smem_addr(sm + (last ? kSpWout : kSpW + l * 8192));
            const uint32_t id = last ? id_o : id_h;
            if (l == 0) {  // K = 64 position encodings from shared memory
              for (int kk = 0; kk < 4; ++kk)
                tc::mma_f16(gacc, tc::sdesc_sw128(a_base + 32 * kk), tc::sdesc_sw128(wb + 32 * kk), id, kk > 0);
            } else {  // K = 64 activations from tensor memory (8 columns per K = 16 step)
              for (int kk = 0; kk < 4; ++kk)
                tc::mma_f16_ta(gacc, tact + 8 * kk, tc::sdesc_sw128(wb + 32 * kk), id, kk > 0);
            }
            tc::mma_commit(mbar);
          }
          if (l == 0 && more) nxt = fetch(c0 + gstep);
          if (l == 1 && more) {  // layer 0 has read the A tile: the next chunk's encodings
            encode_row(nxt);
            tc::fence_proxy_async();
          }
          const bool ok = tid == leader ? tc::mbar_wait(mbar, mphase) : true;
          mphase ^= 1u;
          if (tc::bar_or(gbar, 128, !ok)) {
            gfail = true;
            if (tid == leader) drain.set(mbar, mphase ^ 1u);
            break;
          }
          tc::fence_after_sync();
          if (l < kSpHidden) {
            // bias + LeakyReLU + FP16 pack of 16 columns at a time into this
            // row's lane of the activation columns
#pragma unroll
            for (int part = 0; part < kSpH / 16; ++part) {
              float v[16];
              tc::tmem_ld16(taddr + 16 * part, v);
              tc::tmem_wait_ld();
              uint32_t o[8];
#pragma unroll
              for (int j = 0; j < 8; ++j) {
                const int col = 16 * part + 2 * j;
                float a0 = v[2 * j] + bias[64 * l + col], a1 = v[2 * j + 1] + bias[64 * l + col + 1];
                a0 = a0 < 0.f ? 0.01f * a0 : a0;
                a1 = a1 < 0.f ? 0.01f * a1 : a1;
                o[j] = pack_h2(a0, a1);
              }
              tc::tmem_st8(taddr + kSpH + 8 * part, o);
            }
            tc::tmem_wait_st();
          } else {
            tc::tmem_ld16(taddr, out);
            tc::tmem_ld16(taddr + 16, out + 16);
            tc::tmem_wait_ld();
#pragma unroll
            for (int j = 0; j < kSpOut; ++j) out[j] += bias[64 * kSpHidden + j];
          }
          tc::fence_before_sync();
          tc::bar_sync(gbar, 128);
        }
        if (gfail) break;
        const SpRowOut cur = *my_out;
        if (cur.ori >= 0) {
          const float dx = cur.d[0], dy = cur.d[1], dz = cur.d[2];
          const float inv = rsqrtf(dx * dx + dy * dy + dz * dz);
          const float X = dx * inv, Y = dy * inv, Z = dz * inv;
          const float C0 = 0.28209479177387814f, C1 = 0.4886025119029199f;
          const float C2[5] = {1.0925484305920792f, -1.0925484305920792f, 0.31539156525252005f, -1.0925484305920792f,
                               0.5462742152960396f};
          const float xx = X * X, yy = Y * Y, zz = Z * Z;
          float rgb[3];
#pragma unroll
          for (int i = 0; i < 3; ++i) {
            float v = C0 * out[i] - C1 * Y * out[3 + i] + C1 * Z * out[6 + i] - C1 * X * out[9 + i];
            v += C2[0] * X * Y * out[12 + i] + C2[1] * Y * Z * out[15 + i] + C2[2] * (2.f * zz - xx - yy) * out[18 + i] +
                 C2[3] * X * Z * out[21 + i] + C2[4] * (xx - yy) * out[24 + i];
            rgb[i] = 1.0f / (1.0f + expf(-v));
          }
          results[cur.ori] = make_float4(rgb[0], rgb[1], rgb[2], fmaxf(out[kSpOut - 1], 0.f));
        }
        if (more) keep(nxt);
      }
    }
    if (__syncthreads_or(gfail)) { failed = true; break; }
  }
  bool drained = true;
  if (failed && tid % 128 == 0) {
    if (err && tid == 0) atomicOr(err, kErrTimeout);
    drained = drain.run();
    if (!drained && err) atomicOr(err, kErrDrain);
  }
  tc::fence_before_sync();
  // tensor memory stays allocated when in-flight work did not drain
  if (__syncthreads_or(!drained) == 0 && warp == 0) tc::tmem_dealloc(tmem, 128 * kSpGroups);
}

}  // namespace

cudaError_t launch_sort_by_key(int16_t* keys, int32_t* values, int32_t* starts, int64_t n, int64_t* count_host,
                               cudaStream_t st) {
  if (n <= 0) {
    *count_host = 0;
    return cudaSuccess;
  }
  const int nblocks = (int)((n + kSortBlock - 1) / kSortBlock);
  const size_t hist_n = (size_t)256 * nblocks;
  // temporaries: keys x2, values, starts copy, flags/positions, histogram, count, scan tile sums
  const int scan_nb = max(scan::tiles((int64_t)hist_n), scan::tiles(n));
  const size_t bytes = (size_t)n * 2 * 2 + (size_t)n * 4 * 3 + hist_n * 4 + 64 + (size_t)scan_nb * 4 + 16;
  void* tmp = nullptr;
  cudaError_t e = cudaMallocAsync(&tmp, bytes, st);
  if (e != cudaSuccess) return e;
  uint8_t* q = static_cast<uint8_t*>(tmp);
  int16_t* k1 = reinterpret_cast<int16_t*>(q);
  int16_t* k2 = k1 + n;
  int32_t* v1 = reinterpret_cast<int32_t*>(q + (((size_t)n * 4 + 15) & ~size_t(15)));
  int32_t* s_copy = v1 + n;
  uint32_t* pos = reinterpret_cast<uint32_t*>(s_copy + n);
  uint32_t* hist = pos + n;
  int64_t* cnt = reinterpret_cast<int64_t*>((reinterpret_cast<uintptr_t>(hist + hist_n) + 7) & ~uintptr_t(7));
  uint32_t* scan_sums = reinterpret_cast<uint32_t*>(cnt + 1);
  const int64_t gb = (n + 255) / 256;
  const int g = (int)(gb < 65535 ? gb : 65535);
  do {
    if ((e = cudaMemcpyAsync(s_copy, starts, (size_t)n * 4, cudaMemcpyDeviceToDevice, st)) != cudaSuccess) break;
    // pass 0: keys/values -> k1/v1; pass 1: k1/v1 -> k2/values
    sort_hist_kernel<<<nblocks, kSortThreads, 0, st>>>(keys, n, 0, hist, nblocks);
    scan::exclusive(hist, (int64_t)hist_n, scan_sums, st);
    sort_scatter_kernel<<<nblocks, kSortThreads, 0, st>>>(keys, values, n, 0, hist, nblocks, k1, v1);
    sort_hist_kernel<<<nblocks, kSortThreads, 0, st>>>(k1, n, 1, hist, nblocks);
    scan::exclusive(hist, (int64_t)hist_n, scan_sums, st);
    sort_scatter_kernel<<<nblocks, kSortThreads, 0, st>>>(k1, v1, n, 1, hist, nblocks, k2, values);
    run_flags_kernel<<<g, 256, 0, st>>>(k2, n, pos);
    scan::exclusive(pos, n, scan_sums, st);
    run_compact_kernel<<<g, 256, 0, st>>>(k2, s_copy, pos, n, keys, starts);
    run_keys_kernel<<<g, 256, 0, st>>>(k2, pos, n, keys, cnt);
    if ((e = cudaGetLastError()) != cudaSuccess) break;
    if ((e = cudaMemcpyAsync(count_host, cnt, sizeof(int64_t), cudaMemcpyDeviceToHost, st)) != cudaSuccess) break;
  } while (false);
  cudaError_t e2 = cudaFreeAsync(tmp, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  return e != cudaSuccess ? e : e2;
}

cudaError_t launch_assign_pixels(const int16_t* net, const int32_t* pixel_starts, const int32_t* block_starts,
                                 int64_t num_net, int16_t* new_net, int32_t* new_pixel_starts, cudaStream_t st) {
  if (num_net <= 0) return cudaSuccess;
  const int64_t gb = (num_net + 127) / 128;
  assign_pixels_kernel<<<(int)(gb < 65535 ? gb : 65535), 128, 0, st>>>(
      net, pixel_starts, block_starts, num_net, new_net, new_pixel_starts);
  return cudaGetLastError();
}

int inference_mlp_param_count() { return kSpParams; }

cudaError_t launch_inference_mlp(int spr, int num_block, float inv_far, float trans_stop, const int16_t* net,
                                 int num_groups, const float* transparency, const int32_t* qpix,
                                 const int32_t* pstarts, const float* centers, const float* samples,
                                 const float* rays_d, const uint16_t* params, float* results, int* work,
                                 uint32_t* err, int num_sms, cudaStream_t st) {
  if (num_block <= 0) return cudaSuccess;
  const int smem = kSpSmem + 1024;
  static unsigned long long done = 0;
  cudaError_t e = once_per_device(&done, [&]() {
    return cudaFuncSetAttribute(inference_mlp_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  });
  if (e != cudaSuccess) return e;
  if ((e = cudaMemsetAsync(work, 0, sizeof(int), st)) != cudaSuccess) return e;
  const int grid = min(2 * num_sms, num_block);  // two CTAs of two groups per SM (shared memory ~80 KB each)
  inference_mlp_kernel<<<grid, 128 * kSpGroups, smem, st>>>(spr, num_block, inv_far, trans_stop, net, num_groups, transparency,
                                                qpix, pstarts, centers, samples, rays_d,
                                                reinterpret_cast<const __half*>(params),
                                                reinterpret_cast<float4*>(results), work, err);
  return cudaGetLastError();
}

}  // namespace snisr

using namespace snisr;

extern "C" {

snisr_status snisr_op_sort_by_key(int16_t* keys, int32_t* values, int32_t* starts, int64_t n, int64_t* num_unique,
                                  void* stream) {
  if (n < 0 || !num_unique) return set_error(SNISR_INVALID_ARG, "sort_by_key: bad argument");
  if (n > ((int64_t)1 << 31) - 1) return set_error(SNISR_INVALID_ARG, "sort_by_key: more than 2^31-1 elements");
  if (n > 0 && (!keys || !values || !starts)) return set_error(SNISR_INVALID_ARG, "sort_by_key: null argument");
  cudaError_t e = launch_sort_by_key(keys, values, starts, n, num_unique, (cudaStream_t)stream);
  if (e != cudaSuccess)
    return set_error(e == cudaErrorMemoryAllocation ? SNISR_OOM : SNISR_CUDA_ERROR,
                     std::string("sort_by_key: ") + cudaGetErrorString(e));
  return SNISR_OK;
}

snisr_status snisr_op_assign_pixels(const int16_t* net, const int32_t* pixel_starts, const int32_t* block_starts,
                                    int64_t num_net, int16_t* new_net, int32_t* new_pixel_starts, void* stream) {
  if (num_net < 0) return set_error(SNISR_INVALID_ARG, "assign_pixels: bad size");
  if (num_net == 0) return SNISR_OK;
  if (!net || !pixel_starts || !block_starts || !new_net || !new_pixel_starts)
    return set_error(SNISR_INVALID_ARG, "assign_pixels: null argument");
  cudaError_t e = launch_assign_pixels(net, pixel_starts, block_starts, num_net, new_net, new_pixel_starts,
                                       (cudaStream_t)stream);
  if (e != cudaSuccess) return set_error(SNISR_CUDA_ERROR, std::string("assign_pixels: ") + cudaGetErrorString(e));
  return SNISR_OK;
}

int32_t snisr_op_inference_mlp_param_count(void) { return inference_mlp_param_count(); }

snisr_status snisr_op_inference_mlp(int32_t samples_per_ray, int32_t num_block, float inverse_far, float trans_stop,
                                    const int16_t* net, int32_t num_groups, const float* transparency,
                                    const int32_t* query_pixel_indices, const int32_t* pixel_starts,
                                    const float* group_centers, const float* samples, const float* rays_d,
                                    const uint16_t* params, float* sample_results, uint32_t* err_dev, void* stream) {
  if (samples_per_ray <= 0 || num_block < 0 || num_groups < 0)
    return set_error(SNISR_INVALID_ARG, "inference_mlp: bad size");
  if (num_block == 0) return SNISR_OK;
  if (!net || !transparency || !query_pixel_indices || !pixel_starts || !group_centers || !samples || !rays_d ||
      !params || !sample_results)
    return set_error(SNISR_INVALID_ARG, "inference_mlp: null argument");
  cudaStream_t st = (cudaStream_t)stream;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  int* work = nullptr;
  cudaError_t e = cudaMallocAsync(&work, sizeof(int), st);
  if (e != cudaSuccess) return set_error(SNISR_OOM, std::string("inference_mlp: ") + cudaGetErrorString(e));
  e = launch_inference_mlp(samples_per_ray, num_block, inverse_far, trans_stop, net, num_groups, transparency,
                           query_pixel_indices, pixel_starts, group_centers, samples, rays_d, params, sample_results,
                           work, err_dev, sms > 0 ? sms : 1, st);
  cudaError_t e2 = cudaFreeAsync(work, st);
  if (e == cudaSuccess) e = e2;
  if (e != cudaSuccess) return set_error(SNISR_CUDA_ERROR, std::string("inference_mlp: ") + cudaGetErrorString(e));
  return SNISR_OK;
}

}  // extern "C"
