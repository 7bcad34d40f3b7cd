// Tensor-core (tcgen05, BF16 operands, FP32 accumulation) form of the
// training MLP: forward colours, which also leave each hidden layer's
// activations in global memory, and the backward pass over them.
//
// Samples are processed in chunks of 128 rows of one tile (chunk lists are
// per tile).  Activation tiles are written by the epilogues in the 128-byte
// swizzled layout with one sample per row; the same tiles serve as K-major
// A operands (samples = M) of the forward/backward data GEMMs and as MN-major
// operands (samples = K) of the weight-gradient GEMMs, whose accumulators
// stay in tensor memory across all chunks of a tile and are flushed with
// atomics when the CTA moves to another tile.
//
// Precision.  The forward pass that produces the colours splits its operands
// in three BF16 parts, v = hi + mid + lo (hi = bf16(v), mid = bf16(v - hi),
// lo = bf16(v - hi - mid)), and takes A.B down to the 2^-24 terms:
// A_hi.B_hi + A_mid.B_hi + A_hi.B_mid + A_mid.B_mid + A_lo.B_hi + A_hi.B_lo,
// as accurate as an FP32 evaluation.  The colours feed the loss, whose
// residuals near convergence are small: a two-part split (~2^-17 per
// operand) moved the loss gradient of the MLP parameters by ~1 %.  The
// biases enter in FP32.  The forward stores the hi parts of its hidden
// activations (16 KB per layer and 128-sample chunk, in the swizzled tile
// layout), and the backward loads them instead of recomputing: they give
// the ReLU masks and the weight-gradient operands.  Backward products
// (hidden deltas, weight gradients) use single BF16 operands: their
// rounding error is smooth (~2^-9 per operand).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "device_common.cuh"
#include "kernels.h"
#include "tc_ptx.cuh"

namespace snisr {

namespace {

struct __align__(16) TrainRecT {  // mirror of the record written by the march kernel
  uint32_t rec, ray, tile, pad0;
  float f[3], dv;
  float T, alpha, s, pad1;
};

constexpr uint32_t kBf16One = 0x3F803F80u;     // 1.0, two lanes

__device__ __forceinline__ uint32_t pack_bf2(float lo, float hi) {
  uint32_t d;
  asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(d) : "f"(hi), "f"(lo));
  return d;
}
__device__ __forceinline__ float bf_lo(uint32_t v) { return __uint_as_float(v << 16); }
__device__ __forceinline__ float bf_hi(uint32_t v) { return __uint_as_float(v & 0xFFFF0000u); }
// split of two values into BF16 hi and lo pairs
__device__ __forceinline__ void split_bf2(float a, float b, uint32_t& hi, uint32_t& lo) {
  hi = pack_bf2(a, b);
  lo = pack_bf2(a - bf_lo(hi), b - bf_hi(hi));
}
// three-part split of two values: hi, mid = bf16(v - hi), lo = bf16(v - hi - mid)
__device__ __forceinline__ void split3_bf2(float a, float b, uint32_t& hi, uint32_t& mid, uint32_t& lo) {
  hi = pack_bf2(a, b);
  const float ra = a - bf_lo(hi), rb = b - bf_hi(hi);
  mid = pack_bf2(ra, rb);
  lo = pack_bf2(ra - bf_lo(mid), rb - bf_hi(mid));
}
__device__ __forceinline__ void split3_bf16(float v, uint16_t& hi, uint16_t& mid, uint16_t& lo) {
  const __nv_bfloat16 h = __float2bfloat16_rn(v);
  hi = __bfloat16_as_ushort(h);
  const float r = v - __bfloat162float(h);
  const __nv_bfloat16 m = __float2bfloat16_rn(r);
  mid = __bfloat16_as_ushort(m);
  lo = __bfloat16_as_ushort(__float2bfloat16_rn(r - __bfloat162float(m)));
}
// positive BF16 value in the low / high half (sign clear, not zero)
__device__ __forceinline__ bool pos_lo(uint32_t v) { return (v & 0x8000u) == 0 && (v & 0x7FFFu) != 0; }
__device__ __forceinline__ bool pos_hi(uint32_t v) { return (v & 0x80000000u) == 0 && (v & 0x7FFF0000u) != 0; }

// MN-major 128B-swizzled descriptor: lbo = stride between 64-element MN
// atoms, sbo = stride between 8-row K groups (1024).
__device__ __forceinline__ uint64_t sdesc_mn(uint32_t saddr, uint32_t lbo) {
  return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)(1024u >> 4) << 32) | ((uint64_t)1u << 46) | ((uint64_t)2u << 61);
}

__device__ __forceinline__ uint32_t idesc_bf16(int n, bool a_mn, bool b_mn) {
  return tc::idesc_f16(n, 1) | (a_mn ? (1u << 15) : 0u) | (b_mn ? (1u << 16) : 0u);
}

// ---- per-tile weight image -------------------------------------------------
// All sub-tiles K-major, 128-byte swizzled, 64 K columns:
//   hi part : W_l [H][64] (l < L), W_out [16][64]
//   mid part: the same shapes holding bf16(w - hi)
//   W^T     : per layer l <= L, [64 rows = inputs of l][K = outputs] (hi only)
//   lo part : the shapes of the hi part holding bf16(w - hi - mid)
//   FP32 biases: per layer l <= L, 64 floats
// The forward copies the hi and mid parts, then the lo part and the FP32
// biases; the backward copies the W^T part [t_off, bwd_bytes).
struct ImageLayout {
  int hi_part, mid_off, t_off, bwd_bytes, lo_off, fbias_off, total;
  __host__ __device__ ImageLayout(int H, int L) {
    hi_part = L * H * 128 + 2048;
    mid_off = hi_part;
    t_off = 2 * hi_part;
    bwd_bytes = t_off + (L + 1) * 8192;
    lo_off = bwd_bytes;
    fbias_off = lo_off + hi_part;
    total = fbias_off + (L + 1) * 256;
  }
};

__device__ __forceinline__ uint32_t sw_off(int row, int k) {
  return (uint32_t)(row >> 3) * 1024u + (uint32_t)(row & 7) * 128u + ((uint32_t)((k >> 3) ^ (row & 7)) << 4) +
         (uint32_t)((k & 7) << 1);
}

__global__ void pack_train_weights(const float* __restrict__ mlp, int P, int IN, int H, int L, int stride,
                                   uint8_t* out) {
  const ImageLayout lay(H, L);
  const int tile = blockIdx.y;
  uint8_t* img = out + (size_t)tile * stride;
  const float* p = mlp + (size_t)tile * P;
  // the image was zeroed by the caller; one thread per parameter
  int64_t off = 0;
  for (int l = 0; l <= L; ++l) {
    const int fi = l == 0 ? IN : H, fo = l == L ? 3 : H;
    const int wofs = l < L ? l * H * 128 : L * H * 128;
    uint8_t* whi = img + wofs;
    uint8_t* wmid = img + lay.mid_off + wofs;
    uint8_t* wlo = img + lay.lo_off + wofs;
    uint8_t* tt = img + lay.t_off + l * 8192;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < fo * fi; e += gridDim.x * blockDim.x) {
      const int o = e / fi, i = e % fi;
      uint16_t h, m, lo;
      split3_bf16(p[off + e], h, m, lo);
      *reinterpret_cast<uint16_t*>(whi + sw_off(o, i)) = h;
      *reinterpret_cast<uint16_t*>(wmid + sw_off(o, i)) = m;
      *reinterpret_cast<uint16_t*>(wlo + sw_off(o, i)) = lo;
      *reinterpret_cast<uint16_t*>(tt + sw_off(i, o)) = h;
    }
    for (int o = blockIdx.x * blockDim.x + threadIdx.x; o < fo; o += gridDim.x * blockDim.x)
      reinterpret_cast<float*>(img + lay.fbias_off)[64 * l + o] = p[off + (int64_t)fi * fo + o];
    off += (int64_t)fi * fo + fo;
  }
}

// per-ray view encoding (27 values + 5 zeros) as BF16 hi [0,4), mid [4,8)
// and lo [8,12) uint4s
constexpr int kEncQuads = 12;
__global__ void ray_enc_kernel(const float* __restrict__ dirs, int64_t n, uint4* enc) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    float d[3] = {dirs[3 * i], dirs[3 * i + 1], dirs[3 * i + 2]};
    float e[32];
    dir_encoding(d, 4, e);
    for (int k = 27; k < 32; ++k) e[k] = 0.f;
    for (int q = 0; q < 4; ++q) {
      uint32_t h[4], m[4], l[4];
      for (int j = 0; j < 4; ++j) split3_bf2(e[8 * q + 2 * j], e[8 * q + 2 * j + 1], h[j], m[j], l[j]);
      enc[kEncQuads * i + q] = make_uint4(h[0], h[1], h[2], h[3]);
      enc[kEncQuads * i + 4 + q] = make_uint4(m[0], m[1], m[2], m[3]);
      enc[kEncQuads * i + 8 + q] = make_uint4(l[0], l[1], l[2], l[3]);
    }
  }
}

// chunk lists: chunks of 128 samples (coff) and units of 256 samples (coff2)
// never straddle tiles
__global__ void train_chunks_kernel(const int32_t* __restrict__ tstart, int NT, int32_t* coff, int32_t* coff2) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  int c = 0, c2 = 0;
  for (int t = 0; t < NT; ++t) {
    coff[t] = c;
    coff2[t] = c2;
    c += (tstart[t + 1] - tstart[t] + 127) / 128;
    c2 += (tstart[t + 1] - tstart[t] + 255) / 256;
  }
  coff[NT] = c;
  coff2[NT] = c2;
}

struct ChunkPos {
  int tile, row0, cnt;
};
// chunk c of the lists coff of `rows`-row chunks: its tile, first row and row count
__device__ __forceinline__ ChunkPos chunk_pos(int c, const int32_t* coff, const int32_t* tstart, int NT,
                                              int rows = 128) {
  int lo = 0, hi = NT;
  while (hi - lo > 1) {
    int mid = (lo + hi) >> 1;
    if (__ldg(coff + mid) <= c) lo = mid; else hi = mid;
  }
  ChunkPos p;
  p.tile = lo;
  p.row0 = __ldg(tstart + lo) + (c - __ldg(coff + lo)) * rows;
  p.cnt = min(rows, __ldg(tstart + lo + 1) - p.row0);
  return p;
}

// Gather of the split input rows [0,128) of the chunk into the NP part tiles
// X[0..NP) (hi; mid for NP >= 2; lo for NP = 3): lane (g, row) interpolates 8 FP32
// channels over the 8 corners of each of its rows; view encoding copied from
// the per-ray split table.  Loads are issued in stages across the lane's rows
// (records, then corner ids and encodings, then features) so that each stage
// waits for memory once, not once per row.
template <int NP>
struct PartTiles {
  uint8_t* p[NP];
};

template <int F, int NW, int NP>
__device__ __forceinline__ void gather_x(const SceneDev& S, const float* __restrict__ vfeat,
                                         const TrainRecT* __restrict__ recs, int row0, int cnt,
                                         const uint4* __restrict__ enc, PartTiles<NP> Xt, int warp, int lane) {
  uint8_t* const* X = Xt.p;
  // NW warps share the 128 rows: RPW rows per warp, RPI rows per lane pass
  constexpr int G = F / 8, RPI = 32 / G, RPW = 128 / NW, ITS = RPW / RPI;
  static_assert(RPW % RPI == 0, "rows per warp must be a multiple of rows per pass");
  static_assert(NP >= 1 && NP <= 3, "one to three parts");
  const int my_g = lane / RPI, my_row = lane % RPI;
  const uint4 z = make_uint4(0, 0, 0, 0);
  uint4 head[ITS], fr[ITS];  // {rec, ray, tile, pad}, {f0, f1, f2, dv}
#pragma unroll
  for (int it = 0; it < ITS; ++it) {
    const int r = warp * RPW + it * RPI + my_row;
    if (r < cnt) {
      const uint4* src = reinterpret_cast<const uint4*>(recs + row0 + r);
      head[it] = __ldg(src);
      fr[it] = __ldg(src + 1);
    }
  }
  int4 ca[ITS], cb[ITS];
  uint4 ev[ITS][NP];
#pragma unroll
  for (int it = 0; it < ITS; ++it) {
    const int r = warp * RPW + it * RPI + my_row;
    if (r < cnt) {
      const int4* cn = reinterpret_cast<const int4*>(S.corners + (size_t)head[it].x * 8);
      ca[it] = __ldg(cn);
      cb[it] = __ldg(cn + 1);
      if (my_g < 4) {  // G >= 4 lanes share a row: lane group g copies encoding chunk g (and g + G)
#pragma unroll
        for (int q = 0; q < NP; ++q) ev[it][q] = __ldg(enc + (size_t)head[it].y * kEncQuads + 4 * q + my_g);
      }
    }
  }
#pragma unroll
  for (int it = 0; it < ITS; ++it) {
    const int r = warp * RPW + it * RPI + my_row;
    if (r < cnt) {
      const float f[3] = {__uint_as_float(fr[it].x), __uint_as_float(fr[it].y), __uint_as_float(fr[it].z)};
      float w[8];
      trilinear_weights(f, w);
      const int c[8] = {ca[it].x, ca[it].y, ca[it].z, ca[it].w, cb[it].x, cb[it].y, cb[it].z, cb[it].w};
      float4 v0[8], v1[8];
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        const float4* src = reinterpret_cast<const float4*>(vfeat + (size_t)c[k] * F + 8 * my_g);
        v0[k] = __ldg(src);
        v1[k] = __ldg(src + 1);
      }
      // channel pairs accumulate with packed FP32x2 fused multiply-adds
      uint64_t acc2[4] = {0, 0, 0, 0};
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        const uint64_t w2 = f32x2(w[k], w[k]);
        acc2[0] = ffma2(w2, f32x2(v0[k].x, v0[k].y), acc2[0]);
        acc2[1] = ffma2(w2, f32x2(v0[k].z, v0[k].w), acc2[1]);
        acc2[2] = ffma2(w2, f32x2(v1[k].x, v1[k].y), acc2[2]);
        acc2[3] = ffma2(w2, f32x2(v1[k].z, v1[k].w), acc2[3]);
      }
      float acc[8];
#pragma unroll
      for (int j = 0; j < 4; ++j) split_f32x2(acc2[j], acc[2 * j], acc[2 * j + 1]);
      uint32_t pv[3][4];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        if (NP == 3)
          split3_bf2(acc[2 * j], acc[2 * j + 1], pv[0][j], pv[1][j], pv[2][j]);
        else if (NP == 2)
          split_bf2(acc[2 * j], acc[2 * j + 1], pv[0][j], pv[1][j]);
        else
          pv[0][j] = pack_bf2(acc[2 * j], acc[2 * j + 1]);
      }
#pragma unroll
      for (int q = 0; q < NP; ++q)
        *reinterpret_cast<uint4*>(X[q] + tc::sw128_offset(r, my_g)) = make_uint4(pv[q][0], pv[q][1], pv[q][2], pv[q][3]);
      if (my_g < 4) {
#pragma unroll
        for (int q = 0; q < NP; ++q) *reinterpret_cast<uint4*>(X[q] + tc::sw128_offset(r, G + my_g)) = ev[it][q];
      }
      if (G < 4 && my_g + G < 4) {  // G = 2: the second half of the encoding
#pragma unroll
        for (int q = 0; q < NP; ++q)
          *reinterpret_cast<uint4*>(X[q] + tc::sw128_offset(r, 2 * G + my_g)) =
              __ldg(enc + (size_t)head[it].y * kEncQuads + 4 * q + G + my_g);
      }
#pragma unroll
      for (int ch = G + 4 + my_g; ch < 8; ch += G) {
#pragma unroll
        for (int q = 0; q < NP; ++q) *reinterpret_cast<uint4*>(X[q] + tc::sw128_offset(r, ch)) = z;
      }
    } else {
#pragma unroll
      for (int ch = my_g; ch < 8; ch += G) {
#pragma unroll
        for (int q = 0; q < NP; ++q) *reinterpret_cast<uint4*>(X[q] + tc::sw128_offset(r, ch)) = z;
      }
    }
  }
}

struct Bars {
  uint32_t wbar, mbar;
  uint32_t wphase, mphase;
};

__device__ __forceinline__ bool wait_mma(Bars& b, int tid) {
  bool ok = tid == 0 ? tc::mbar_wait(b.mbar, b.mphase) : true;
  b.mphase ^= 1u;
  ok = !__syncthreads_or(!ok);
  tc::fence_after_sync();
  return ok;
}

// ---------------------------------------------------------------------------
// Forward: per-sample colour c = sigmoid(MLP(x)) on tcgen05, three-part
// split operands.  One CTA per SM of NG groups of 4 warps: a work unit is
// NG x 128 rows of one tile, group g gathers, and runs the epilogues of,
// rows [128 g, 128 g + 128) with its own part tiles and tensor-memory
// accumulators; the weight image (hi, mid, lo parts, FP32 biases) is shared.
// Within a unit the groups run their layer chains apart: each has its own
// MMA issuer (its first thread), mbarrier and named barrier, so that one
// group's epilogue overlaps the other group's MMAs.
//
// Accumulation.  The tensor core's FP32 accumulation is not a
// round-to-nearest sum: chained into one accumulator over the 24 MMAs of a
// layer, its error was biased and moved the loss gradient by ~0.5 %.  So
// the products A_hi.W_hi, the bulk of the value, go to two accumulators of
// their own (K steps [0, ks/2) and [ks/2, ks), two MMAs each), the five
// smaller terms of all K steps to a third (their error is 2^-8 smaller),
// and the epilogue adds them and the FP32 bias on the CUDA cores.  Per
// group, 3 x 64 tensor-memory columns at 256 g.
// ---------------------------------------------------------------------------
constexpr int kFwdTileBytes = 3 * 16384;  // hi, mid, lo part tiles of one group

int fwd_smem_bytes(const ImageLayout& lay, int ng) {
  return 1024 + ng * kFwdTileBytes + (lay.total - lay.lo_off) + 2 * lay.hi_part + 64;  // + 3 mbarriers, slots
}

// one layer's MMAs for one group: acc + 0 / acc + 64 = the hi.hi products of
// the first / second half of the K steps, acc + 128 = the smaller terms
__device__ __forceinline__ void issue_fwd_layer(uint32_t acc, const uint32_t (&a)[3], const uint32_t (&w)[3], int n,
                                                int ksteps) {
  const uint32_t id = idesc_bf16(n, false, false);
  const int half = ksteps / 2;
  for (int kk = 0; kk < ksteps; ++kk) {
    const uint64_t ah = tc::sdesc_sw128(a[0] + 32 * kk), am = tc::sdesc_sw128(a[1] + 32 * kk);
    const uint64_t al = tc::sdesc_sw128(a[2] + 32 * kk);
    const uint64_t wh = tc::sdesc_sw128(w[0] + 32 * kk), wm = tc::sdesc_sw128(w[1] + 32 * kk);
    const uint64_t wl = tc::sdesc_sw128(w[2] + 32 * kk);
    tc::mma_f16(acc + 64u * (uint32_t)(kk / half), ah, wh, id, kk % half != 0);
    tc::mma_f16(acc + 128u, am, wh, id, kk > 0);
    tc::mma_f16(acc + 128u, ah, wm, id, 1u);
    tc::mma_f16(acc + 128u, am, wm, id, 1u);
    tc::mma_f16(acc + 128u, al, wh, id, 1u);
    tc::mma_f16(acc + 128u, ah, wl, id, 1u);
  }
}

// columns [col, col + 16) of this thread's row: the two hi.hi accumulators,
// the small-term accumulator and the FP32 bias, summed
__device__ __forceinline__ void fwd_sum16(uint32_t taddr, int col, const float* bias, float (&x)[16]) {
  float u[16], t[16];
  tc::tmem_ld16(taddr + col, x);
  tc::tmem_ld16(taddr + 64 + col, u);
  tc::tmem_ld16(taddr + 128 + col, t);
  tc::tmem_wait_ld();
#pragma unroll
  for (int j = 0; j < 16; ++j) x[j] = ((x[j] + u[j]) + t[j]) + bias[col + j];
}

// hidden-layer epilogue: ReLU of the summed accumulators, three-part split
// into the group's part tiles
template <int H>
__device__ __forceinline__ void epi_fwd_hidden(uint32_t taddr, const float* bias, uint8_t* const (&dst)[3],
                                               int row) {
#pragma unroll
  for (int col = 0; col < H; col += 16) {
    float x[16];
    fwd_sum16(taddr, col, bias, x);
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      uint32_t pv[3][4];
#pragma unroll
      for (int j = 0; j < 4; ++j)
        split3_bf2(fmaxf(x[8 * q + 2 * j], 0.f), fmaxf(x[8 * q + 2 * j + 1], 0.f), pv[0][j], pv[1][j], pv[2][j]);
#pragma unroll
      for (int k = 0; k < 3; ++k)
        *reinterpret_cast<uint4*>(dst[k] + tc::sw128_offset(row, col / 8 + q)) =
            make_uint4(pv[k][0], pv[k][1], pv[k][2], pv[k][3]);
    }
  }
}

template <int F, int H, int L, int NG>
__global__ void __launch_bounds__(128 * NG, 1) tr_mlp_fwd_tc(SceneDev S, const float* __restrict__ vfeat,
                                                             const TrainRecT* __restrict__ recs,
                                                             const int32_t* __restrict__ tstart,
                                                             const int32_t* __restrict__ uoff,
                                                             const int32_t* __restrict__ coff, int* work,
                                                             const uint4* __restrict__ enc,
                                                             const uint8_t* __restrict__ wimg, int img_stride,
                                                             float4* cout, uint8_t* htiles) {
  constexpr int KH = H / 16, NTMEM = NG == 1 ? 256 : 512;
  static_assert(NG == 1 || NG == 2, "one or two groups");
  static_assert(KH % 2 == 0 && H <= 64, "two hi.hi accumulators of up to 64 columns");
  const ImageLayout lay(H, L);
  extern __shared__ uint8_t smem_raw[];
  uint8_t* base = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int grp = warp >> 2, gw = warp & 3, row = tid & 127;
  const int leader = 128 * grp;  // the group's MMA issuer
  const uint32_t gbar = 1u + (uint32_t)grp;
  uint8_t* gbase = base + grp * kFwdTileBytes;
  uint8_t* const A[3] = {gbase, gbase + 16384, gbase + 32768};  // this group's hi, mid, lo part tiles
  uint8_t* Wsm = base + NG * kFwdTileBytes;                    // image: hi, mid parts, then lo part, FP32 biases
  const float* fbias = reinterpret_cast<const float*>(Wsm + 3 * lay.hi_part);
  uint64_t* bars = reinterpret_cast<uint64_t*>(Wsm + 2 * lay.hi_part + (lay.total - lay.lo_off));
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 3);
  int* unit_slot = reinterpret_cast<int*>(tmem_slot + 1);
  const int NT = S.num_tiles;
  const uint32_t wbar = tc::smem_addr(bars), mbar = tc::smem_addr(bars + 1 + grp);
  uint32_t wphase = 0, mphase = 0;
  if (tid == 0) {
    tc::mbar_init(wbar, 1);
    for (int g = 0; g < NG; ++g) tc::mbar_init(tc::smem_addr(bars + 1 + g), 1);
    tc::fence_mbar_init();
  }
  if (warp == 0) {
    tc::tmem_alloc(tc::smem_addr(tmem_slot), NTMEM);
    tc::tmem_relinquish();
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *tmem_slot;
  const uint32_t gacc = tmem + 256u * (uint32_t)grp;  // the group's accumulators
  const uint32_t taddr = gacc + ((uint32_t)(gw * 32) << 16);  // this thread's row (lane quarter gw)
  const uint32_t a3[3] = {tc::smem_addr(A[0]), tc::smem_addr(A[1]), tc::smem_addr(A[2])};
  const int total = uoff[NT];
  int cur_tile = -1;
  bool failed = false;
  tc::Drain drain;  // on the group leaders: in-flight weight copy or MMAs at a timeout
  for (;;) {
    if (tid == 0) *unit_slot = atomicAdd(work, 1);
    __syncthreads();
    const int c = *unit_slot;
    if (c >= total) break;
    const ChunkPos cp = chunk_pos(c, uoff, tstart, NT, 128 * NG);
    const int my_cnt = min(128, cp.cnt - 128 * grp);  // rows of this group (uniform per group)
    // this group's 128-row chunk in the backward's chunk list (units of NG
    // chunks start at the same rows), where its hidden activations go
    const int my_chunk = NG == 1 ? c : __ldg(coff + cp.tile) + NG * (c - __ldg(uoff + cp.tile)) + grp;
    uint8_t* my_htiles = htiles + (size_t)my_chunk * L * 16384;
    const bool new_w = cp.tile != cur_tile;
    if (new_w && tid == 0) {
      const uint8_t* img = wimg + (size_t)cp.tile * img_stride;
      const uint32_t tail = (uint32_t)(lay.total - lay.lo_off);
      tc::mbar_arrive_expect_tx(wbar, (uint32_t)(2 * lay.hi_part) + tail);
      tc::bulk_g2s(tc::smem_addr(Wsm), img, (uint32_t)(2 * lay.hi_part), wbar);
      tc::bulk_g2s(tc::smem_addr(Wsm + 2 * lay.hi_part), img + lay.lo_off, tail, wbar);
    }
    cur_tile = cp.tile;
    if (my_cnt > 0)
      gather_x<F, 4, 3>(S, vfeat, recs, cp.row0 + 128 * grp, my_cnt, enc, PartTiles<3>{{A[0], A[1], A[2]}}, gw, lane);
    tc::fence_proxy_async();
    if (new_w) {
      bool ok = tid == 0 ? tc::mbar_wait(wbar, wphase) : true;
      wphase ^= 1u;
      if (__syncthreads_or(!ok)) {
        failed = true;
        if (tid == 0) drain.set(wbar, wphase ^ 1u);
        break;
      }
    } else {
      __syncthreads();
    }
    // the group's layer chain
    const uint32_t w = tc::smem_addr(Wsm);
    float out3[3] = {0.f, 0.f, 0.f};
    bool gfail = false;
    if (my_cnt > 0) {
      for (int l = 0; l <= L; ++l) {
        if (tid == leader) {
          tc::fence_after_sync();
          const uint32_t wofs = (uint32_t)(l < L ? l * H * 128 : L * H * 128);
          const uint32_t w3[3] = {w + wofs, w + lay.hi_part + wofs, w + 2 * lay.hi_part + wofs};
          issue_fwd_layer(gacc, a3, w3, l < L ? H : 16, l == 0 ? 4 : KH);
          tc::mma_commit(mbar);
          // the previous layer's activation tile has been read out before
          // this layer's epilogue overwrites it
          if (l > 0) tc::bulk_wait_read();
        }
        const bool ok = tid == leader ? tc::mbar_wait(mbar, mphase) : true;
        mphase ^= 1u;
        if (tc::bar_or(gbar, 128, !ok)) {
          gfail = true;
          if (tid == leader) drain.set(mbar, mphase ^ 1u);
          break;
        }
        tc::fence_after_sync();
        if (l < L) {
          epi_fwd_hidden<H>(taddr, fbias + 64 * l, A, row);  // the output layer also takes split inputs
          tc::fence_proxy_async();
        } else {
          float x[16];
          fwd_sum16(taddr, 0, fbias + 64 * L, x);
          out3[0] = x[0]; out3[1] = x[1]; out3[2] = x[2];
        }
        tc::fence_before_sync();
        tc::bar_sync(gbar, 128);
        if (l < L && tid == leader) {  // the hi activations of hidden layer l, for the backward
          tc::bulk_s2g(my_htiles + (size_t)l * 16384, a3[0], 16384u);
          tc::bulk_commit();
        }
      }
    }
    if (__syncthreads_or(gfail)) { failed = true; break; }
    if (row < my_cnt)
      cout[cp.row0 + 128 * grp + row] =
          make_float4(sigmoidf_(out3[0]), sigmoidf_(out3[1]), sigmoidf_(out3[2]), 0.f);
  }
  if (tid == leader) tc::bulk_wait_all();  // the activation tiles are written
  bool drained = true;
  if (failed && tid % 128 == 0) {
    if (tid == 0) atomicOr(S.err, ERR_TIMEOUT);
    drained = drain.run();
    if (!drained) atomicOr(S.err, ERR_DRAIN);
  }
  tc::fence_before_sync();
  // tensor memory stays allocated when in-flight work did not drain
  if (__syncthreads_or(!drained) == 0 && warp == 0) tc::tmem_dealloc(tmem, NTMEM);
}

// ---------------------------------------------------------------------------
// Backward on tcgen05.  Tensor memory (512 columns): [0,64) data-GEMM
// accumulator, then per layer l = 0..L a weight-gradient accumulator
// (128 lanes = output units, 64 columns = inputs) and a 16-column bias
// accumulator (column 0 used), both living across the chunks of a tile.
//
// Shared memory tiles (16 KB, one sample per 128-byte row), in this order:
//   D (hidden delta), X (input hi), H1..HL (activation hi: the forward's,
//   bulk-loaded per chunk), DO (output-logit gradient); then the weight
//   image's W^T part.
// An MN-major M = 128 operand spans two 64-wide atoms 16 KB apart: for D and
// DO the second atom is the next tile, whose products land in accumulator
// lanes 64..127 (output units that do not exist) and are never read.
// ---------------------------------------------------------------------------
constexpr int kBwdRun = 4;
// weight-gradient staging per tile: per layer 64 rows x 64 columns, then 64
// biases (16-byte aligned rows for vector reductions)
constexpr int kDwStageLayer = 64 * 64 + 64, kDwStageTile = 4 * kDwStageLayer;

// gmlp[t][P] += the staged weight gradients (one thread per parameter)
__global__ void apply_dw_kernel(const float* __restrict__ gstage, int NT, int IN, int H, int L, int P,
                                float* gmlp) {
  const int64_t total = (int64_t)NT * P;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int t = (int)(idx / P);
    int j = (int)(idx % P);
    for (int l = 0; l <= L; ++l) {
      const int fi = l == 0 ? IN : H, fo = l == L ? 3 : H;
      const float* Gl = gstage + (size_t)t * kDwStageTile + (size_t)l * kDwStageLayer;
      if (j < fi * fo) {
        gmlp[idx] += Gl[(j / fi) * 64 + j % fi];
        break;
      }
      j -= fi * fo;
      if (j < fo) {
        gmlp[idx] += Gl[4096 + j];
        break;
      }
      j -= fo;
    }
  }
}

template <int F, int H, int L>
__global__ void __launch_bounds__(256, 1) tr_mlp_bwd_tc(SceneDev S, const float* __restrict__ vfeat,
                                                        const TrainRecT* __restrict__ recs,
                                                        const int32_t* __restrict__ tstart,
                                                        const int32_t* __restrict__ coff, int* work,
                                                        const uint4* __restrict__ enc, const uint8_t* __restrict__ wimg,
                                                        int img_stride, const float4* __restrict__ dout, float* gvfeat,
                                                        float* gstage, const uint8_t* __restrict__ htiles) {
  constexpr int IN = F + 27;
  constexpr int kTiles = 3 + L;
  const ImageLayout lay(H, L);
  extern __shared__ uint8_t smem_raw[];
  uint8_t* base = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint8_t* Dt = base;
  uint8_t* Xt = base + 16384;
  uint8_t* Ht = base + 2 * 16384;  // H_l at Ht + (l-1)*16384, l = 1..L
  uint8_t* DOt = base + (2 + L) * 16384;
  uint8_t* Wsm = base + kTiles * 16384;  // the weight image's W^T part
  const int wt_bytes = lay.bwd_bytes - lay.t_off;
  uint8_t* ones = Wsm + ((wt_bytes + 1023) & ~1023);  // 1 KB of 1.0
  uint64_t* bars = reinterpret_cast<uint64_t*>(ones + 1024);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 3);
  int* chunk_slot = reinterpret_cast<int*>(tmem_slot + 1);
  // 8 warps: warps w and w + 4 read the same tensor-memory lane quarter
  // (rows 32 (w % 4) ..) and split the accumulator columns (part = w / 4)
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int row = tid & 127, part = tid >> 7;
  const int NT = S.num_tiles;
  Bars B{tc::smem_addr(bars), tc::smem_addr(bars + 1), 0u, 0u};
  const uint32_t hbar = tc::smem_addr(bars + 2);  // the chunk's activation tiles
  uint32_t hphase = 0;
  if (tid == 0) {
    tc::mbar_init(B.wbar, 1);
    tc::mbar_init(B.mbar, 1);
    tc::mbar_init(hbar, 1);
    tc::fence_mbar_init();
  }
  if (warp == 0) {
    tc::tmem_alloc(tc::smem_addr(tmem_slot), 512);
    tc::tmem_relinquish();
  }
  for (int k = tid; k < 64; k += 256)
    reinterpret_cast<uint4*>(ones)[k] = make_uint4(kBf16One, kBf16One, kBf16One, kBf16One);
  // all tiles start zeroed: DO columns beyond 3 and the columns beyond H of
  // the activation / delta tiles are never written afterwards
  for (int k = tid; k < kTiles * 16384 / 16; k += 256) reinterpret_cast<uint4*>(base)[k] = make_uint4(0, 0, 0, 0);
  tc::fence_proxy_async();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *tmem_slot;
  const uint32_t tw = tmem;  // data accumulator
  auto tdw = [&](int l) { return tmem + 64u + 64u * (uint32_t)l; };
  auto tdb = [&](int l) { return tmem + 64u + 64u * (uint32_t)(L + 1) + 16u * (uint32_t)l; };
  const uint64_t ones1 = tc::sdesc_sw128_sbo(tc::smem_addr(ones), 0);
  const int total = coff[NT];
  int cur_tile = -1;
  bool failed = false, have_acc = false;
  tc::Drain drain;
  const uint32_t taddr = tmem + ((uint32_t)((warp & 3) * 32) << 16);
  int run_c = 0, run_left = 0;

  // flush the weight/bias gradient accumulators of `tile` to global memory
  // (lanes = output units: threads 0..fo-1 of the first part)
  // into the aligned staging rows (64 columns per output unit; the input
  // columns past fi accumulate zeros), by vector reductions: part p adds
  // columns [32 p, 32 p + 32) of rows 0..fo-1, part 0 the biases
  (void)IN;
  auto flush = [&](int tile) {
    float* G = gstage + (size_t)tile * kDwStageTile;
    for (int l = 0; l <= L; ++l) {
      const int fo = l == L ? 3 : H;
      float* Gl = G + l * kDwStageLayer;
#pragma unroll
      for (int cc = 0; cc < 32; cc += 16) {
        const int col = part * 32 + cc;
        float v[16];
        tc::tmem_ld16(taddr + 64u + 64u * l + col, v);
        tc::tmem_wait_ld();
        if (row < fo) {
#pragma unroll
          for (int q = 0; q < 16; q += 4)
            red_add_v4(Gl + row * 64 + col + q, v[q], v[q + 1], v[q + 2], v[q + 3]);
        }
      }
      if (part == 0) {
        float bv[4];
        tc::tmem_ld4(taddr + 64u + 64u * (L + 1) + 16u * l, bv);
        tc::tmem_wait_ld();
        if (row < fo) atomicAdd(Gl + 4096 + row, bv[0]);
      }
    }
  };

  for (;;) {
    // chunks are claimed in runs of kBwdRun consecutive ones (mostly of one
    // tile), so that the weight-gradient accumulators are flushed less often
    if (run_left == 0) {
      if (tid == 0) *chunk_slot = atomicAdd(work, kBwdRun);
      __syncthreads();
      run_c = *chunk_slot;
      run_left = kBwdRun;
      __syncthreads();  // every thread has read the slot before it is claimed again
    }
    const int c = run_c++;
    --run_left;
    if (c >= total) break;
    const ChunkPos cp = chunk_pos(c, coff, tstart, NT);
    const bool new_w = cp.tile != cur_tile;
    if (new_w && have_acc) {
      tc::fence_after_sync();
      flush(cur_tile);
      tc::fence_before_sync();
      __syncthreads();
    }
    if (new_w && tid == 0) {
      tc::mbar_arrive_expect_tx(B.wbar, (uint32_t)wt_bytes);
      tc::bulk_g2s(tc::smem_addr(Wsm), wimg + (size_t)cp.tile * img_stride + lay.t_off, (uint32_t)wt_bytes, B.wbar);
    }
    const bool first_of_tile = new_w;
    cur_tile = cp.tile;
    // this thread's own row: output gradient, and the record and corner ids
    // the feature-gradient scatter needs at the end of the chunk (loaded now,
    // consumed after the MMA chain)
    const bool mine = row < cp.cnt;
    float4 dmine = make_float4(0.f, 0.f, 0.f, 0.f);
    uint4 my_fr = make_uint4(0, 0, 0, 0);
    int4 my_cn = make_int4(0, 0, 0, 0);  // corners 4 part .. 4 part + 3 (each part scatters four)
    if (mine) {
      if (part == 0) dmine = __ldg(dout + cp.row0 + row);
      const uint4* src = reinterpret_cast<const uint4*>(recs + cp.row0 + row);
      const uint32_t my_rec = __ldg(src).x;
      my_fr = __ldg(src + 1);
      my_cn = __ldg(reinterpret_cast<const int4*>(S.corners + (size_t)my_rec * 8) + part);
    }
    // the forward's hidden activations of this chunk (hi parts, swizzled tiles)
    if (tid == 0) {
      tc::mbar_arrive_expect_tx(hbar, (uint32_t)(L * 16384));
      for (int l = 0; l < L; ++l)
        tc::bulk_g2s(tc::smem_addr(Ht + l * 16384), htiles + ((size_t)c * L + l) * 16384, 16384u, hbar);
    }
    gather_x<F, 8, 1>(S, vfeat, recs, cp.row0, cp.cnt, enc, PartTiles<1>{{Xt}}, warp, lane);
    // output-gradient rows (3 values, BF16) of the DO tile; other columns stay 0
    if (part == 0)
      *reinterpret_cast<uint2*>(DOt + tc::sw128_offset(row, 0)) =
          make_uint2(pack_bf2(dmine.x, dmine.y), pack_bf2(dmine.z, 0.f));
    tc::fence_proxy_async();
    __syncthreads();
    if (new_w) {
      bool ok = tid == 0 ? tc::mbar_wait(B.wbar, B.wphase) : true;
      B.wphase ^= 1u;
      if (__syncthreads_or(!ok)) { failed = true; drain.set(B.wbar, B.wphase ^ 1u); break; }
    }
    {
      bool ok = tid == 0 ? tc::mbar_wait(hbar, hphase) : true;
      hphase ^= 1u;
      if (__syncthreads_or(!ok)) { failed = true; drain.set(hbar, hphase ^ 1u); break; }
      tc::fence_after_sync();
    }
    const uint32_t w = tc::smem_addr(Wsm);
    // backward: layer L (output) down to 0.  delta of layer l's output is in
    // DO (l = L) or D; its input activation is HL..H1 or X.
    for (int l = L; l >= 0; --l) {
      const uint32_t dlt = tc::smem_addr(l == L ? DOt : Dt);
      const uint32_t act = tc::smem_addr(l == 0 ? Xt : Ht + (l - 1) * 16384);
      if (tid == 0) {
        tc::fence_after_sync();
        const bool acc0 = !first_of_tile;
        // weight gradient: dW_l[o][i] += sum_s delta[s][o] act[s][i]  (K = 128 samples)
        const uint32_t idw = idesc_bf16(64, true, true);
        for (int kk = 0; kk < 8; ++kk)
          tc::mma_f16(tdw(l), sdesc_mn(dlt + 2048 * kk, 16384), sdesc_mn(act + 2048 * kk, 16384), idw,
                      (acc0 || kk > 0) ? 1u : 0u);
        // bias gradient: db_l[o] += sum_s delta[s][o]  (B = ones, K-major)
        const uint32_t idb = idesc_bf16(16, true, false);
        for (int kk = 0; kk < 8; ++kk)
          tc::mma_f16(tdb(l), sdesc_mn(dlt + 2048 * kk, 16384), ones1, idb, (acc0 || kk > 0) ? 1u : 0u);
        // data gradient w.r.t. the layer input: delta x W_l^T (N = 64 inputs)
        const uint32_t wt = w + 8192u * (uint32_t)l;
        const uint32_t idd = idesc_bf16(64, false, false);
        const int ksteps = l == L ? 1 : H / 16;
        for (int kk = 0; kk < ksteps; ++kk)
          tc::mma_f16(tw, tc::sdesc_sw128(dlt + 32 * kk), tc::sdesc_sw128(wt + 32 * kk), idd, kk > 0);
        tc::mma_commit(B.mbar);
      }
      if (!wait_mma(B, tid)) { failed = true; drain.set(B.mbar, B.mphase ^ 1u); break; }
      if (l > 0) {
        // delta of layer l-1's output = (delta W_l) * [act > 0], BF16 into D;
        // this thread's part: columns [part H/2, (part+1) H/2)
        constexpr int CP = H / 2;
        float v[CP];
#pragma unroll
        for (int j = 0; j < CP; j += 16) tc::tmem_ld16(taddr + part * CP + j, v + j);
        tc::tmem_wait_ld();
#pragma unroll
        for (int q = 0; q < CP / 8; ++q) {
          const int chunk = part * (CP / 8) + q;
          const uint4 hv = *reinterpret_cast<const uint4*>(Ht + (l - 1) * 16384 + tc::sw128_offset(row, chunk));
          const uint32_t hw[4] = {hv.x, hv.y, hv.z, hv.w};
          uint32_t o[4];
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            const float a0 = pos_lo(hw[j]) ? v[8 * q + 2 * j] : 0.f;
            const float a1 = pos_hi(hw[j]) ? v[8 * q + 2 * j + 1] : 0.f;
            o[j] = pack_bf2(a0, a1);
          }
          *reinterpret_cast<uint4*>(Dt + tc::sw128_offset(row, chunk)) = make_uint4(o[0], o[1], o[2], o[3]);
        }
        tc::fence_proxy_async();
      } else {
        // feature gradient: first F inputs (the TMEM load is warp-collective,
        // so every thread loads), scattered to the 8 corner vertices
        float dx[F];
#pragma unroll
        for (int cc = 0; cc < F; cc += 16) tc::tmem_ld16(taddr + cc, dx + cc);
        tc::tmem_wait_ld();
        if (mine) {
          const float f[3] = {__uint_as_float(my_fr.x), __uint_as_float(my_fr.y), __uint_as_float(my_fr.z)};
          float wk[8];
          trilinear_weights(f, wk);
          const int cn[4] = {my_cn.x, my_cn.y, my_cn.z, my_cn.w};
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            const float wkk = wk[4 * part + k];
            float* g = gvfeat + (size_t)cn[k] * F;  // 16-byte aligned rows (F a multiple of 4)
#pragma unroll
            for (int q = 0; q < F; q += 4)
              red_add_v4(g + q, wkk * dx[q], wkk * dx[q + 1], wkk * dx[q + 2], wkk * dx[q + 3]);
          }
        }
      }
      tc::fence_before_sync();
      __syncthreads();
    }
    if (failed) break;
    have_acc = true;
  }
  if (!failed && have_acc) {
    tc::fence_after_sync();
    flush(cur_tile);
  }
  bool drained = true;
  if (failed && tid == 0) {
    atomicOr(S.err, ERR_TIMEOUT);
    drained = drain.run();
    if (!drained) atomicOr(S.err, ERR_DRAIN);
  }
  tc::fence_before_sync();
  // tensor memory stays allocated when in-flight work did not drain
  if (__syncthreads_or(!drained) == 0 && warp == 0) tc::tmem_dealloc(tmem, 512);
}

}  // namespace

int train_tc_image_bytes(int H, int L) { return ImageLayout(H, L).total; }

// dynamic shared memory of the backward kernel (checked against the 227 KB limit)
int train_tc_bwd_smem_bytes(int H, int L) {
  const ImageLayout lay(H, L);
  return 1024 + 16384 * (3 + L) + ((lay.bwd_bytes - lay.t_off + 1023) & ~1023) + 1024 + 64;
}

template <int F, int H, int L>
cudaError_t launch_train_tc_t(const SceneDev& S, const TrainTcArgs& a, bool backward, cudaStream_t st) {
  const ImageLayout lay(H, L);
  cudaError_t e;
  if (!backward) {
    e = cudaMemsetAsync(a.wimg, 0, (size_t)a.img_stride * S.num_tiles, st);
    if (e != cudaSuccess) return e;
    pack_train_weights<<<dim3(32, S.num_tiles), 256, 0, st>>>(a.mlp, S.params_per_tile, F + 27, H, L, a.img_stride,
                                                              a.wimg);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    ray_enc_kernel<<<(int)((a.n + 127) / 128 < 65536 ? (a.n + 127) / 128 : 65536), 128, 0, st>>>(a.dirs, a.n, a.enc);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    train_chunks_kernel<<<1, 32, 0, st>>>(a.tstart, S.num_tiles, a.coff, a.coff + S.num_tiles + 2);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  e = cudaMemsetAsync(a.work, 0, sizeof(int), st);
  if (e != cudaSuccess) return e;
  if (!backward) {
    // one CTA per SM of one or two 4-warp groups (128 or 256 rows per work unit)
    const int ng = a.fwd_warps == 4 ? 1 : 2;
    const int smem = fwd_smem_bytes(lay, ng);
    static unsigned long long cfg1 = 0, cfg2 = 0;
    e = once_per_device(ng == 1 ? &cfg1 : &cfg2, [&]() {
      return cudaFuncSetAttribute(ng == 1 ? tr_mlp_fwd_tc<F, H, L, 1> : tr_mlp_fwd_tc<F, H, L, 2>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    });
    if (e != cudaSuccess) return e;
    const int32_t* uoff = ng == 1 ? a.coff : a.coff + S.num_tiles + 2;
    (ng == 1 ? tr_mlp_fwd_tc<F, H, L, 1> : tr_mlp_fwd_tc<F, H, L, 2>)<<<a.num_sms, 128 * ng, smem, st>>>(
        S, a.vfeat, (const TrainRecT*)a.recs, a.tstart, uoff, a.coff, a.work, a.enc, a.wimg, a.img_stride, a.cout,
        a.htiles);
  } else {
    const int smem = train_tc_bwd_smem_bytes(H, L);
    static unsigned long long cfg = 0;
    e = once_per_device(&cfg, [&]() {
      return cudaFuncSetAttribute(tr_mlp_bwd_tc<F, H, L>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    });
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(a.gstage, 0, (size_t)S.num_tiles * kDwStageTile * sizeof(float), st);
    if (e != cudaSuccess) return e;
    tr_mlp_bwd_tc<F, H, L><<<a.num_sms, 256, smem, st>>>(S, a.vfeat, (const TrainRecT*)a.recs, a.tstart, a.coff,
                                                         a.work, a.enc, a.wimg, a.img_stride, a.dout, a.gvfeat,
                                                         a.gstage, a.htiles);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    const int64_t np = (int64_t)S.num_tiles * S.params_per_tile;
    apply_dw_kernel<<<(int)((np + 255) / 256 < 65536 ? (np + 255) / 256 : 65536), 256, 0, st>>>(
        a.gstage, S.num_tiles, F + 27, H, L, S.params_per_tile, a.gmlp);
  }
  return cudaGetLastError();
}

cudaError_t launch_train_tc(const SceneDev& S, const TrainTcArgs& a, bool backward, cudaStream_t st) {
  const int F = S.feat_dim, H = S.mlp_hidden, L = S.mlp_layers;
  if (F == 32 && H == 64 && L == 3) return launch_train_tc_t<32, 64, 3>(S, a, backward, st);
  if (F == 16 && H == 32 && L == 2) return launch_train_tc_t<16, 32, 2>(S, a, backward, st);
  return cudaErrorInvalidValue;
}

}  // namespace snisr
