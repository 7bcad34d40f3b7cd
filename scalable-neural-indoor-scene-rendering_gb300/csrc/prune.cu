// Occupancy pruning after a training epoch, on the reference's dilated
// per-tile grids (D = N + 2 cells per side, [x][y][z] order, one cell of
// border):
//   transparency_statistic (training/src/Helper_kernel.cu:108-172,272-303):
//     per training ray, a fixed-step march through the tile; at every sample
//     whose cell is flagged 1 the trilinear weights times the transmittance
//     before the sample are max-combined into T_voxels at the 8 corners, and
//     the transmittance is advanced with the trilinear density;
//   dilate_boundary (Helper_kernel.cu:174-270): every -1 cell with a 1 cell
//     in its 3^3 neighbourhood becomes 0;
//   prune_flags (training/scripts/tile/tile.py:325-372): 3^3 max filter of
//     T_voxels, per-block maximum of the density at the voxel centres, the
//     two thresholds, then dilate_boundary;
//   pack_occupancy: the 1 cells of the inner N^3 as this library's 64-bit
//     occupancy words (bit v of word v / 64, v = (x * N + y) * N + z).
//
// GB300 design: one thread per ray for the statistic, with the 8 corner
// maxima of the current trilinear cell held in registers and written with
// one atomic max each when the march leaves the cell (about 10 samples per
// cell at the reference's step of 0.1 voxel: a tenth of the atomics, same
// result because a maximum does not depend on grouping).  All values are
// transmittances times weights, never negative, so the atomic is a signed
// integer max on their bit patterns.  Positions and the trilinear density
// use the fused multiply-adds of the compiled reference (ffma), the density
// exponential is expf, as in the reference.
#include <cuda_runtime.h>

#include <string>

#include "device_common.cuh"
#include "snisr.h"
#include "snisr_internal.h"

namespace snisr {
namespace {

inline int blocks_for_n(int64_t n, int threads) {
  int64_t b = (n + threads - 1) / threads;
  return (int)(b < (1 << 20) ? b : (1 << 20));
}

__device__ __forceinline__ void max_into(float* addr, float v) {
  if (!(v >= 0.0f)) return;  // NaN (the reference's fmaxf ignores it)
  atomicMax(reinterpret_cast<int*>(addr), __float_as_int(v));
}

__global__ void transparency_stat_kernel(const float* __restrict__ ro, const float* __restrict__ rd, int64_t n,
                                         int D, const float* __restrict__ center, float tile_size, float vs,
                                         float step, const float* __restrict__ sigma,
                                         const int16_t* __restrict__ nodes, float* T_voxels) {
  const int DD = D * D;
  const float c[3] = {__ldg(center), __ldg(center + 1), __ldg(center + 2)};
  const float hs = fdiv(tile_size, 2.0f);
  const float h3[3] = {hs, hs, hs};
  const float inv_vs = fdiv(1.0f, vs);  // float3 / float multiplies by the reciprocal (cutil_math.h:396-400)
  float tcorner[3], dcorner[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    tcorner[a] = fsub(c[a], hs);
    dcorner[a] = fsub(tcorner[a], vs);
  }
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    const float o[3] = {ro[3 * r], ro[3 * r + 1], ro[3 * r + 2]};
    const float d[3] = {rd[3 * r], rd[3 * r + 1], rd[3 * r + 2]};
    const float2 b = slab(o, d, c, h3);
    float z = b.x, T = 1.0f;
    int cell = -1;  // v000 of the cell whose maxima are held
    float m[8];
    while (z < b.y) {
      float pts[3];
      int p[3];
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        pts[a] = ffma(z, d[a], o[a]);
        p[a] = (int)fmul(fsub(pts[a], dcorner[a]), inv_vs);
      }
      if (p[0] < 0 || p[1] < 0 || p[2] < 0 || p[0] >= D || p[1] >= D || p[2] >= D ||
          __ldg(nodes + p[0] * DD + p[1] * D + p[2]) != 1) {
        z = march_next(z, step);
        continue;
      }
      float f[3], x[3];
      int x0[3];
      bool ok = true;
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        f[a] = ffma(fsub(pts[a], tcorner[a]), inv_vs, 0.5f);
        x0[a] = (int)f[a];
        x[a] = fsub(f[a], (float)x0[a]);
        ok = ok && x0[a] >= 0 && x0[a] + 1 < D;
      }
      if (!ok) {  // flagged border cell: the reference asserts here; the sample is skipped
        z = march_next(z, step);
        continue;
      }
      const float ux = fsub(1.0f, x[0]), uy = fsub(1.0f, x[1]), uz = fsub(1.0f, x[2]);
      float w[8];
      w[0] = fmul(fmul(ux, uy), uz);
      w[1] = fmul(fmul(ux, uy), x[2]);
      w[2] = fmul(fmul(ux, x[1]), uz);
      w[3] = fmul(fmul(ux, x[1]), x[2]);
      w[4] = fmul(fmul(x[0], uy), uz);
      w[5] = fmul(fmul(x[0], uy), x[2]);
      w[6] = fmul(fmul(x[0], x[1]), uz);
      w[7] = fmul(fmul(x[0], x[1]), x[2]);
      const int v000 = x0[0] * DD + x0[1] * D + x0[2];
      const int off[8] = {0, 1, D, D + 1, DD, DD + 1, DD + D, DD + D + 1};
      if (v000 != cell) {
        if (cell >= 0) {
#pragma unroll
          for (int k = 0; k < 8; ++k) max_into(T_voxels + cell + off[k], m[k]);
        }
        cell = v000;
#pragma unroll
        for (int k = 0; k < 8; ++k) m[k] = fmul(T, w[k]);
      } else {
#pragma unroll
        for (int k = 0; k < 8; ++k) m[k] = fmaxf(m[k], fmul(T, w[k]));
      }
      // v0*w0 + v1*w1 + ... + v7*w7 compiles to fma(v0, w0, v1*w1), then fma(vk, wk, s)
      float s = ffma(__ldg(sigma + v000 + off[0]), w[0], fmul(__ldg(sigma + v000 + off[1]), w[1]));
#pragma unroll
      for (int k = 2; k < 8; ++k) s = ffma(__ldg(sigma + v000 + off[k]), w[k], s);
      const float alpha = fsub(1.0f, expf(fmul(fmul(-1.0f, s), step)));
      T = fmul(T, fsub(1.0f, alpha));
      if (T < 0.00000001f) break;
      z = march_next(z, step);
    }
    if (cell >= 0) {
      const int off[8] = {0, 1, D, D + 1, DD, DD + 1, DD + D, DD + D + 1};
#pragma unroll
      for (int k = 0; k < 8; ++k) max_into(T_voxels + cell + off[k], m[k]);
    }
  }
}

// In place: a cell only ever changes from -1 to 0 and the test reads "== 1",
// so the order in which threads see their neighbours' updates does not
// matter (the reference writes a copy and copies it back).
__global__ void dilate_kernel(int16_t* flags, int D) {
  const int64_t total = (int64_t)D * D * D;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    if (flags[i] != -1) continue;
    const int x = (int)(i / ((int64_t)D * D)), rem = (int)(i % ((int64_t)D * D)), y = rem / D, z = rem % D;
    bool near1 = false;
    for (int a = max(x - 1, 0); a <= min(x + 1, D - 1) && !near1; ++a)
      for (int b = max(y - 1, 0); b <= min(y + 1, D - 1) && !near1; ++b)
        for (int cc = max(z - 1, 0); cc <= min(z + 1, D - 1); ++cc)
          if (flags[((int64_t)a * D + b) * D + cc] == 1) {
            near1 = true;
            break;
          }
    if (near1) flags[i] = 0;
  }
}

// tile.py:337-372 without the model query: flags of the inner N^3 from the
// initial flags, the block maxima of the voxel-centre density and the 3^3
// max filter of T_voxels; border cells -1.
__global__ void prune_flags_kernel(const float* __restrict__ T_voxels, const float* __restrict__ voxel_sigma,
                                   const int16_t* __restrict__ init_flags, int N, int block, float th, float T_th,
                                   int16_t* flags) {
  const int D = N + 2;
  const int64_t total = (int64_t)D * D * D;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int x = (int)(i / ((int64_t)D * D)), rem = (int)(i % ((int64_t)D * D)), y = rem / D, z = rem % D;
    if (x == 0 || y == 0 || z == 0 || x == D - 1 || y == D - 1 || z == D - 1) {
      flags[i] = -1;
      continue;
    }
    const int vx = x - 1, vy = y - 1, vz = z - 1;
    int16_t f = init_flags ? init_flags[((int64_t)vx * N + vy) * N + vz] : (int16_t)1;
    // block maximum of the density at the voxel centres
    const int bx = vx / block * block, by = vy / block * block, bz = vz / block * block;
    float smax = __ldg(voxel_sigma + ((int64_t)bx * N + by) * N + bz);
    for (int a = 0; a < block; ++a)
      for (int b = 0; b < block; ++b)
        for (int cc = 0; cc < block; ++cc)
          smax = fmaxf(smax, __ldg(voxel_sigma + ((int64_t)(bx + a) * N + (by + b)) * N + (bz + cc)));
    if (expf(-smax) > th) f = -1;
    float tmax = __ldg(T_voxels + ((int64_t)(x - 1) * D + (y - 1)) * D + (z - 1));
    for (int a = x - 1; a <= x + 1; ++a)
      for (int b = y - 1; b <= y + 1; ++b)
        for (int cc = z - 1; cc <= z + 1; ++cc) tmax = fmaxf(tmax, __ldg(T_voxels + ((int64_t)a * D + b) * D + cc));
    if (tmax <= T_th) f = -1;
    flags[i] = f;
  }
}

// One warp per 64-bit word: lanes take bits 2l and 2l+1 of the word.
__global__ void pack_occupancy_kernel(const int16_t* __restrict__ flags, int N, unsigned long long* words,
                                      int64_t* count) {
  const int D = N + 2;
  const int64_t nwords = ((int64_t)N * N * N + 63) / 64;
  const int lane = threadIdx.x & 31;
  const int64_t warp0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int64_t nvox = (int64_t)N * N * N;
  unsigned long long local = 0;
  for (int64_t w = warp0; w < nwords; w += nwarps) {
    unsigned bits2 = 0;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int64_t v = w * 64 + h * 32 + lane;
      bool on = false;
      if (v < nvox) {
        const int x = (int)(v / ((int64_t)N * N)), rem = (int)(v % ((int64_t)N * N)), y = rem / N, z = rem % N;
        on = flags[((int64_t)(x + 1) * D + (y + 1)) * D + (z + 1)] == 1;
      }
      const unsigned m = __ballot_sync(0xFFFFFFFFu, on);
      if (h == 0) bits2 = m;
      else if (lane == 0) {
        words[w] = (unsigned long long)bits2 | ((unsigned long long)m << 32);
        local += (unsigned long long)(__popc(bits2) + __popc(m));
      }
    }
  }
  if (lane == 0 && local) atomicAdd(reinterpret_cast<unsigned long long*>(count), local);
}

}  // namespace
}  // namespace snisr

using namespace snisr;

#define PRUNE_CHECK(name)                                                                    \
  do {                                                                                       \
    cudaError_t e = cudaGetLastError();                                                      \
    if (e != cudaSuccess) return set_error(SNISR_CUDA_ERROR, std::string(name ": ") + cudaGetErrorString(e)); \
  } while (0)

extern "C" {

snisr_status snisr_op_transparency_statistic(const float* rays_start, const float* rays_dir, int64_t n,
                                             int32_t num_voxel, const float* tile_center, float tile_size,
                                             float voxel_size, float sample_step, const float* voxels,
                                             const int16_t* nodes, float* T_voxels, void* stream) {
  if (n < 0 || num_voxel < 2 || num_voxel > 1024 || !(tile_size > 0) || !(voxel_size > 0) || !(sample_step > 0))
    return set_error(SNISR_INVALID_ARG, "transparency_statistic: bad size (2 <= num_voxel <= 1024)");
  if (!(sample_step >= voxel_size * kMinStepVox))
    return set_error(SNISR_INVALID_ARG, "transparency_statistic: sample_step below voxel_size / 1024");
  if (n == 0) return SNISR_OK;
  if (!rays_start || !rays_dir || !tile_center || !voxels || !nodes || !T_voxels)
    return set_error(SNISR_INVALID_ARG, "transparency_statistic: null argument");
  transparency_stat_kernel<<<blocks_for_n(n, 128), 128, 0, (cudaStream_t)stream>>>(
      rays_start, rays_dir, n, num_voxel, tile_center, tile_size, voxel_size, sample_step, voxels, nodes, T_voxels);
  PRUNE_CHECK("transparency_statistic");
  return SNISR_OK;
}

snisr_status snisr_op_dilate_boundary(int16_t* nodes_flag, int32_t num_voxel, void* stream) {
  if (num_voxel <= 0 || num_voxel > 2048) return set_error(SNISR_INVALID_ARG, "dilate_boundary: bad size");
  if (!nodes_flag) return set_error(SNISR_INVALID_ARG, "dilate_boundary: null argument");
  const int64_t total = (int64_t)num_voxel * num_voxel * num_voxel;
  dilate_kernel<<<blocks_for_n(total, 256), 256, 0, (cudaStream_t)stream>>>(nodes_flag, num_voxel);
  PRUNE_CHECK("dilate_boundary");
  return SNISR_OK;
}

snisr_status snisr_op_prune_flags(const float* T_voxels, const float* voxel_sigma, const int16_t* init_flags,
                                  int32_t num_voxel, int32_t block, float th, float T_th, int16_t* nodes_flag,
                                  void* stream) {
  if (num_voxel <= 0 || num_voxel > 2046 || block <= 0 || num_voxel % block != 0)
    return set_error(SNISR_INVALID_ARG, "prune_flags: bad size (num_voxel a multiple of block)");
  if (!T_voxels || !voxel_sigma || !nodes_flag) return set_error(SNISR_INVALID_ARG, "prune_flags: null argument");
  const int D = num_voxel + 2;
  const int64_t total = (int64_t)D * D * D;
  prune_flags_kernel<<<blocks_for_n(total, 256), 256, 0, (cudaStream_t)stream>>>(
      T_voxels, voxel_sigma, init_flags, num_voxel, block, th, T_th, nodes_flag);
  PRUNE_CHECK("prune_flags");
  dilate_kernel<<<blocks_for_n(total, 256), 256, 0, (cudaStream_t)stream>>>(nodes_flag, D);
  PRUNE_CHECK("prune_flags");
  return SNISR_OK;
}

snisr_status snisr_op_pack_occupancy(const int16_t* nodes_flag, int32_t num_voxel, uint64_t* words,
                                     int64_t* count, void* stream) {
  if (num_voxel <= 0 || num_voxel > 2046) return set_error(SNISR_INVALID_ARG, "pack_occupancy: bad size");
  if (!nodes_flag || !words || !count) return set_error(SNISR_INVALID_ARG, "pack_occupancy: null argument");
  const int64_t nwords = ((int64_t)num_voxel * num_voxel * num_voxel + 63) / 64;
  cudaError_t e = cudaMemsetAsync(count, 0, sizeof(int64_t), (cudaStream_t)stream);
  if (e != cudaSuccess) return set_error(SNISR_CUDA_ERROR, std::string("pack_occupancy: ") + cudaGetErrorString(e));
  pack_occupancy_kernel<<<blocks_for_n(nwords * 32, 256), 256, 0, (cudaStream_t)stream>>>(
      nodes_flag, num_voxel, reinterpret_cast<unsigned long long*>(words), count);
  PRUNE_CHECK("pack_occupancy");
  return SNISR_OK;
}

}  // extern "C"
