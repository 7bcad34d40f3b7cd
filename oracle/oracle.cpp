// ORACLE — test infrastructure only.  Scalar CPU restatement of the
// reference's algorithm for the tiled sparse-voxel hot path, used by tests/,
// __graft_entry__.smoke() and bench.py's CPU baseline as the checker.  It is
// never linked into, loaded by or called from the product library.
//
// Independent of the GPU code: written from the algorithm, not from the
// kernels.  Traversal is evaluated in IEEE binary32 with every operation
// rounded separately (compile with -ffp-contract=off), which is the
// specification of the visited-voxel sequence; shading (trilinear, MLP,
// compositing) runs in float (mode 0) or double (mode 1, the FP64 oracle).
//
// The restatements of the reference's own CUDA ops (oracle_op_*, sample_bg,
// train_tracing) also state the fused multiply-adds of the reference's nvcc
// build, which contracts a product feeding an add into one fma (the left
// product when both operands are products: a*b + c*d + e is
// fma(a, b, c*d) + e).  fmac() below marks each of them; running the
// reference's compiled kernels on the GPU showed them at these places.
// The low-level helpers pinned against the reference headers compiled for
// the host (ray_aabb, voxel traversal of the tile grid in the render path,
// ray-triangle, FP32 trilinear) stay unfused, like that host build.
//
// Reference functions restated (paths inside the reference project):
//   safe_divide / signf            rendering/src/include/cutil_math.h:856-876
//   RayAABBIntersection            rendering/src/include/cuda_utils.h:506-598
//   voxel_traversal (tie rules)    rendering/src/include/cuda_utils.h:158-238
//   RayTriangleIntersection        rendering/src/include/cuda_utils.h:403-436
//   tracing_tiles_kernel           rendering/src/raytile_tracing.cu:9-60
//   per-tile clip + march          rendering/src/raydiffuse_render_octree_fp16.cu:20-139,199-225
//   voxel DDA of Sample_sparse     training/src/Sample_kernel.cu:181-394
//   compute_rays / get_direction   rendering/src/compute_rays.cu:7-44
//   inverse_z_sampling_kernel      rendering/src/sampling.cu:5-45
//   integrate_points_kernel        rendering/src/volume_rendering.cu:5-58
//   volume_rendering (cumprod)     training/scripts/utils.py:823-837
//   Positional_Encoding / MLP      training/scripts/networks.py:4-41
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <type_traits>
#include <vector>

#include "snisr.h"

namespace {

const float kInf = 100000000.0f;

// One fused multiply-add, rounded once (a contraction of the reference's build).
inline float fmac(float a, float b, float c) { return std::fma(a, b, c); }

float f16_to_f32(uint16_t h) {
  uint32_t sign = (uint32_t)(h & 0x8000u) << 16;
  uint32_t exp = (h >> 10) & 0x1F, mant = h & 0x3FFu, x;
  if (exp == 0) {
    if (mant == 0) x = sign;
    else {
      int e = -1;
      do { mant <<= 1; ++e; } while (!(mant & 0x400u));
      x = sign | ((uint32_t)(127 - 15 - e) << 23) | ((mant & 0x3FFu) << 13);
    }
  } else if (exp == 31) x = sign | 0x7F800000u | (mant << 13);
  else x = sign | ((exp - 15 + 127) << 23) | (mant << 13);
  float f;
  std::memcpy(&f, &x, 4);
  return f;
}

// round to nearest-even FP16, returned as float
float round_f16(float f) {
  uint32_t x;
  std::memcpy(&x, &f, 4);
  uint32_t sign = (x >> 16) & 0x8000u;
  int32_t exp = (int32_t)((x >> 23) & 0xFF) - 127 + 15;
  uint32_t mant = x & 0x7FFFFFu;
  uint16_t h;
  if (((x >> 23) & 0xFF) == 0xFF) h = (uint16_t)(sign | 0x7C00u | (mant ? 0x200u : 0u));
  else if (exp >= 31) h = (uint16_t)(sign | 0x7C00u);
  else if (exp <= 0) {
    if (exp < -10) h = (uint16_t)sign;
    else {
      mant |= 0x800000u;
      int shift = 14 - exp;
      uint32_t half = mant >> shift, rem = mant & ((1u << shift) - 1u), mid = 1u << (shift - 1);
      if (rem > mid || (rem == mid && (half & 1u))) ++half;
      h = (uint16_t)(sign | half);
    }
  } else {
    uint32_t half = sign | ((uint32_t)exp << 10) | (mant >> 13), rem = mant & 0x1FFFu;
    if (rem > 0x1000u || (rem == 0x1000u && (half & 1u))) ++half;
    h = (uint16_t)half;
  }
  return f16_to_f32(h);
}

// reference safe_divide (cutil_math.h:867-869)
inline float safe_divide(float a, float b) { return b != 0.0f ? a / b : kInf; }

struct Bound { float lo, hi; };

// reference RayAABBIntersection (cuda_utils.h:553-598), per-axis half size
Bound ray_aabb(const float o[3], const float d[3], const float c[3], const float h[3]) {
  float f_low = 0.0f, f_high = 100000.0f;
  for (int a = 0; a < 3; ++a) {
    float inv = safe_divide(1.0f, d[a]);
    float lo = ((c[a] - h[a]) - o[a]) * inv;
    float hi = ((c[a] + h[a]) - o[a]) * inv;
    if (hi < lo) std::swap(lo, hi);
    if (hi < f_low) return {-1.0f, -1.0f};
    if (lo > f_high) return {-1.0f, -1.0f};
    f_low = (lo > f_low) ? lo : f_low;
    f_high = (hi < f_high) ? hi : f_high;
    if (f_low > f_high) return {-1.0f, -1.0f};
  }
  return {f_low, f_high};
}

// Amanatides-Woo axis choice with the reference tie rule (cuda_utils.h:195-216)
inline int dda_axis(const float m[3]) {
  if (m[0] < m[1]) return (m[0] < m[2]) ? 0 : 2;
  return (m[1] < m[2]) ? 1 : 2;
}

// Node of the oracle's own bounding-volume hierarchy over the proxy mesh
// (only to time the host path on the full mesh; the nearest hit it returns is
// the brute-force one).  Leaf: count > 0 triangles from `first` in `tri`.
struct HostBvhNode {
  float lo[3], hi[3];
  int32_t first, count;  // inner node: children first, first + 1 (count 0)
};

struct Scene {
  const snisr_scene_desc* d;
  int N, NT, F, H, L, in, P;
  int64_t words;
  float tile, voxel, inv_voxel, step_len, early, start_off;
  std::vector<float> centers;      // [NT][3]
  std::vector<uint32_t> base;      // [NT*words] first global voxel of a word
  std::vector<float> vfeat, vdens; // vertex data as float
  std::vector<HostBvhNode> bvh;    // built on first use by oracle_proxy_bvh
  std::vector<int32_t> bvh_tri;
};

bool occupied(const Scene& s, int tile, int vid, uint32_t& rec) {
  int64_t w = (int64_t)tile * s.words + (vid >> 6);
  uint64_t bits = s.d->occupancy[w];
  int b = vid & 63;
  if (!((bits >> b) & 1ull)) return false;
  rec = s.base[(size_t)w] + (uint32_t)__builtin_popcountll(bits & ((1ull << b) - 1ull));
  return true;
}

// ---------------------------------------------------------------------------
// Per-ray traversal: callback on every occupied voxel segment, in order.
// visit(tile, rec, vc[3], near, far, t_in, q[3]) returns false to stop.
// ---------------------------------------------------------------------------
template <class Visit>
void march(const Scene& s, const float o[3], const float d[3], float t_start, Visit&& visit) {
  const snisr_scene_desc* D = s.d;
  const int g[3] = {D->grid[0], D->grid[1], D->grid[2]};
  float size[3], half[3], cen[3];
  for (int a = 0; a < 3; ++a) {
    size[a] = (float)g[a] * s.tile;
    half[a] = size[a] * 0.5f;
    cen[a] = D->scene_min[a] + half[a];
  }
  Bound b = ray_aabb(o, d, cen, half);
  if (b.lo == -1.0f) return;
  float t0 = std::max(b.lo, t_start);
  if (!(t0 < b.hi)) return;
  int tc[3], ts[3];
  float tmax[3], tdel[3];
  for (int a = 0; a < 3; ++a) {
    float p = (o[a] + t0 * d[a]) - D->scene_min[a];
    p = std::min(std::max(p, 0.0f), size[a] - 0.000001f);
    int c = (int)std::floor(p / s.tile);
    tc[a] = std::min(std::max(c, 0), g[a] - 1);
    ts[a] = d[a] >= 0.0f ? 1 : -1;
    float nb = (float)(tc[a] + ts[a]) * s.tile;
    if (ts[a] < 0) nb = nb + s.tile;
    tmax[a] = d[a] != 0.0f ? (nb - p) / d[a] : kInf;
    tdel[a] = d[a] != 0.0f ? (s.tile / d[a]) * (float)ts[a] : kInf;
  }
  const int N = s.N;
  for (;;) {
    int id = D->tile_index[((int64_t)tc[0] * g[1] + tc[1]) * g[2] + tc[2]];
    if (id >= 0) {
      float c[3], h[3];
      for (int a = 0; a < 3; ++a) { c[a] = s.centers[(size_t)id * 3 + a]; h[a] = s.tile * 0.5f; }
      Bound tb = ray_aabb(o, d, c, h);
      float ti = std::max(tb.lo, t_start);
      if (tb.lo != -1.0f && ti < tb.hi) {
        float q[3], vmax[3], vdel[3];
        int vc[3], vs[3];
        for (int a = 0; a < 3; ++a) {
          float corner = c[a] - h[a];
          q[a] = (o[a] + ti * d[a]) - corner;
          q[a] = std::min(std::max(q[a], 0.0f), s.tile - 0.00001f);
          int v = (int)(q[a] / s.voxel);
          vc[a] = std::min(std::max(v, 0), N - 1);
          vs[a] = d[a] >= 0.0f ? 1 : -1;
          float nb = (float)(vc[a] + vs[a]) * s.voxel;
          if (vs[a] < 0) nb = nb + s.voxel;
          vmax[a] = safe_divide(nb - q[a], d[a]);
          vdel[a] = safe_divide((float)vs[a] * s.voxel, d[a]);
        }
        float near_ = 0.0f;
        for (;;) {
          float far_ = std::min(std::min(vmax[0], vmax[1]), vmax[2]);
          int vid = (vc[0] * N + vc[1]) * N + vc[2];
          uint32_t rec;
          if (occupied(s, id, vid, rec))
            if (!visit(id, rec, vc, near_, far_, ti, q)) return;
          int a = dda_axis(vmax);
          vc[a] += vs[a];
          vmax[a] = vmax[a] + vdel[a];
          near_ = far_;
          if (vc[a] < 0 || vc[a] >= N) break;
        }
      }
    }
    int a = dda_axis(tmax);
    tc[a] += ts[a];
    tmax[a] = tmax[a] + tdel[a];
    if (tc[a] < 0 || tc[a] >= g[a]) return;
  }
}

template <class T>
T softplus(T x) { return std::max(x, T(0)) + std::log1p(std::exp(-std::fabs(x))); }

// The render march's own single-precision exponential and log1p, as the
// kernels define them (the transmittance they produce is specified bit for
// bit, so these are the same operations in the same order; every float
// operation here is one IEEE single-precision rounding: -ffp-contract=off,
// std::fma is the fused multiply-add).
//
// e^x for x <= 0: Cody-Waite reduction x = k ln2 + r (ln2 = 16-bit head +
// tail), degree-7 Taylor polynomial of e^r by Horner's rule, scaling by 2^k.
// 0 below -80; NaN propagates.
float exp_nonpos(float x) {
  if (!(x >= -80.0f)) return x != x ? x : 0.0f;
  const float k = std::nearbyint(x * 1.44269504088896341f);
  float r = std::fma(-k, 0.693145751953125f, x);
  r = std::fma(-k, 1.42860682030941723212e-6f, r);
  const float c[8] = {1.98412698412698413e-4f, 1.38888888888888889e-3f, 8.33333333333333333e-3f,
                      4.16666666666666667e-2f, 1.66666666666666667e-1f, 0.5f, 1.0f, 1.0f};
  float p = c[0];
  for (int i = 1; i < 8; ++i) p = std::fma(p, r, c[i]);
  const uint32_t bits = (uint32_t)((int)k + 127) << 23;
  float scale;
  std::memcpy(&scale, &bits, 4);
  return p * scale;
}

// log(1 + y), y in [0, 1]: 2 atanh(y / (2 + y)) by its odd series to s^19.
float log1p_unit(float y) {
  const float s = y / (2.0f + y);
  const float s2 = s * s;
  const float c[10] = {5.26315789473684211e-2f, 5.88235294117647059e-2f, 6.66666666666666667e-2f,
                       7.69230769230769231e-2f, 9.09090909090909091e-2f, 1.11111111111111111e-1f,
                       1.42857142857142857e-1f, 2.0e-1f, 3.33333333333333333e-1f, 1.0f};
  float q = c[0];
  for (int i = 1; i < 10; ++i) q = std::fma(q, s2, c[i]);
  const float t = s * q;
  return t + t;
}

float softplus_march(float x) { return std::max(x, 0.0f) + log1p_unit(exp_nonpos(-std::fabs(x))); }
template <class T>
T sigmoid(T x) { return T(1) / (T(1) + std::exp(-x)); }

// view encoding [d, sin(2^i d), cos(2^i d)] (networks.py:4-15)
template <class T>
void dir_enc(const float d[3], T* out) {
  for (int a = 0; a < 3; ++a) out[a] = (T)d[a];
  T scale = 1;
  for (int i = 0; i < 4; ++i) {
    for (int a = 0; a < 3; ++a) {
      out[3 + 6 * i + a] = std::sin(scale * (T)d[a]);
      out[3 + 6 * i + 3 + a] = std::cos(scale * (T)d[a]);
    }
    scale *= 2;
  }
}

// MLP of one tile: Linear -> ReLU (L times) -> Linear; layout per Linear
// W[out][in] then b[out].  `half_inputs`: emulate the tensor-core form --
// every Linear's weights, inputs and bias rounded to FP16, products summed
// exactly (FP32 accumulation in hardware; the oracle sums in T).
template <class T>
void mlp(const Scene& s, int tile, const T* x, T out[3], bool half_inputs = false) {
  const float* p = s.d->mlp_params + (int64_t)tile * s.P;
  std::vector<T> cur(x, x + s.in), nxt;
  int64_t off = 0;
  for (int l = 0; l <= s.L; ++l) {
    int fi = l == 0 ? s.in : s.H, fo = l == s.L ? 3 : s.H;
    nxt.assign((size_t)fo, T(0));
    for (int o = 0; o < fo; ++o) {
      T acc = 0;
      for (int i = 0; i < fi; ++i) {
        T w = (T)p[off + (int64_t)o * fi + i];
        T xi = cur[(size_t)i];
        if (half_inputs) { w = (T)round_f16((float)w); xi = (T)round_f16((float)xi); }
        acc += w * xi;
      }
      T bias = (T)p[off + (int64_t)fi * fo + o];
      if (half_inputs) bias = (T)round_f16((float)bias);
      nxt[(size_t)o] = acc + bias;
    }
    off += (int64_t)fi * fo + fo;
    if (l < s.L)
      for (auto& v : nxt) v = std::max(v, T(0));
    cur.swap(nxt);
  }
  for (int c = 0; c < 3; ++c) out[c] = cur[(size_t)c];
}

struct SampleGeom {
  float f[3];
  float interval;
  float t;
};

// Fixed-step samples inside one occupied voxel segment
// (block_traversal_rendering's march, raydiffuse_render_octree_fp16.cu:67-106).
template <class Emit>
bool voxel_samples(const Scene& s, const int vc[3], float near_, float far_, float t_in, const float q[3], const float d[3],
                   Emit&& emit) {
  for (float z = near_; z < far_; z = z + s.step_len) {
    SampleGeom g;
    for (int a = 0; a < 3; ++a) {
      float pos = q[a] + z * d[a];
      float f = pos * s.inv_voxel - (float)vc[a];
      g.f[a] = std::min(std::max(f, 0.0f), 1.0f);
    }
    g.interval = std::min(s.step_len, far_ - z);
    g.t = t_in + z;
    if (!emit(g)) return false;
  }
  return true;
}

template <class T>
void trilinear_w(const float f[3], T w[8]) {
  T wx[2] = {T(1) - (T)f[0], (T)f[0]}, wy[2] = {T(1) - (T)f[1], (T)f[1]}, wz[2] = {T(1) - (T)f[2], (T)f[2]};
  for (int k = 0; k < 8; ++k) w[k] = wx[(k >> 2) & 1] * wy[(k >> 1) & 1] * wz[k & 1];
}

struct RayStats {
  int64_t samples = 0;
  int64_t voxels = 0;
  uint8_t* touched = nullptr;  // optional [num_voxels] marks of sampled voxels
};

// form: 0 plain FP32 semantics, 1 FP64, 2 tensor-core emulation (FP16-rounded
// MLP inputs, FP64 arithmetic)
template <class T>
void render_ray(const Scene& s, const float o[3], const float d[3], float t_start, int form, float rgb[3], float& depth,
                float& opac, RayStats& st) {
  T C[3] = {0, 0, 0}, Dp = 0, Tr = 1;
  std::vector<T> x((size_t)s.in, T(0));
  dir_enc<T>(d, x.data() + s.F);
  if (form == 2)
    for (int i = s.F; i < s.in; ++i) x[(size_t)i] = (T)round_f16((float)x[(size_t)i]);
  bool stop = false;
  march(s, o, d, t_start, [&](int tile, uint32_t rec, const int* vc, float nr, float fr, float ti, const float* q) {
    st.voxels++;
    return voxel_samples(s, vc, nr, fr, ti, q, d, [&](const SampleGeom& g) {
      T w[8];
      trilinear_w<T>(g.f, w);
      const int32_t* cn = s.d->voxel_corners + (int64_t)rec * 8;
      T logit = 0;
      for (int k = 0; k < 8; ++k) logit += w[k] * (T)s.vdens[(size_t)cn[k]];
      T sigma, alpha;
      if constexpr (std::is_same<T, float>::value) {  // the kernels' transmittance, bit for bit
        sigma = softplus_march(logit);
        alpha = 1.0f - exp_nonpos(-sigma * (g.interval * s.inv_voxel));
      } else {
        sigma = softplus<T>(logit);
        alpha = T(1) - std::exp(-sigma * (T)(g.interval * s.inv_voxel));
      }
      T wt = Tr * alpha;
      for (int c = 0; c < s.F; ++c) {
        T acc = 0;
        for (int k = 0; k < 8; ++k) acc += w[k] * (T)s.vfeat[(size_t)cn[k] * s.F + c];
        x[(size_t)c] = form == 2 ? (T)round_f16((float)acc) : acc;
      }
      T out[3];
      mlp<T>(s, tile, x.data(), out, form == 2);
      for (int c = 0; c < 3; ++c) C[c] += wt * sigmoid<T>(out[c]);
      Dp += wt * (T)g.t;
      Tr *= (T(1) - alpha);
      st.samples++;
      if (st.touched) st.touched[rec] = 1;
      if (Tr < (T)s.early) { stop = true; return false; }
      return true;
    });
  });
  (void)stop;
  for (int c = 0; c < 3; ++c) rgb[c] = (float)C[c];
  depth = (float)Dp;
  opac = (float)(T(1) - Tr);
}

// ---------------------------------------------------------------------------
// Proxy mesh: brute-force nearest hit, FP32 Moller-Trumbore two-sided with the
// FP64 re-test band (ties -> lower triangle id).
// ---------------------------------------------------------------------------
const float kDetBand = 1e-7f, kBaryBand = 1e-5f;

inline float dot3(const float a[3], const float b[3]) { return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]; }
inline void cross3(const float a[3], const float b[3], float c[3]) {
  c[0] = a[1] * b[2] - a[2] * b[1];
  c[1] = a[2] * b[0] - a[0] * b[2];
  c[2] = a[0] * b[1] - a[1] * b[0];
}
inline double ddot3(const double a[3], const double b[3]) { return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]; }
inline void dcross3(const double a[3], const double b[3], double c[3]) {
  c[0] = a[1] * b[2] - a[2] * b[1];
  c[1] = a[2] * b[0] - a[0] * b[2];
  c[2] = a[0] * b[1] - a[1] * b[0];
}

bool tri_hit(const float o[3], const float d[3], const float* A, const float* B, const float* C, float& th) {
  float e1[3], e2[3], s[3], p[3], q[3];
  for (int a = 0; a < 3; ++a) { e1[a] = B[a] - A[a]; e2[a] = C[a] - A[a]; s[a] = o[a] - A[a]; }
  cross3(d, e2, p);
  float det = dot3(e1, p);
  cross3(s, e1, q);
  float un = dot3(s, p), vn = dot3(d, q), tn = dot3(e2, q);
  bool band = !(std::fabs(det) >= kDetBand);
  float u = 0, v = 0, t = 0, uv = 0;
  if (!band) {
    float inv = 1.0f / det;
    u = un * inv; v = vn * inv; t = tn * inv;
    uv = u + v;
    band = std::fabs(u) < kBaryBand || std::fabs(v) < kBaryBand || std::fabs(uv - 1.0f) < kBaryBand;
  }
  if (!band) {
    if (u >= 0.0f && v >= 0.0f && uv <= 1.0f && t > 0.0f) { th = t; return true; }
    return false;
  }
  double de1[3], de2[3], ds[3], dd[3], dp[3], dq[3];
  for (int a = 0; a < 3; ++a) {
    de1[a] = (double)B[a] - (double)A[a];
    de2[a] = (double)C[a] - (double)A[a];
    ds[a] = (double)o[a] - (double)A[a];
    dd[a] = d[a];
  }
  dcross3(dd, de2, dp);
  double ddet = ddot3(de1, dp);
  if (ddet == 0.0) return false;
  dcross3(ds, de1, dq);
  double du = ddot3(ds, dp) / ddet, dv = ddot3(dd, dq) / ddet, dt = ddot3(de2, dq) / ddet;
  if (du >= 0.0 && dv >= 0.0 && du + dv <= 1.0 && dt > 0.0) {
    th = (float)dt;
    return th > 0.0f;
  }
  return false;
}

float nearest_hit(const snisr_scene_desc* D, const float o[3], const float d[3], int& tri) {
  float best = 3.0e38f;
  int bid = -1;
  for (int64_t t = 0; t < D->num_triangles; ++t) {
    const float* A = D->mesh_vertices + 3 * (int64_t)D->mesh_faces[3 * t];
    const float* B = D->mesh_vertices + 3 * (int64_t)D->mesh_faces[3 * t + 1];
    const float* C = D->mesh_vertices + 3 * (int64_t)D->mesh_faces[3 * t + 2];
    float th;
    if (tri_hit(o, d, A, B, C, th) && (th < best || (th == best && t < bid))) { best = th; bid = (int)t; }
  }
  tri = bid;
  return bid >= 0 ? best : -1.0f;
}

// Median-split hierarchy over triangle centroids, at most 4 triangles per
// leaf; node boxes are padded by 1e-4 of the mesh extent (plus 1e-5) so that
// a hit whose rounded t lies a little outside its triangle's exact box is
// still reached.
void build_host_bvh(Scene& s) {
  const snisr_scene_desc* D = s.d;
  const int64_t nt = D->num_triangles;
  s.bvh_tri.resize((size_t)nt);
  std::vector<float> cen((size_t)nt * 3), tlo((size_t)nt * 3), thi((size_t)nt * 3);
  float mlo[3] = {3e38f, 3e38f, 3e38f}, mhi[3] = {-3e38f, -3e38f, -3e38f};
  for (int64_t t = 0; t < nt; ++t) {
    s.bvh_tri[(size_t)t] = (int32_t)t;
    for (int a = 0; a < 3; ++a) {
      float lo = 3e38f, hi = -3e38f;
      for (int k = 0; k < 3; ++k) {
        const float v = D->mesh_vertices[3 * (int64_t)D->mesh_faces[3 * t + k] + a];
        lo = std::min(lo, v);
        hi = std::max(hi, v);
      }
      tlo[(size_t)t * 3 + a] = lo;
      thi[(size_t)t * 3 + a] = hi;
      cen[(size_t)t * 3 + a] = 0.5f * (lo + hi);
      mlo[a] = std::min(mlo[a], lo);
      mhi[a] = std::max(mhi[a], hi);
    }
  }
  float pad = 1e-5f;
  for (int a = 0; a < 3; ++a) pad = std::max(pad, 1e-4f * (mhi[a] - mlo[a]) + 1e-5f);
  struct Job { int32_t node, begin, end; };
  s.bvh.clear();
  s.bvh.push_back(HostBvhNode{});
  std::vector<Job> jobs{{0, 0, (int32_t)nt}};
  while (!jobs.empty()) {
    const Job j = jobs.back();
    jobs.pop_back();
    HostBvhNode nd{};
    float clo[3] = {3e38f, 3e38f, 3e38f}, chi[3] = {-3e38f, -3e38f, -3e38f};
    for (int a = 0; a < 3; ++a) { nd.lo[a] = 3e38f; nd.hi[a] = -3e38f; }
    for (int32_t i = j.begin; i < j.end; ++i) {
      const int32_t t = s.bvh_tri[(size_t)i];
      for (int a = 0; a < 3; ++a) {
        nd.lo[a] = std::min(nd.lo[a], tlo[(size_t)t * 3 + a]);
        nd.hi[a] = std::max(nd.hi[a], thi[(size_t)t * 3 + a]);
        clo[a] = std::min(clo[a], cen[(size_t)t * 3 + a]);
        chi[a] = std::max(chi[a], cen[(size_t)t * 3 + a]);
      }
    }
    for (int a = 0; a < 3; ++a) { nd.lo[a] -= pad; nd.hi[a] += pad; }
    if (j.end - j.begin <= 4) {
      nd.first = j.begin;
      nd.count = j.end - j.begin;
      s.bvh[(size_t)j.node] = nd;
      continue;
    }
    int axis = 0;
    for (int a = 1; a < 3; ++a)
      if (chi[a] - clo[a] > chi[axis] - clo[axis]) axis = a;
    const int32_t mid = (j.begin + j.end) / 2;
    std::nth_element(s.bvh_tri.begin() + j.begin, s.bvh_tri.begin() + mid, s.bvh_tri.begin() + j.end,
                     [&](int32_t x, int32_t y) {
                       const float cx = cen[(size_t)x * 3 + axis], cy = cen[(size_t)y * 3 + axis];
                       return cx < cy || (cx == cy && x < y);
                     });
    nd.first = (int32_t)s.bvh.size();
    nd.count = 0;
    s.bvh[(size_t)j.node] = nd;
    s.bvh.push_back(HostBvhNode{});
    s.bvh.push_back(HostBvhNode{});
    jobs.push_back({nd.first, j.begin, mid});
    jobs.push_back({nd.first + 1, mid, j.end});
  }
}

// Nearest hit through the hierarchy: the same triangle tests and the same
// rule as nearest_hit (smallest t, ties to the lower triangle id); boxes
// entered beyond the best t so far are skipped.
float nearest_hit_bvh(const Scene& s, const float o[3], const float d[3], int& tri) {
  const snisr_scene_desc* D = s.d;
  float inv[3];
  for (int a = 0; a < 3; ++a) inv[a] = d[a] != 0.0f ? 1.0f / d[a] : (std::signbit(d[a]) ? -kInf : kInf);
  float best = 3.0e38f;
  int bid = -1;
  int32_t stack[128];
  int sp = 0;
  stack[sp++] = 0;
  while (sp > 0) {
    const HostBvhNode& nd = s.bvh[(size_t)stack[--sp]];
    float t0 = 0.0f, t1 = best;
    bool miss = false;
    for (int a = 0; a < 3 && !miss; ++a) {
      float ta = (nd.lo[a] - o[a]) * inv[a], tb = (nd.hi[a] - o[a]) * inv[a];
      if (ta != ta) ta = -kInf;  // 0 * inf: the ray runs inside the slab's plane
      if (tb != tb) tb = kInf;
      if (ta > tb) std::swap(ta, tb);
      t0 = std::max(t0, ta);
      t1 = std::min(t1, tb);
      miss = t0 > t1;
    }
    if (miss) continue;
    if (nd.count > 0) {
      for (int32_t i = nd.first; i < nd.first + nd.count; ++i) {
        const int64_t t = s.bvh_tri[(size_t)i];
        const float* A = D->mesh_vertices + 3 * (int64_t)D->mesh_faces[3 * t];
        const float* B = D->mesh_vertices + 3 * (int64_t)D->mesh_faces[3 * t + 1];
        const float* C = D->mesh_vertices + 3 * (int64_t)D->mesh_faces[3 * t + 2];
        float th;
        if (tri_hit(o, d, A, B, C, th) && (th < best || (th == best && t < bid))) { best = th; bid = (int)t; }
      }
    } else if (sp + 2 <= 128) {
      stack[sp++] = nd.first;
      stack[sp++] = nd.first + 1;
    }
  }
  tri = bid;
  return bid >= 0 ? best : -1.0f;
}

template <class F>
void parallel_for(int64_t n, int threads, F&& fn) {
  if (threads <= 1 || n < 64) {
    for (int64_t i = 0; i < n; ++i) fn(i);
    return;
  }
  std::atomic<int64_t> next(0);
  std::vector<std::thread> pool;
  for (int t = 0; t < threads; ++t)
    pool.emplace_back([&]() {
      for (;;) {
        int64_t i0 = next.fetch_add(64);
        if (i0 >= n) break;
        for (int64_t i = i0; i < std::min(n, i0 + 64); ++i) fn(i);
      }
    });
  for (auto& th : pool) th.join();
}

}  // namespace

extern "C" {

struct oracle_scene;

oracle_scene* oracle_scene_create(const snisr_scene_desc* d) {
  Scene* s = new Scene();
  s->d = d;
  s->N = d->res;
  s->NT = d->num_tiles;
  s->F = d->feat_dim;
  s->H = d->mlp_hidden;
  s->L = d->mlp_layers;
  s->in = s->F + 3 + 6 * d->dir_freqs;
  s->P = 0;
  for (int l = 0; l <= s->L; ++l) {
    int fi = l == 0 ? s->in : s->H, fo = l == s->L ? 3 : s->H;
    s->P += fi * fo + fo;
  }
  s->words = (int64_t)s->N * s->N * s->N / 64;
  s->tile = d->tile_size;
  s->voxel = d->tile_size / (float)s->N;
  s->inv_voxel = (float)s->N / d->tile_size;
  s->step_len = d->step_vox * s->voxel;
  s->early = d->early_stop;
  s->start_off = d->start_offset_vox * s->voxel;
  s->centers.assign((size_t)s->NT * 3, 0.0f);
  for (int x = 0; x < d->grid[0]; ++x)
    for (int y = 0; y < d->grid[1]; ++y)
      for (int z = 0; z < d->grid[2]; ++z) {
        int id = d->tile_index[((int64_t)x * d->grid[1] + y) * d->grid[2] + z];
        if (id < 0) continue;
        const int tc[3] = {x, y, z};
        for (int a = 0; a < 3; ++a) s->centers[(size_t)id * 3 + a] = d->scene_min[a] + ((float)tc[a] + 0.5f) * d->tile_size;
      }
  s->base.assign((size_t)(s->NT * s->words), 0u);
  uint64_t acc = 0;
  for (int64_t w = 0; w < (int64_t)s->NT * s->words; ++w) {
    s->base[(size_t)w] = (uint32_t)acc;
    acc += (uint64_t)__builtin_popcountll(d->occupancy[w]);
  }
  const int64_t nv = d->num_vertices;
  s->vfeat.resize((size_t)(nv * s->F));
  s->vdens.resize((size_t)nv);
  for (int64_t i = 0; i < nv * s->F; ++i)
    s->vfeat[(size_t)i] = d->feat_type == SNISR_F16 ? f16_to_f32(((const uint16_t*)d->vertex_feat)[i]) : ((const float*)d->vertex_feat)[i];
  for (int64_t i = 0; i < nv; ++i)
    s->vdens[(size_t)i] = d->feat_type == SNISR_F16 ? f16_to_f32(((const uint16_t*)d->vertex_density)[i]) : ((const float*)d->vertex_density)[i];
  return reinterpret_cast<oracle_scene*>(s);
}

void oracle_scene_destroy(oracle_scene* s) { delete reinterpret_cast<Scene*>(s); }

// Normalised camera directions, same operation order as the GPU ray setup.
// The march's single-precision functions on an array (fn 0: e^x for x <= 0,
// 1: log(1 + y) for y in [0, 1], 2: softplus), for checks of the kernels'
// transmittance arithmetic.
void oracle_march_math(int fn, const float* x, int64_t n, float* out) {
  for (int64_t i = 0; i < n; ++i)
    out[i] = fn == 0 ? exp_nonpos(x[i]) : fn == 1 ? log1p_unit(x[i]) : softplus_march(x[i]);
}

void oracle_camera_dirs(const snisr_camera* cam, float* dirs) {
  for (int64_t i = 0; i < (int64_t)cam->width * cam->height; ++i) {
    int py = (int)(i / cam->width), px = (int)(i % cam->width);
    float x = ((float)px - cam->cx) * cam->inv_focal, y = ((float)py - cam->cy) * cam->inv_focal;
    float r[3];
    for (int a = 0; a < 3; ++a) r[a] = (cam->c2w[4 * a] * x + cam->c2w[4 * a + 1] * y) + cam->c2w[4 * a + 2];
    float n = std::sqrt((r[0] * r[0] + r[1] * r[1]) + r[2] * r[2]);
    for (int a = 0; a < 3; ++a) dirs[3 * i + a] = r[a] / n;
  }
}

// Proxy-mesh start distances: t_start = max(hit - offset, 0), 0 on a miss or
// without a mesh.  t_hit / tri may be null.
void oracle_proxy(const oracle_scene* os, const float* o, const float* d, int64_t n, float* t_start, float* t_hit,
                  int32_t* tri, int threads) {
  const Scene& s = *reinterpret_cast<const Scene*>(os);
  parallel_for(n, threads, [&](int64_t i) {
    int id = -1;
    float th = s.d->num_triangles > 0 ? nearest_hit(s.d, o + 3 * i, d + 3 * i, id) : -1.0f;
    if (t_hit) t_hit[i] = th;
    if (tri) tri[i] = id;
    if (t_start) t_start[i] = th >= 0.0f ? std::max(th - s.start_off, 0.0f) : 0.0f;
  });
}

// oracle_proxy through the host hierarchy (same results; used to time the
// host path with the same work per ray as the GPU's BVH walk).
void oracle_proxy_bvh(oracle_scene* os, const float* o, const float* d, int64_t n, float* t_start, float* t_hit,
                      int32_t* tri, int threads) {
  Scene& s = *reinterpret_cast<Scene*>(os);
  if (s.d->num_triangles > 0 && s.bvh.empty()) build_host_bvh(s);
  parallel_for(n, threads, [&](int64_t i) {
    int id = -1;
    float th = s.d->num_triangles > 0 ? nearest_hit_bvh(s, o + 3 * i, d + 3 * i, id) : -1.0f;
    if (t_hit) t_hit[i] = th;
    if (tri) tri[i] = id;
    if (t_start) t_start[i] = th >= 0.0f ? std::max(th - s.start_off, 0.0f) : 0.0f;
  });
}

// Start distance from a proxy-mesh hit distance (the rule of oracle_proxy).
void oracle_start_from_hit(const oracle_scene* os, const float* t_hit, int64_t n, float* t_start) {
  const Scene& s = *reinterpret_cast<const Scene*>(os);
  for (int64_t i = 0; i < n; ++i) t_start[i] = t_hit[i] >= 0.0f ? std::max(t_hit[i] - s.start_off, 0.0f) : 0.0f;
}

// Occupied-voxel sequence per ray (no transmittance).
void oracle_trace(const oracle_scene* os, const float* o, const float* d, const float* t_start, int64_t n, int K,
                  int32_t* visited, int32_t* count, int threads) {
  const Scene& s = *reinterpret_cast<const Scene*>(os);
  parallel_for(n, threads, [&](int64_t i) {
    int c = 0;
    march(s, o + 3 * i, d + 3 * i, t_start ? t_start[i] : 0.0f,
          [&](int, uint32_t rec, const int*, float, float, float, const float*) {
            if (c < K) visited[i * K + c] = (int32_t)rec;
            ++c;
            return true;
          });
    for (int k = c; k < K; ++k) visited[i * K + k] = -1;
    count[i] = c;
  });
}

// Render rays.  form: 0 plain FP32, 1 FP64, 2 tensor-core emulation in FP64.
// stats (optional, [2]): total samples, total occupied voxels visited.
void oracle_render(const oracle_scene* os, const float* o, const float* d, const float* t_start, int64_t n, int form,
                   float* rgb, float* depth, float* opac, int64_t* stats, int threads) {
  const Scene& s = *reinterpret_cast<const Scene*>(os);
  std::vector<RayStats> per((size_t)n);
  parallel_for(n, threads, [&](int64_t i) {
    float ts = t_start ? t_start[i] : 0.0f;
    if (form == 0) render_ray<float>(s, o + 3 * i, d + 3 * i, ts, 0, rgb + 3 * i, depth[i], opac[i], per[(size_t)i]);
    else render_ray<double>(s, o + 3 * i, d + 3 * i, ts, form, rgb + 3 * i, depth[i], opac[i], per[(size_t)i]);
  });
  if (stats) {
    stats[0] = stats[1] = 0;
    for (const auto& p : per) { stats[0] += p.samples; stats[1] += p.voxels; }
  }
}

// Voxels holding at least one sample of the rays (plain FP32 render,
// single-threaded): touched [num_voxels] is set to 1 for each.
void oracle_touched_voxels(const oracle_scene* os, const float* o, const float* d, const float* t_start, int64_t n,
                           uint8_t* touched) {
  const Scene& s = *reinterpret_cast<const Scene*>(os);
  RayStats st;
  st.touched = touched;
  for (int64_t i = 0; i < n; ++i) {
    float rgb[3], dep, op;
    render_ray<float>(s, o + 3 * i, d + 3 * i, t_start ? t_start[i] : 0.0f, 0, rgb, dep, op, st);
  }
}

// ---------------------------------------------------------------------------
// Training: forward and adjoint of one ray segment inside one tile, FP64.
// Replaces the autograd graph of Tile.train_batch (training/scripts/tile/
// tile.py:667-704: sparse sampling, query_voxel, volume_rendering) for the
// per-corner feature model: rgb = sigmoid(MLP([trilinear F, enc(d)])),
// sigma = softplus(trilinear G), alpha = 1 - exp(-sigma * delta / voxel).
// ---------------------------------------------------------------------------
}  // extern "C"
namespace {
struct TrainSample {
  int32_t corners[8];
  double w[8];
  double s;            // density logit
  double sigma, alpha, T, dv;  // dv = delta / voxel
  double c[3];
  int32_t rec;                       // global voxel id
  double pos[3];                     // tile-local position in voxel units (voxel coordinate + fraction)
  std::vector<double> x;             // MLP input
  std::vector<std::vector<double>> h;  // hidden activations (post-ReLU)
};

// Occupied-voxel segments of a ray inside one tile (no tile DDA): the tile's
// own slab clip and voxel DDA, as in march().
template <class Visit>
void march_one_tile(const Scene& s, int id, const float o[3], const float d[3], Visit&& visit) {
  float c[3], h[3];
  for (int a = 0; a < 3; ++a) { c[a] = s.centers[(size_t)id * 3 + a]; h[a] = s.tile * 0.5f; }
  Bound tb = ray_aabb(o, d, c, h);
  if (tb.lo == -1.0f || !(tb.lo < tb.hi)) return;
  const float ti = tb.lo;
  const int N = s.N;
  float q[3], vmax[3], vdel[3];
  int vc[3], vs[3];
  for (int a = 0; a < 3; ++a) {
    float corner = c[a] - h[a];
    q[a] = (o[a] + ti * d[a]) - corner;
    q[a] = std::min(std::max(q[a], 0.0f), s.tile - 0.00001f);
    int v = (int)(q[a] / s.voxel);
    vc[a] = std::min(std::max(v, 0), N - 1);
    vs[a] = d[a] >= 0.0f ? 1 : -1;
    float nb = (float)(vc[a] + vs[a]) * s.voxel;
    if (vs[a] < 0) nb = nb + s.voxel;
    vmax[a] = safe_divide(nb - q[a], d[a]);
    vdel[a] = safe_divide((float)vs[a] * s.voxel, d[a]);
  }
  float near_ = 0.0f;
  for (;;) {
    float far_ = std::min(std::min(vmax[0], vmax[1]), vmax[2]);
    int vid = (vc[0] * N + vc[1]) * N + vc[2];
    uint32_t rec;
    if (occupied(s, id, vid, rec))
      if (!visit(id, rec, vc, near_, far_, ti, q)) return;
    int a = dda_axis(vmax);
    vc[a] += vs[a];
    vmax[a] = vmax[a] + vdel[a];
    near_ = far_;
    if (vc[a] < 0 || vc[a] >= N) return;
  }
}

// round to nearest-even BF16, returned as float
float round_bf16(float f) {
  uint32_t x;
  std::memcpy(&x, &f, 4);
  if ((x & 0x7F800000u) == 0x7F800000u) return f;
  x += 0x7FFFu + ((x >> 16) & 1u);
  x &= 0xFFFF0000u;
  std::memcpy(&f, &x, 4);
  return f;
}

struct TrainParams {
  const float* vfeat;  // [NV][F]
  const float* vdens;  // [NV]
  const float* mlp;    // [NT][P]
  // emul = 5: operand emulation of the tensor-core training form.  The
  // forward pass splits its operands in three BF16 parts, v = hi + mid + lo
  // (hi = bf16(v), mid = bf16(v - hi), lo = bf16(v - hi - mid)): MLP inputs,
  // weights and post-ReLU activations (rf); biases are exact.  A product of
  // two split operands is taken down to the 2^-24 terms, hi.hi + hi.mid +
  // mid.hi + hi.lo + lo.hi + mid.mid (six MMAs per K step).  The backward
  // takes the forward's activations (their hi parts are stored by the
  // kernels): they set the ReLU masks and, rounded to BF16, the
  // weight-gradient operands.  Backward products use single BF16 operands
  // (rb): the output-logit gradient, each hidden delta, W^T in the data
  // gradient and the activation in the weight gradient.
  // emul = 1: the two-part split (v = hi + lo, three products) with
  // two-part biases; 4: emul = 5 with three-part biases; 2 / 3: only the
  // forward / only the backward rounding of emul = 1 (these attribute the
  // tensor-core form's error).
  int emul = 0;
  // parts of the forward operand split: 0 (exact), 2 or 3; `colour` selects
  // the pass that produces the colours, otherwise the one whose activations
  // the backward uses (the same pass in every mode now)
  int split(bool colour) const {
    (void)colour;
    switch (emul) {
      case 1: case 2: return 2;
      case 4: case 5: return 3;
      default: return 0;
    }
  }
  int bias_split(bool colour) const { return emul == 5 ? 0 : split(colour); }
  bool bwd_r() const { return emul == 1 || emul == 3 || emul == 4 || emul == 5; }
  static double rf(double v, int parts) {
    if (parts == 0) return v;
    const float hi = round_bf16((float)v);
    if (parts == 3) {
      const float mid = round_bf16((float)v - hi);
      return (double)hi + (double)mid + (double)round_bf16(((float)v - hi) - mid);
    }
    return (double)hi + (double)round_bf16((float)v - hi);
  }
  double rb(double v) const { return bwd_r() ? (double)round_bf16((float)v) : v; }
  // w * x for the forward products (exact without forward rounding)
  static double product(double w, double x, int parts) {
    if (parts == 0) return w * x;
    const float wh = round_bf16((float)w), xh = round_bf16((float)x);
    if (parts == 3) {
      const float wm = round_bf16((float)w - wh), xm = round_bf16((float)x - xh);
      const double wl = (double)round_bf16(((float)w - wh) - wm), xl = (double)round_bf16(((float)x - xh) - xm);
      return (double)wh * xh + (double)wh * xm + (double)wm * xh + (double)wh * xl + wl * (double)xh +
             (double)wm * xm;
    }
    const double wl = (double)round_bf16((float)w - wh), xl = (double)round_bf16((float)x - xh);
    return (double)wh * (double)xh + (double)wh * xl + wl * (double)xh;
  }
};

// Forward of one segment; returns the samples (with activations) and colour.
void train_forward_ray(const Scene& s, const TrainParams& p, int tile, const float o[3], const float d[3],
                       std::vector<TrainSample>& out, double C[3]) {
  out.clear();
  C[0] = C[1] = C[2] = 0;
  double T = 1.0;
  std::vector<double> enc(27);
  dir_enc<double>(d, enc.data());
  const float* W = p.mlp + (int64_t)tile * s.P;
  march_one_tile(s, tile, o, d, [&](int, uint32_t rec, const int* vc, float nr, float fr, float ti, const float* q) {
    return voxel_samples(s, vc, nr, fr, ti, q, d, [&](const SampleGeom& g) {
      TrainSample ts;
      trilinear_w<double>(g.f, ts.w);
      ts.rec = (int32_t)rec;
      for (int a = 0; a < 3; ++a) ts.pos[a] = (double)vc[a] + (double)g.f[a];
      const int32_t* cn = s.d->voxel_corners + (int64_t)rec * 8;
      ts.s = 0;
      for (int k = 0; k < 8; ++k) {
        ts.corners[k] = cn[k];
        ts.s += ts.w[k] * (double)p.vdens[cn[k]];
      }
      ts.sigma = softplus<double>(ts.s);
      ts.dv = (double)(g.interval * s.inv_voxel);
      ts.alpha = 1.0 - std::exp(-ts.sigma * ts.dv);
      ts.T = T;
      std::vector<double> xe((size_t)s.in, 0.0);  // exact inputs
      for (int c = 0; c < s.F; ++c)
        for (int k = 0; k < 8; ++k) xe[(size_t)c] += ts.w[k] * (double)p.vfeat[(int64_t)cn[k] * s.F + c];
      for (int i = 0; i < 27; ++i) xe[(size_t)(s.F + i)] = enc[(size_t)i];
      // MLP with operands split in `parts`; the hidden activations go to hs
      auto mlp = [&](int parts, int bparts, std::vector<double>& x, std::vector<std::vector<double>>* hs) {
        x.resize(xe.size());
        for (size_t i = 0; i < xe.size(); ++i) x[i] = TrainParams::rf(xe[i], parts);
        std::vector<double> cur = x;
        int64_t off = 0;
        for (int l = 0; l <= s.L; ++l) {
          int fi = l == 0 ? s.in : s.H, fo = l == s.L ? 3 : s.H;
          std::vector<double> nx((size_t)fo);
          for (int oo = 0; oo < fo; ++oo) {
            double acc = TrainParams::rf(W[off + (int64_t)fi * fo + oo], bparts);
            for (int i = 0; i < fi; ++i) acc += TrainParams::product(W[off + (int64_t)oo * fi + i], cur[(size_t)i], parts);
            nx[(size_t)oo] = l < s.L ? TrainParams::rf(std::max(acc, 0.0), parts) : acc;
          }
          off += (int64_t)fi * fo + fo;
          if (l < s.L && hs) hs->push_back(nx);
          cur.swap(nx);
        }
        return cur;
      };
      // stored activations: the backward's recomputation; colours: the forward
      std::vector<double> cur = mlp(p.split(false), p.bias_split(false), ts.x, &ts.h);
      if (p.split(true) != p.split(false) || p.bias_split(true) != p.bias_split(false)) {
        std::vector<double> xc;
        cur = mlp(p.split(true), p.bias_split(true), xc, nullptr);
      }
      for (int c = 0; c < 3; ++c) {
        ts.c[c] = sigmoid<double>(cur[(size_t)c]);
        C[c] += T * ts.alpha * ts.c[c];
      }
      T *= (1.0 - ts.alpha);
      out.push_back(std::move(ts));
      return !(T < (double)s.early);
    });
  });
}

// Adjoint of one segment given dL/dC (g); accumulates into the gradients.
void train_backward_ray(const Scene& s, const TrainParams& p, int tile, const std::vector<TrainSample>& S,
                        const double g[3], double* gF, double* gG, double* gW) {
  const float* W = p.mlp + (int64_t)tile * s.P;
  double* GW = gW + (int64_t)tile * s.P;
  const int n = (int)S.size();
  std::vector<double> suffix((size_t)n * 3 + 3, 0.0);  // S_i = sum_{j>i} T_j alpha_j c_j
  for (int i = n - 1; i >= 0; --i)
    for (int c = 0; c < 3; ++c) {
      double next = (i + 1 < n) ? S[(size_t)i + 1].T * S[(size_t)i + 1].alpha * S[(size_t)i + 1].c[c] : 0.0;
      suffix[(size_t)i * 3 + c] = suffix[(size_t)(i + 1) * 3 + c] + next;
    }
  for (int i = 0; i < n; ++i) {
    const TrainSample& t = S[(size_t)i];
    double gc = 0, gs = 0;
    for (int c = 0; c < 3; ++c) { gc += g[c] * t.c[c]; gs += g[c] * suffix[(size_t)i * 3 + c]; }
    double dsigma = t.dv * ((1.0 - t.alpha) * t.T * gc - gs);
    double ds = sigmoid<double>(t.s) * dsigma;
    for (int k = 0; k < 8; ++k) gG[t.corners[k]] += t.w[k] * ds;
    // MLP backward
    std::vector<double> delta(3);
    for (int c = 0; c < 3; ++c) delta[(size_t)c] = p.rb(g[c] * t.T * t.alpha * t.c[c] * (1.0 - t.c[c]));
    // layer offsets
    std::vector<int64_t> offs;
    int64_t off = 0;
    for (int l = 0; l <= s.L; ++l) {
      int fi = l == 0 ? s.in : s.H, fo = l == s.L ? 3 : s.H;
      offs.push_back(off);
      off += (int64_t)fi * fo + fo;
    }
    for (int l = s.L; l >= 0; --l) {
      int fi = l == 0 ? s.in : s.H, fo = l == s.L ? 3 : s.H;
      const std::vector<double>& in = l == 0 ? t.x : t.h[(size_t)l - 1];
      for (int oo = 0; oo < fo; ++oo) {
        GW[offs[(size_t)l] + (int64_t)fi * fo + oo] += delta[(size_t)oo];
        for (int ii = 0; ii < fi; ++ii) GW[offs[(size_t)l] + (int64_t)oo * fi + ii] += delta[(size_t)oo] * p.rb(in[(size_t)ii]);
      }
      std::vector<double> prev((size_t)fi, 0.0);
      for (int ii = 0; ii < fi; ++ii) {
        double acc = 0;
        for (int oo = 0; oo < fo; ++oo) acc += p.rb(W[offs[(size_t)l] + (int64_t)oo * fi + ii]) * delta[(size_t)oo];
        if (l > 0) acc = t.h[(size_t)l - 1][(size_t)ii] > 0.0 ? p.rb(acc) : 0.0;
        prev[(size_t)ii] = acc;
      }
      delta.swap(prev);
    }
    for (int c = 0; c < s.F; ++c)
      for (int k = 0; k < 8; ++k) gF[(int64_t)t.corners[k] * s.F + c] += t.w[k] * delta[(size_t)c];
  }
}
}  // namespace
extern "C" {

// ---------------------------------------------------------------------------
// Reference-op restatements (bit-exact specification of the drop-in ops).
// ---------------------------------------------------------------------------
void oracle_op_compute_rays(const float* intr, const float* rot, int H, int W, float* rays_d) {
  for (int64_t i = 0; i < (int64_t)H * W; ++i) {
    int py = (int)(i / W), px = (int)(i % W);
    float x = ((float)px - intr[0]) * intr[2], y = ((float)py - intr[1]) * intr[2];
    for (int a = 0; a < 3; ++a) rays_d[3 * i + a] = fmac(rot[3 * a], x, rot[3 * a + 1] * y) + rot[3 * a + 2];
  }
}

void oracle_op_tracing_tiles(const float* rays_d, int64_t npix, const int32_t* imap, const float* origin,
                             const int32_t* shape, const float* smin, const float* ssize, float tile, int K,
                             int32_t* visited) {
  for (int64_t i = 0; i < npix; ++i) {
    int32_t* vis = visited + i * K;
    for (int j = 0; j < K; ++j) vis[j] = -1;
    const float* d = rays_d + 3 * i;
    float p[3];
    for (int a = 0; a < 3; ++a) p[a] = origin[a] - smin[a];
    if (p[0] < 0 || p[0] >= ssize[0] || p[1] < 0 || p[1] >= ssize[1] || p[2] < 0 || p[2] >= ssize[2]) {
      float c[3], h[3];
      for (int a = 0; a < 3; ++a) { h[a] = ssize[a] / 2.0f; c[a] = smin[a] + h[a]; }
      Bound b = ray_aabb(origin, d, c, h);
      for (int a = 0; a < 3; ++a) {
        p[a] = fmac(b.lo, d[a], p[a]);
        p[a] = std::min(std::max(p[a], 0.0f), ssize[a] - 0.000001f);
      }
    }
    int cur[3], st[3];
    float tmax[3], tdel[3];
    for (int a = 0; a < 3; ++a) {
      cur[a] = std::min(std::max((int)std::floor(p[a] / tile), 0), shape[a] - 1);
      st[a] = d[a] >= 0 ? 1 : -1;
      float nb = (float)(cur[a] + st[a]) * tile;
      if (st[a] < 0) nb = nb + tile;
      tmax[a] = d[a] != 0 ? (nb - p[a]) / d[a] : kInf;
      tdel[a] = d[a] != 0 ? (tile / d[a]) * (float)st[a] : kInf;
    }
    int idx = 0;
    int id = imap[((int64_t)cur[0] * shape[1] + cur[1]) * shape[2] + cur[2]];
    if (id != -1) vis[idx++] = id;
    while (idx < K) {
      int a = dda_axis(tmax);
      cur[a] += st[a];
      tmax[a] = tmax[a] + tdel[a];
      if (cur[a] < 0 || cur[a] >= shape[a]) break;
      id = imap[((int64_t)cur[0] * shape[1] + cur[1]) * shape[2] + cur[2]];
      if (id != -1) vis[idx++] = id;
    }
  }
}

static void uniform_v3(float* z, float* dist, float near_, float far_, int n) {
  float interval = (far_ - near_) / (float)n;
  for (int i = 0; i < n; ++i) {
    z[i] = fmac((float)i, interval, near_);
    dist[i] = interval;
  }
}

void oracle_op_sample_sparse(const float* ro, const float* rd, int64_t B, const int16_t* flags, float cx, float cy,
                             float cz, float tile, int N, int ns, float* zv, float* dv) {
  const float half = tile * 0.5f, vs = tile / (float)N;
  const float inv_vs = 1.0f / vs;  // float3 / float multiplies by the reciprocal (cutil_math.h:396-400)
  const float center[3] = {cx, cy, cz};
  float minc[3];
  for (int a = 0; a < 3; ++a) minc[a] = center[a] - half;
  const float hh[3] = {half, half, half};
  for (int64_t i = 0; i < B; ++i) {
    float* z = zv + i * ns;
    float* dd = dv + i * ns;
    const float* o = ro + 3 * i;
    const float* d = rd + 3 * i;
    Bound nf = ray_aabb(o, d, center, hh);
    if (nf.lo == -1.0f && nf.hi == -1.0f) continue;
    float near_ = nf.lo, far_ = nf.hi, total = 0.0f;
    float loc[3], nb[3], tmax[3], tdel[3];
    int cur[3], st[3];
    for (int a = 0; a < 3; ++a) {
      loc[a] = fmac(near_, d[a], o[a]) - minc[a];
      loc[a] = std::min(std::max(loc[a], 0.0f), tile - 0.000001f);
      cur[a] = std::min(std::max((int)(loc[a] * inv_vs), 0), N - 1);
      st[a] = d[a] >= 0 ? 1 : -1;
      nb[a] = (float)(cur[a] + st[a]) * vs;
      if (st[a] < 0) nb[a] = nb[a] + vs;
      tmax[a] = safe_divide(nb[a] - loc[a], d[a]);
      tdel[a] = safe_divide((float)st[a] * vs, d[a]);
    }
    auto vbound = [&]() {
      float vc[3];
      for (int a = 0; a < 3; ++a) vc[a] = fmac((float)cur[a], vs, minc[a]) + 0.5f * vs;
      const float h5 = 0.5f * vs;
      const float h3[3] = {h5, h5, h5};
      return ray_aabb(o, d, vc, h3);
    };
    auto step = [&]() {
      int a = dda_axis(tmax);
      cur[a] += st[a];
      tmax[a] = tmax[a] + tdel[a];
      return !(cur[a] < 0 || cur[a] >= N);
    };
    for (;;) {
      if (flags[((int64_t)cur[0] * N + cur[1]) * N + cur[2]] == 1) {
        Bound b = vbound();
        total = total + (b.hi - b.lo);
      }
      if (!step()) break;
    }
    if (total == 0.0f) continue;
    for (int a = 0; a < 3; ++a) {
      cur[a] = std::min(std::max((int)(loc[a] * inv_vs), 0), N - 1);
      tmax[a] = safe_divide(nb[a] - loc[a], d[a]);
    }
    int count = 0, bsm = 4;
    bool acc = false, first = false;
    const int ins = ns - 2 * bsm;
    for (;;) {
      if (flags[((int64_t)cur[0] * N + cur[1]) * N + cur[2]] == 1) {
        Bound b = vbound();
        if (b.lo != -1.0f && b.hi != -1.0f) {
          if (acc) far_ = b.hi;
          else {
            near_ = b.lo;
            far_ = b.hi;
            acc = true;
            if (!first) {
              first = true;
              uniform_v3(z + count, dd + count, near_ - vs, near_ - 0.000001f, bsm);
              count += bsm;
            }
          }
        }
      } else if (acc) {
        int num = (int)std::ceil(((float)ins * (far_ - near_)) / total);
        num = std::min(ns - count, num);
        uniform_v3(z + count, dd + count, near_, far_, num);
        count += num;
        acc = false;
      }
      if (!step()) break;
    }
    if (acc) {
      int num = (int)std::ceil(((float)ins * (far_ - near_)) / total);
      num = std::min(ns - count, num);
      uniform_v3(z + count, dd + count, near_, far_, num);
      count += num;
    }
    bsm = std::min(ns - count, bsm);
    uniform_v3(z + count, dd + count, far_ + 0.000001f, far_ + vs, bsm);
  }
}

void oracle_op_inverse_z(const float* rays_d, const float* origin, const float* inv_near, const float* inv_bound,
                         int64_t npix, int offset, int spr, float* pts, float* steps) {
  for (int64_t t = 0; t < npix * spr; ++t) {
    int64_t p = t / spr;
    int j = (int)(t % spr);
    float z = 1.0f / fmac((float)(offset + j), inv_bound[p], inv_near[p]);
    float zn = 1.0f / fmac((float)(offset + j + 1), inv_bound[p], inv_near[p]);
    steps[t] = std::max(zn - z, 0.0f);
    for (int a = 0; a < 3; ++a) pts[3 * t + a] = fmac(z, rays_d[3 * p + a], origin[a]);
  }
}

void oracle_op_integrate(const float* rgba, const float* dz, int64_t npix, float early, float* frame, float* trans) {
  for (int64_t i = 0; i < npix; ++i) {
    float T = trans[i];
    if (T < early) continue;
    float c[3] = {0, 0, 0};
    for (int s = 0; s < 16; ++s) {
      const float* v = rgba + (i * 16 + s) * 4;
      float alpha = 1.0f - std::exp((-1.0f * v[3]) * dz[i * 16 + s]);
      float w = alpha * T;
      for (int a = 0; a < 3; ++a) c[a] = fmac(w, v[a], c[a]);
      T = T * (1.0f - alpha);
    }
    trans[i] = T;
    for (int a = 0; a < 3; ++a) frame[3 * i + a] = frame[3 * i + a] + c[a];
  }
}

// Training forward (FP64): rgb [n][3] of ray segments (ray i inside tile
// ray_tile[i]); counts [n] (optional) = samples per segment.  emul: 1 =
// operand emulation of the tensor-core form (TrainParams), 0 = exact.
void oracle_train_forward(const oracle_scene* os, const float* vfeat, const float* vdens, const float* mlp,
                          const float* o, const float* d, const int32_t* ray_tile, int64_t n, double* rgb,
                          int32_t* counts, int threads, int emul) {
  const Scene& s = *reinterpret_cast<const Scene*>(os);
  TrainParams p{vfeat, vdens, mlp, emul};
  parallel_for(n, threads, [&](int64_t i) {
    std::vector<TrainSample> S;
    train_forward_ray(s, p, ray_tile[i], o + 3 * i, d + 3 * i, S, rgb + 3 * i);
    if (counts) counts[i] = (int32_t)S.size();
  });
}

// Sample geometry of the training forward (the samples train_forward_ray
// takes, early stop included): per sample the global voxel id, the
// tile-local position in voxel units and delta / voxel.  offsets [n+1]:
// prefix sums of the counts returned by oracle_train_forward.
void oracle_train_samples(const oracle_scene* os, const float* vfeat, const float* vdens, const float* mlp,
                          const float* o, const float* d, const int32_t* ray_tile, int64_t n, const int64_t* offsets,
                          int32_t* vox, double* pos, double* dv) {
  const Scene& s = *reinterpret_cast<const Scene*>(os);
  TrainParams p{vfeat, vdens, mlp};
  std::vector<TrainSample> S;
  for (int64_t i = 0; i < n; ++i) {
    double C[3];
    train_forward_ray(s, p, ray_tile[i], o + 3 * i, d + 3 * i, S, C);
    const int64_t b = offsets[i];
    if ((int64_t)S.size() != offsets[i + 1] - b) continue;  // counts from another call: leave untouched
    for (size_t k = 0; k < S.size(); ++k) {
      vox[b + (int64_t)k] = S[k].rec;
      for (int a = 0; a < 3; ++a) pos[3 * (b + (int64_t)k) + a] = S[k].pos[a];
      dv[b + (int64_t)k] = S[k].dv;
    }
  }
}

// Training adjoint (FP64): gradients of L = sum(grad_rgb * rgb) accumulated
// into gF [NV][F], gG [NV], gW [NT][P] (zero them first).  Single-threaded
// (deterministic accumulation order).
void oracle_train_backward(const oracle_scene* os, const float* vfeat, const float* vdens, const float* mlp,
                           const float* o, const float* d, const int32_t* ray_tile, int64_t n,
                           const double* grad_rgb, double* gF, double* gG, double* gW, int emul) {
  const Scene& s = *reinterpret_cast<const Scene*>(os);
  TrainParams p{vfeat, vdens, mlp, emul};
  std::vector<TrainSample> S;
  for (int64_t i = 0; i < n; ++i) {
    double C[3];
    train_forward_ray(s, p, ray_tile[i], o + 3 * i, d + 3 * i, S, C);
    train_backward_ray(s, p, ray_tile[i], S, grad_rgb + 3 * i, gF, gG, gW);
  }
}

// Compositing of the training graph (training/scripts/utils.py:823-837):
// alpha = 1 - exp(-sigma*dist); T = cumprod([init_T, 1 - alpha + 1e-10])[:-1];
// out = sum(alpha * T * rgb).  Double precision.
void oracle_volume_rendering(const float* rgb, const float* sigma, const float* dists, int64_t B, int ns, float init_T,
                             double* out, double* trans, double* alpha) {
  for (int64_t b = 0; b < B; ++b) {
    double T = init_T, c[3] = {0, 0, 0};
    for (int i = 0; i < ns; ++i) {
      int64_t k = b * ns + i;
      double a = 1.0 - std::exp(-(double)sigma[k] * (double)dists[k]);
      alpha[k] = a;
      trans[k] = T;
      for (int j = 0; j < 3; ++j) c[j] += a * T * (double)rgb[3 * k + j];
      T *= (1.0 - a + 1e-10);
    }
    for (int j = 0; j < 3; ++j) out[3 * b + j] = c[j];
  }
}

// Positional encoding [x, sin(2^i x), cos(2^i x)] (training/scripts/networks.py:4-15),
// applied to n 3-vectors with L frequencies; out [n][3 + 6L].  Double precision.
void oracle_positional_encoding(const float* x, int64_t n, int L, double* out) {
  const int W = 3 + 6 * L;
  for (int64_t i = 0; i < n; ++i) {
    double* o = out + i * W;
    for (int a = 0; a < 3; ++a) o[a] = x[3 * i + a];
    for (int l = 0; l < L; ++l) {
      double sc = std::ldexp(1.0, l);
      for (int a = 0; a < 3; ++a) {
        o[3 + 6 * l + a] = std::sin(sc * (double)x[3 * i + a]);
        o[3 + 6 * l + 3 + a] = std::cos(sc * (double)x[3 * i + a]);
      }
    }
  }
}

// Trilinear lookup of query_voxel (training/scripts/tile/tile.py:225-236):
// grid_sample(align_corners=True, zeros padding) of a [C][D][H][W] volume
// (x indexes W) at index-space points (x - min_corner)/voxel - 0.5.
void oracle_grid_sample(const float* vol, int C, int D, int H, int W, const float* idx, int64_t n, double* out) {
  for (int64_t i = 0; i < n; ++i) {
    double p[3] = {idx[3 * i], idx[3 * i + 1], idx[3 * i + 2]};  // (x->W, y->H, z->D)
    int i0[3];
    double f[3];
    for (int a = 0; a < 3; ++a) { double fl = std::floor(p[a]); i0[a] = (int)fl; f[a] = p[a] - fl; }
    for (int c = 0; c < C; ++c) {
      double acc = 0;
      for (int k = 0; k < 8; ++k) {
        int dx = (k >> 2) & 1, dy = (k >> 1) & 1, dz = k & 1;
        int x = i0[0] + dx, y = i0[1] + dy, z = i0[2] + dz;
        if (x < 0 || x >= W || y < 0 || y >= H || z < 0 || z >= D) continue;
        double w = (dx ? f[0] : 1 - f[0]) * (dy ? f[1] : 1 - f[1]) * (dz ? f[2] : 1 - f[2]);
        acc += w * (double)vol[(((int64_t)c * D + z) * H + y) * W + x];
      }
      out[i * C + c] = acc;
    }
  }
}

// Pieces exposed for the reference-harness cross-check.
void oracle_ray_aabb(const float* o, const float* d, const float* c, float h, float* out) {
  const float hh[3] = {h, h, h};
  Bound b = ray_aabb(o, d, c, hh);
  out[0] = b.lo;
  out[1] = b.hi;
}
int oracle_voxel_traversal(const float* o, const float* d, const int32_t* imap, int32_t* visited, int K, int Mx, int My,
                           int Mz, float vs) {
  int cur[3], st[3];
  float tmax[3], tdel[3];
  const int M[3] = {Mx, My, Mz};
  for (int a = 0; a < 3; ++a) {
    cur[a] = (int)std::floor(o[a] / vs);
    st[a] = d[a] >= 0 ? 1 : -1;
    float nb = (float)(cur[a] + st[a]) * vs;
    if (st[a] < 0) nb = nb + vs;
    tmax[a] = d[a] != 0 ? (nb - o[a]) / d[a] : kInf;
    tdel[a] = d[a] != 0 ? (vs / d[a]) * (float)st[a] : kInf;
  }
  int idx = 0;
  int id = imap[((int64_t)cur[0] * My + cur[1]) * Mz + cur[2]];
  if (id != -1) visited[idx++] = id;
  while (idx < K) {
    int a = dda_axis(tmax);
    cur[a] += st[a];
    tmax[a] = tmax[a] + tdel[a];
    if (cur[a] < 0 || cur[a] >= M[a]) break;
    id = imap[((int64_t)cur[0] * My + cur[1]) * Mz + cur[2]];
    if (id != -1) visited[idx++] = id;
  }
  return idx;
}
float oracle_ray_triangle_onesided(const float* o, const float* d, const float* A, const float* B, const float* C) {
  // the reference's single-sided test with blur 0 (cuda_utils.h:403-436)
  float e1[3], e2[3], s[3], p[3], q[3];
  for (int a = 0; a < 3; ++a) { e1[a] = B[a] - A[a]; e2[a] = C[a] - A[a]; s[a] = o[a] - A[a]; }
  cross3(d, e2, p);
  float det = dot3(e1, p);
  if (det < 0.00000001f) return -kInf;
  det = 1.0f / det;
  float u = dot3(s, p) * det;
  if (u < 0.0f || u > 1.0f) return -kInf;
  cross3(s, e1, q);
  float v = dot3(d, q) * det;
  if (v < 0.0f || v > 1.0f) return -kInf;
  if ((u + v) < 0.0f || (u + v) > 1.0f) return -kInf;
  return dot3(e2, q) * det;
}
void oracle_trilinear_base(const float* voxels, int Mx, int My, int Mz, const float* point, float* out) {
  // FP32 trilinear with edge fallbacks (interpolation.h:41-116), float4 voxels
  int MYZ = My * Mz;
  int x0 = (int)point[0], y0 = (int)point[1], z0 = (int)point[2];
  int x1 = x0 + 1, y1 = y0 + 1, z1 = z0 + 1;
  float x = point[0] - x0, y = point[1] - y0, z = point[2] - z0;
  if (x < 0) x = 0;
  if (y < 0) y = 0;
  if (z < 0) z = 0;
  auto V = [&](int i, int j, int k, int c) { return voxels[((int64_t)i * MYZ + j * Mz + k) * 4 + c]; };
  auto i1 = [](float a, float b, float t) { return a * (1.0f - t) + b * t; };
  for (int c = 0; c < 4; ++c) {
    float r;
    if (x1 >= Mx) {
      if (y1 >= My) r = (z1 >= Mz) ? V(x0, y0, z0, c) : i1(V(x0, y0, z0, c), V(x0, y0, z1, c), z);
      else if (z1 >= Mz) r = i1(V(x0, y0, z0, c), V(x0, y1, z0, c), y);
      else r = i1(i1(V(x0, y0, z0, c), V(x0, y1, z0, c), y), i1(V(x0, y0, z1, c), V(x0, y1, z1, c), y), z);
    } else {
      if (y1 >= My) {
        if (z1 >= Mz) r = i1(V(x0, y0, z0, c), V(x1, y0, z0, c), x);
        else r = i1(i1(V(x0, y0, z0, c), V(x1, y0, z0, c), x), i1(V(x0, y0, z1, c), V(x1, y0, z1, c), x), z);
      } else if (z1 >= Mz) {
        r = i1(i1(V(x0, y0, z0, c), V(x1, y0, z0, c), x), i1(V(x0, y1, z0, c), V(x1, y1, z0, c), x), y);
      } else {
        float s = i1(i1(V(x0, y0, z0, c), V(x1, y0, z0, c), x), i1(V(x0, y1, z0, c), V(x1, y1, z0, c), x), y);
        float t = i1(i1(V(x0, y0, z1, c), V(x1, y0, z1, c), x), i1(V(x0, y1, z1, c), V(x1, y1, z1, c), x), y);
        r = i1(s, t, z);
      }
    }
    out[c] = r;
  }
}


// ---------------------------------------------------------------------------
// Specular pass ops (rendering/src/reorder.cu, rendering/src/rayreflection_render.cu)
// ---------------------------------------------------------------------------
// FASTRENDERING.sort_by_key (reorder.cu:10-22): stable sort of (keys,
// values) by key, then unique_by_key over (keys, starts): keys[k] = the k-th
// distinct key, starts[k] = starts[first position of its run].  Returns the
// number of runs.
int64_t oracle_op_sort_by_key(int16_t* keys, int32_t* values, int32_t* starts, int64_t n) {
  std::vector<int64_t> idx((size_t)n);
  for (int64_t i = 0; i < n; ++i) idx[(size_t)i] = i;
  std::stable_sort(idx.begin(), idx.end(), [&](int64_t a, int64_t b) { return keys[a] < keys[b]; });
  std::vector<int16_t> k2((size_t)n);
  std::vector<int32_t> v2((size_t)n);
  for (int64_t i = 0; i < n; ++i) {
    k2[(size_t)i] = keys[idx[(size_t)i]];
    v2[(size_t)i] = values[idx[(size_t)i]];
  }
  int64_t k = 0;
  for (int64_t i = 0; i < n; ++i) {
    keys[i] = k2[(size_t)i];
    values[i] = v2[(size_t)i];
  }
  for (int64_t i = 0; i < n; ++i)
    if (i == 0 || keys[i] != keys[i - 1]) {
      keys[k] = keys[i];
      starts[k] = starts[i];
      ++k;
    }
  return k;
}

// FASTRENDERING.assign_pixels (reorder.cu:24-94): per network k, blocks
// [block_starts[k], block_starts[k+1]) share its pixels, the first
// (count mod blocks) blocks taking one pixel more.
void oracle_op_assign_pixels(const int16_t* net, const int32_t* pixel_starts, const int32_t* block_starts,
                             int64_t num_net, int16_t* new_net, int32_t* new_pixel_starts) {
  for (int64_t k = 0; k < num_net; ++k) {
    int32_t ps = pixel_starts[k];
    const int32_t num = pixel_starts[k + 1] - pixel_starts[k];
    const int32_t nb = block_starts[k + 1] - block_starts[k];
    if (nb <= 0) continue;
    const int32_t base = num / nb, add = num - base * nb;
    for (int32_t i = 0; i < nb; ++i) {
      new_net[block_starts[k] + i] = net[k];
      new_pixel_starts[block_starts[k] + i] = ps;
      ps += i < add ? base + 1 : base;
    }
  }
}

}  // extern "C"
namespace {
constexpr int kSpecIn = 63, kSpecH = 64, kSpecHidden = 5, kSpecOut = 28, kSpecParams = 22556;
inline float h16(float v) { return round_f16(v); }
// double -> FP16, round to nearest even (one rounding)
inline float round_f16_d(double x) {
  if (x == 0.0 || !std::isfinite(x)) return round_f16((float)x);
  const double ax = std::fabs(x);
  int e;
  std::frexp(ax, &e);
  const int lead = std::max(e - 1, -14);
  const double q = std::ldexp(1.0, lead - 10);
  double r = std::nearbyint(ax / q) * q;
  if (r > 65504.0) r = INFINITY;
  return (float)std::copysign(r, x);
}
// FP16 fused multiply-add, rounded once
inline float hfma(float a, float b, float c) { return round_f16_d((double)a * (double)b + (double)c); }
inline float hmul(float a, float b) { return round_f16((float)((double)a * (double)b)); }
inline float hadd(float a, float b) { return round_f16((float)((double)a + (double)b)); }
inline float hsub(float a, float b) { return round_f16((float)((double)a - (double)b)); }
const double kSH[] = {0.28209479177387814, 0.4886025119029199, 1.0925484305920792, -1.0925484305920792,
                      0.31539156525252005, -1.0925484305920792, 0.5462742152960396};

// SH degree 2 in FP64, coefficients c[3 * basis + channel] (the device
// layout of rayreflection_render.cu:61-108; formula of training/scripts/sh.py
// eval_sh), unit direction (X, Y, Z).
void sh2_eval(const double* c, double X, double Y, double Z, double out[3]) {
  for (int i = 0; i < 3; ++i) {
    double v = kSH[0] * c[i] - kSH[1] * Y * c[3 + i] + kSH[1] * Z * c[6 + i] - kSH[1] * X * c[9 + i];
    v += kSH[2] * X * Y * c[12 + i] + kSH[3] * Y * Z * c[15 + i] + kSH[4] * (2 * Z * Z - X * X - Y * Y) * c[18 + i] +
         kSH[5] * X * Z * c[21 + i] + kSH[6] * (X * X - Y * Y) * c[24 + i];
    out[i] = v;
  }
}

// One specular sample (rayreflection_render.cu:176-287).  mode 0: the
// reference's FP16 arithmetic (each HFMA and SH operation rounded to FP16;
// the reference's fast __sinf/__cosf are replaced by the exact sine/cosine
// rounded to float, a difference FP16 rounding absorbs almost always).
// mode 1: FP64 accumulation with FP16-rounded inputs, weights and hidden
// activations (the tensor-core form's semantics); SH and sigmoid in FP64.
void spec_sample(const float pt[3], const float c[3], float inv_far, const float dir[3], const uint16_t* W, int mode,
                 float out[4]) {
  float p[3];
  for (int a = 0; a < 3; ++a) p[a] = (pt[a] - c[a]) * inv_far;
  double x[kSpecH] = {0};
  for (int a = 0; a < 3; ++a) x[a] = h16(p[a]);
  for (int i = 0; i < 10; ++i) {
    const float f = (float)(1 << i);
    for (int a = 0; a < 3; ++a) {
      const float arg = f * p[a];
      x[3 + 6 * i + a] = h16((float)std::sin((double)arg));
      x[6 + 6 * i + a] = h16((float)std::cos((double)arg));
    }
  }
  auto w = [&](size_t k) { return (double)f16_to_f32(W[k]); };
  size_t off = 0;
  double cur[kSpecH], nx[kSpecH];
  for (int i = 0; i < kSpecH; ++i) cur[i] = x[i];
  int fin = kSpecIn;
  for (int l = 0; l <= kSpecHidden; ++l) {
    const int fo = l == kSpecHidden ? kSpecOut : kSpecH;
    for (int j = 0; j < fo; ++j) {
      double acc = w(off + (size_t)j);
      if (mode == 0) {
        float a = (float)acc;
        for (int i = 0; i < fin; ++i) a = hfma((float)cur[i], (float)w(off + fo + (size_t)i * fo + j), a);
        acc = a;
      } else {
        for (int i = 0; i < fin; ++i) acc += cur[i] * w(off + fo + (size_t)i * fo + j);
      }
      if (l < kSpecHidden) {
        if (mode == 0) acc = acc < 0.0 ? hmul((float)acc, h16(0.01f)) : acc;
        else acc = h16((float)(acc < 0.0 ? acc * 0.01 : acc));
      }
      nx[j] = acc;
    }
    off += (size_t)fo + (size_t)fin * fo;
    for (int j = 0; j < fo; ++j) cur[j] = nx[j];
    fin = kSpecH;
  }
  out[3] = (float)std::max(cur[kSpecOut - 1], 0.0);
  // SH degree 2 (PlenOctree convention, coefficient layout [basis][rgb])
  if (mode == 0) {
    const float inv = 1.0f / std::sqrt(dir[0] * dir[0] + dir[1] * dir[1] + dir[2] * dir[2]);
    const float X = h16(dir[0] * inv), Y = h16(dir[1] * inv), Z = h16(dir[2] * inv);
    float col[3];
    for (int i = 0; i < 3; ++i) col[i] = hmul(h16((float)kSH[0]), (float)cur[i]);
    const float C1 = h16((float)kSH[1]);
    for (int i = 0; i < 3; ++i) {
      const float t1 = hmul(hmul(C1, Y), (float)cur[3 + i]);
      const float t2 = hmul(hmul(C1, Z), (float)cur[6 + i]);
      const float t3 = hmul(hmul(C1, X), (float)cur[9 + i]);
      col[i] = hsub(hadd(hsub(col[i], t1), t2), t3);
    }
    const float xx = hmul(X, X), yy = hmul(Y, Y), zz = hmul(Z, Z), xy = hmul(X, Y), yz = hmul(Y, Z), xz = hmul(X, Z);
    const float t = hsub(hsub(hmul(h16(2.0f), zz), xx), yy), t2 = hsub(xx, yy);
    for (int i = 0; i < 3; ++i) {
      col[i] = hadd(col[i], hmul(hmul(h16((float)kSH[2]), xy), (float)cur[12 + i]));
      col[i] = hadd(col[i], hmul(hmul(h16((float)kSH[3]), yz), (float)cur[15 + i]));
      col[i] = hadd(col[i], hmul(hmul(h16((float)kSH[4]), t), (float)cur[18 + i]));
      col[i] = hadd(col[i], hmul(hmul(h16((float)kSH[5]), xz), (float)cur[21 + i]));
      col[i] = hadd(col[i], hmul(hmul(h16((float)kSH[6]), t2), (float)cur[24 + i]));
    }
    for (int i = 0; i < 3; ++i) out[i] = 1.0f / (1.0f + std::exp(-col[i]));
  } else {
    const double nrm = std::sqrt((double)dir[0] * dir[0] + (double)dir[1] * dir[1] + (double)dir[2] * dir[2]);
    double v[3];
    sh2_eval(cur, dir[0] / nrm, dir[1] / nrm, dir[2] / nrm, v);
    for (int i = 0; i < 3; ++i) out[i] = (float)(1.0 / (1.0 + std::exp(-v[i])));
  }
}
}  // namespace
extern "C" {

// SH degree 2 (FP64) of n unit directions; coeff [n][27] basis-major.
void oracle_eval_sh2(const double* coeff, const double* dirs, int64_t n, double* out) {
  for (int64_t i = 0; i < n; ++i) sh2_eval(coeff + 27 * i, dirs[3 * i], dirs[3 * i + 1], dirs[3 * i + 2], out + 3 * i);
}

// FASTRENDERING.inference_mlp (rayreflection_render.cu:111-301): block b
// evaluates network net[b] on the samples of pixels [pstarts[b],
// pstarts[b+1]) of the sorted pixel list (query_pixel_indices maps them to
// frame pixels); pixels whose transparency is below trans_stop are skipped
// (their results are not written).  params: [G][22556] FP16 bit patterns.
// mode as in spec_sample.
void oracle_op_inference_mlp(int spr, int64_t num_block, float inverse_far, float trans_stop, const int16_t* net,
                             const float* transparency, const int32_t* qpix, const int32_t* pstarts,
                             const float* centers, const float* samples, const float* rays_d, const uint16_t* params,
                             float* results, int mode, int threads) {
  parallel_for(num_block, threads, [&](int64_t b) {
    const int g = net[b];
    if (g == -1) return;
    for (int64_t task = (int64_t)pstarts[b] * spr; task < (int64_t)pstarts[b + 1] * spr; ++task) {
      const int64_t pix = qpix[task / spr];
      if (transparency[pix] < trans_stop) continue;
      const int64_t ori = pix * spr + task % spr;
      spec_sample(samples + 3 * ori, centers + 3 * (int64_t)g, inverse_far, rays_d + 3 * pix,
                  params + (size_t)g * kSpecParams, mode, results + 4 * ori);
    }
  });
}

}  // extern "C"
namespace {
// ---------------------------------------------------------------------------
// FASTRENDERING.rendering_diffuse_octree_fp16 (rendering/src/
// raydiffuse_render_octree_fp16.cu:10-235): per pixel, the visited tiles in
// order; per tile a DDA over its 4^3 blocks; in a block with a node, samples
// every sample_step from the block entry, taken where the node's sample flag
// is set; FP16 trilinear of the node's half4 RGBA through its short index map
// (half_ope.h:222-296) and FP16 compositing (hexp); early stop on the FP16
// transmittance; the first sample with transmittance below trans_th records
// 1/(z + tile entry) and the tile's group; with soft_hit a pixel without a
// first hit takes the last examined tile's group and 1/(its exit distance)
// (:223-228).  Each FP16 operation rounds once
// (round to nearest even); hexp is exp rounded to FP16.  The fused
// multiply-adds of the compiled reference are stated: FP32 positions (entry
// point, sample point, dilated corner), each linear interpolation
// (fma(v1, 1 - x, v2 * x) in FP16) and the colour accumulation.  Reads outside a node's
// 18^3 grid (not reached by in-block samples) are skipped.
struct OctreeView {
  const int32_t* group_map;    // [NT]
  const uint16_t* data;        // [Nv][4] FP16
  const int32_t* block_map;    // [NT][64]
  const int16_t* node_map;     // [Nn][D^3]
  const uint8_t* sample_flag;  // [Nn][D^3]
  const int64_t* vstart;       // [Nn]
  const float* centers;        // [NT][3]
  float tile_size, voxel_size, sample_step;
  int D;                       // dilated voxels per block side (18)
};
constexpr int kOctBlocks = 4;

inline float hexp16(float x) { return round_f16((float)std::exp((double)x)); }

void octree_pixel(const OctreeView& V, const float o[3], const float d[3], const int32_t* vis, int K,
                  float trans_th_h, float early, bool soft_hit, float out_rgb[3], float* inv_near, int16_t* net) {
  float col[3] = {0.f, 0.f, 0.f};
  float T = 1.0f;  // FP16 values held in float
  const float early_h = round_f16(early);
  bool first_hit = false;
  int last_group = -1;
  float last_exit = 0.0f;
  const float bs = V.tile_size / (float)kOctBlocks;
  // float3 / float multiplies by the reciprocal (cutil_math.h:397-401)
  const float inv_bs = 1.0f / bs, inv_vs = 1.0f / V.voxel_size;
  const int D = V.D, DD = D * D, D3 = D * D * D;
  for (int i = 0; i < K; ++i) {
    const int tile = vis[i];
    if (tile == -1) break;
    if (T < early_h) break;
    const int group = V.group_map[tile];
    const float* c = V.centers + 3 * (int64_t)tile;
    const float hs = V.tile_size / 2.0f;
    const float h3[3] = {hs, hs, hs};
    const Bound b = ray_aabb(o, d, c, h3);
    last_group = group;
    last_exit = b.hi;
    if (b.lo == -1.0f) continue;
    float ro[3];
    for (int a = 0; a < 3; ++a) {
      const float corner = c[a] - hs;
      ro[a] = fmac(b.lo, d[a], o[a]) - corner;
      ro[a] = std::min(std::max(ro[a], 0.0f), V.tile_size - 0.00001f);
    }
    // block DDA (raydiffuse_render_octree_fp16.cu:39-131)
    int cb[3], st[3];
    float tmax[3], tdel[3];
    for (int a = 0; a < 3; ++a) {
      cb[a] = (int)(ro[a] * inv_bs);
      st[a] = d[a] >= 0.0f ? 1 : -1;
      float nb = (float)(cb[a] + st[a]) * bs;
      if (st[a] < 0) nb = nb + bs;
      tmax[a] = safe_divide(nb - ro[a], d[a]);
      tdel[a] = safe_divide(bs * (float)st[a], d[a]);
    }
    if (cb[0] < 0 || cb[1] < 0 || cb[2] < 0 || cb[0] >= kOctBlocks || cb[1] >= kOctBlocks || cb[2] >= kOctBlocks)
      continue;  // entry rounded onto the far face: skipped (the reference reads out of range there)
    float near_ = 0.0f, far_ = std::fmin(std::fmin(tmax[0], tmax[1]), tmax[2]);
    const int32_t* bmap = V.block_map + (int64_t)tile * kOctBlocks * kOctBlocks * kOctBlocks;
    for (;;) {
      const int nidx = bmap[(cb[0] * kOctBlocks + cb[1]) * kOctBlocks + cb[2]];
      if (nidx != -1) {
        const int16_t* nodes = V.node_map + (int64_t)nidx * D3;
        const uint8_t* flags = V.sample_flag + (int64_t)nidx * D3;
        const uint16_t* vox = V.data + 4 * V.vstart[nidx];
        float dc[3];
        for (int a = 0; a < 3; ++a) dc[a] = fmac((float)cb[a], bs, -V.voxel_size);
        float z = near_;
        while (z < far_) {
          float pts[3], rel[3];
          int vl[3];
          for (int a = 0; a < 3; ++a) {
            pts[a] = fmac(z, d[a], ro[a]);
            rel[a] = (pts[a] - dc[a]) * inv_vs;
            vl[a] = (int)rel[a];
          }
          const bool inside = vl[0] >= 0 && vl[1] >= 0 && vl[2] >= 0 && vl[0] < D && vl[1] < D && vl[2] < D;
          if (!inside || !flags[vl[0] * DD + vl[1] * D + vl[2]]) {
            z = z + V.sample_step;
            continue;
          }
          if (!first_hit && T < trans_th_h) {
            first_hit = true;
            *inv_near = 1.0f / (z + b.lo);
            *net = (int16_t)group;
          }
          float f[3];
          int x0[3];
          for (int a = 0; a < 3; ++a) {
            f[a] = rel[a] - 0.5f;  // the product is shared with vl: not fused
            x0[a] = (int)f[a];
          }
          bool ok = true;
          for (int a = 0; a < 3; ++a) ok = ok && x0[a] >= 0 && x0[a] + 1 < D;
          if (ok) {
            float w[3];
            for (int a = 0; a < 3; ++a) w[a] = std::max(f[a] - (float)x0[a], 0.0f);
            // corner k: (dx, dy, dz) = ((k >> 0) & 1, (k >> 1) & 1, (k >> 2) & 1) in the reference's v1..v8 order
            float v[8][4];
            for (int k = 0; k < 8; ++k) {
              const int xi = x0[0] + (k & 1), yi = x0[1] + ((k >> 1) & 1), zi = x0[2] + ((k >> 2) & 1);
              const int idx = nodes[xi * DD + yi * D + zi];
              for (int q = 0; q < 4; ++q) v[k][q] = f16_to_f32(vox[4 * (int64_t)idx + q]);
            }
            // half_interpolate1D, v1 * (1 - x) + v2 * x: the compiled reference
            // fuses the left product into the add (one FP16 rounding less)
            auto lerp = [](float a, float bb, float x) { return hfma(a, h16(1.0f - x), hmul(bb, h16(x))); };
            float rgba[4];
            for (int q = 0; q < 4; ++q) {
              const float s0 = lerp(lerp(v[0][q], v[1][q], w[0]), lerp(v[2][q], v[3][q], w[0]), w[1]);
              const float s1 = lerp(lerp(v[4][q], v[5][q], w[0]), lerp(v[6][q], v[7][q], w[0]), w[1]);
              rgba[q] = lerp(s0, s1, w[2]);
            }
            const float interval = std::min(V.sample_step, far_ - z);
            const float step_h = h16(interval);
            const float alpha = hsub(1.0f, hexp16(hmul(hmul(rgba[3], -1.0f), step_h)));
            const float wgt = hmul(alpha, T);
            for (int a = 0; a < 3; ++a) col[a] = hfma(wgt, rgba[a], col[a]);  // color + weight * rgb, fused
            T = hmul(T, hsub(1.0f, alpha));
          }
          z = z + V.sample_step;
        }
      }
      const int a = dda_axis(tmax);
      cb[a] += st[a];
      tmax[a] = tmax[a] + tdel[a];
      near_ = far_;
      far_ = std::fmin(std::fmin(tmax[0], tmax[1]), tmax[2]);
      if (cb[0] < 0 || cb[1] < 0 || cb[2] < 0 || cb[0] >= kOctBlocks || cb[1] >= kOctBlocks || cb[2] >= kOctBlocks) break;
    }
  }
  if (soft_hit && !first_hit && last_group != -1) {
    *inv_near = 1.0f / last_exit;
    *net = (int16_t)last_group;
  }
  for (int a = 0; a < 3; ++a) out_rgb[a] = col[a];
}
}  // namespace
extern "C" {

void oracle_op_rendering_diffuse_octree(const float* rays_d, const int32_t* visited, int64_t npix, int K,
                                        const float* origin, const int32_t* group_map, const uint16_t* data,
                                        const int32_t* block_map, const int16_t* node_map, const uint8_t* flags,
                                        const int64_t* vstart, const float* centers, float tile_size,
                                        float voxel_size, float sample_step, int D, float trans_th, float early,
                                        int soft_hit, float* frame, float* inv_near, int16_t* net, int threads) {
  OctreeView V{group_map, data, block_map, node_map, flags, vstart, centers, tile_size, voxel_size, sample_step, D};
  const float th = round_f16(trans_th);
  parallel_for(npix, threads, [&](int64_t i) {
    octree_pixel(V, origin, rays_d + 3 * i, visited + i * K, K, th, early, soft_hit != 0, frame + 3 * i, inv_near + i,
                 net + i);
  });
}
}  // extern "C"

// ---------------------------------------------------------------------------
// Pruning after a training epoch, on the reference's dilated [x][y][z] grids
// (D = N + 2 cells per side).
//   transparency_statistic: transparency_statistic_cuda_kernel and
//     transparency_interpolation (training/src/Helper_kernel.cu:30-172):
//     per ray a march at sample_step from the tile entry; at samples whose
//     cell ((pts - tile corner + voxel) * (1/voxel), truncated) is flagged 1
//     the 8 corner cells of the trilinear cell ((pts - tile corner) *
//     (1/voxel) + 0.5) get max(T_voxels, T * w); then T *= exp(-sigma *
//     step) through alpha = 1 - exp(-sigma * step); stop when T < 1e-8.
//     Rays run one after another (max-combining is order-free).
//   dilate_boundary: dilate_boundary_cuda_kernel (Helper_kernel.cu:174-226).
//   prune_flags: training/scripts/tile/tile.py:337-372 (with the density at
//     the voxel centres given): block maximum, exp(-s) > th -> -1, 3^3 max
//     filter of T_voxels <= T_th -> -1, then dilate_boundary.
//   pack_occupancy: flags == 1 of the inner N^3 as 64-bit words.
// Float operations round one at a time except for the fused multiply-adds of
// the compiled reference (fmac: sample positions, the cell coordinate and
// the trilinear density sum of the statistic); exp is
// std::exp in single precision.
// ---------------------------------------------------------------------------
extern "C" {

void oracle_op_transparency_statistic(const float* ro, const float* rd, int64_t n, int D, const float* center,
                                      float tile_size, float vs, float step, const float* sigma,
                                      const int16_t* nodes, float* T_voxels) {
  const int DD = D * D;
  const float hs = tile_size / 2.0f;
  const float h3[3] = {hs, hs, hs};
  const float inv_vs = 1.0f / vs;
  float tcorner[3], dcorner[3];
  for (int a = 0; a < 3; ++a) {
    tcorner[a] = center[a] - hs;
    dcorner[a] = tcorner[a] - vs;
  }
  for (int64_t r = 0; r < n; ++r) {
    const float* o = ro + 3 * r;
    const float* d = rd + 3 * r;
    const Bound b = ray_aabb(o, d, center, h3);
    float z = b.lo, T = 1.0f;
    while (z < b.hi) {
      float pts[3];
      int p[3];
      for (int a = 0; a < 3; ++a) {
        pts[a] = fmac(z, d[a], o[a]);
        p[a] = (int)((pts[a] - dcorner[a]) * inv_vs);
      }
      if (p[0] < 0 || p[1] < 0 || p[2] < 0 || p[0] >= D || p[1] >= D || p[2] >= D ||
          nodes[p[0] * DD + p[1] * D + p[2]] != 1) {
        z = z + step;
        continue;
      }
      float x[3];
      int x0[3];
      bool ok = true;
      for (int a = 0; a < 3; ++a) {
        const float f = fmac(pts[a] - tcorner[a], inv_vs, 0.5f);
        x0[a] = (int)f;
        x[a] = f - (float)x0[a];
        ok = ok && x0[a] >= 0 && x0[a] + 1 < D;
      }
      if (!ok) {
        z = z + step;
        continue;
      }
      const float ux = 1.0f - x[0], uy = 1.0f - x[1], uz = 1.0f - x[2];
      const float w[8] = {(ux * uy) * uz,     (ux * uy) * x[2],     (ux * x[1]) * uz,     (ux * x[1]) * x[2],
                          (x[0] * uy) * uz,   (x[0] * uy) * x[2],   (x[0] * x[1]) * uz,   (x[0] * x[1]) * x[2]};
      const int v000 = x0[0] * DD + x0[1] * D + x0[2];
      const int off[8] = {0, 1, D, D + 1, DD, DD + 1, DD + D, DD + D + 1};
      float s = 0.0f;
      for (int k = 0; k < 8; ++k) {
        const float t = T * w[k];
        float& slot = T_voxels[v000 + off[k]];
        if (t > slot) slot = t;
        if (k == 1) s = fmac(sigma[v000], w[0], sigma[v000 + off[1]] * w[1]);
        else if (k > 1) s = fmac(sigma[v000 + off[k]], w[k], s);
      }
      const float alpha = 1.0f - std::exp((-1.0f * s) * step);
      T = T * (1.0f - alpha);
      if (T < 0.00000001f) break;
      z = z + step;
    }
  }
}

void oracle_op_dilate_boundary(int16_t* flags, int D) {
  const int64_t total = (int64_t)D * D * D;
  std::vector<int16_t> out(flags, flags + total);
  for (int64_t i = 0; i < total; ++i) {
    if (flags[i] != -1) continue;
    const int x = (int)(i / ((int64_t)D * D)), y = (int)(i / D % D), z = (int)(i % D);
    for (int a = std::max(x - 1, 0); a <= std::min(x + 1, D - 1); ++a)
      for (int b = std::max(y - 1, 0); b <= std::min(y + 1, D - 1); ++b)
        for (int c = std::max(z - 1, 0); c <= std::min(z + 1, D - 1); ++c)
          if (flags[((int64_t)a * D + b) * D + c] == 1) out[i] = 0;
  }
  std::memcpy(flags, out.data(), sizeof(int16_t) * total);
}

void oracle_op_prune_flags(const float* T_voxels, const float* voxel_sigma, const int16_t* init_flags, int N,
                           int block, float th, float T_th, int16_t* flags) {
  const int D = N + 2;
  for (int x = 0; x < D; ++x)
    for (int y = 0; y < D; ++y)
      for (int z = 0; z < D; ++z) {
        int16_t& f = flags[((int64_t)x * D + y) * D + z];
        if (x == 0 || y == 0 || z == 0 || x == D - 1 || y == D - 1 || z == D - 1) {
          f = -1;
          continue;
        }
        const int vx = x - 1, vy = y - 1, vz = z - 1;
        f = init_flags ? init_flags[((int64_t)vx * N + vy) * N + vz] : (int16_t)1;
        float smax = voxel_sigma[((int64_t)(vx / block * block) * N + vy / block * block) * N + vz / block * block];
        for (int a = vx / block * block; a < vx / block * block + block; ++a)
          for (int b = vy / block * block; b < vy / block * block + block; ++b)
            for (int c = vz / block * block; c < vz / block * block + block; ++c)
              smax = std::max(smax, voxel_sigma[((int64_t)a * N + b) * N + c]);
        if (std::exp(-smax) > th) f = -1;
        float tmax = T_voxels[((int64_t)(x - 1) * D + (y - 1)) * D + (z - 1)];
        for (int a = x - 1; a <= x + 1; ++a)
          for (int b = y - 1; b <= y + 1; ++b)
            for (int c = z - 1; c <= z + 1; ++c) tmax = std::max(tmax, T_voxels[((int64_t)a * D + b) * D + c]);
        if (tmax <= T_th) f = -1;
      }
  oracle_op_dilate_boundary(flags, D);
}

int64_t oracle_op_pack_occupancy(const int16_t* flags, int N, uint64_t* words) {
  const int D = N + 2;
  const int64_t nvox = (int64_t)N * N * N;
  std::memset(words, 0, sizeof(uint64_t) * ((nvox + 63) / 64));
  int64_t count = 0;
  for (int64_t v = 0; v < nvox; ++v) {
    const int x = (int)(v / ((int64_t)N * N)), y = (int)(v / N % N), z = (int)(v % N);
    if (flags[((int64_t)(x + 1) * D + (y + 1)) * D + (z + 1)] == 1) {
      words[v >> 6] |= 1ull << (v & 63);
      ++count;
    }
  }
  return count;
}
}  // extern "C"

// ---------------------------------------------------------------------------
// Training-ray preparation (get_trainData_v3, training/src/cuda_func.cu:
// 1341-1686): get_rays (training/src/include/cuda_utils.h:143-155),
// tracingTile_kernel (cuda_func.cu:52-128), ray_doubleHit_inTile_kernel
// (:284-444) as the two nearest hits with the same two-sided triangle test
// as the proxy hit and the hit point inside the tile +- 1e-5, get_trainData_
// kernel (:587-663), gen_diffuse_in_tile_kernel (:1197-1339), Sample_bg
// (training/src/Sample_kernel.cu:481-542), the patch loop (:1545-1600) and
// compute_project_matrix (cuda_utils.h:37-58).  Normalisation uses
// 1 / sqrt in double rounded once to float (the reference: rsqrtf).
// ---------------------------------------------------------------------------
namespace {
inline float rinv_sqrt(float x) { return (float)(1.0 / std::sqrt((double)x)); }
inline void normalize3(const float v[3], float out[3]) {
  const float inv = rinv_sqrt((v[0] * v[0] + v[1] * v[1]) + v[2] * v[2]);
  for (int a = 0; a < 3; ++a) out[a] = v[a] * inv;
}
const float kThreshPrep = 0.00001f;
inline int patch_count(int L, int P) {
  const int half = P / 2;
  return L - P > half ? (L - P - half + P - 1) / P : 0;
}
}  // namespace

extern "C" {

void oracle_project_matrix(const float* K, const float* C, float* m) {
  const float fx = K[0], fy = K[4], cx = K[2], cy = K[5];
  const float t1 = -1.0f * ((C[0] * C[3] + C[4] * C[7]) + C[8] * C[11]);
  const float t2 = -1.0f * ((C[1] * C[3] + C[5] * C[7]) + C[9] * C[11]);
  const float t3 = -1.0f * ((C[2] * C[3] + C[6] * C[7]) + C[10] * C[11]);
  m[0] = fx * C[0] + cx * C[2];
  m[1] = fx * C[4] + cx * C[6];
  m[2] = fx * C[8] + cx * C[10];
  m[3] = fx * t1 + cx * t3;
  m[4] = fy * C[1] + cy * C[2];
  m[5] = fy * C[5] + cy * C[6];
  m[6] = fy * C[9] + cy * C[10];
  m[7] = fy * t2 + cy * t3;
  m[8] = C[2];
  m[9] = C[6];
  m[10] = C[10];
  m[11] = t3;
}

void oracle_train_rays(const float* K, const float* C, int H, int W, float* ro, float* rd) {
  for (int64_t i = 0; i < (int64_t)H * W; ++i) {
    const int y = (int)(i / W), x = (int)(i % W);
    const float u = ((float)x - K[2]) / K[0], v = ((float)y - K[5]) / K[4];
    for (int a = 0; a < 3; ++a) {
      // the reference build fuses the left product: fma(C0, u, C1 * v) + C2
      rd[3 * i + a] = fmac(C[4 * a], u, C[4 * a + 1] * v) + C[4 * a + 2];
      ro[3 * i + a] = C[4 * a + 3];
    }
  }
}

void oracle_train_tracing(const float* ro, const float* rd, int64_t n, const int32_t* imap, const int32_t* shape,
                          const float* smin, float tile, int K, int32_t* visited) {
  float size[3], c[3], h[3];
  for (int a = 0; a < 3; ++a) {
    size[a] = (float)shape[a] * tile;
    h[a] = size[a] * 0.5f;
    c[a] = smin[a] + h[a];
  }
  for (int64_t i = 0; i < n; ++i) {
    int32_t* vis = visited + i * K;
    for (int j = 0; j < K; ++j) vis[j] = -1;
    const float* o = ro + 3 * i;
    float d[3], p[3];
    normalize3(rd + 3 * i, d);
    for (int a = 0; a < 3; ++a) p[a] = o[a] - smin[a];
    if (p[0] < 0 || p[0] >= size[0] || p[1] < 0 || p[1] >= size[1] || p[2] < 0 || p[2] >= size[2]) {
      const Bound b = ray_aabb(o, d, c, h);
      for (int a = 0; a < 3; ++a) p[a] = fmac(b.lo, d[a], p[a]);
    }
    for (int a = 0; a < 3; ++a) p[a] = std::max(0.0f, std::min(p[a], size[a] - 0.000001f));
    // voxel_traversal with the start cell clamped into the grid (p / tile can
    // round up to the grid size at the far face)
    int cur[3], st[3];
    float tmax[3], tdel[3];
    for (int a = 0; a < 3; ++a) {
      cur[a] = std::min(std::max((int)std::floor(p[a] / tile), 0), shape[a] - 1);
      st[a] = d[a] >= 0 ? 1 : -1;
      float nb = (float)(cur[a] + st[a]) * tile;
      if (st[a] < 0) nb = nb + tile;
      tmax[a] = d[a] != 0 ? (nb - p[a]) / d[a] : kInf;
      tdel[a] = d[a] != 0 ? (tile / d[a]) * (float)st[a] : kInf;
    }
    int idx = 0;
    int id = imap[((int64_t)cur[0] * shape[1] + cur[1]) * shape[2] + cur[2]];
    if (id != -1) vis[idx++] = id;
    while (idx < K) {
      const int a = dda_axis(tmax);
      cur[a] += st[a];
      tmax[a] = tmax[a] + tdel[a];
      if (cur[a] < 0 || cur[a] >= shape[a]) break;
      id = imap[((int64_t)cur[0] * shape[1] + cur[1]) * shape[2] + cur[2]];
      if (id != -1) vis[idx++] = id;
    }
  }
}

void oracle_double_hits(const oracle_scene* os, const float* ro, const float* rd, const int32_t* visited, int64_t n,
                        int K, float* hits, int threads) {
  const Scene& s = *reinterpret_cast<const Scene*>(os);
  const snisr_scene_desc* D = s.d;
  const float hs = s.tile / 2.0f;
  // per tile: triangles whose bounding box meets the tile box +- 2e-5 (a
  // conservative prefilter; the hit test below decides)
  std::vector<std::vector<int64_t>> cand((size_t)s.NT);
  for (int64_t t = 0; t < D->num_triangles; ++t) {
    float lo[3], hi[3];
    for (int a = 0; a < 3; ++a) {
      lo[a] = hi[a] = D->mesh_vertices[3 * (int64_t)D->mesh_faces[3 * t] + a];
      for (int k = 1; k < 3; ++k) {
        const float v = D->mesh_vertices[3 * (int64_t)D->mesh_faces[3 * t + k] + a];
        lo[a] = std::min(lo[a], v);
        hi[a] = std::max(hi[a], v);
      }
    }
    for (int tile = 0; tile < s.NT; ++tile) {
      bool meet = true;
      for (int a = 0; a < 3; ++a) {
        const float c = s.centers[(size_t)tile * 3 + a];
        meet = meet && hi[a] >= (c - hs) - 2.0f * kThreshPrep && lo[a] <= (c + hs) + 2.0f * kThreshPrep;
      }
      if (meet) cand[(size_t)tile].push_back(t);
    }
  }
  parallel_for(n * K, threads, [&](int64_t i) {
    float* out = hits + 2 * i;
    out[0] = out[1] = -1.0f;
    const int tile = visited[i];
    if (tile < 0 || tile >= s.NT || D->num_triangles == 0) return;
    const int64_t r = i / K;
    const float* o = ro + 3 * r;
    const float* d = rd + 3 * r;
    const float* c = s.centers.data() + (size_t)tile * 3;
    float near1 = kInf, near2 = kInf;
    for (int64_t t : cand[(size_t)tile]) {
      const float* A = D->mesh_vertices + 3 * (int64_t)D->mesh_faces[3 * t];
      const float* B = D->mesh_vertices + 3 * (int64_t)D->mesh_faces[3 * t + 1];
      const float* Cc = D->mesh_vertices + 3 * (int64_t)D->mesh_faces[3 * t + 2];
      float th;
      if (!tri_hit(o, d, A, B, Cc, th) || !(th < near2)) continue;
      bool in = true;
      for (int a = 0; a < 3; ++a) in = in && std::fabs((o[a] + th * d[a]) - c[a]) - hs <= kThreshPrep;
      if (!in) continue;
      if (th < near1) {
        near2 = near1;
        near1 = th;
      } else {
        near2 = th;
      }
    }
    if (near1 != kInf) {
      out[0] = near1;
      if (near2 != kInf) out[1] = near2;
    }
  });
}

void oracle_train_bgdepth(int train_tile, const int32_t* visited, const float* hits, int64_t n, int K,
                          float* bgdepth, int32_t* valid) {
  for (int64_t i = 0; i < n; ++i) {
    const float* h = hits + 2 * i * K;
    const int32_t* vis = visited + i * K;
    float first = -1.0f, second = -1.0f;
    int ff = -1;
    for (int j = 0; j < K; ++j)
      if (h[2 * j] != -1.0f) {
        if (ff == -1) {
          ff = j;
          first = h[2 * j];
        } else {
          second = h[2 * j];
          break;
        }
      }
    bgdepth[i] = -1.0f;
    valid[i] = 0;
    for (int j = 0; j <= ff; ++j)
      if (vis[j] == train_tile) {
        bgdepth[i] = j == ff ? second : first;
        valid[i] = 1;
        break;
      }
  }
}

// Multi-view diffuse estimate of gen_diffuse_in_tile_kernel
// (training/src/cuda_func.cu:1197-1339) with the fused multiply-adds of the
// reference's build: in `a*b + c*d + e*f + g` the first add fuses its left
// product and each further product is fused into the running sum
// (fma(e, f, fma(a, b, c*d)) + g); `p + t*d` is fma(t, d, p).  normalize()
// multiplies by 1/sqrt of the squared length: correctly rounded here, CUDA's
// rsqrtf in the reference and in the library's kernel.  The two agree except
// where rsqrtf is off by an ulp; that decides only the training view's own
// weight (1 - cos)^2, a rounding residue that rsqrtf leaves non-zero for most
// pixels (the pixel then takes its own colour when no other view sees its
// hit) and that is often exactly 0 here (the pixel keeps 0).
void oracle_gen_diffuse(const float* origins, int train_tile, const float* ro, const float* rd, const float* hits,
                        const int32_t* visited, const float* images, const float* depths, const float* ms, int K,
                        int nimg, int H, int W, float* diffuse, float* bgdepth, int threads) {
  const int64_t npix = (int64_t)H * W;
  auto dot_f = [](const float* a, const float* b) { return fmac(a[2], b[2], fmac(a[0], b[0], a[1] * b[1])); };
  auto project = [&](const float* m, const float p[3], float& z, float& px, float& py) {
    const float x = fmac(m[2], p[2], fmac(m[0], p[0], m[1] * p[1])) + m[3];
    const float y = fmac(m[6], p[2], fmac(m[4], p[0], m[5] * p[1])) + m[7];
    z = fmac(m[10], p[2], fmac(m[8], p[0], m[9] * p[1])) + m[11];
    if (z <= 0.0f) return false;
    px = x / z;
    py = y / z;
    return !(px < 0.0f || px >= (float)(W - 1) || py < 0.0f || py >= (float)(H - 1));
  };
  auto normalize = [&](const float* v, float* out) {
    const float inv = (float)(1.0 / std::sqrt((double)dot_f(v, v)));
    for (int a = 0; a < 3; ++a) out[a] = v[a] * inv;
  };
  parallel_for(npix, threads, [&](int64_t i) {
    const float* h = hits + 2 * i * K;
    const int32_t* vis = visited + i * K;
    const float* o = ro + 3 * i;
    const float* d = rd + 3 * i;
    diffuse[3 * i] = diffuse[3 * i + 1] = diffuse[3 * i + 2] = 0.0f;
    float first = -1.0f;
    for (int j = 0; j < K; ++j)
      if (h[2 * j] != -1.0f && vis[j] == train_tile) {
        first = h[2 * j];
        break;
      }
    if (first == -1.0f) return;
    if (bgdepth[i] != -1.0f) {
      float p[3];
      for (int a = 0; a < 3; ++a) p[a] = fmac(bgdepth[i], d[a], o[a]);
      bool visible = false;
      for (int j = 0; j < nimg && !visible; ++j) {
        float z, px, py;
        if (!project(ms + 12 * j, p, z, px, py)) continue;
        const float dep = depths[(int64_t)j * npix + (int64_t)(int)((double)py + 0.5) * W + (int)((double)px + 0.5)];
        if (std::fabs(z - dep) > 0.01f) continue;
        visible = true;
      }
      if (!visible) bgdepth[i] = -1.0f;
    }
    float hp[3], dn[3];
    for (int a = 0; a < 3; ++a) hp[a] = fmac(first, d[a], o[a]);
    normalize(d, dn);
    float sum[3] = {0.0f, 0.0f, 0.0f}, weight = 0.0f;
    for (int j = 0; j < nimg; ++j) {
      float z, px, py;
      if (!project(ms + 12 * j, hp, z, px, py)) continue;
      const float dep = depths[(int64_t)j * npix + (int64_t)(int)((double)py + 0.5) * W + (int)((double)px + 0.5)];
      if (std::fabs(z - dep) > 0.01f) continue;
      float v[3], vp[3];
      for (int a = 0; a < 3; ++a) v[a] = hp[a] - origins[3 * j + a];
      normalize(v, vp);
      const int x0 = (int)px, y0 = (int)py;
      const float fx = px - (float)x0, fy = py - (float)y0;
      const float w00 = (1.0f - fx) * (1.0f - fy), w11 = fx * fy, w01 = (1.0f - fx) * fy, w10 = fx * (1.0f - fy);
      const int64_t i00 = (int64_t)j * npix + (int64_t)y0 * W + x0, i10 = i00 + 1, i01 = i00 + W, i11 = i01 + 1;
      float wc = 1.0f - dot_f(dn, vp);
      wc = wc * wc;
      for (int a = 0; a < 3; ++a) {
        const float c = fmac(images[3 * i11 + a], w11,
                             fmac(images[3 * i10 + a], w10, fmac(images[3 * i00 + a], w00, images[3 * i01 + a] * w01)));
        sum[a] = fmac(wc, c, sum[a]);
      }
      weight = weight + wc;
    }
    if (weight != 0.0f) {
      const float inv = 1.0f / weight;
      for (int a = 0; a < 3; ++a) diffuse[3 * i + a] = sum[a] * inv;
    }
  });
}

void oracle_sample_bg(const float* ro, const float* rd, const float* bgz, int64_t n, int ns, float range,
                      const float* center, float tile, float* z) {
  const float hs = tile / 2.0f;
  const float h3[3] = {hs, hs, hs};
  for (int64_t i = 0; i < n; ++i) {
    const float bg = bgz[i];
    if (bg == -1.0f) continue;
    const float half = range / 2.0f;
    const Bound b = ray_aabb(ro + 3 * i, rd + 3 * i, center, h3);
    float near_ = bg - half, far_ = bg + half;
    if (near_ <= b.hi) {
      near_ = b.hi + 0.00001f;
      far_ = near_ + range;
    }
    const float interval = (far_ - near_) / (float)(ns - 1);
    for (int k = 0; k < ns; ++k) z[i * ns + k] = fmac((float)k, interval, near_);
  }
}

int64_t oracle_patch_rows(const int32_t* valid, int H, int W, int P, const float* ro, const float* rd,
                          const float* bgdepth, const float* gt, const float* diffuse, float* rows) {
  const int half = P / 2, ny = patch_count(H, P), nx = patch_count(W, P);
  int64_t count = 0;
  for (int qy = 0; qy < ny; ++qy)
    for (int qx = 0; qx < nx; ++qx) {
      const int y = half + qy * P, x = half + qx * P;
      bool any = false;
      for (int dy = -half; dy <= half && !any; ++dy)
        for (int dx = -half; dx <= half && !any; ++dx) any = valid[(int64_t)(y + dy) * W + (x + dx)] != 0;
      if (!any) continue;
      for (int dy = -half; dy <= half; ++dy)
        for (int dx = -half; dx <= half; ++dx) {
          const int64_t idx = (int64_t)(y + dy) * W + (x + dx);
          float* r = rows + (count * P * P + (dy + half) * P + (dx + half)) * 14;
          for (int a = 0; a < 3; ++a) {
            r[a] = ro[3 * idx + a];
            r[3 + a] = rd[3 * idx + a];
            r[7 + a] = gt[3 * idx + a];
            r[10 + a] = diffuse[3 * idx + a];
          }
          r[6] = bgdepth[idx];
          r[13] = (float)valid[idx];
        }
      ++count;
    }
  return count;
}
}  // extern "C"
