// Proxy-mesh nearest hit: BVH traversal with an FP32 Moller-Trumbore test
// and an FP64 re-test inside the near-degenerate band.
//
// The triangle test follows RayTriangleIntersection
// (rendering/src/include/cuda_utils.h:403-436) made two-sided: the reference
// flips the winding by the sign of the face normal against the ray
// (training/src/cuda_func.cu:224-231) so that every face is front-facing,
// which is the same as testing |det|.  Hits need u, v >= 0, u + v <= 1 and
// t > 0; the nearest hit wins, ties go to the lower triangle id.
#pragma once

#include "device_common.cuh"

namespace snisr {

constexpr float kDetBand = 1e-7f;   // |det| below this: re-test in FP64
constexpr float kBaryBand = 1e-5f;  // u, v or u+v-1 within this of 0: re-test in FP64

__device__ __forceinline__ float dot3(const float a[3], const float b[3]) {
  return fadd(fadd(fmul(a[0], b[0]), fmul(a[1], b[1])), fmul(a[2], b[2]));
}
__device__ __forceinline__ void cross3(const float a[3], const float b[3], float c[3]) {
  c[0] = fsub(fmul(a[1], b[2]), fmul(a[2], b[1]));
  c[1] = fsub(fmul(a[2], b[0]), fmul(a[0], b[2]));
  c[2] = fsub(fmul(a[0], b[1]), fmul(a[1], b[0]));
}
__device__ __forceinline__ double ddot3(const double a[3], const double b[3]) {
  return __dadd_rn(__dadd_rn(__dmul_rn(a[0], b[0]), __dmul_rn(a[1], b[1])), __dmul_rn(a[2], b[2]));
}
__device__ __forceinline__ void dcross3(const double a[3], const double b[3], double c[3]) {
  c[0] = __dsub_rn(__dmul_rn(a[1], b[2]), __dmul_rn(a[2], b[1]));
  c[1] = __dsub_rn(__dmul_rn(a[2], b[0]), __dmul_rn(a[0], b[2]));
  c[2] = __dsub_rn(__dmul_rn(a[0], b[1]), __dmul_rn(a[1], b[0]));
}

// Returns true and the hit distance if the ray hits the triangle.
__device__ __forceinline__ bool tri_hit(const float o[3], const float d[3], const float A[3], const float B[3],
                                        const float C[3], float& t_hit) {
  float e1[3], e2[3], s[3], p[3], qv[3];
  for (int a = 0; a < 3; ++a) { e1[a] = fsub(B[a], A[a]); e2[a] = fsub(C[a], A[a]); s[a] = fsub(o[a], A[a]); }
  cross3(d, e2, p);
  float det = dot3(e1, p);
  cross3(s, e1, qv);
  float un = dot3(s, p), vn = dot3(d, qv), tn = dot3(e2, qv);
  bool band = !(fabsf(det) >= kDetBand);
  float u = 0.f, v = 0.f, t = 0.f, uv = 0.f;
  if (!band) {
    float inv = fdiv(1.0f, det);
    u = fmul(un, inv); v = fmul(vn, inv); t = fmul(tn, inv);
    uv = fadd(u, v);
    band = fabsf(u) < kBaryBand || fabsf(v) < kBaryBand || fabsf(fsub(uv, 1.0f)) < kBaryBand;
  }
  if (!band) {
    if (u >= 0.0f && v >= 0.0f && uv <= 1.0f && t > 0.0f) { t_hit = t; return true; }
    return false;
  }
  double de1[3], de2[3], ds[3], dd[3], dp[3], dq[3];
  for (int a = 0; a < 3; ++a) {
    de1[a] = __dsub_rn((double)B[a], (double)A[a]);
    de2[a] = __dsub_rn((double)C[a], (double)A[a]);
    ds[a] = __dsub_rn((double)o[a], (double)A[a]);
    dd[a] = (double)d[a];
  }
  dcross3(dd, de2, dp);
  double ddet = ddot3(de1, dp);
  if (ddet == 0.0) return false;
  dcross3(ds, de1, dq);
  double du = __ddiv_rn(ddot3(ds, dp), ddet);
  double dv = __ddiv_rn(ddot3(dd, dq), ddet);
  double dt = __ddiv_rn(ddot3(de2, dq), ddet);
  if (du >= 0.0 && dv >= 0.0 && __dadd_rn(du, dv) <= 1.0 && dt > 0.0) {
    t_hit = (float)dt;
    return t_hit > 0.0f;
  }
  return false;
}

// Slab test of a BVH node box against [0, tmax]; NaN from 0*inf is dropped
// by fminf/fmaxf.  The far bound is widened by a few ulps so that rounding
// never culls a box whose triangles the exact test would hit.
__device__ __forceinline__ bool box_hit(const float o[3], const float inv[3], const float* bmin, const float* bmax,
                                        float tmax, float& tnear) {
  float lo = 0.0f, hi = tmax;
  for (int a = 0; a < 3; ++a) {
    float t0 = fmul(fsub(bmin[a], o[a]), inv[a]);
    float t1 = fmul(fsub(bmax[a], o[a]), inv[a]);
    lo = fmaxf(lo, fminf(t0, t1));
    hi = fminf(hi, fmaxf(t0, t1));
  }
  tnear = lo;
  return lo <= fmul(hi, 1.0000005f);
}

// Nearest hit of the ray with the proxy mesh.  Returns the hit distance or
// -1, and the original triangle id (or -1).  A node goes on the stack with
// the distance at which the ray enters its box, tested when it was pushed,
// and its child index / triangle range (first << 5 | count; leaves hold at
// most 16 triangles): popped, it needs no load and only the comparison of
// that distance with the current best (the box's exit passed the test when
// pushed), the same test as re-testing the box.
__device__ __forceinline__ float bvh_nearest(const SceneDev& S, const float o[3], const float d[3], int& tri_out) {
  float inv[3];
  for (int a = 0; a < 3; ++a) inv[a] = fdiv(1.0f, d[a]);
  float best = 3.0e38f;
  int best_id = -1;
  uint32_t stack[64];
  float snear[64];
  int sp = 0;
  {
    const BvhNodeDev r = S.bvh[0];
    float tn;
    if (box_hit(o, inv, r.bmin, r.bmax, best, tn)) {
      stack[0] = ((uint32_t)r.first << 5) | (uint32_t)r.count;
      snear[0] = tn;
      sp = 1;
    }
  }
  while (sp > 0) {
    --sp;
    if (!(snear[sp] <= fmul(best, 1.0000005f))) continue;
    const int first = (int)(stack[sp] >> 5), count = (int)(stack[sp] & 31u);
    if (count > 0) {
      for (int k = 0; k < count; ++k) {
        int slot = first + k;
        float4 a4 = __ldg(S.tri + 3 * slot), b4 = __ldg(S.tri + 3 * slot + 1), c4 = __ldg(S.tri + 3 * slot + 2);
        float A[3] = {a4.x, a4.y, a4.z}, B[3] = {b4.x, b4.y, b4.z}, C[3] = {c4.x, c4.y, c4.z};
        float t;
        if (tri_hit(o, d, A, B, C, t)) {
          int id = __ldg(S.tri_id + slot);
          if (t < best || (t == best && id < best_id)) { best = t; best_id = id; }
        }
      }
    } else {
      const BvhNodeDev l = S.bvh[first], r = S.bvh[first + 1];
      float tl, tr;
      const bool hl = box_hit(o, inv, l.bmin, l.bmax, best, tl);
      const bool hr = box_hit(o, inv, r.bmin, r.bmax, best, tr);
      if (sp + 2 > 64) { atomicOr(S.err, ERR_OVERFLOW); break; }
      const uint32_t el = ((uint32_t)l.first << 5) | (uint32_t)l.count, er = ((uint32_t)r.first << 5) | (uint32_t)r.count;
      if (hl && hr) {  // the nearer child on top
        if (tl <= tr) { stack[sp] = er; snear[sp++] = tr; stack[sp] = el; snear[sp++] = tl; }
        else { stack[sp] = el; snear[sp++] = tl; stack[sp] = er; snear[sp++] = tr; }
      } else if (hl) {
        stack[sp] = el; snear[sp++] = tl;
      } else if (hr) {
        stack[sp] = er; snear[sp++] = tr;
      }
    }
  }
  tri_out = best_id;
  return best_id >= 0 ? best : -1.0f;
}

}  // namespace snisr
