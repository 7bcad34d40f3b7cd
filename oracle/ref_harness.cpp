// Host harness around the reference's header-only helpers, compiled from the
// reference tree by oracle/build_ref.py into oracle/_ref/libref.so.  Test
// infrastructure only: it lets tests compare the oracle's restatements with
// the reference's own code (RayAABBIntersection, voxel_traversal,
// RayTriangleIntersection, trilinear_base, uniform_sample_bound_v3,
// inverse_z_sample_bound, safe_divide, signf) on the same inputs.
#include <cuda_runtime.h>

// The helpers are declared __device__ (some __host__ __device__); build them
// as plain host functions.
#undef __device__
#undef __host__
#undef __forceinline__
#define __device__
#define __host__
#define __forceinline__ inline

#include "cutil_math.h"
#include "cuda_utils.h"
#include "interpolation.h"

extern "C" {

void ref_ray_aabb(const float* o, const float* d, const float* c, float h, float* out) {
  float2 b = RayAABBIntersection(make_float3(o[0], o[1], o[2]), make_float3(d[0], d[1], d[2]),
                                 make_float3(c[0], c[1], c[2]), h);
  out[0] = b.x;
  out[1] = b.y;
}

int ref_voxel_traversal(const float* o, const float* d, const int* imap, int* visited, int K, int Mx, int My, int Mz,
                        float vs) {
  for (int i = 0; i < K; ++i) visited[i] = -1;
  voxel_traversal(o, d, imap, visited, K, Mx, My, Mz, vs);
  int n = 0;
  while (n < K && visited[n] != -1) ++n;
  return n;
}

float ref_ray_triangle(const float* o, const float* d, const float* A, const float* B, const float* C) {
  return RayTriangleIntersection(make_float3(o[0], o[1], o[2]), make_float3(d[0], d[1], d[2]),
                                 make_float3(A[0], A[1], A[2]), make_float3(B[0], B[1], B[2]),
                                 make_float3(C[0], C[1], C[2]), 0.0f);
}

void ref_trilinear_base(const float* vox, int Mx, int My, int Mz, const float* p, float* out) {
  float4 r = trilinear_base(reinterpret_cast<const float4*>(vox), Mx, My, Mz, make_float3(p[0], p[1], p[2]));
  out[0] = r.x;
  out[1] = r.y;
  out[2] = r.z;
  out[3] = r.w;
}

void ref_uniform_sample_bound_v3(float* z, float* dist, float near, float far, int n) {
  uniform_sample_bound_v3(z, dist, near, far, n);
}

void ref_inverse_z_sample_bound(float* z, float near, float far, int n) { inverse_z_sample_bound(z, near, far, n); }

float ref_safe_divide(float a, float b) { return safe_divide(a, b); }
int ref_signf(float a) { return signf(a); }

}  // extern "C"
