// aov_kernels.cu — one primary pass producing the normal, albedo and depth
// passes (RenderToy NormalRenderer / AlbedoRenderer / DepthBufferRenderer,
// src/renderer.cpp:138-229, 391-427) and the raw hit records used for parity
// (BVH::Intersect of the primary rays), plus BVH::Intersect of arbitrary rays.
//
// Pixels are mapped in 8 x 8 tiles per 64-thread block so that a warp's
// primary rays are coherent and share BVH node fetches in L1.
#include "traverse.cuh"

namespace rtx {

enum PrimaryMode { kModeAov = 1, kModeHits = 2 };

__global__ void __launch_bounds__(64) k_primary(DeviceScene s, CamParams cam, int mode,
                                                float near_, float inv_range, float* normal,
                                                float* albedo, float* depth, int* tri_out,
                                                float* tuv_out, int* err) {
  int tiles_x = (cam.W + 7) >> 3;
  int tile = blockIdx.x;
  int x = (tile % tiles_x) * 8 + (threadIdx.x & 7);
  int y = (tile / tiles_x) * 8 + (threadIdx.x >> 3);
  if (x >= cam.W || y >= cam.H) return;
  F3 o, d;
  camera_ray(cam, x, y, o, d);
  float t, u, v;
  VisitCount vc;
  int h = closest_hit<false>(s, o, d, -1, t, u, v, err, vc);
  size_t p = (size_t)y * cam.W + x;
  if (mode & kModeHits) {
    tri_out[p] = h;
    tuv_out[3 * p] = t;
    tuv_out[3 * p + 1] = u;
    tuv_out[3 * p + 2] = v;
  }
  if (mode & kModeAov) {
    F3 nv = f3s(0.0f), av = f3s(0.0f), dv = f3s(1.0f);
    if (h >= 0) {
      float4 s0 = __ldg(s.shade + 4 * (size_t)h);
      float4 s1 = __ldg(s.shade + 4 * (size_t)h + 1);
      int info = __float_as_int(s1.w);
      bool smooth = info < 0;
      int mat = info & 0x7fffffff;
      F3 n = shading_normal(s, h, u, v, s0, s1, smooth);
      // NormalRenderer: flip to face the viewer by the geometric normal
      if (dot(f3(s0.x, s0.y, s0.z), -d) < 0.0f) n = -n;
      nv = (n + f3s(1.0f)) / 2.0f;
      const float* m = s.mats + 24 * (size_t)mat;
      av = f3(__ldg(m), __ldg(m + 1), __ldg(m + 2));
      if (__ldg(m + 21) != 0.0f) av = textured_base(m, o + d * t, n, s.perm);
      dv = f3s(clamp01((t - near_) * inv_range));
    }
    if (normal) {
      normal[3 * p] = nv.x;
      normal[3 * p + 1] = nv.y;
      normal[3 * p + 2] = nv.z;
    }
    if (albedo) {
      albedo[3 * p] = av.x;
      albedo[3 * p + 1] = av.y;
      albedo[3 * p + 2] = av.z;
    }
    if (depth) {
      depth[3 * p] = dv.x;
      depth[3 * p + 1] = dv.y;
      depth[3 * p + 2] = dv.z;
    }
  }
}

__global__ void __launch_bounds__(128) k_intersect(DeviceScene s, int n, const float* rays,
                                                   const int* exclude, int* tri_out,
                                                   float* tuv_out, int* err) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float* r = rays + 6 * (size_t)i;
  F3 o = f3(r[0], r[1], r[2]), d = f3(r[3], r[4], r[5]);
  float t, u, v;
  VisitCount vc;
  int h = closest_hit<false>(s, o, d, exclude ? exclude[i] : -1, t, u, v, err, vc);
  tri_out[i] = h;
  tuv_out[3 * (size_t)i] = t;
  tuv_out[3 * (size_t)i + 1] = u;
  tuv_out[3 * (size_t)i + 2] = v;
}

cudaError_t launch_primary(const DeviceScene& s, const CamParams& cam, int mode, float near_,
                           float far_, float* normal, float* albedo, float* depth, int* tri,
                           float* tuv, int* err, cudaStream_t st, int* launches) {
  int tiles = ((cam.W + 7) >> 3) * ((cam.H + 7) >> 3);
  // DepthBufferRenderer: div_far_minus_near = 1 / (far - near), in float
  float inv_range = 1.0f / (far_ - near_);
  k_primary<<<tiles, 64, 0, st>>>(s, cam, mode, near_, inv_range, normal, albedo, depth, tri,
                                  tuv, err);
  ++*launches;
  return cudaGetLastError();
}

cudaError_t launch_intersect(const DeviceScene& s, int n, const float* rays, const int* exclude,
                             int* tri, float* tuv, int* err, cudaStream_t st, int* launches) {
  if (n <= 0) return cudaSuccess;
  k_intersect<<<(n + 127) / 128, 128, 0, st>>>(s, n, rays, exclude, tri, tuv, err);
  ++*launches;
  return cudaGetLastError();
}

// RenderToy's procedural textures sampled at points (the shading code's
// samplers): out[i] = Sample(uv[2 i], uv[2 i + 1])
__global__ void k_texture_sample(int kind, float param, const uint8_t* __restrict__ perm, int n,
                                 const float* __restrict__ uv, float* __restrict__ out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = texture_sample(kind, param, perm, uv[2 * i], uv[2 * i + 1]);
}

cudaError_t launch_texture_sample(int kind, float param, const uint8_t* perm, int n, const float* uv,
                                  float* out, cudaStream_t st) {
  if (n > 0) k_texture_sample<<<(n + 255) / 256, 256, 0, st>>>(kind, param, perm, n, uv, out);
  return cudaGetLastError();
}

}  // namespace rtx
