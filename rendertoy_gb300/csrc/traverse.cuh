// traverse.cuh — closest-hit and occlusion traversal of the binary BVH.
//
// Closest hit restates the result of BVH::Intersect (RenderToy
// src/bvh.cpp:266-341): the nearest triangle whose two-sided Moller-Trumbore
// test (src/object.cpp:107-167, restated operation for operation in
// tri_hit below) accepts the ray with 0 <= t < 1e7, skipping one excluded
// triangle.  The reference's best-first octree walk is replaced by a
// depth-first walk with a per-thread stack; equal distances resolve to the
// lower triangle id, so the result does not depend on the walk order.
//
// Loads: a node is four 16-byte __ldg loads (both children), a triangle three.
#pragma once
#include "device_math.cuh"
#include "rtx_internal.h"

namespace rtx {

// Triangle::Intersect (object.cpp:107-167), same operations and order
RTX_DEV bool tri_hit(F3 o, F3 d, F3 v0, F3 e1, F3 e2, float& t, float& u, float& v) {
  F3 pvec = cross(d, e2);
  float det = dot(e1, pvec);
  if (det > 0.0f) {
    F3 tvec = o - v0;
    float alpha = dot(pvec, tvec);
    if (alpha < 0.0f || alpha > det) return false;
    F3 qvec = cross(tvec, e1);
    float beta = dot(qvec, d);
    if (beta < 0.0f || alpha + beta > det) return false;
    float inv_det = 1.0f / det;
    t = dot(e2, qvec) * inv_det;
    if (t < 0.0f) return false;
    u = alpha * inv_det;
    v = beta * inv_det;
    return true;
  } else if (det < 0.0f) {
    F3 tvec = o - v0;
    float alpha = dot(pvec, tvec);
    if (alpha > 0.0f || alpha < det) return false;
    F3 qvec = cross(tvec, e1);
    float beta = dot(qvec, d);
    if (beta > 0.0f || alpha + beta < det) return false;
    float inv_det = 1.0f / det;
    t = dot(e2, qvec) * inv_det;
    if (t < 0.0f) return false;
    u = alpha * inv_det;
    v = beta * inv_det;
    return true;
  }
  return false;
}

struct RayBox {
  float ox, oy, oz, ix, iy, iz;
};

RTX_DEV float safe_inv(float d) {
  // 1/d with zero components mapped to a huge finite value of the same sign
  return fabsf(d) > 1e-30f ? 1.0f / d : copysignf(1e30f, d);
}

RTX_DEV RayBox make_raybox(F3 o, F3 d) {
  return RayBox{o.x, o.y, o.z, safe_inv(d.x), safe_inv(d.y), safe_inv(d.z)};
}

// Slab test of the two children stored in one node; returns entry distances.
RTX_DEV void box2(const RayBox& r, float4 n0, float4 n1, float4 n2, float tmax, bool& h0,
                  bool& h1, float& t0, float& t1) {
  float a0 = (n0.x - r.ox) * r.ix, a1 = (n0.y - r.ox) * r.ix;
  float b0 = (n0.z - r.oy) * r.iy, b1 = (n0.w - r.oy) * r.iy;
  float c0 = (n2.x - r.oz) * r.iz, c1 = (n2.y - r.oz) * r.iz;
  float lo0 = fmaxf(fmaxf(fminf(a0, a1), fminf(b0, b1)), fmaxf(fminf(c0, c1), 0.0f));
  float hi0 = fminf(fminf(fmaxf(a0, a1), fmaxf(b0, b1)), fminf(fmaxf(c0, c1), tmax));
  float d0 = (n1.x - r.ox) * r.ix, d1 = (n1.y - r.ox) * r.ix;
  float e0 = (n1.z - r.oy) * r.iy, e1 = (n1.w - r.oy) * r.iy;
  float f0 = (n2.z - r.oz) * r.iz, f1 = (n2.w - r.oz) * r.iz;
  float lo1 = fmaxf(fmaxf(fminf(d0, d1), fminf(e0, e1)), fmaxf(fminf(f0, f1), 0.0f));
  float hi1 = fminf(fminf(fmaxf(d0, d1), fmaxf(e0, e1)), fminf(fmaxf(f0, f1), tmax));
  h0 = lo0 <= hi0;
  h1 = lo1 <= hi1;
  t0 = lo0;
  t1 = lo1;
}

struct VisitCount {
  unsigned nodes = 0, tris = 0;
};

// Closest hit.  Returns the triangle id or -1; t/u/v as BVH::Intersect
// (t = 1e7 on a miss).
template <bool kCount>
RTX_DEV int closest_hit(const DeviceScene& s, F3 o, F3 d, int exclude, float& t, float& u,
                        float& v, int* err, VisitCount& vc) {
  t = kInf;
  u = 0.0f;
  v = 0.0f;
  int best = -1;
  if (s.root == kEmptyRoot) return -1;
  RayBox rb = make_raybox(o, d);
  int stack[kStackSize];
  int sp = 0;
  int node = s.root;
  while (true) {
    if (node >= 0) {
      const float4* n = s.nodes + 4 * (size_t)node;
      float4 n0 = __ldg(n), n1 = __ldg(n + 1), n2 = __ldg(n + 2), n3 = __ldg(n + 3);
      if (kCount) vc.nodes++;
      bool h0, h1;
      float t0, t1;
      box2(rb, n0, n1, n2, t, h0, h1, t0, t1);
      int c0 = __float_as_int(n3.x), c1 = __float_as_int(n3.y);
      if (h0 && h1) {
        int nearc = c0, farc = c1;
        if (t1 < t0) {
          nearc = c1;
          farc = c0;
        }
        if (sp >= kStackSize) {
          atomicOr(err, kErrStackOverflow);
          return best;
        }
        stack[sp++] = farc;
        node = nearc;
        continue;
      } else if (h0) {
        node = c0;
        continue;
      } else if (h1) {
        node = c1;
        continue;
      }
    } else {
      int ref = ~node;
      int first = ref >> 3, cnt = (ref & 7) + 1;
      for (int k = 0; k < cnt; ++k) {
        const float4* tp = s.tris + 3 * (size_t)(first + k);
        float4 a = __ldg(tp), b = __ldg(tp + 1), c = __ldg(tp + 2);
        if (kCount) vc.tris++;
        int id = __float_as_int(a.w);
        if (id == exclude) continue;
        float tt, uu, vv;
        if (tri_hit(o, d, f3(a.x, a.y, a.z), f3(b.x, b.y, b.z), f3(c.x, c.y, c.z), tt, uu, vv)) {
          if (tt < t || (tt == t && id < best)) {
            t = tt;
            u = uu;
            v = vv;
            best = id;
          }
        }
      }
    }
    if (sp == 0) break;
    node = stack[--sp];
  }
  return best;
}

// Occlusion: is there a triangle other than `exclude` and `target` that the
// exact test accepts at t < tmax, or at t == tmax with an id below `target`
// (the tie rule of closest_hit)?
template <bool kCount>
RTX_DEV bool occluded(const DeviceScene& s, F3 o, F3 d, int exclude, int target, float tmax,
                      int* err, VisitCount& vc) {
  if (s.root == kEmptyRoot) return false;
  RayBox rb = make_raybox(o, d);
  int stack[kStackSize];
  int sp = 0;
  int node = s.root;
  while (true) {
    if (node >= 0) {
      const float4* n = s.nodes + 4 * (size_t)node;
      float4 n0 = __ldg(n), n1 = __ldg(n + 1), n2 = __ldg(n + 2), n3 = __ldg(n + 3);
      if (kCount) vc.nodes++;
      bool h0, h1;
      float t0, t1;
      box2(rb, n0, n1, n2, tmax, h0, h1, t0, t1);
      int c0 = __float_as_int(n3.x), c1 = __float_as_int(n3.y);
      if (h0 && h1) {
        int nearc = c0, farc = c1;
        if (t1 < t0) {
          nearc = c1;
          farc = c0;
        }
        if (sp >= kStackSize) {
          atomicOr(err, kErrStackOverflow);
          return true;
        }
        stack[sp++] = farc;
        node = nearc;
        continue;
      } else if (h0) {
        node = c0;
        continue;
      } else if (h1) {
        node = c1;
        continue;
      }
    } else {
      int ref = ~node;
      int first = ref >> 3, cnt = (ref & 7) + 1;
      for (int k = 0; k < cnt; ++k) {
        const float4* tp = s.tris + 3 * (size_t)(first + k);
        float4 a = __ldg(tp), b = __ldg(tp + 1), c = __ldg(tp + 2);
        if (kCount) vc.tris++;
        int id = __float_as_int(a.w);
        if (id == exclude || id == target) continue;
        float tt, uu, vv;
        if (tri_hit(o, d, f3(a.x, a.y, a.z), f3(b.x, b.y, b.z), f3(c.x, c.y, c.z), tt, uu, vv)) {
          if (tt < tmax || (tt == tmax && id < target)) return true;
        }
      }
    }
    if (sp == 0) break;
    node = stack[--sp];
  }
  return false;
}

// Shading normal (Triangle::NormalC, src/object.cpp:207-217)
RTX_DEV F3 shading_normal(const DeviceScene& s, int tri, float u, float v, float4 s0, float4 s1,
                          bool smooth) {
  if (smooth) {
    float4 s2 = __ldg(s.shade + 4 * (size_t)tri + 2);
    float4 s3 = __ldg(s.shade + 4 * (size_t)tri + 3);
    float w = 1.0f - u - v;
    return normalized((f3(s1.x, s1.y, s1.z) * w + f3(s2.x, s2.y, s2.z) * u) +
                      f3(s3.x, s3.y, s3.z) * v);
  }
  return f3(s0.x, s0.y, s0.z);
}

// Primary ray (src/renderer.cpp:252-259, Geometry::O2WTransform object.cpp:58-64)
RTX_DEV void camera_ray(const CamParams& c, int x, int y, F3& o, F3& d) {
  float nx = float(x) * c.inv_w, ny = float(y) * c.inv_h;
  float sx = 2.0f * c.right * nx - c.right;
  float sy = 2.0f * c.top * ny - c.top;
  float oo[3], pp[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const float* r = c.m + 4 * i;
    float a = 0.0f;
    a = a + r[0] * 0.0f;
    a = a + r[1] * 0.0f;
    a = a + r[2] * 0.0f;
    a = a + r[3] * 1.0f;
    oo[i] = a;
    float b = 0.0f;
    b = b + r[0] * sx;
    b = b + r[1] * sy;
    b = b + r[2] * -1.0f;
    b = b + r[3] * 1.0f;
    pp[i] = b;
  }
  o = f3(oo[0], oo[1], oo[2]);
  d = normalized(f3(pp[0], pp[1], pp[2]) - o);
}

}  // namespace rtx
