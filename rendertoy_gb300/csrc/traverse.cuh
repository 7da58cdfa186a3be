// traverse.cuh — closest-hit and occlusion traversal of the binary and the
// 4-wide BVH.
//
// Closest hit restates the result of BVH::Intersect (RenderToy
// src/bvh.cpp:266-341): the nearest triangle whose two-sided Moller-Trumbore
// test (src/object.cpp:107-167, restated operation for operation in
// tri_hit below) accepts the ray with 0 <= t < 1e7, skipping one excluded
// triangle.  The reference's best-first octree walk is replaced by a
// depth-first walk with a per-thread stack; equal distances resolve to the
// lower triangle id, so the result does not depend on the walk order.
//
// Loads: a binary node is four 16-byte __ldg loads (both children), a 4-wide
// node seven, a triangle three.
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

// Slab-test form of a ray: t = plane * inv - origin * inv, one FMA per plane.
// The box test need not be exact: boxes are widened far beyond its rounding.
struct RayBox {
  float ox, oy, oz, ix, iy, iz;  // ox.. hold -origin * inv
};

RTX_DEV float safe_inv(float d) {
  // 1/d with zero components mapped to a huge finite value of the same sign
  return fabsf(d) > 1e-30f ? 1.0f / d : copysignf(1e30f, d);
}

RTX_DEV RayBox make_raybox(F3 o, F3 d) {
  float ix = safe_inv(d.x), iy = safe_inv(d.y), iz = safe_inv(d.z);
  return RayBox{-o.x * ix, -o.y * iy, -o.z * iz, ix, iy, iz};
}

// Slab test of the two children stored in one node; returns entry distances.
RTX_DEV void box2(const RayBox& r, float4 n0, float4 n1, float4 n2, float tmax, bool& h0,
                  bool& h1, float& t0, float& t1) {
  float a0 = __fmaf_rn(n0.x, r.ix, r.ox), a1 = __fmaf_rn(n0.y, r.ix, r.ox);
  float b0 = __fmaf_rn(n0.z, r.iy, r.oy), b1 = __fmaf_rn(n0.w, r.iy, r.oy);
  float c0 = __fmaf_rn(n2.x, r.iz, r.oz), c1 = __fmaf_rn(n2.y, r.iz, r.oz);
  float lo0 = fmaxf(fmaxf(fminf(a0, a1), fminf(b0, b1)), fmaxf(fminf(c0, c1), 0.0f));
  float hi0 = fminf(fminf(fmaxf(a0, a1), fmaxf(b0, b1)), fminf(fmaxf(c0, c1), tmax));
  float d0 = __fmaf_rn(n1.x, r.ix, r.ox), d1 = __fmaf_rn(n1.y, r.ix, r.ox);
  float e0 = __fmaf_rn(n1.z, r.iy, r.oy), e1 = __fmaf_rn(n1.w, r.iy, r.oy);
  float f0 = __fmaf_rn(n2.z, r.iz, r.oz), f1 = __fmaf_rn(n2.w, r.iz, r.oz);
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
        if (sp >= s.stack_limit) {
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
        if (sp >= s.stack_limit) {
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

// ---------------------------------------------------------------------------
// 4-wide tree: one node = seven 16-byte loads, four slab tests; the children
// hit are visited nearest first (sorted by entry distance).
// ---------------------------------------------------------------------------
RTX_DEV void cswap(float& ka, int& ra, float& kb, int& rb) {
  if (kb < ka) {
    float tk = ka;
    ka = kb;
    kb = tk;
    int tr = ra;
    ra = rb;
    rb = tr;
  }
}

// The ray as the 4-wide box test reads it: each axis' inverse direction and
// -origin * inverse, twice (one packed pair serves two children), and which
// of a node's two plane vectors is the near one on each axis (the max planes
// when the direction is negative).  Choosing the near and far planes by load
// address once per ray replaces a min and a max per child and axis.
struct RayBox4 {
  f2_t ix, iy, iz;
  f2_t ox, oy, oz;
  int sx, sy, sz;
};

RTX_DEV RayBox4 make_raybox4(F3 o, F3 d) {
  const float ix = safe_inv(d.x), iy = safe_inv(d.y), iz = safe_inv(d.z);
  const float ox = -o.x * ix, oy = -o.y * iy, oz = -o.z * iz;
  RayBox4 r;
  r.ix = f2_pack(ix, ix);
  r.iy = f2_pack(iy, iy);
  r.iz = f2_pack(iz, iz);
  r.ox = f2_pack(ox, ox);
  r.oy = f2_pack(oy, oy);
  r.oz = f2_pack(oz, oz);
  r.sx = ix < 0.0f;
  r.sy = iy < 0.0f;
  r.sz = iz < 0.0f;
  return r;
}

// Plane distances of the four children on one axis: two packed FMAs.
RTX_DEV void slab4(float4 p, f2_t inv, f2_t org, float (&t)[4]) {
  f2_unpack(f2_fma(f2_pack(p.x, p.y), inv, org), t[0], t[1]);
  f2_unpack(f2_fma(f2_pack(p.z, p.w), inv, org), t[2], t[3]);
}

// Children of a 4-wide node hit before tmax; returns how many, in c0.. .
// kSort: nearest entry distance first (closest hit); otherwise in node order
// (an occlusion query's answer does not depend on the order, and skipping
// the sort measured 1.3 % faster frames).  Node: min x, max x, min y, max y,
// min z, max z of the four children (one float4 each), then the four child
// refs.
template <bool kSort>
RTX_DEV int node4(const RayBox4& r, const float4* n, float tmax, int& c0, int& c1, int& c2, int& c3) {
  const float4 px0 = __ldg(n + r.sx), px1 = __ldg(n + 1 - r.sx);
  const float4 py0 = __ldg(n + 2 + r.sy), py1 = __ldg(n + 3 - r.sy);
  const float4 pz0 = __ldg(n + 4 + r.sz), pz1 = __ldg(n + 5 - r.sz);
  const float4 rf = __ldg(n + 6);
  float nx[4], fx[4], ny[4], fy[4], nz[4], fz[4];
  slab4(px0, r.ix, r.ox, nx);
  slab4(px1, r.ix, r.ox, fx);
  slab4(py0, r.iy, r.oy, ny);
  slab4(py1, r.iy, r.oy, fy);
  slab4(pz0, r.iz, r.oz, nz);
  slab4(pz1, r.iz, r.oz, fz);
  const float kMiss = __int_as_float(0x7f800000);
  float k[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const float tn = fmax3(nx[i], ny[i], fmaxf(nz[i], 0.0f));
    const float tf = fmin3(fx[i], fy[i], fminf(fz[i], tmax));
    k[i] = tn <= tf ? tn : kMiss;
  }
  float k0 = k[0], k1 = k[1], k2 = k[2], k3 = k[3];
  c0 = __float_as_int(rf.x);
  c1 = __float_as_int(rf.y);
  c2 = __float_as_int(rf.z);
  c3 = __float_as_int(rf.w);
  if (!kSort) {
    // hit children first, in node order (an occlusion query needs no order)
    int h[4] = {c0, c1, c2, c3};
    bool v[4] = {k0 < kMiss, k1 < kMiss, k2 < kMiss, k3 < kMiss};
    int n = 0;
    int o0 = 0, o1 = 0, o2 = 0, o3 = 0;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      if (v[i]) {
        if (n == 0) o0 = h[i];
        else if (n == 1) o1 = h[i];
        else if (n == 2) o2 = h[i];
        else o3 = h[i];
        ++n;
      }
    }
    c0 = o0;
    c1 = o1;
    c2 = o2;
    c3 = o3;
    return n;
  }
  cswap(k0, c0, k1, c1);
  cswap(k2, c2, k3, c3);
  cswap(k0, c0, k2, c2);
  cswap(k1, c1, k3, c3);
  cswap(k1, c1, k2, c2);
  return (k0 < kMiss) + (k1 < kMiss) + (k2 < kMiss) + (k3 < kMiss);
}

// Closest hit over the 4-wide tree; same result as closest_hit.
template <bool kAnyHit, bool kCount>
RTX_DEV int trace4(const DeviceScene& s, F3 o, F3 d, int exclude, int target, float& t, float& u,
                   float& v, int* err, VisitCount& vc) {
  // closest hit: t starts at 1e7, returns the triangle; occlusion: t is the
  // limit, returns 1 when occluded, -1 otherwise
  if (!kAnyHit) t = kInf;
  u = 0.0f;
  v = 0.0f;
  int best = -1;
  int node = s.root4;
  if (node == kEmptyRoot) return -1;
  const RayBox4 rb = make_raybox4(o, d);
  // Pending nodes: the newest in the register `top`, the older ones in
  // stack[0 .. sp - 2].  A pop hands over `top` at once and reloads the
  // entry below it for the next pop, so the stack's memory latency stays off
  // the pop -> node fetch dependency chain.
  int stack[kStackSize];
  int sp = 0, top = 0;
  auto push = [&](int x) {
    if (sp > 0) stack[sp - 1] = top;
    top = x;
    ++sp;
  };
  while (true) {
    if (node >= 0) {
      if (kCount) vc.nodes++;
      int c0, c1, c2, c3;
      int nh = node4<!kAnyHit>(rb, s.nodes4 + kNode4Vecs * (size_t)node, t, c0, c1, c2, c3);
      if (nh > 0) {
        if (sp + 3 > s.stack_limit) {
          atomicOr(err, kErrStackOverflow);
          return kAnyHit ? 1 : best;
        }
        if (nh >= 4) push(c3);
        if (nh >= 3) push(c2);
        if (nh >= 2) push(c1);
        node = c0;
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
        if (id == exclude || (kAnyHit && id == target)) continue;
        float tt, uu, vv;
        if (tri_hit(o, d, f3(a.x, a.y, a.z), f3(b.x, b.y, b.z), f3(c.x, c.y, c.z), tt, uu, vv)) {
          if (kAnyHit) {
            if (tt < t || (tt == t && id < target)) return 1;
          } else if (tt < t || (tt == t && id < best)) {
            t = tt;
            u = uu;
            v = vv;
            best = id;
          }
        }
      }
    }
    if (sp == 0) break;
    node = top;
    if (--sp > 0) top = stack[sp - 1];
  }
  return best;
}

// ---------------------------------------------------------------------------
// Resumable traversal for persistent kernels (Aila & Laine, HPG 2009:
// while-while loop, speculative postponement of the first leaf, and an exit
// when too few lanes of the warp are still busy so that the kernel can hand
// finished lanes new rays).  One lane's ray lives in a Trav; trav_run advances
// it and returns true once it has finished.
// ---------------------------------------------------------------------------
constexpr int kSentinel = 0x76543210;  // bottom of the stack: "nothing left"

struct Trav {
  F3 o, d;
  RayBox rb;
  float tmax;  // closest hit: the nearest t so far; occlusion: the fixed limit
  float u, v;
  int best;    // closest hit: triangle id (-1); occlusion: 1 once occluded
  int exclude, target;
  int node, leaf, sp;
};

// `stack` is the lane's traversal stack (kStackSize ints, kept apart from the
// scalar state so that the latter stays in registers).
RTX_DEV void trav_begin(Trav& r, int* stack, const DeviceScene& s, F3 o, F3 d, int exclude,
                        int target, float tmax) {
  r.o = o;
  r.d = d;
  r.rb = make_raybox(o, d);
  r.exclude = exclude;
  r.target = target;
  r.tmax = tmax;
  r.u = 0.0f;
  r.v = 0.0f;
  r.best = -1;
  r.sp = 0;
  stack[0] = kSentinel;
  r.leaf = 0;
  r.node = s.root;
  if (s.root == kEmptyRoot) {
    r.node = kSentinel;
  } else if (s.root < 0) {  // the whole tree is one leaf
    r.leaf = s.root;
    r.node = kSentinel;
  }
}

template <bool kAnyHit, bool kCount>
RTX_DEV bool trav_run(Trav& r, int* stack, const DeviceScene& s, int* err, VisitCount& vc,
                      int min_busy) {
  do {
    // inner nodes: 0 <= node < kSentinel
    while ((unsigned)r.node < (unsigned)kSentinel) {
      const float4* n = s.nodes + 4 * (size_t)r.node;
      float4 n0 = __ldg(n), n1 = __ldg(n + 1), n2 = __ldg(n + 2), n3 = __ldg(n + 3);
      if (kCount) vc.nodes++;
      bool h0, h1;
      float t0, t1;
      box2(r.rb, n0, n1, n2, r.tmax, h0, h1, t0, t1);
      int c0 = __float_as_int(n3.x), c1 = __float_as_int(n3.y);
      if (!h0 && !h1) {
        r.node = stack[r.sp--];
      } else {
        r.node = h0 ? c0 : c1;
        if (h0 && h1) {
          int farc = c1;
          if (t1 < t0) {
            r.node = c1;
            farc = c0;
          }
          if (r.sp + 1 >= s.stack_limit) {
            atomicOr(err, kErrStackOverflow);
            r.node = kSentinel;
            r.leaf = 0;
            return true;
          }
          stack[++r.sp] = farc;
        }
      }
      if (r.node < 0 && r.leaf >= 0) {  // first leaf: postpone it, keep descending
        r.leaf = r.node;
        r.node = stack[r.sp--];
      }
      if (!__any_sync(__activemask(), r.leaf >= 0)) break;  // every busy lane holds a leaf
    }
    // postponed leaves
    while (r.leaf < 0) {
      int ref = ~r.leaf;
      int first = ref >> 3, cnt = (ref & 7) + 1;
      for (int k = 0; k < cnt; ++k) {
        const float4* tp = s.tris + 3 * (size_t)(first + k);
        float4 a = __ldg(tp), b = __ldg(tp + 1), c = __ldg(tp + 2);
        if (kCount) vc.tris++;
        int id = __float_as_int(a.w);
        if (id == r.exclude || (kAnyHit && id == r.target)) continue;
        float tt, uu, vv;
        if (tri_hit(r.o, r.d, f3(a.x, a.y, a.z), f3(b.x, b.y, b.z), f3(c.x, c.y, c.z), tt, uu, vv)) {
          if (kAnyHit) {
            if (tt < r.tmax || (tt == r.tmax && id < r.target)) {
              r.best = 1;
              r.node = kSentinel;
              break;
            }
          } else if (tt < r.tmax || (tt == r.tmax && id < r.best)) {
            r.tmax = tt;
            r.u = uu;
            r.v = vv;
            r.best = id;
          }
        }
      }
      if (kAnyHit && r.best == 1) {
        r.leaf = 0;
        break;
      }
      r.leaf = r.node;
      if (r.node < 0) r.node = stack[r.sp--];
    }
    if (__popc(__activemask()) < min_busy) break;  // let the warp refill idle lanes
  } while (r.node != kSentinel);
  return r.node == kSentinel;
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
