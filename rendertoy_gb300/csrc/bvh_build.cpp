// bvh_build.cpp — host binned-SAH builder of the binary BVH that the GPU
// traverses (layout in rtx_internal.h).
//
// This replaces the reference's loose octree (RenderToy src/bvh.cpp:127-264:
// centroid insertion, refit, best-first priority-queue traversal) with a
// structure suited to a GPU: SAH-split binary tree, both child boxes stored in
// the parent so one 64-byte fetch tests two children, and triangles copied in
// leaf order so a leaf is one contiguous run of 48-byte records.  Any
// conservative acceleration structure returns the same closest hit, because
// the exact Moller-Trumbore test decides every hit; child boxes are widened by
// a few parts per million of the scene size so rounding in the box test never
// culls a triangle the exact test accepts.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>

#include "rtx_internal.h"

namespace rtx {
namespace {

struct AABB {
  float lo[3], hi[3];
  void reset() {
    for (int k = 0; k < 3; ++k) {
      lo[k] = INFINITY;
      hi[k] = -INFINITY;
    }
  }
  void grow(const AABB& b) {
    for (int k = 0; k < 3; ++k) {
      lo[k] = std::min(lo[k], b.lo[k]);
      hi[k] = std::max(hi[k], b.hi[k]);
    }
  }
  void grow_pt(const float* p) {
    for (int k = 0; k < 3; ++k) {
      lo[k] = std::min(lo[k], p[k]);
      hi[k] = std::max(hi[k], p[k]);
    }
  }
  float area() const {
    float d0 = hi[0] - lo[0], d1 = hi[1] - lo[1], d2 = hi[2] - lo[2];
    if (!(d0 >= 0.0f) || !(d1 >= 0.0f) || !(d2 >= 0.0f)) return 0.0f;
    return 2.0f * (d0 * d1 + d1 * d2 + d2 * d0);
  }
};

struct Prim {
  AABB box;
  float c[3];
};

constexpr int kBins = 16;

struct Builder {
  const float* verts;
  std::vector<Prim> prims;
  std::vector<int> idx;
  std::vector<float4> nodes;
  std::vector<float4> tris;
  int max_leaf;
  float pad_abs;
  int n_leaves = 0;
  int max_depth = 0;

  int make_leaf(int begin, int end) {
    int first = (int)(tris.size() / 3);
    for (int i = begin; i < end; ++i) {
      int t = idx[i];
      const float* v = verts + 9 * (size_t)t;
      float4 a, b, c;
      // Triangle::UpdateCache, object.cpp:238-239
      a = make_float4(v[0], v[1], v[2], 0.0f);
      std::memcpy(&a.w, &t, 4);
      b = make_float4(v[3] - v[0], v[4] - v[1], v[5] - v[2], 0.0f);
      c = make_float4(v[6] - v[0], v[7] - v[1], v[8] - v[2], 0.0f);
      tris.push_back(a);
      tris.push_back(b);
      tris.push_back(c);
    }
    ++n_leaves;
    return ~((first << 3) | (end - begin - 1));
  }

  int build(int begin, int end, int depth) {
    max_depth = std::max(max_depth, depth);
    int n = end - begin;
    AABB cb;
    cb.reset();
    AABB bb;
    bb.reset();
    for (int i = begin; i < end; ++i) {
      cb.grow_pt(prims[idx[i]].c);
      bb.grow(prims[idx[i]].box);
    }
    if (n == 1) return make_leaf(begin, end);

    // SAH over 3 axes, kBins bins each.  From depth 40 on the split is the
    // median by index, which bounds the depth (and so the traversal stack).
    int best_axis = -1, best_split = -1;
    float best_cost = INFINITY;
    for (int ax = 0; ax < 3 && depth < 40; ++ax) {
      float ext = cb.hi[ax] - cb.lo[ax];
      if (!(ext > 0.0f)) continue;
      float scale = kBins / ext;
      AABB bins[kBins];
      int cnt[kBins] = {};
      for (int b = 0; b < kBins; ++b) bins[b].reset();
      for (int i = begin; i < end; ++i) {
        const Prim& p = prims[idx[i]];
        int b = std::min(kBins - 1, (int)((p.c[ax] - cb.lo[ax]) * scale));
        cnt[b]++;
        bins[b].grow(p.box);
      }
      float right_area[kBins];
      int right_cnt[kBins];
      AABB acc;
      acc.reset();
      int c = 0;
      for (int b = kBins - 1; b > 0; --b) {
        acc.grow(bins[b]);
        c += cnt[b];
        right_area[b] = acc.area();
        right_cnt[b] = c;
      }
      acc.reset();
      c = 0;
      for (int b = 0; b < kBins - 1; ++b) {
        acc.grow(bins[b]);
        c += cnt[b];
        if (c == 0 || right_cnt[b + 1] == 0) continue;
        float cost = acc.area() * c + right_area[b + 1] * right_cnt[b + 1];
        if (cost < best_cost) {
          best_cost = cost;
          best_axis = ax;
          best_split = b;
        }
      }
    }
    float parent_area = bb.area();
    float leaf_cost = (float)n;
    float split_cost = parent_area > 0.0f ? 1.0f + best_cost / parent_area : INFINITY;
    if (n <= max_leaf && (best_axis < 0 || leaf_cost <= split_cost)) return make_leaf(begin, end);

    int mid;
    if (best_axis < 0) {
      mid = begin + n / 2;  // all centroids coincide: split by index
    } else {
      float ext = cb.hi[best_axis] - cb.lo[best_axis];
      float scale = kBins / ext;
      int ax = best_axis;
      auto it = std::partition(idx.begin() + begin, idx.begin() + end, [&](int t) {
        int b = std::min(kBins - 1, (int)((prims[t].c[ax] - cb.lo[ax]) * scale));
        return b <= best_split;
      });
      mid = (int)(it - idx.begin());
      if (mid == begin || mid == end) mid = begin + n / 2;
    }
    int node = (int)(nodes.size() / 4);
    nodes.resize(nodes.size() + 4);
    AABB lb, rb;
    lb.reset();
    rb.reset();
    for (int i = begin; i < mid; ++i) lb.grow(prims[idx[i]].box);
    for (int i = mid; i < end; ++i) rb.grow(prims[idx[i]].box);
    int l = build(begin, mid, depth + 1);
    int r = build(mid, end, depth + 1);
    auto lo = [&](float v) { return v - (std::fabs(v) * 4e-7f + pad_abs); };
    auto hi = [&](float v) { return v + (std::fabs(v) * 4e-7f + pad_abs); };
    float4* nd = &nodes[4 * (size_t)node];
    nd[0] = make_float4(lo(lb.lo[0]), hi(lb.hi[0]), lo(lb.lo[1]), hi(lb.hi[1]));
    nd[1] = make_float4(lo(rb.lo[0]), hi(rb.hi[0]), lo(rb.lo[1]), hi(rb.hi[1]));
    nd[2] = make_float4(lo(lb.lo[2]), hi(lb.hi[2]), lo(rb.lo[2]), hi(rb.hi[2]));
    float4 m = make_float4(0, 0, 0, 0);
    std::memcpy(&m.x, &l, 4);
    std::memcpy(&m.y, &r, 4);
    nd[3] = m;
    return node;
  }
};

// Collapse the binary tree into a 4-wide one: a 4-wide node takes a binary
// node's two children and keeps replacing its largest-area inner child by
// that child's two children until it has four (or only leaves remain).
struct Collapser {
  const std::vector<float4>& bin;
  std::vector<float4>& out;
  int max_depth = 0;

  struct Child {
    float lo[3], hi[3];
    int ref;
  };

  Child child_of(int b, int k) const {
    const float4* n = &bin[4 * (size_t)b];
    Child c;
    if (k == 0) {
      c.lo[0] = n[0].x; c.hi[0] = n[0].y; c.lo[1] = n[0].z; c.hi[1] = n[0].w;
      c.lo[2] = n[2].x; c.hi[2] = n[2].y;
      std::memcpy(&c.ref, &n[3].x, 4);
    } else {
      c.lo[0] = n[1].x; c.hi[0] = n[1].y; c.lo[1] = n[1].z; c.hi[1] = n[1].w;
      c.lo[2] = n[2].z; c.hi[2] = n[2].w;
      std::memcpy(&c.ref, &n[3].y, 4);
    }
    return c;
  }

  static float area(const Child& c) {
    float d0 = c.hi[0] - c.lo[0], d1 = c.hi[1] - c.lo[1], d2 = c.hi[2] - c.lo[2];
    return d0 * d1 + d1 * d2 + d2 * d0;
  }

  int collapse(int b, int depth) {
    max_depth = std::max(max_depth, depth);
    int idx = (int)(out.size() / kNode4Vecs);
    out.resize(out.size() + kNode4Vecs);
    Child ch[4];
    int n = 2;
    ch[0] = child_of(b, 0);
    ch[1] = child_of(b, 1);
    while (n < 4) {
      int best = -1;
      float best_area = -1.0f;
      for (int k = 0; k < n; ++k)
        if (ch[k].ref >= 0 && area(ch[k]) > best_area) {
          best = k;
          best_area = area(ch[k]);
        }
      if (best < 0) break;
      int bb = ch[best].ref;
      ch[best] = child_of(bb, 0);
      ch[n++] = child_of(bb, 1);
    }
    int refs[4];
    for (int k = 0; k < 4; ++k) refs[k] = k < n ? (ch[k].ref >= 0 ? collapse(ch[k].ref, depth + 1) : ch[k].ref) : 0;
    float4* nd = &out[kNode4Vecs * (size_t)idx];
    float v[6][4];
    for (int k = 0; k < 4; ++k)
      for (int a = 0; a < 3; ++a) {
        v[2 * a][k] = k < n ? ch[k].lo[a] : 1e30f;
        v[2 * a + 1][k] = k < n ? ch[k].hi[a] : 1e30f;
      }
    for (int r = 0; r < 6; ++r) nd[r] = make_float4(v[r][0], v[r][1], v[r][2], v[r][3]);
    float4 m;
    std::memcpy(&m.x, &refs[0], 4);
    std::memcpy(&m.y, &refs[1], 4);
    std::memcpy(&m.z, &refs[2], 4);
    std::memcpy(&m.w, &refs[3], 4);
    nd[6] = m;
    return idx;
  }
};

}  // namespace

BvhBuildResult build_bvh(const float* verts, int n, int max_leaf) {
  auto t0 = std::chrono::steady_clock::now();
  BvhBuildResult res;
  if (n <= 0) return res;
  Builder b;
  b.verts = verts;
  b.max_leaf = std::min(std::max(max_leaf, 1), kMaxLeaf);
  b.prims.resize(n);
  b.idx.resize(n);
  AABB scene;
  scene.reset();
  for (int i = 0; i < n; ++i) {
    Prim& p = b.prims[i];
    p.box.reset();
    for (int k = 0; k < 3; ++k) p.box.grow_pt(verts + 9 * (size_t)i + 3 * k);
    for (int k = 0; k < 3; ++k) p.c[k] = 0.5f * (p.box.lo[k] + p.box.hi[k]);
    scene.grow(p.box);
    b.idx[i] = i;
  }
  float ext = 0.0f;
  for (int k = 0; k < 3; ++k) ext = std::max(ext, scene.hi[k] - scene.lo[k]);
  if (!std::isfinite(ext)) ext = 0.0f;
  b.pad_abs = ext * 2e-6f + 1e-30f;
  b.nodes.reserve((size_t)8 * n / std::max(1, b.max_leaf) + 8);
  b.tris.reserve((size_t)3 * n);
  res.root = b.build(0, n, 0);
  res.nodes.swap(b.nodes);
  res.tris.swap(b.tris);
  res.n_nodes = (int)(res.nodes.size() / 4);
  res.n_leaves = b.n_leaves;
  res.depth = b.max_depth;
  if (res.root >= 0) {
    Collapser col{res.nodes, res.nodes4};
    res.nodes4.reserve(res.nodes.size() * kNode4Vecs / 4 / 2 + kNode4Vecs);
    res.root4 = col.collapse(res.root, 0);
    res.depth4 = col.max_depth;
  } else {
    res.root4 = res.root;
  }
  res.n_nodes4 = (int)(res.nodes4.size() / kNode4Vecs);
  res.ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  return res;
}

}  // namespace rtx
