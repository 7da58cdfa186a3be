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
//
// The build runs on host threads and gives the same bits as one thread:
// the passes over the first levels' large ranges are cut into chunks whose
// results merge in chunk order; below them the halves of each split go to
// threads of their own, each subtree into its own arrays; the arrays are
// then numbered depth first and copied into place, offsetting their node
// and triangle indices.  The 4-wide collapse is split the same way.
// Triangles with non-finite vertices are accepted (their centroids go to
// the first bin) and can never be hit.
#include <algorithm>
#include <atomic>
#include <cfloat>
#include <chrono>
#include <cmath>
#include <cstring>
#include <exception>
#include <memory>
#include <mutex>
#include <system_error>
#include <thread>

#include "host_threads.h"
#include "rtx_internal.h"

namespace rtx {
namespace {

// A box; the fourth lane (always empty) lets the compiler grow a box with
// whole-vector minimum and maximum instructions.
struct alignas(16) AABB {
  float lo[4], hi[4];
  void reset() {
    for (int k = 0; k < 4; ++k) {
      lo[k] = INFINITY;
      hi[k] = -INFINITY;
    }
  }
  void grow(const AABB& b) {
    for (int k = 0; k < 4; ++k) {
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
  float c[3];  // centroid of the box
  int tri;     // triangle id
};

constexpr int kBins = 16;
// Ranges of fewer triangles than this are built by one thread from start to
// end, into arrays of their own
constexpr int kTaskPrims = 1 << 14;
// Above them, a half of a split of at least this many triangles gets a
// thread of its own; scenes with fewer triangles are built on one thread
constexpr int kThreadPrims = 1 << 16;

// Bin of a centroid coordinate along one axis.  A centroid that is not a
// number (a triangle with a non-finite vertex) goes to bin 0.
inline int bin_of(float c, float lo, float scale) {
  float x = (c - lo) * scale;
  if (!(x >= 0.0f)) return 0;
  return x < (float)kBins ? (int)x : kBins - 1;
}

// A range of prims with the bounds of their boxes and of their centroids
struct Range {
  int begin, end;
  AABB bb, cb;
};

// A pass over a range is cut into chunks of at least this many prims, one
// thread each; the chunks' results are merged in chunk order, which gives
// the serial pass's values bit for bit (a box keeps the first of equal
// minima or maxima in either form, counts are integers).
constexpr int kChunkPrims = 1 << 16;

int chunk_count(int n, unsigned n_threads) {
  return (int)std::max(1u, std::min(n_threads, (unsigned)(n / kChunkPrims)));
}

void range_bounds(const Prim* prims, Range& r, unsigned n_threads) {
  auto bound_chunk = [&](AABB& bb_out, AABB& cb_out, int b0, int e0) {
    AABB bb, cb;  // local, so that threads never write one cache line
    bb.reset();
    cb.reset();
    for (int i = b0; i < e0; ++i) {
      cb.grow_pt(prims[i].c);
      bb.grow(prims[i].box);
    }
    bb_out = bb;
    cb_out = cb;
  };
  int n = r.end - r.begin, chunks = chunk_count(n, n_threads);
  if (chunks == 1) {
    bound_chunk(r.bb, r.cb, r.begin, r.end);
    return;
  }
  std::vector<AABB> bb(chunks), cb(chunks);
  run_parallel(chunks, chunks, [&](size_t c) {
    bound_chunk(bb[c], cb[c], r.begin + (int)((int64_t)n * (int64_t)c / chunks),
                r.begin + (int)((int64_t)n * (int64_t)(c + 1) / chunks));
  });
  r.bb.reset();
  r.cb.reset();
  for (int c = 0; c < chunks; ++c) {
    r.bb.grow(bb[c]);
    r.cb.grow(cb[c]);
  }
}

// SAH over 3 axes, kBins bins each, for one range.  Returns -1 when the range
// becomes a leaf; otherwise partitions prims[begin, end) and returns the
// first index of the right half, with both halves' bounds.
int split_range(Prim* prims, const Range& r, int depth, int max_leaf, Range& left, Range& right,
                unsigned n_threads = 1) {
  int n = r.end - r.begin;
  if (n == 1) return -1;
  const AABB& cb = r.cb;
  // From depth 40 on the split is the median by index, which bounds the
  // depth (and so the traversal stack).
  float scale[3];
  bool use[3];
  for (int ax = 0; ax < 3; ++ax) {
    float ext = cb.hi[ax] - cb.lo[ax];
    use[ax] = depth < 40 && ext > 0.0f;
    scale[ax] = use[ax] ? kBins / ext : 0.0f;
  }
  struct Bins {
    AABB box[3][kBins];
    int cnt[3][kBins];
  };
  auto bin_chunk = [&](Bins& B, int b0, int e0) {  // one pass bins all three axes
    for (int ax = 0; ax < 3; ++ax)
      for (int b = 0; b < kBins; ++b) {
        B.box[ax][b].reset();
        B.cnt[ax][b] = 0;
      }
    for (int i = b0; i < e0; ++i) {
      const Prim& p = prims[i];
      for (int ax = 0; ax < 3; ++ax) {
        if (!use[ax]) continue;
        int b = bin_of(p.c[ax], cb.lo[ax], scale[ax]);
        B.cnt[ax][b]++;
        B.box[ax][b].grow(p.box);
      }
    }
  };
  Bins all;
  int chunks = chunk_count(n, n_threads);
  if (chunks == 1) {
    bin_chunk(all, r.begin, r.end);
  } else {
    std::vector<Bins> part(chunks);
    run_parallel(chunks, chunks, [&](size_t c) {
      Bins B;  // local, so that threads never write one cache line
      bin_chunk(B, r.begin + (int)((int64_t)n * (int64_t)c / chunks),
                r.begin + (int)((int64_t)n * (int64_t)(c + 1) / chunks));
      part[c] = B;
    });
    all = part[0];
    for (int c = 1; c < chunks; ++c)
      for (int ax = 0; ax < 3; ++ax)
        for (int b = 0; b < kBins; ++b) {
          all.box[ax][b].grow(part[c].box[ax][b]);
          all.cnt[ax][b] += part[c].cnt[ax][b];
        }
  }
  auto& bins = all.box;
  auto& cnt = all.cnt;
  int best_axis = -1, best_split = -1;
  float best_cost = INFINITY;
  for (int ax = 0; ax < 3; ++ax) {
    if (!use[ax]) continue;
    // the sweep visits occupied bins only: an empty bin adds nothing to
    // either side, so a split after it costs the same as one after the
    // occupied bin before it, which the strict comparison below keeps
    int occ[kBins], n_occ = 0;
    for (int b = 0; b < kBins; ++b)
      if (cnt[ax][b]) occ[n_occ++] = b;
    float right_area[kBins];
    int right_cnt[kBins];
    AABB acc;
    acc.reset();
    int c = 0;
    for (int j = n_occ - 1; j > 0; --j) {
      acc.grow(bins[ax][occ[j]]);
      c += cnt[ax][occ[j]];
      right_area[j] = acc.area();
      right_cnt[j] = c;
    }
    acc.reset();
    c = 0;
    for (int j = 0; j < n_occ - 1; ++j) {
      acc.grow(bins[ax][occ[j]]);
      c += cnt[ax][occ[j]];
      float cost = acc.area() * c + right_area[j + 1] * right_cnt[j + 1];
      if (cost < best_cost) {
        best_cost = cost;
        best_axis = ax;
        best_split = occ[j];
      }
    }
  }
  float parent_area = r.bb.area();
  float leaf_cost = (float)n;
  float split_cost = parent_area > 0.0f ? 1.0f + best_cost / parent_area : INFINITY;
  if (n <= max_leaf && (best_axis < 0 || leaf_cost <= split_cost)) return -1;

  int mid;
  if (best_axis < 0) {
    mid = r.begin + n / 2;  // all centroids coincide: split by index
  } else {
    int ax = best_axis;
    float lo = cb.lo[ax], sc = scale[ax];
    Prim* it = std::partition(prims + r.begin, prims + r.end,
                              [&](const Prim& p) { return bin_of(p.c[ax], lo, sc) <= best_split; });
    mid = (int)(it - prims);
    if (mid == r.begin || mid == r.end) mid = r.begin + n / 2;
  }
  left.begin = r.begin;
  left.end = mid;
  right.begin = mid;
  right.end = r.end;
  range_bounds(prims, left, n_threads);
  range_bounds(prims, right, n_threads);
  return mid;
}

// An inner node: both children's boxes, widened by a few parts per million
void write_node(float4* nd, const AABB& lb, const AABB& rb, int l, int r, float pad_abs) {
  auto lo = [&](float v) { return v - (std::fabs(v) * 4e-7f + pad_abs); };
  auto hi = [&](float v) { return v + (std::fabs(v) * 4e-7f + pad_abs); };
  nd[0] = make_float4(lo(lb.lo[0]), hi(lb.hi[0]), lo(lb.lo[1]), hi(lb.hi[1]));
  nd[1] = make_float4(lo(rb.lo[0]), hi(rb.hi[0]), lo(rb.lo[1]), hi(rb.hi[1]));
  nd[2] = make_float4(lo(lb.lo[2]), hi(lb.hi[2]), lo(rb.lo[2]), hi(rb.hi[2]));
  float4 m = make_float4(0, 0, 0, 0);
  std::memcpy(&m.x, &l, 4);
  std::memcpy(&m.y, &r, 4);
  nd[3] = m;
}

// One subtree built by one thread: its nodes and leaf triangles numbered
// from 0, in depth-first order (a node before its left subtree, the left
// subtree before the right one)
struct Subtree {
  const float* verts = nullptr;
  Prim* prims = nullptr;
  int max_leaf = 1;
  float pad_abs = 0.0f;
  Float4Array nodes;
  Float4Array tris;
  int root = 0;
  int n_leaves = 0;
  int max_depth = 0;

  int make_leaf(int begin, int end) {
    int first = (int)(tris.size() / 3);
    for (int i = begin; i < end; ++i) {
      int t = prims[i].tri;
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

  int build(const Range& r, int depth) {
    max_depth = std::max(max_depth, depth);
    Range L, R;
    if (split_range(prims, r, depth, max_leaf, L, R) < 0) return make_leaf(r.begin, r.end);
    int node = (int)(nodes.size() / 4);
    nodes.resize(nodes.size() + 4);
    int l = build(L, depth + 1);
    int rr = build(R, depth + 1);
    write_node(&nodes[4 * (size_t)node], L.bb, R.bb, l, rr, pad_abs);
    return node;
  }
};

// The tree above the subtrees.  A part is an inner node whose two children
// are parts, or a subtree built by one thread.  The parts of the first few
// levels are split on threads of their own; numbering comes last.
struct Part {
  bool inner = false;
  AABB lb, rb;  // inner: the children's boxes
  std::unique_ptr<Part> l, r;
  Subtree sub;  // otherwise
  int depth = 0;
  int node_base = 0, tri_base = 0, ref = 0;  // set when numbering
};

struct Builder {
  const float* verts;
  std::vector<Prim> prims;
  int max_leaf;
  float pad_abs;
  unsigned n_threads = 1;

  void split_part(Part& p, const Range& r, int depth) {
    p.depth = depth;
    // threads working on this part's passes: its share of the triangles
    // (the parts of one level run at once)
    unsigned share = (unsigned)std::max<int64_t>(1, (int64_t)n_threads * (r.end - r.begin) / (int64_t)prims.size());
    Range L, R;
    if (r.end - r.begin < kTaskPrims || split_range(prims.data(), r, depth, max_leaf, L, R, share) < 0) {
      p.sub.verts = verts;
      p.sub.prims = prims.data();
      p.sub.max_leaf = max_leaf;
      p.sub.pad_abs = pad_abs;
      p.sub.root = p.sub.build(r, depth);
      return;
    }
    p.inner = true;
    p.lb = L.bb;
    p.rb = R.bb;
    p.l = std::make_unique<Part>();
    p.r = std::make_unique<Part>();
    // the right half on a thread of its own while this one takes the left,
    // as long as it is large enough to be worth a thread
    std::thread right;
    std::exception_ptr right_err;
    if (n_threads > 1 && R.end - R.begin >= kThreadPrims) {
      try {
        right = std::thread([&] {
          try {
            split_part(*p.r, R, depth + 1);
          } catch (...) {
            right_err = std::current_exception();
          }
        });
      } catch (const std::system_error&) {
      }
    }
    try {
      split_part(*p.l, L, depth + 1);
    } catch (...) {
      if (right.joinable()) right.join();
      throw;
    }
    if (right.joinable()) {
      right.join();
      if (right_err) std::rethrow_exception(right_err);
    } else {
      split_part(*p.r, R, depth + 1);
    }
  }

  // Numbers nodes and triangles depth first, as one thread building the
  // whole tree would (a node before its left subtree, the left subtree
  // before the right one); lists the subtrees.
  void number(Part& p, int& n_nodes, int& n_tris, std::vector<Part*>& subs, int& n_leaves, int& max_depth) {
    max_depth = std::max(max_depth, p.depth);
    if (!p.inner) {
      p.node_base = n_nodes;
      p.tri_base = n_tris;
      n_nodes += (int)(p.sub.nodes.size() / 4);
      n_tris += (int)(p.sub.tris.size() / 3);
      n_leaves += p.sub.n_leaves;
      max_depth = std::max(max_depth, p.sub.max_depth);
      p.ref = reloc(p, p.sub.root);
      subs.push_back(&p);
      return;
    }
    p.node_base = n_nodes++;
    p.ref = p.node_base;
    number(*p.l, n_nodes, n_tris, subs, n_leaves, max_depth);
    number(*p.r, n_nodes, n_tris, subs, n_leaves, max_depth);
  }

  static int reloc(const Part& p, int c) {
    if (c >= 0) return c + p.node_base;
    unsigned u = ~(unsigned)c;
    return ~(int)((((u >> 3) + (unsigned)p.tri_base) << 3) | (u & 7u));
  }

  void write_inner(const Part& p, float4* nodes) {
    if (!p.inner) return;
    write_node(&nodes[4 * (size_t)p.node_base], p.lb, p.rb, p.l->ref, p.r->ref, pad_abs);
    write_inner(*p.l, nodes);
    write_inner(*p.r, nodes);
  }

  // Copies each subtree into its block with its indices offset
  static void place(Part& p, float4* nodes, float4* tris) {
    Subtree& s = p.sub;
    if (!s.nodes.empty()) {  // (a subtree that is one leaf has no nodes)
      float4* nd = nodes + 4 * (size_t)p.node_base;
      std::memcpy(nd, s.nodes.data(), s.nodes.size() * sizeof(float4));
      for (size_t i = 3; i < s.nodes.size(); i += 4) {
        int c0, c1;
        std::memcpy(&c0, &nd[i].x, 4);
        std::memcpy(&c1, &nd[i].y, 4);
        c0 = reloc(p, c0);
        c1 = reloc(p, c1);
        std::memcpy(&nd[i].x, &c0, 4);
        std::memcpy(&nd[i].y, &c1, 4);
      }
    }
    std::memcpy(tris + 3 * (size_t)p.tri_base, s.tris.data(), s.tris.size() * sizeof(float4));
    Float4Array().swap(s.nodes);
    Float4Array().swap(s.tris);
  }
};

// Collapse the binary tree into a 4-wide one: a 4-wide node takes a binary
// node's two children and keeps replacing its largest-area inner child by
// that child's two children until it has four (or only leaves remain).
struct Child {
  float lo[3], hi[3];
  int ref;
};

Child child_of(const Float4Array& bin, int b, int k) {
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

float child_area(const Child& c) {
  float d0 = c.hi[0] - c.lo[0], d1 = c.hi[1] - c.lo[1], d2 = c.hi[2] - c.lo[2];
  return d0 * d1 + d1 * d2 + d2 * d0;
}

// The children of the 4-wide node made from binary node b; returns how many
int expand(const Float4Array& bin, int b, Child ch[4]) {
  int n = 2;
  ch[0] = child_of(bin, b, 0);
  ch[1] = child_of(bin, b, 1);
  while (n < 4) {
    int best = -1;
    float best_area = -1.0f;
    for (int k = 0; k < n; ++k)
      if (ch[k].ref >= 0 && child_area(ch[k]) > best_area) {
        best = k;
        best_area = child_area(ch[k]);
      }
    if (best < 0) break;
    int bb = ch[best].ref;
    ch[best] = child_of(bin, bb, 0);
    ch[n++] = child_of(bin, bb, 1);
  }
  return n;
}

void write_node4(float4* nd, const Child ch[4], int n, const int refs[4]) {
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
}

// One thread's collapse of the subtree under one binary node, numbered from
// 0 depth first (a node, then its children's subtrees in slot order)
struct Collapser {
  const Float4Array* bin = nullptr;
  Float4Array out;
  int max_depth = 0;

  int collapse(int b, int depth) {
    max_depth = std::max(max_depth, depth);
    int idx = (int)(out.size() / kNode4Vecs);
    out.resize(out.size() + kNode4Vecs);
    Child ch[4];
    int n = expand(*bin, b, ch);
    int refs[4];
    for (int k = 0; k < 4; ++k) refs[k] = k < n ? (ch[k].ref >= 0 ? collapse(ch[k].ref, depth + 1) : ch[k].ref) : 0;
    write_node4(&out[kNode4Vecs * (size_t)idx], ch, n, refs);
    return idx;
  }
};

// The 4-wide tree's first levels, made on the calling thread; below them
// each subtree is collapsed by one thread and the blocks are numbered as one
// thread collapsing the whole tree would number them.
constexpr int kTopLevels4 = 4;

struct Part4 {
  bool inner = false;
  int depth = 0;
  // inner
  Child ch[4];
  int n = 0;
  std::unique_ptr<Part4> kid[4];  // null for leaf slots
  // subtree
  int b = 0;
  Collapser col;
  int root = 0;
  int node_base = 0, ref = 0;
};

void split4(const Float4Array& bin, Part4& p, int b, int depth, std::vector<Part4*>& subs) {
  p.depth = depth;
  p.b = b;
  if (depth >= kTopLevels4) {
    p.col.bin = &bin;
    subs.push_back(&p);
    return;
  }
  p.inner = true;
  p.n = expand(bin, b, p.ch);
  for (int k = 0; k < p.n; ++k)
    if (p.ch[k].ref >= 0) {
      p.kid[k] = std::make_unique<Part4>();
      split4(bin, *p.kid[k], p.ch[k].ref, depth + 1, subs);
    }
}

void number4(Part4& p, int& n_nodes, int& max_depth) {
  max_depth = std::max(max_depth, p.depth);
  p.node_base = n_nodes;
  p.ref = n_nodes;
  if (!p.inner) {
    n_nodes += (int)(p.col.out.size() / kNode4Vecs);
    max_depth = std::max(max_depth, p.col.max_depth);
    p.ref += p.root;
    return;
  }
  ++n_nodes;
  for (int k = 0; k < p.n; ++k)
    if (p.kid[k]) number4(*p.kid[k], n_nodes, max_depth);
}

void write4(const Part4& p, float4* out) {
  if (!p.inner) return;
  int refs[4];
  for (int k = 0; k < 4; ++k) refs[k] = k < p.n ? (p.kid[k] ? p.kid[k]->ref : p.ch[k].ref) : 0;
  write_node4(out + kNode4Vecs * (size_t)p.node_base, p.ch, p.n, refs);
  for (int k = 0; k < p.n; ++k)
    if (p.kid[k]) write4(*p.kid[k], out);
}

void place4(Part4& p, float4* out) {
  float4* nd = out + kNode4Vecs * (size_t)p.node_base;
  size_t len = p.col.out.size();
  std::memcpy(nd, p.col.out.data(), len * sizeof(float4));
  for (size_t i = kNode4Vecs - 1; i < len; i += kNode4Vecs) {
    int r[4];
    std::memcpy(r, &nd[i], 16);
    for (int k = 0; k < 4; ++k)
      if (r[k] > 0) r[k] += p.node_base;  // inner child (never the block's root, 0)
    std::memcpy(&nd[i], r, 16);
  }
  Float4Array().swap(p.col.out);
}

}  // namespace

BvhBuildResult build_bvh(const float* verts, int n, int max_leaf, int threads) {
  auto t0 = std::chrono::steady_clock::now();
  BvhBuildResult res;
  if (n <= 0) return res;
  Builder b;
  b.verts = verts;
  b.max_leaf = std::min(std::max(max_leaf, 1), kMaxLeaf);
  b.prims.resize(n);
  Range all{0, n, {}, {}};
  // threads only where there is enough work to pay for starting them
  unsigned want = threads > 0 ? (unsigned)threads : std::thread::hardware_concurrency();
  b.n_threads = n >= kThreadPrims ? std::max(1u, std::min(want, 64u)) : 1u;
  int chunks = chunk_count(n, b.n_threads);
  std::vector<AABB> finite(chunks);  // bounds of the finite coordinates
  run_parallel(chunks, chunks, [&](size_t c) {
    AABB fin;
    fin.reset();
    int e = (int)((int64_t)n * (int64_t)(c + 1) / chunks);
    for (int i = (int)((int64_t)n * (int64_t)c / chunks); i < e; ++i) {
      Prim& p = b.prims[i];
      const float* v = verts + 9 * (size_t)i;
      p.box.reset();
      for (int k = 0; k < 3; ++k) p.box.grow_pt(v + 3 * k);
      for (int k = 0; k < 3; ++k) p.c[k] = 0.5f * (p.box.lo[k] + p.box.hi[k]);
      p.tri = i;
      for (int k = 0; k < 9; ++k)
        if (std::isfinite(v[k])) {
          fin.lo[k % 3] = std::min(fin.lo[k % 3], v[k]);
          fin.hi[k % 3] = std::max(fin.hi[k % 3], v[k]);
        }
    }
    finite[c] = fin;
  });
  range_bounds(b.prims.data(), all, b.n_threads);
  // The absolute widening of every box scales with the scene's extent, over
  // its finite coordinates (a non-finite vertex must not shrink it to
  // nothing); an extent that overflows widens every box without limit,
  // which keeps the tree conservative.
  AABB fin;
  fin.reset();
  for (const AABB& f : finite) fin.grow(f);
  float ext = 0.0f;
  for (int k = 0; k < 3; ++k) ext = std::max(ext, fin.hi[k] - fin.lo[k]);
  if (!(ext <= FLT_MAX)) ext = FLT_MAX;
  b.pad_abs = ext * 2e-6f + 1e-30f;
  Part root;
  b.split_part(root, all, 0);
  int n_nodes = 0, n_tris = 0;
  std::vector<Part*> subs;
  b.number(root, n_nodes, n_tris, subs, res.n_leaves, res.depth);
  res.nodes.resize(4 * (size_t)n_nodes);
  res.tris.resize(3 * (size_t)n_tris);
  run_parallel(subs.size(), b.n_threads, [&](size_t k) { Builder::place(*subs[k], res.nodes.data(), res.tris.data()); });
  b.write_inner(root, res.nodes.data());
  res.root = root.ref;
  res.n_nodes = n_nodes;
  if (res.root >= 0) {
    Part4 top;
    std::vector<Part4*> subs4;
    split4(res.nodes, top, res.root, 0, subs4);
    run_parallel(subs4.size(), b.n_threads, [&](size_t k) { subs4[k]->root = subs4[k]->col.collapse(subs4[k]->b, subs4[k]->depth); });
    int n4 = 0;
    number4(top, n4, res.depth4);
    res.nodes4.resize(kNode4Vecs * (size_t)n4);
    run_parallel(subs4.size(), b.n_threads, [&](size_t k) { place4(*subs4[k], res.nodes4.data()); });
    write4(top, res.nodes4.data());
    res.root4 = top.ref;
  } else {
    res.root4 = res.root;
  }
  res.n_nodes4 = (int)(res.nodes4.size() / kNode4Vecs);
  res.ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  return res;
}

}  // namespace rtx
