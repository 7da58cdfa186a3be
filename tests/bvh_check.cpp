// Checks the host thread pool, then builds the BVH of a triangle file (n x 9
// float32) with 1, 3 and 8 threads and checks each result: both trees
// (binary and 4-wide) hold every triangle exactly once, every child box
// contains its subtree's finite vertices, and the bits are the same for
// every thread count.  Prints one line:
//   "<hash> nodes <n> nodes4 <n> ok" or the first failure.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <vector>

#include "host_threads.h"
#include "rtx_internal.h"

using rtx::BvhBuildResult;

static uint64_t fnv(const void* p, size_t n, uint64_t h) {
  const unsigned char* b = static_cast<const unsigned char*>(p);
  for (size_t i = 0; i < n; ++i) {
    h ^= b[i];
    h *= 1099511628211ull;
  }
  return h;
}

static uint64_t hash_of(const BvhBuildResult& r) {
  uint64_t h = 1469598103934665603ull;
  h = fnv(r.nodes.data(), r.nodes.size() * 16, h);
  h = fnv(r.nodes4.data(), r.nodes4.size() * 16, h);
  h = fnv(r.tris.data(), r.tris.size() * 16, h);
  int meta[7] = {r.root, r.root4, r.n_nodes, r.n_nodes4, r.n_leaves, r.depth, r.depth4};
  return fnv(meta, sizeof meta, h);
}

struct Checker {
  const BvhBuildResult& r;
  const std::vector<float>& v;
  std::vector<int> seen;
  const char* err = nullptr;

  // marks a leaf's triangles; returns their finite vertex bounds in lo/hi
  void leaf(int ref, float lo[3], float hi[3]) {
    unsigned u = ~(unsigned)ref;
    int first = (int)(u >> 3), count = (int)(u & 7u) + 1;
    if (first < 0 || (size_t)(first + count) * 3 > r.tris.size()) {
      err = "leaf out of range";
      return;
    }
    for (int i = first; i < first + count; ++i) {
      int id;
      std::memcpy(&id, &r.tris[3 * (size_t)i].w, 4);
      if (id < 0 || (size_t)id >= seen.size()) {
        err = "bad triangle id";
        return;
      }
      seen[id]++;
      for (int k = 0; k < 9; ++k) {
        float x = v[9 * (size_t)id + k];
        if (std::isfinite(x)) {
          lo[k % 3] = std::fmin(lo[k % 3], x);
          hi[k % 3] = std::fmax(hi[k % 3], x);
        }
      }
    }
  }

  static bool covers(const float blo[3], const float bhi[3], const float lo[3], const float hi[3]) {
    for (int a = 0; a < 3; ++a)
      if (lo[a] <= hi[a] && !(blo[a] <= lo[a] && bhi[a] >= hi[a])) return false;
    return true;
  }

  void walk2(int ref, float lo[3], float hi[3], int depth = 0) {
    if (err) return;
    if (depth > 256) {
      err = "binary tree deeper than 256 levels (a cycle?)";
      return;
    }
    if (ref < 0) return leaf(ref, lo, hi);
    if ((size_t)ref * 4 + 4 > r.nodes.size()) {
      err = "binary node out of range";
      return;
    }
    const float4* n = &r.nodes[4 * (size_t)ref];
    float blo[2][3] = {{n[0].x, n[0].z, n[2].x}, {n[1].x, n[1].z, n[2].z}};
    float bhi[2][3] = {{n[0].y, n[0].w, n[2].y}, {n[1].y, n[1].w, n[2].w}};
    int c[2];
    std::memcpy(&c[0], &n[3].x, 4);
    std::memcpy(&c[1], &n[3].y, 4);
    for (int k = 0; k < 2; ++k) {
      float clo[3] = {INFINITY, INFINITY, INFINITY}, chi[3] = {-INFINITY, -INFINITY, -INFINITY};
      walk2(c[k], clo, chi, depth + 1);
      if (!err && !covers(blo[k], bhi[k], clo, chi)) err = "binary child box misses a vertex";
      for (int a = 0; a < 3; ++a) {
        lo[a] = std::fmin(lo[a], clo[a]);
        hi[a] = std::fmax(hi[a], chi[a]);
      }
    }
  }

  void walk4(int ref, float lo[3], float hi[3], int depth = 0) {
    if (err) return;
    if (depth > 256) {
      err = "4-wide tree deeper than 256 levels (a cycle?)";
      return;
    }
    if (ref < 0) return leaf(ref, lo, hi);
    if ((size_t)ref * rtx::kNode4Vecs + rtx::kNode4Vecs > r.nodes4.size()) {
      err = "4-wide node out of range";
      return;
    }
    const float4* n = &r.nodes4[rtx::kNode4Vecs * (size_t)ref];
    int c[4];
    std::memcpy(c, &n[6], 16);
    for (int k = 0; k < 4; ++k) {
      const float* f = reinterpret_cast<const float*>(n);
      float blo[3] = {f[0 * 4 + k], f[2 * 4 + k], f[4 * 4 + k]};
      float bhi[3] = {f[1 * 4 + k], f[3 * 4 + k], f[5 * 4 + k]};
      if (blo[0] == 1e30f) {  // unused slot
        if (c[k] != 0) err = "unused slot with a child";
        continue;
      }
      float clo[3] = {INFINITY, INFINITY, INFINITY}, chi[3] = {-INFINITY, -INFINITY, -INFINITY};
      walk4(c[k], clo, chi, depth + 1);
      if (!err && !covers(blo, bhi, clo, chi)) err = "4-wide child box misses a vertex";
      for (int a = 0; a < 3; ++a) {
        lo[a] = std::fmin(lo[a], clo[a]);
        hi[a] = std::fmax(hi[a], chi[a]);
      }
    }
  }

  const char* check() {
    int n = (int)(v.size() / 9);
    for (int pass = 0; pass < 2 && !err; ++pass) {
      seen.assign(n, 0);
      float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
      if (pass == 0)
        walk2(r.root, lo, hi);
      else
        walk4(r.root4, lo, hi);
      for (int i = 0; i < n && !err; ++i)
        if (seen[i] != 1) err = pass == 0 ? "binary tree: a triangle not held once" : "4-wide tree: a triangle not held once";
    }
    return err;
  }
};

// run_parallel (host_threads.h): every index runs once, and an exception on
// a worker reaches the caller after all threads have joined
static const char* check_pool() {
  std::vector<int> hits(1000, 0);
  rtx::run_parallel(hits.size(), 8, [&](size_t k) { hits[k]++; });
  for (int h : hits)
    if (h != 1) return "an index did not run exactly once";
  try {
    rtx::run_parallel(1000, 8, [&](size_t k) {
      if (k == 517) throw std::runtime_error("planted");
    });
  } catch (const std::runtime_error&) {
    return nullptr;
  }
  return "a worker's exception did not reach the caller";
}

int main(int argc, char** argv) {
  if (const char* e = check_pool()) {
    std::printf("fail %s\n", e);
    return 1;
  }
  if (argc < 3) return 2;
  FILE* f = std::fopen(argv[1], "rb");
  if (!f) return 2;
  std::fseek(f, 0, SEEK_END);
  long bytes = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  std::vector<float> v(bytes / 4);
  if (std::fread(v.data(), 4, v.size(), f) != v.size()) return 2;
  std::fclose(f);
  int leaf = std::atoi(argv[2]);
  int n = (int)(v.size() / 9);
  uint64_t h0 = 0;
  for (int threads : {1, 3, 8}) {
    BvhBuildResult r = rtx::build_bvh(v.data(), n, leaf, threads);
    uint64_t h = hash_of(r);
    if (threads == 1) {
      h0 = h;
      Checker c{r, v, {}};
      if (const char* e = c.check()) {
        std::printf("fail %s\n", e);
        return 1;
      }
    } else if (h != h0) {
      std::printf("fail %d threads give other bits\n", threads);
      return 1;
    }
    if (threads == 8) std::printf("%016llx nodes %d nodes4 %d ok\n", (unsigned long long)h, r.n_nodes, r.n_nodes4);
  }
  return 0;
}
