// RenderToy/bvh.h — BVH is the GPU-resident scene of a RenderContext (in
// RenderToy, include/RenderToy/bvh.h:74-86, the CPU octree).  It owns one
// librtx context; Intersect traces rays on the GPU.
#ifndef RTX_COMPAT_BVH_H
#define RTX_COMPAT_BVH_H
#include <cstdint>
#include <unordered_map>
#include <vector>

#include "ray.h"
#include "rtmath.h"

struct rtx_context;

namespace RenderToy {
class Triangle;
struct World;

struct BoundingBox {
  Vector3f vmin, vmax;
  BoundingBox() : vmin(Vector3f::O), vmax(Vector3f::O) {}
  BoundingBox(const Vector3f& a, const Vector3f& b) : vmin(a), vmax(b) {}
};

class BVH {
 public:
  // Uploads the world's triangles (World::triangles order), materials and
  // emitters.
  explicit BVH(World* world);
  BVH(const BVH&) = delete;
  ~BVH();
  // Closest hit of one ray (BVH::Intersect): the triangle or nullptr.
  const Triangle* Intersect(const Ray& ray, Vector3f& position, float& t, float& u, float& v,
                            const Triangle* const exclude) const;
  rtx_context* Device() const { return ctx; }
  // Re-upload when the world's materials or emitters changed
  void Refresh();

 private:
  friend struct RenderContext;
  World* world;
  rtx_context* ctx = nullptr;
  // materials, mesh table, emitters and environment as uploaded: float bits
  // and emitter addresses, compared exactly
  std::vector<uint64_t> snapshot;
  // World::triangles index of each triangle, made on the first Intersect
  // that excludes one (instead of a search of the whole list per call)
  mutable std::unordered_map<const Triangle*, int32_t> tri_ids;
  void Upload();
  std::vector<uint64_t> Signature() const;
};
}  // namespace RenderToy
#endif
