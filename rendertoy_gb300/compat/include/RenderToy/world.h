// RenderToy/world.h — the scene container (RenderToy
// include/RenderToy/world.h:13-43).
#ifndef RTX_COMPAT_WORLD_H
#define RTX_COMPAT_WORLD_H
#include <vector>

#include "material.h"
#include "object.h"
#include "rtmath.h"

namespace RenderToy {
struct World {
  std::vector<Mesh*> meshes;
  std::vector<Triangle*> triangles;
  std::vector<Camera> cameras;
  std::vector<PrincipledBSDF*> materials;

  // Emissive triangles in mesh order, then each mesh's triangle order
  void PrepareDirectLightSampling();
  int CountEmitters() const;
  const std::vector<const Triangle*>& Emitters() const { return emissive_triangles; }

  Vector3f sky_emission;
  Vector3f ground_reflection;
  const Vector3f GetDefaultEmission(const Vector3f& back_dir) const;

 private:
  std::vector<const Triangle*> emissive_triangles;
};
}  // namespace RenderToy
#endif
