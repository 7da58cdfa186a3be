// intersect_exclude.cpp — BVH::Intersect through the RenderToy-compatible API
// with and without an excluded triangle.
//
// Two parallel unit quads (z = 1 and z = 2, two triangles each) and a ray
// along +z through them: the closest hit is a front triangle; excluding it
// gives the back triangle behind it; excluding a back triangle changes
// nothing.  Prints "ok" or the first mismatch.
#include <RenderToy/rendertoy.h>

#include <array>
#include <cstdio>

using namespace RenderToy;

int main() {
  World world;
  PrincipledBSDF white;
  Mesh* mesh = new Mesh();
  mesh->tex = &white;
  world.meshes.push_back(mesh);
  std::array<Vector2f, 3> uv = {Vector2f::O, Vector2f::O, Vector2f::O};
  std::array<Vector3f, 3> nn = {Vector3f(0, 0, -1), Vector3f(0, 0, -1), Vector3f(0, 0, -1)};
  for (float z : {1.0f, 2.0f}) {
    std::array<std::array<Vector3f, 3>, 2> quad = {
        std::array<Vector3f, 3>{Vector3f(-1, -1, z), Vector3f(1, -1, z), Vector3f(1, 1, z)},
        std::array<Vector3f, 3>{Vector3f(-1, -1, z), Vector3f(1, 1, z), Vector3f(-1, 1, z)}};
    for (auto& v : quad) {
      Triangle* t = new Triangle(v, nn, uv, mesh);
      world.triangles.push_back(t);
      mesh->tris.push_back(t);
    }
  }
  RenderContext rc(&world, FormatSettings(SizeN(4, 4), Vector2f(1.0f, 1.0f)));
  Ray ray(Vector3f(0.3f, -0.4f, 0.0f), Vector3f(0.0f, 0.0f, 1.0f));  // below the diagonal: triangles 0 and 2
  Vector3f pos;
  float t, u, v;
  const Triangle* a = rc.bvh->Intersect(ray, pos, t, u, v, nullptr);
  if (a != world.triangles[0] || !(t > 0.99f && t < 1.01f)) {
    std::printf("closest hit is not the front triangle\n");
    return 1;
  }
  const Triangle* b = rc.bvh->Intersect(ray, pos, t, u, v, world.triangles[0]);
  if (b != world.triangles[2] || !(t > 1.99f && t < 2.01f)) {
    std::printf("with the front triangle excluded the hit is not the back one\n");
    return 1;
  }
  const Triangle* c = rc.bvh->Intersect(ray, pos, t, u, v, world.triangles[3]);
  if (c != world.triangles[0]) {
    std::printf("excluding an unrelated triangle changed the hit\n");
    return 1;
  }
  std::printf("ok\n");
  return 0;
}
