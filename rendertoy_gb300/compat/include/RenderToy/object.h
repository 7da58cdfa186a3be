// RenderToy/object.h — Geometry, Camera, Triangle, Mesh (RenderToy
// include/RenderToy/object.h:27-214): same public members and methods.
#ifndef RTX_COMPAT_OBJECT_H
#define RTX_COMPAT_OBJECT_H
#include <array>
#include <string>
#include <vector>

#include "material.h"
#include "ray.h"
#include "rtmath.h"

namespace RenderToy {
class Mesh;
struct BoundingBox;

class Geometry {
 protected:
  Matrix4x4f object_to_world;
  Matrix4x4f world_to_object;

 public:
  std::string name;
  Geometry();
  virtual ~Geometry() = default;
  virtual void SetO2W(const Matrix4x4f& object_to_world_);
  const Matrix4x4f& GetO2W() const;
  const Matrix4x4f& GetW2O() const;
  const Vector3f O2WTransform(const Vector3f& vec) const;
  const Vector3f W2OTransform(const Vector3f& vec) const;
  const Ray O2WTransform(const Ray& ray) const;
  const Ray W2OTransform(const Ray& ray) const;
};

class Camera : public Geometry {
 public:
  float focal_length;       // mm
  Vector2f gate_dimension;  // inches
  float near_clipping_plane;
  float far_clipping_plane;
  // As in RenderToy (src/object.cpp:74-81) the matrix argument is not applied:
  // the camera starts at the identity and is placed with SetO2W.
  Camera(Matrix4x4f object_to_world_, float focal_length_, Vector2f gate_dimension_,
         float near_clipping_plane_, float far_clipping_plane_);
};

static const Camera academy_format = Camera(Matrix4x4f::I, 35.0f, Vector2f(0.868f, 0.631f), 0.1f, 1000.0f);
static const Camera imax_hd = Camera(Matrix4x4f::I, 65.0f, Vector2f(2.772f, 2.072f), 0.1f, 1000.0f);
static const Camera maxivision = Camera(Matrix4x4f::I, 35.0f, Vector2f(0.980f, 0.546f), 0.1f, 1000.0f);

class Triangle {
 public:
  std::array<Vector3f, 3> vert;
  std::array<Vector3f, 3> norm;
  std::array<Vector2f, 3> uv;
  Mesh* parent;

  Triangle(const std::array<Vector3f, 3>& vert_, const std::array<Vector3f, 3>& norm_,
           const std::array<Vector2f, 3>& uv_, Mesh* const parent_);
  const float AreaC() const;
  const Vector3f NormalC(const float u, const float v) const;
  const Vector3f GeometricalNormalC() const;
  // Recompute the world-space vertices after the parent's O2W changed
  void UpdateCache();
  // World-space vertex i (Triangle::vert_w)
  const Vector3f& WorldVertex(int i) const { return vert_w[i]; }

 private:
  std::array<Vector3f, 3> vert_w;
  Vector3f v0v1_w, v0v2_w;
  float area;
  Vector3f normal;
};

class Mesh : public Geometry {
 public:
  std::vector<Triangle*> tris;
  PrincipledBSDF* tex = nullptr;
  bool smooth{false};
  virtual void SetO2W(const Matrix4x4f& object_to_world_) override;
};
}  // namespace RenderToy
#endif
