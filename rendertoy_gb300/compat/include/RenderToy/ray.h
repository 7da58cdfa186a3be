// RenderToy/ray.h — Ray and RayState (RenderToy include/RenderToy/ray.h:9-30).
#ifndef RTX_COMPAT_RAY_H
#define RTX_COMPAT_RAY_H
#include "rtmath.h"

namespace RenderToy {
struct Ray {
  Ray() = delete;
  Ray(Vector3f src_, Vector3f normalized_direction_) : src(src_), direction(normalized_direction_) {}
  Vector3f src;
  Vector3f direction;
  const Ray operator-(const Ray& ray) { return Ray(src, -direction); }
};

struct RayState {
  float eta;
  Vector3f absorption;
  Vector3f ffnormal;
};
}  // namespace RenderToy
#endif
