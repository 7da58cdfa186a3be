// RenderToy/material.h — PrincipledBSDF parameters (RenderToy
// include/RenderToy/material.h:12-77): same fields, defaults and constructor
// (roughness clamped to at least 0.001).  Evaluation and sampling run on the
// GPU inside the renderers; the struct is the material record they read.
#ifndef RTX_COMPAT_MATERIAL_H
#define RTX_COMPAT_MATERIAL_H
#include <string>

#include "ray.h"
#include "rtmath.h"

namespace RenderToy {
struct PrincipledBSDF {
  std::string name = "unnamed";
  Vector3f base_color = Vector3f::White;
  Vector3f emission = Vector3f::O;
  float roughness = 0.5f;
  float metallic = 0.0f;
  float anisotropic = 0.0f;
  float subsurface = 0.0f;
  float specular_tint = 0.0f;
  float sheen = 0.0f;
  float sheen_tint = 0.5f;
  float clearcoat = 0.0f;
  float clearcoat_roughness = 0.03f;
  float spec_trans = 0.0f;
  float ior = 1.45f;
  float at_distance = 1.0f;
  Vector3f extinction = Vector3f::White;

  PrincipledBSDF() = default;
  PrincipledBSDF(const Vector3f& base_color_, const Vector3f& emission_ = Vector3f::O,
                 const float roughness_ = 0.5f, const float metallic_ = 0.0f,
                 const float spec_trans_ = 0.0f, const float ior_ = 1.45f,
                 const float anisotropic_ = 0.0f, const float subsurface_ = 0.0f,
                 const float specular_tint_ = 0.0f, const float sheen_ = 0.0f,
                 const float sheen_tint_ = 0.0f, const float clearcoat_ = 0.0f,
                 const float clearcoat_roughness_ = 0.0f, const float at_distance_ = 1.0f,
                 const Vector3f& extinction_ = Vector3f::White);

  // The 24-float record of the C ABI (include/rtx.h)
  void ToRecord(float* out) const;
};

struct ITexture {
  virtual void Sample(const float u, const float v) const = 0;
};
}  // namespace RenderToy
#endif
