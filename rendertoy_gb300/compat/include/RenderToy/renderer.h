// RenderToy/renderer.h — RenderContext and the renderers (RenderToy
// include/RenderToy/renderer.h:14-135): same classes, members and
// constructors.  Render() runs on the GPU through librtx (include/rtx.h).
//
// RenderContext uploads the world (flattened triangles, materials, emitters)
// when it is constructed, where RenderToy builds its BVH; if the materials or
// the emitter list differ at Render() time the scene is uploaded again.
// Failures of the GPU library raise Exception::DeviceException.
#ifndef RTX_COMPAT_RENDERER_H
#define RTX_COMPAT_RENDERER_H
#include <cstdint>
#include <ostream>

#include "bvh.h"
#include "rtmath.h"
#include "world.h"

struct rtx_context;

namespace RenderToy {
enum class RenderTech { kTest = 0, kIntersectTest, kDepthBuffer, kNormal, kPathTracing, kAlbedo, kLineEdge };
enum class ProjectionMode { kPerspective = 0, kParallel };

struct FormatSettings {
  SizeN resolution = SizeN(1920, 1080);
  Vector2f aspect = Vector2f(1.0f, 1.0f);
  FormatSettings() = default;
  FormatSettings(SizeN resolution_, Vector2f aspect_);
};

struct RenderContext {
  World* world;
  BVH* bvh;  // the world as uploaded to the GPU
  Vector3f* buffer;
  FormatSettings format_settings;
  int camera_id = 0;

  RenderContext(World* world_, FormatSettings format_settings_);
  ~RenderContext();
  Vector3f& operator()(const std::size_t x, const std::size_t y);
  const Vector3f& operator()(const std::size_t x, const std::size_t y) const;
};

class Renderer {
 protected:
  void PrepareScreenSpace(Camera* cam, float& top, float& right);

 public:
  RenderContext* render_context;
  Renderer() = delete;
  Renderer(const Renderer&) = delete;
  Renderer(const Renderer&&) = delete;
  Renderer(RenderContext* render_context_);
  virtual ~Renderer() = default;
  virtual void Render() = 0;
};

class TestRenderer : public Renderer {
 public:
  TestRenderer(const SizeN& resolution_);
  virtual void Render() override final;
};

class IntersectTestRenderer : public Renderer {
 public:
  IntersectTestRenderer(RenderContext* render_context_);
  virtual void Render() override final;
};

class DepthBufferRenderer : public Renderer {
 public:
  float near, far;
  DepthBufferRenderer(RenderContext* render_context_);
  DepthBufferRenderer(RenderContext* render_context_, float near_, float far_);
  virtual void Render() override final;
};

class NormalRenderer : public Renderer {
 public:
  NormalRenderer(RenderContext* render_context_);
  virtual void Render() override final;
};

// Adds the mean of iteration_count samples per pixel to the buffer, as
// RenderToy's does.  max_depth (shaded vertices per path; RenderToy fixes 5)
// and seed (of the counter-based random stream) are additions.
class PathTracingRenderer : public Renderer {
  int iteration_count;

 public:
  int max_depth = 5;
  uint64_t seed = 0;
  PathTracingRenderer(RenderContext* render_context_, const int iteration_count_);
  virtual void Render() override final;
};

class AlbedoRenderer : public Renderer {
 public:
  AlbedoRenderer(RenderContext* render_context_);
  virtual void Render() override final;
};
}  // namespace RenderToy
#endif
