// rendertoy_compat.cpp — the RenderToy-compatible C++ API over librtx.
//
// Host arithmetic (transforms, triangle caches, camera film extents, the
// black-body colour) keeps RenderToy's operation order; build with
// -ffp-contract=off.  Each function names the RenderToy function whose
// behaviour it keeps (paths relative to the RenderToy source tree).
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <unordered_map>
#include <mutex>
#include <random>
#include <string>

#include "../../../include/rtx.h"
#include "RenderToy/rendertoy.h"

namespace RenderToy {

namespace {

void check(int code, rtx_context* ctx, const char* what) {
  if (code != RTX_OK) {
    std::string m = std::string(what) + ": " + (ctx ? rtx_last_error(ctx) : "no GPU context");
    throw Exception::DeviceException(code, m);
  }
}

int device_index() {
  const char* e = std::getenv("RTX_DEVICE");
  return e ? std::atoi(e) : 0;
}

rtx_context* new_context() {
  rtx_context* c = nullptr;
  int r = rtx_create(&c, device_index());
  if (r != RTX_OK) throw Exception::DeviceException(r, "rtx_create: no usable CUDA device");
  return c;
}

// Context for the Image filters, created on first use
rtx_context* image_context() {
  static std::once_flag once;
  static rtx_context* ctx = nullptr;
  std::call_once(once, [] {
    ctx = new_context();
    std::atexit([] { rtx_destroy(ctx); });
  });
  return ctx;
}

void camera_record(const Camera& cam, float* out) {
  const Matrix4x4f& m = cam.GetO2W();
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) out[4 * i + j] = m[i][j];
  out[16] = cam.focal_length;
  out[17] = cam.gate_dimension.x();
  out[18] = cam.gate_dimension.y();
  out[19] = cam.near_clipping_plane;
  out[20] = cam.far_clipping_plane;
}

}  // namespace

// ---- rtmath ------------------------------------------------------------------
PointN::PointN() : x(0), y(0) {}
PointN::PointN(int x_, int y_) : x(x_), y(y_) {}
PointN::PointN(const Vector2f& v) : x(int(v.x())), y(int(v.y())) {}
PointN::PointN(const std::array<int, 2>& t) : x(t[0]), y(t[1]) {}
PointN PointN::operator+(const PointN& p) const { return PointN(x + p.x, y + p.y); }
void PointN::SizeClamp(const SizeN& s) {
  x = std::clamp(x, 0, static_cast<int>(s.width));
  y = std::clamp(y, 0, static_cast<int>(s.height));
}
SizeN::SizeN() : width(0), height(0) {}
SizeN::SizeN(std::size_t w, std::size_t h) : width(w), height(h) {}
SizeN::SizeN(const Vector2f& v) : width(std::size_t(v.x())), height(std::size_t(v.y())) {}
SizeN::SizeN(const std::array<std::size_t, 2>& t) : width(t[0]), height(t[1]) {}
std::size_t SizeN::Area() const { return width * height; }
float SizeN::AspectRatio() const { return float(width) / float(height); }
PointN SizeN::Center() const { return PointN(static_cast<int>(width) >> 1, static_cast<int>(height) >> 1); }
bool SizeN::operator==(const SizeN& a) const { return width == a.width && height == a.height; }
bool SizeN::operator!=(const SizeN& a) const { return !(*this == a); }

namespace Convert {
// CIE XYZ -> linear sRGB (D65), the matrix published by B. Lindbloom
Vector3f XYZToSRGB(const Vector3f& x) {
  const Matrix3x3f m(Vector3f(3.2404542f, -1.5371385f, -0.4985314f),
                     Vector3f(-0.9692660f, 1.8760108f, 0.0415560f),
                     Vector3f(0.0556434f, -0.2040259f, 1.0572252f));
  return m * x;
}
// Krystek's rational approximation of the Planckian locus in CIE 1960 (u, v),
// evaluated in double and narrowed to float at the same points as RenderToy's
// Convert::BlackBody (src/rtmath.cpp:34-56)
Vector3f BlackBody(const float t) {
  float tt = t * t;
  float u = (0.860117757 + 1.54118254e-4 * t + 1.28641212e-7 * tt) /
            (1.0 + 8.42420235e-4 * t + 7.08145163e-7 * tt);
  float v = (0.317398726 + 4.22806245e-5 * t + 4.20481691e-8 * tt) /
            (1.0 - 2.89741816e-5 * t + 1.61456053e-7 * tt);
  Vector2f xy = Vector2f(3.0f * u, 2.0f * v) / (float)(2.0 * u - 8.0 * v + 4.0);
  Vector3f xyz(xy.x() / xy.y(), 1.0f, (1.0f - xy.x() - xy.y()) / xy.y());
  Vector3f rgb = XYZToSRGB(xyz);
  return rgb / std::max(rgb.x(), std::max(rgb.y(), rgb.z()));
}
}  // namespace Convert

namespace AffineTransformation {
Matrix4x4f Translation(const Vector3f& o) {
  Matrix4x4f r(Matrix4x4f::I);
  for (int i = 0; i < 3; ++i) r[i][3] = o[i];
  return r;
}
// src/rtmath.cpp:144-167: Z * Y * X
Matrix4x4f RotationEulerXYZ(const Vector3f& e) {
  float x = e.x(), y = e.y(), z = e.z();
  Matrix4x4f Z(Vector4f(std::cos(z), -std::sin(z), 0.0f, 0.0f), Vector4f(std::sin(z), std::cos(z), 0.0f, 0.0f),
               Vector4f(0.0f, 0.0f, 1.0f, 0.0f), Vector4f(0.0f, 0.0f, 0.0f, 1.0f));
  Matrix4x4f Y(Vector4f(std::cos(y), 0.0f, -std::sin(y), 0.0f), Vector4f(0.0f, 1.0f, 0.0f, 0.0f),
               Vector4f(std::sin(y), 0.0f, std::cos(y), 0.0f), Vector4f(0.0f, 0.0f, 0.0f, 1.0f));
  Matrix4x4f X(Vector4f(1.0f, 0.0f, 0.0f, 0.0f), Vector4f(0.0f, std::cos(x), -std::sin(x), 0.0f),
               Vector4f(0.0f, std::sin(x), std::cos(x), 0.0f), Vector4f(0.0f, 0.0f, 0.0f, 1.0f));
  return Z * Y * X;
}
}  // namespace AffineTransformation

namespace Random {
static thread_local std::mt19937 engine;
int Int(int min, int max) { return std::uniform_int_distribution<>(min, max)(engine); }
float Float() { return std::uniform_real_distribution<float>(0.0f, 1.0f)(engine); }
}  // namespace Random

// ---- material ------------------------------------------------------------------
PrincipledBSDF::PrincipledBSDF(const Vector3f& base_color_, const Vector3f& emission_,
                               const float roughness_, const float metallic_, const float spec_trans_,
                               const float ior_, const float anisotropic_, const float subsurface_,
                               const float specular_tint_, const float sheen_, const float sheen_tint_,
                               const float clearcoat_, const float clearcoat_roughness_,
                               const float at_distance_, const Vector3f& extinction_)
    : base_color(base_color_), emission(emission_), roughness(roughness_), metallic(metallic_),
      anisotropic(anisotropic_), subsurface(subsurface_), specular_tint(specular_tint_), sheen(sheen_),
      sheen_tint(sheen_tint_), clearcoat(clearcoat_), clearcoat_roughness(clearcoat_roughness_),
      spec_trans(spec_trans_), ior(ior_), at_distance(at_distance_), extinction(extinction_) {
  if (roughness < 0.001f) roughness = 0.001f;  // src/material.cpp:29-32
}

void PrincipledBSDF::ToRecord(float* m) const {
  std::memset(m, 0, RTX_MATERIAL_FLOATS * sizeof(float));
  for (int k = 0; k < 3; ++k) {
    m[k] = base_color[k];
    m[3 + k] = emission[k];
    m[18 + k] = extinction[k];
  }
  m[6] = roughness;
  m[7] = metallic;
  m[8] = anisotropic;
  m[9] = subsurface;
  m[10] = specular_tint;
  m[11] = sheen;
  m[12] = sheen_tint;
  m[13] = clearcoat;
  m[14] = clearcoat_roughness;
  m[15] = spec_trans;
  m[16] = ior;
  m[17] = at_distance;
}

// ---- objects (src/object.cpp) -------------------------------------------------
Geometry::Geometry() : object_to_world(Matrix4x4f::I), world_to_object(Matrix4x4f::I) {}
void Geometry::SetO2W(const Matrix4x4f& m) {
  object_to_world = m;
  // inverse of a rigid transform: R^T and -R^T c
  Matrix3x3f R = m.ComplementMinor(3, 3).Transposed();
  Vector3f C = {m[0][3], m[1][3], m[2][3]};
  C = (-1.0f) * (R * C);
  world_to_object = Matrix4x4f::O;
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 3; ++j) world_to_object[i][j] = R[i][j];
    world_to_object[i][3] = C[i];
  }
  world_to_object[3][3] = 1.0f;
}
const Matrix4x4f& Geometry::GetO2W() const { return object_to_world; }
const Matrix4x4f& Geometry::GetW2O() const { return world_to_object; }
const Vector3f Geometry::O2WTransform(const Vector3f& v) const {
  Vector4f p = object_to_world * Vector4f(v.x(), v.y(), v.z(), 1.0f);
  return Vector3f(p[0], p[1], p[2]);
}
const Vector3f Geometry::W2OTransform(const Vector3f& v) const {
  Vector4f p = world_to_object * Vector4f(v.x(), v.y(), v.z(), 1.0f);
  return Vector3f(p[0], p[1], p[2]);
}
const Ray Geometry::O2WTransform(const Ray& r) const {
  Ray o(O2WTransform(r.src), O2WTransform(r.direction));
  o.direction -= o.src;
  o.direction.Normalize();
  return o;
}
const Ray Geometry::W2OTransform(const Ray& r) const {
  Ray o(W2OTransform(r.src), W2OTransform(r.direction));
  o.direction -= o.src;
  o.direction.Normalize();
  return o;
}

Camera::Camera(Matrix4x4f, float f, Vector2f g, float n, float fa)
    : focal_length(f), gate_dimension(g), near_clipping_plane(n), far_clipping_plane(fa) {
  Geometry::SetO2W(object_to_world);
}

Triangle::Triangle(const std::array<Vector3f, 3>& v, const std::array<Vector3f, 3>& n,
                   const std::array<Vector2f, 3>& t, Mesh* const p)
    : vert(v), norm(n), uv(t), parent(p), vert_w(v) {
  UpdateCache();
}
// src/object.cpp:224-243
void Triangle::UpdateCache() {
  for (int i = 0; i < 3; ++i) vert_w[i] = parent ? parent->O2WTransform(vert[i]) : vert[i];
  v0v1_w = vert_w[1] - vert_w[0];
  v0v2_w = vert_w[2] - vert_w[0];
  area = v0v1_w.Cross(v0v2_w).Length() * 0.5f;
  normal = v0v1_w.Normalized().Cross(vert_w[2] - vert_w[1]).Normalized();
}
const float Triangle::AreaC() const { return area; }
const Vector3f Triangle::GeometricalNormalC() const { return normal; }
const Vector3f Triangle::NormalC(const float u, const float v) const {
  if (parent && parent->smooth) return ((1 - u - v) * norm[0] + u * norm[1] + v * norm[2]).Normalized();
  return normal;
}

void Mesh::SetO2W(const Matrix4x4f& m) {
  Geometry::SetO2W(m);
  for (auto t : tris) t->UpdateCache();
}

// ---- world (src/world.cpp) -------------------------------------------------------
void World::PrepareDirectLightSampling() {
  emissive_triangles.clear();
  for (auto m : meshes)
    if (m->tex && m->tex->emission != Vector3f::O)
      for (auto t : m->tris) emissive_triangles.push_back(t);
}
int World::CountEmitters() const { return (int)emissive_triangles.size(); }
const Vector3f World::GetDefaultEmission(const Vector3f& back_dir) const {
  return (back_dir[2] < 0.0f) ? sky_emission : ground_reflection;
}

// ---- BVH: the world on the GPU ------------------------------------------------------
BVH::BVH(World* w) : world(w) {
  ctx = new_context();
  try {
    Upload();
  } catch (...) {
    rtx_destroy(ctx);
    throw;
  }
}
BVH::~BVH() { rtx_destroy(ctx); }

std::vector<uint64_t> BVH::Signature() const {
  // exact: a float by its bits (a NaN field equals itself), an emitter by
  // its full address (a float of an address would merge nearby ones)
  std::vector<uint64_t> s;
  auto put = [&](float f) {
    uint32_t b;
    std::memcpy(&b, &f, 4);
    s.push_back(b);
  };
  float rec[RTX_MATERIAL_FLOATS];
  for (auto m : world->meshes) {
    if (m->tex) {
      m->tex->ToRecord(rec);
      for (float f : rec) put(f);
    }
    s.push_back(m->smooth ? 1 : 0);
  }
  for (auto t : world->Emitters()) s.push_back((uint64_t)(uintptr_t)t);
  for (int k = 0; k < 3; ++k) {
    put(world->sky_emission[k]);
    put(world->ground_reflection[k]);
  }
  return s;
}

void BVH::Upload() {
  tri_ids.clear();
  const auto& tris = world->triangles;
  int n = (int)tris.size();
  std::unordered_map<const Mesh*, int> mesh_id;
  std::vector<const Mesh*> meshes;
  for (auto m : world->meshes)
    if (!mesh_id.count(m)) {
      mesh_id[m] = (int)meshes.size();
      meshes.push_back(m);
    }
  std::vector<float> verts((size_t)n * 9), norms((size_t)n * 9);
  std::vector<int32_t> tri_mesh(n);
  // ids are looked up only for the emitters
  std::unordered_map<const Triangle*, int> tri_id;
  for (auto t : world->Emitters()) tri_id.emplace(t, -1);
  const Mesh* last = nullptr;
  int last_id = -1;
  for (int i = 0; i < n; ++i) {
    const Triangle* t = tris[i];
    if (!t->parent) throw Exception::DeviceException(RTX_ERR_INVALID, "triangle without a parent mesh");
    if (t->parent != last) {  // a mesh's triangles usually come together
      auto it = mesh_id.find(t->parent);
      if (it == mesh_id.end()) {
        it = mesh_id.emplace(t->parent, (int)meshes.size()).first;
        meshes.push_back(t->parent);
      }
      last = t->parent;
      last_id = it->second;
    }
    tri_mesh[i] = last_id;
    if (!tri_id.empty()) {
      auto it = tri_id.find(t);
      if (it != tri_id.end() && it->second < 0) it->second = i;
    }
    for (int k = 0; k < 3; ++k)
      for (int c = 0; c < 3; ++c) {
        verts[9 * (size_t)i + 3 * k + c] = t->WorldVertex(k)[c];
        norms[9 * (size_t)i + 3 * k + c] = t->norm[k][c];
      }
  }
  std::map<const PrincipledBSDF*, int> mat_id;
  std::vector<float> mats;
  std::vector<int32_t> mesh_mat(meshes.size());
  std::vector<uint8_t> mesh_smooth(meshes.size());
  for (size_t m = 0; m < meshes.size(); ++m) {
    const PrincipledBSDF* b = meshes[m]->tex;
    if (!b) throw Exception::DeviceException(RTX_ERR_INVALID, "mesh without a material (Mesh::tex)");
    if (!mat_id.count(b)) {
      mat_id[b] = (int)(mats.size() / RTX_MATERIAL_FLOATS);
      mats.resize(mats.size() + RTX_MATERIAL_FLOATS);
      b->ToRecord(&mats[mats.size() - RTX_MATERIAL_FLOATS]);
    }
    mesh_mat[m] = mat_id[b];
    mesh_smooth[m] = meshes[m]->smooth ? 1 : 0;
  }
  float sky[3] = {world->sky_emission[0], world->sky_emission[1], world->sky_emission[2]};
  float ground[3] = {world->ground_reflection[0], world->ground_reflection[1], world->ground_reflection[2]};
  check(rtx_scene_upload(ctx, n, verts.data(), norms.data(), tri_mesh.data(), (int)meshes.size(),
                         mesh_mat.data(), mesh_smooth.data(), (int)(mats.size() / RTX_MATERIAL_FLOATS),
                         mats.data(), sky, ground),
        ctx, "rtx_scene_upload");
  // the emitter list is the world's own (empty unless PrepareDirectLightSampling ran)
  std::vector<int32_t> em;
  for (auto t : world->Emitters()) {
    auto it = tri_id.find(t);
    if (it == tri_id.end() || it->second < 0)
      throw Exception::DeviceException(RTX_ERR_INVALID, "emitter triangle missing from World::triangles");
    em.push_back(it->second);
  }
  check(rtx_scene_set_emitters(ctx, em.data(), (int)em.size()), ctx, "rtx_scene_set_emitters");
  snapshot = Signature();
}

void BVH::Refresh() {
  if (Signature() != snapshot) Upload();
}

const Triangle* BVH::Intersect(const Ray& ray, Vector3f& position, float& t, float& u, float& v,
                               const Triangle* const exclude) const {
  float r[6] = {ray.src[0], ray.src[1], ray.src[2], ray.direction[0], ray.direction[1], ray.direction[2]};
  int32_t ex = -1;
  if (exclude) {
    const auto& tris = world->triangles;
    if (tri_ids.empty()) {  // emptied by each upload
      tri_ids.reserve(tris.size());
      for (size_t i = 0; i < tris.size(); ++i) tri_ids[tris[i]] = (int32_t)i;  // the last of repeats, as before
    }
    auto it = tri_ids.find(exclude);
    if (it != tri_ids.end()) ex = it->second;
  }
  int32_t tri = -1;
  float tuv[3];
  check(rtx_intersect(ctx, 1, r, &ex, &tri, tuv), ctx, "rtx_intersect");
  t = tuv[0];
  if (tri < 0) return nullptr;
  u = tuv[1];
  v = tuv[2];
  position = ray.src + t * ray.direction;
  return world->triangles[tri];
}

// ---- renderers (src/renderer.cpp) -------------------------------------------------------
FormatSettings::FormatSettings(SizeN r, Vector2f a) : resolution(r), aspect(a) {}

RenderContext::RenderContext(World* w, FormatSettings f) : world(w), bvh(nullptr), format_settings(f) {
  if (world) bvh = new BVH(world);
  buffer = new Vector3f[format_settings.resolution.Area()];
}
RenderContext::~RenderContext() {
  delete[] buffer;
  delete bvh;
}
Vector3f& RenderContext::operator()(const std::size_t x, const std::size_t y) {
  return buffer[y * format_settings.resolution.width + x];
}
const Vector3f& RenderContext::operator()(const std::size_t x, const std::size_t y) const {
  return buffer[y * format_settings.resolution.width + x];
}

Renderer::Renderer(RenderContext* rc) : render_context(rc) {}

// src/renderer.cpp:103-124
void Renderer::PrepareScreenSpace(Camera* cam, float& top, float& right) {
  top = (Convert::InchToMM(cam->gate_dimension.y()) / 2.0f) / cam->focal_length;
  right = (Convert::InchToMM(cam->gate_dimension.x()) / 2.0f) / cam->focal_length;
  float gate_aspr = cam->gate_dimension.x() / cam->gate_dimension.y();
  float film_aspr = render_context->format_settings.resolution.AspectRatio();
  float xscale = 1.0f, yscale = 1.0f;
  if (gate_aspr >= film_aspr)
    xscale = film_aspr / gate_aspr;
  else
    yscale = gate_aspr / film_aspr;
  right *= xscale;
  top *= yscale;
}

namespace {
struct Frame {
  rtx_context* ctx;
  float cam[RTX_CAMERA_FLOATS];
  int W, H;
};
Frame frame_of(RenderContext* rc) {
  if (!rc->world || !rc->bvh) throw Exception::DeviceException(RTX_ERR_NO_SCENE, "render context without a world");
  rc->bvh->Refresh();
  Frame f;
  f.ctx = rc->bvh->Device();
  camera_record(rc->world->cameras.at(rc->camera_id), f.cam);
  f.W = (int)rc->format_settings.resolution.width;
  f.H = (int)rc->format_settings.resolution.height;
  return f;
}
}  // namespace

TestRenderer::TestRenderer(const SizeN& r) : Renderer(new RenderContext(nullptr, FormatSettings(r, Vector2f::O))) {}
void TestRenderer::Render() {
  auto& r = render_context->format_settings.resolution;
  for (std::size_t y = 0; y < r.height; ++y)
    for (std::size_t x = 0; x < r.width; ++x)
      render_context->buffer[y * r.width + x] = Vector3f(float(x) / float(r.width), 1.0f, 1.0f);
}

IntersectTestRenderer::IntersectTestRenderer(RenderContext* rc) : Renderer(rc) {}
void IntersectTestRenderer::Render() {
  Frame f = frame_of(render_context);
  std::vector<int32_t> tri((size_t)f.W * f.H);
  std::vector<float> tuv((size_t)f.W * f.H * 3);
  check(rtx_primary_hits(f.ctx, f.cam, f.W, f.H, tri.data(), tuv.data()), f.ctx, "rtx_primary_hits");
  for (size_t p = 0; p < tri.size(); ++p) render_context->buffer[p] = tri[p] >= 0 ? Vector3f::White : Vector3f::O;
}

DepthBufferRenderer::DepthBufferRenderer(RenderContext* rc) : Renderer(rc) {
  near = rc->world->cameras[rc->camera_id].near_clipping_plane;
  far = rc->world->cameras[rc->camera_id].far_clipping_plane;
}
DepthBufferRenderer::DepthBufferRenderer(RenderContext* rc, float n, float f) : Renderer(rc), near(n), far(f) {}
void DepthBufferRenderer::Render() {
  Frame f = frame_of(render_context);
  check(rtx_render_aov(f.ctx, f.cam, f.W, f.H, near, far, nullptr, nullptr, (float*)render_context->buffer),
        f.ctx, "rtx_render_aov");
}

NormalRenderer::NormalRenderer(RenderContext* rc) : Renderer(rc) {}
void NormalRenderer::Render() {
  Frame f = frame_of(render_context);
  check(rtx_render_aov(f.ctx, f.cam, f.W, f.H, 0.0f, 1.0f, (float*)render_context->buffer, nullptr, nullptr),
        f.ctx, "rtx_render_aov");
}

AlbedoRenderer::AlbedoRenderer(RenderContext* rc) : Renderer(rc) {}
void AlbedoRenderer::Render() {
  Frame f = frame_of(render_context);
  check(rtx_render_aov(f.ctx, f.cam, f.W, f.H, 0.0f, 1.0f, nullptr, (float*)render_context->buffer, nullptr),
        f.ctx, "rtx_render_aov");
}

PathTracingRenderer::PathTracingRenderer(RenderContext* rc, const int n) : Renderer(rc), iteration_count(n) {}
void PathTracingRenderer::Render() {
  if (iteration_count <= 0) return;
  Frame f = frame_of(render_context);
  check(rtx_set_option(f.ctx, RTX_OPT_ACCUMULATE, 1), f.ctx, "rtx_set_option");
  int r = rtx_render_pt(f.ctx, f.cam, f.W, f.H, iteration_count, max_depth, seed,
                        (float*)render_context->buffer);
  rtx_set_option(f.ctx, RTX_OPT_ACCUMULATE, 0);
  check(r, f.ctx, "rtx_render_pt");
}

// ---- Image (src/compositor.cpp, include/RenderToy/compositor.h) -------------------------
Image::Image(const SizeN& r) : resolution(r) { buffer = new Vector3f[resolution.Area()]; }
Image::Image(const RenderContext* const rc) : resolution(rc->format_settings.resolution) {
  buffer = new Vector3f[resolution.Area()];
  std::memcpy((void*)buffer, (const void*)rc->buffer, resolution.Area() * sizeof(Vector3f));
}
Image::Image(const Image& o) : resolution(o.resolution) {
  buffer = new Vector3f[resolution.Area()];
  std::memcpy((void*)buffer, (const void*)o.buffer, resolution.Area() * sizeof(Vector3f));
}
Image::~Image() { delete[] buffer; }
Vector3f& Image::operator()(const std::size_t x, const std::size_t y) { return buffer[y * resolution.width + x]; }
const Vector3f& Image::operator()(const std::size_t x, const std::size_t y) const {
  return buffer[y * resolution.width + x];
}
Vector3f*& Image::GetBuffer() { return buffer; }
const Vector3f* const& Image::GetBuffer() const { return buffer; }

const Image Image::Extract(const std::function<bool(const Vector3f&)>& f, const Vector3f& d) {
  Image r(resolution);
  for (std::size_t i = 0; i < resolution.Area(); ++i) r.buffer[i] = f(buffer[i]) ? buffer[i] : d;
  return r;
}
const void Image::Transform(const std::function<void(Vector3f&)>& f) {
  for (std::size_t i = 0; i < resolution.Area(); ++i) f(buffer[i]);
}

void Image::Convolve(const IConvolutionKernel<float>& k, bool normalize, bool length, bool absval) {
  const auto& m = k.kernel_mat;
  std::vector<float> w(m.row * m.column);
  for (std::size_t i = 0; i < m.row; ++i)
    for (std::size_t j = 0; j < m.column; ++j) w[i * m.column + j] = m[i][j];
  rtx_context* c = image_context();
  check(rtx_image_convolve(c, (const float*)buffer, (float*)buffer, (int)resolution.width,
                           (int)resolution.height, w.data(), (int)m.row, (int)m.column, normalize, length,
                           absval),
        c, "rtx_image_convolve");
}
Image& Image::GaussianBlur(const std::size_t size, const float sigma) {
  rtx_context* c = image_context();
  check(rtx_image_gaussian_blur(c, (const float*)buffer, (float*)buffer, (int)resolution.width,
                                (int)resolution.height, (int)size, sigma),
        c, "rtx_image_gaussian_blur");
  return *this;
}
void Image::EdgeDetectionAll() {
  rtx_context* c = image_context();
  check(rtx_image_edge_detect(c, (const float*)buffer, (float*)buffer, (int)resolution.width,
                              (int)resolution.height),
        c, "rtx_image_edge_detect");
}
Image& Image::Bloom(const std::size_t size, const float sigma, const float threshold) {
  rtx_context* c = image_context();
  check(rtx_image_bloom(c, (const float*)buffer, (float*)buffer, (int)resolution.width,
                        (int)resolution.height, (int)size, sigma, threshold),
        c, "rtx_image_bloom");
  return *this;
}
Image& Image::GammaCorrection(const float gamma) {
  rtx_context* c = image_context();
  check(rtx_image_gamma(c, (const float*)buffer, (float*)buffer, (int)resolution.width, (int)resolution.height,
                        gamma),
        c, "rtx_image_gamma");
  return *this;
}

// ---- files --------------------------------------------------------------------------
void PPMExporter::Export(std::ostream& os) {
  rtx_context* c = image_context();
  int W = (int)image.resolution.width, H = (int)image.resolution.height;
  const float* px = (const float*)&image(0, 0);
  size_t n = 0;
  check(rtx_encode_ppm(c, px, W, H, nullptr, 0, &n), c, "rtx_encode_ppm");
  std::vector<char> buf(n);
  check(rtx_encode_ppm(c, px, W, H, buf.data(), n, &n), c, "rtx_encode_ppm");
  os.write(buf.data(), (std::streamsize)n);
}

void BMPExporter::Export(std::ostream& os) {
  rtx_context* c = image_context();
  int W = (int)image.resolution.width, H = (int)image.resolution.height;
  const float* px = (const float*)&image(0, 0);
  size_t n = 0;
  check(rtx_encode_bmp(c, px, W, H, nullptr, 0, &n), c, "rtx_encode_bmp");
  std::vector<uint8_t> buf(n);
  check(rtx_encode_bmp(c, px, W, H, buf.data(), n, &n), c, "rtx_encode_bmp");
  os.write((const char*)buf.data(), (std::streamsize)n);
}

// ---- import -------------------------------------------------------------------------
void OBJModelImporter::Import(World& world, const std::string& path) {
  rtx_obj* o = nullptr;
  char msg[512] = {0};
  int r = rtx_obj_import(path.c_str(), nullptr, &o, msg, sizeof msg);
  if (r != RTX_OK) throw Exception::DeviceException(r, std::string("OBJ import: ") + msg);
  int nt = 0, nm = 0;
  rtx_obj_info(o, &nt, &nm, nullptr);
  std::vector<float> v((size_t)nt * 9), n((size_t)nt * 9), t((size_t)nt * 6);
  std::vector<int32_t> tm((size_t)nt);
  rtx_obj_triangles(o, v.data(), n.data(), t.data(), tm.data());
  std::vector<Mesh*> meshes;
  for (int m = 0; m < nm; ++m) {
    const char* name = nullptr;
    uint8_t sm = 0;
    rtx_obj_mesh(o, m, &name, &sm, nullptr, nullptr);
    Mesh* mesh = new Mesh();
    mesh->name = name;
    mesh->smooth = sm != 0;
    meshes.push_back(mesh);
  }
  size_t base = world.triangles.size();
  for (int i = 0; i < nt; ++i) {
    const float* p = &v[9 * (size_t)i];
    const float* q = &n[9 * (size_t)i];
    const float* w = &t[6 * (size_t)i];
    Triangle* tri = new Triangle({Vector3f(p[0], p[1], p[2]), Vector3f(p[3], p[4], p[5]), Vector3f(p[6], p[7], p[8])},
                                 {Vector3f(q[0], q[1], q[2]), Vector3f(q[3], q[4], q[5]), Vector3f(q[6], q[7], q[8])},
                                 {Vector2f(w[0], w[1]), Vector2f(w[2], w[3]), Vector2f(w[4], w[5])}, meshes[tm[i]]);
    world.triangles.push_back(tri);
  }
  for (int m = 0; m < nm; ++m) {
    int k = 0;
    rtx_obj_mesh(o, m, nullptr, nullptr, nullptr, &k);
    std::vector<int32_t> ids((size_t)k);
    rtx_obj_mesh(o, m, nullptr, nullptr, ids.data(), &k);
    for (int32_t id : ids) meshes[m]->tris.push_back(world.triangles[base + id]);
    world.meshes.push_back(meshes[m]);
  }
  rtx_obj_free(o);
}

void MTLImporter::Import(World& world, const std::string& path) {
  rtx_obj* o = nullptr;
  char msg[512] = {0};
  int r = rtx_obj_import(nullptr, path.c_str(), &o, msg, sizeof msg);
  if (r != RTX_OK) throw Exception::DeviceException(r, std::string("MTL import: ") + msg);
  int nmat = 0;
  rtx_obj_info(o, nullptr, nullptr, &nmat);
  for (int i = 0; i < nmat; ++i) {
    const char* name = nullptr;
    float m[24];
    rtx_obj_material(o, i, &name, m);
    PrincipledBSDF* b = new PrincipledBSDF();
    b->name = name;
    b->base_color = Vector3f(m[0], m[1], m[2]);
    b->emission = Vector3f(m[3], m[4], m[5]);
    b->roughness = m[6];
    b->metallic = m[7];
    b->anisotropic = m[8];
    b->subsurface = m[9];
    b->specular_tint = m[10];
    b->sheen = m[11];
    b->sheen_tint = m[12];
    b->clearcoat = m[13];
    b->clearcoat_roughness = m[14];
    b->spec_trans = m[15];
    b->ior = m[16];
    b->at_distance = m[17];
    b->extinction = Vector3f(m[18], m[19], m[20]);
    world.materials.push_back(b);
  }
  rtx_obj_free(o);
}

#define RTX_IMAGE_OP(op, name)                                                        \
  const Image Image::operator op(const Image& img) {                                  \
    if (resolution != img.resolution)                                                 \
      throw Exception::ImageSizeNotMatchException(                                    \
          "The " name " operator of two images requires two images have the same resolution."); \
    Image r(resolution);                                                              \
    for (std::size_t i = 0; i < resolution.Area(); ++i) r.buffer[i] = buffer[i] op img.buffer[i]; \
    return r;                                                                         \
  }
RTX_IMAGE_OP(+, "+")
RTX_IMAGE_OP(-, "-")
RTX_IMAGE_OP(*, "*")
RTX_IMAGE_OP(/, "/")
#undef RTX_IMAGE_OP

const void Image::operator=(const Image& img) {
  if (resolution != img.resolution)
    throw Exception::ImageSizeNotMatchException(
        "The = operator of two images requires two images have the same resolution.");
  std::memcpy((void*)buffer, (const void*)img.buffer, resolution.Area() * sizeof(Vector3f));
}

// Line and rectangle drawing (src/compositor.cpp:176-259): integer stepping
// along the major axis with an error term, clamped to the image.
void Image::DrawLine(PointN p1, PointN p2, const Vector3f& color) {
  p1.SizeClamp(resolution);
  p2.SizeClamp(resolution);
  const bool flat = std::abs(p2.y - p1.y) < std::abs(p2.x - p1.x);
  if (flat ? p1.x > p2.x : p1.y > p2.y) std::swap(p1, p2);
  int major0 = flat ? p1.x : p1.y, major1 = flat ? p2.x : p2.y;
  int minor = flat ? p1.y : p1.x;
  int dminor = flat ? p2.y - p1.y : p2.x - p1.x;
  int step = dminor < 0 ? -1 : 1;
  dminor = std::abs(dminor);
  int dmajor = major1 - major0;
  int err = 0;
  for (int i = major0; i < major1; ++i) {
    if (err > dmajor) {
      minor += step;
      err -= 2 * dmajor;
    }
    if (flat)
      buffer[minor * resolution.width + i] = color;
    else
      buffer[i * resolution.width + minor] = color;
    err += 2 * dminor;
  }
}
void Image::Fill(PointN p1, PointN p2, const Vector3f& color) {
  p1.SizeClamp(resolution);
  p2.SizeClamp(resolution);
  if (p1.x > p2.x) std::swap(p1.x, p2.x);
  if (p1.y > p2.y) std::swap(p1.y, p2.y);
  for (int i = p1.x; i < p2.x; ++i)
    for (int j = p1.y; j < p2.y; ++j) buffer[j * resolution.width + i] = color;
}

}  // namespace RenderToy
