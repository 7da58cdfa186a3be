/*
 * ref_harness.cpp — drives the REFERENCE's own compiled sources (RenderToy
 * src/*.cpp, built by oracle/build_ref.sh into oracle/_ref/) through the same
 * C API as the restatement in rt_oracle.cpp, with prefix ref_ instead of orc_.
 *
 * TEST INFRASTRUCTURE ONLY: used to generate and check the golden vectors in
 * tests/golden.  Only buildable where the RenderToy sources are present.
 *
 * Deterministic RNG: the link wraps RenderToy::Random::Float / Int
 * (src/rtmath.cpp:361-373) with the Philox stream below, keyed per path by a
 * thread-local (seed, pixel, sample) and a draw counter.
 *
 * Per-path driver: the primary ray of src/renderer.cpp:252-259 is rebuilt
 * here and PathTracingRenderer::Radiance (renderer.cpp:272) is called once per
 * (pixel, sample), serially per path, which avoids the shared-buffer race of
 * renderer.cpp:247-261.  The recursion cap is the build-time patched literal
 * of renderer.cpp:274 (see ref_depthcap.h).
 */
#include <malloc.h>

#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <functional>
#include <map>
#include <optional>
#include <queue>
#include <random>
#include <sstream>
#include <string>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

#define private public
#define protected public
#include <RenderToy/rendertoy.h>
#undef private
#undef protected

#include "ref_depthcap.h"

using namespace RenderToy;

int rtx_ref_depth_cap = 4;

namespace {

inline void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1) {
  for (int r = 0; r < 10; ++r) {
    uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
    uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    uint32_t n0 = hi1 ^ c[1] ^ k0;
    uint32_t n2 = hi0 ^ c[3] ^ k1;
    c[0] = n0;
    c[1] = lo1;
    c[2] = n2;
    c[3] = lo0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
}

struct PathKey {
  uint64_t seed = 0;
  uint32_t pixel = 0, sample = 0, draw = 0;
};
thread_local PathKey g_key;

uint32_t next_u32() {
  uint32_t c[4] = {g_key.draw >> 2, g_key.sample, g_key.pixel, 0u};
  philox4x32_10(c, (uint32_t)g_key.seed, (uint32_t)(g_key.seed >> 32));
  uint32_t w = c[g_key.draw & 3u];
  ++g_key.draw;
  return w;
}

struct Ctx;

struct RefScene {
  World world;
  std::vector<PrincipledBSDF*> mats;
  std::vector<Mesh*> meshes;
  std::map<const Triangle*, int> id;
  BVH* bvh = nullptr;
  // The RenderContext of the last per-path call, kept while the camera and
  // film stay the same: its constructor builds an octree (renderer.cpp:77-85),
  // which repeated calls need not pay again.
  Ctx* path_ctx = nullptr;
  std::vector<float> path_key;
  ~RefScene();
};

void destroy_scene_contents(RefScene* s) {
    delete s->bvh;
    for (auto t : s->world.triangles) delete t;
    for (auto m : s->meshes) delete m;
    for (auto m : s->mats) delete m;
}

Camera make_camera(const float* c) {
  Camera cam(Matrix4x4f::I, c[16], Vector2f(c[17], c[18]), c[19], c[20]);
  Matrix4x4f m;
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) m[i][j] = c[4 * i + j];
  cam.SetO2W(m);
  return cam;
}

struct Ctx {
  RenderContext* rc;
  Ctx(RefScene* s, const float* cam, int W, int H) {
    s->world.cameras.clear();
    s->world.cameras.push_back(make_camera(cam));
    rc = new RenderContext(&s->world, FormatSettings(SizeN(W, H), Vector2f(1.0f, 1.0f)));
  }
  ~Ctx() { delete rc; }
};

RefScene::~RefScene() {
  delete path_ctx;
  destroy_scene_contents(this);
}

// The cached per-path context for (camera, W, H), rebuilt when they change.
Ctx& path_context(RefScene* s, const float* cam, int W, int H) {
  std::vector<float> key(cam, cam + 21);
  key.push_back((float)W);
  key.push_back((float)H);
  if (!s->path_ctx || key != s->path_key) {
    delete s->path_ctx;
    s->path_ctx = new Ctx(s, cam, W, H);
    s->path_key = key;
  } else {
    // other calls may have installed their own camera in the shared World
    s->world.cameras.clear();
    s->world.cameras.push_back(make_camera(cam));
  }
  return *s->path_ctx;
}

Ray primary_ray(Renderer& r, int W, int H, int x, int y) {
  Camera* cam = &(r.render_context->world->cameras[r.render_context->camera_id]);
  float top, right;
  r.PrepareScreenSpace(cam, top, right);
  float dw = 1.0f / float(W);
  float dh = 1.0f / float(H);
  Vector2f ndc = {float(x) * dw, float(y) * dh};
  Vector2f sc = {2.0f * right * ndc.x() - right, 2.0f * top * ndc.y() - top};
  Ray ray(Vector3f::O, Vector3f(sc.x(), sc.y(), -1.0f));
  return cam->O2WTransform(ray);
}

int nthreads(int threads) {
#ifdef _OPENMP
  return threads > 0 ? threads : omp_get_max_threads();
#else
  (void)threads;
  return 1;
#endif
}

}  // namespace

extern "C" {

// --wrap targets: RenderToy::Random::Float() and RenderToy::Random::Int(int,int)
float __wrap__ZN9RenderToy6Random5FloatEv() {
  return (float)(next_u32() >> 8) * (1.0f / 16777216.0f);
}
int __wrap__ZN9RenderToy6Random3IntEii(int a, int b) {
  uint32_t n = (uint32_t)(b - a + 1);
  return a + (int)(((uint64_t)next_u32() * (uint64_t)n) >> 32);
}

void* ref_scene_create(int n_tris, const float* verts, const float* norms,
                       const int32_t* tri_mesh, int n_meshes,
                       const int32_t* mesh_mat, const uint8_t* mesh_smooth,
                       int n_mat, const float* mats, const float* sky,
                       const float* ground) {
  // Compositor taps may read one row past an image (compositor.h:25-39);
  // keep image buffers on the heap so that read stays inside mapped memory.
  mallopt(M_MMAP_THRESHOLD, 1 << 30);
  RefScene* s = new RefScene();
  for (int i = 0; i < n_mat; ++i) {
    const float* m = mats + 24 * (size_t)i;
    PrincipledBSDF* b = new PrincipledBSDF();
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
    s->mats.push_back(b);
  }
  for (int i = 0; i < n_meshes; ++i) {
    Mesh* me = new Mesh();
    me->tex = s->mats[mesh_mat[i]];
    me->smooth = mesh_smooth[i] != 0;
    s->meshes.push_back(me);
    s->world.meshes.push_back(me);
  }
  for (int i = 0; i < n_tris; ++i) {
    const float* p = verts + 9 * (size_t)i;
    std::array<Vector3f, 3> v = {Vector3f(p[0], p[1], p[2]), Vector3f(p[3], p[4], p[5]),
                                 Vector3f(p[6], p[7], p[8])};
    std::array<Vector3f, 3> n = {Vector3f::O, Vector3f::O, Vector3f::O};
    if (norms) {
      const float* q = norms + 9 * (size_t)i;
      n = {Vector3f(q[0], q[1], q[2]), Vector3f(q[3], q[4], q[5]), Vector3f(q[6], q[7], q[8])};
    }
    std::array<Vector2f, 3> uv = {Vector2f::O, Vector2f::O, Vector2f::O};
    Triangle* t = new Triangle(v, n, uv, s->meshes[tri_mesh[i]]);
    s->world.triangles.push_back(t);
    s->meshes[tri_mesh[i]]->tris.push_back(t);
    s->id[t] = i;
  }
  s->world.sky_emission = Vector3f(sky[0], sky[1], sky[2]);
  s->world.ground_reflection = Vector3f(ground[0], ground[1], ground[2]);
  s->world.PrepareDirectLightSampling();
  s->bvh = new BVH(s->world.triangles);
  return s;
}

void ref_scene_destroy(void* scene) { delete (RefScene*)scene; }

int ref_scene_emitters(void* scene, int32_t* out, int cap) {
  RefScene* s = (RefScene*)scene;
  int n = (int)s->world.emissive_triangles.size();
  for (int i = 0; i < n && i < cap; ++i) out[i] = s->id[s->world.emissive_triangles[i]];
  return n;
}

void ref_intersect(void* scene, int n, const float* rays, const int32_t* exclude,
                   int32_t* out_tri, float* out_tuv, int threads) {
  RefScene* s = (RefScene*)scene;
#pragma omp parallel for num_threads(nthreads(threads)) schedule(dynamic, 64)
  for (int i = 0; i < n; ++i) {
    const float* r = rays + 6 * (size_t)i;
    Ray ray(Vector3f(r[0], r[1], r[2]), Vector3f(r[3], r[4], r[5]));
    const Triangle* ex = (exclude && exclude[i] >= 0) ? s->world.triangles[exclude[i]] : nullptr;
    Vector3f pos;
    float t, u = 0.0f, v = 0.0f;
    const Triangle* h = s->bvh->Intersect(ray, pos, t, u, v, ex);
    out_tri[i] = h ? s->id.at(h) : -1;
    out_tuv[3 * i] = t;
    out_tuv[3 * i + 1] = h ? u : 0.0f;
    out_tuv[3 * i + 2] = h ? v : 0.0f;
  }
}

void ref_primary(void* scene, const float* cam, int W, int H, int32_t* out_tri,
                 float* out_tuv, int threads) {
  RefScene* s = (RefScene*)scene;
  Ctx c(s, cam, W, H);
  IntersectTestRenderer r(c.rc);
#pragma omp parallel for num_threads(nthreads(threads)) schedule(dynamic, 4)
  for (int y = 0; y < H; ++y)
    for (int x = 0; x < W; ++x) {
      Ray ray = primary_ray(r, W, H, x, y);
      Vector3f pos;
      float t, u = 0.0f, v = 0.0f;
      const Triangle* h = c.rc->bvh->Intersect(ray, pos, t, u, v, nullptr);
      size_t p = (size_t)y * W + x;
      out_tri[p] = h ? s->id.at(h) : -1;
      out_tuv[3 * p] = t;
      out_tuv[3 * p + 1] = h ? u : 0.0f;
      out_tuv[3 * p + 2] = h ? v : 0.0f;
    }
}

static void copy_buffer(const RenderContext* rc, int W, int H, float* out) {
  for (size_t p = 0; p < (size_t)W * H; ++p) {
    out[3 * p] = rc->buffer[p].x();
    out[3 * p + 1] = rc->buffer[p].y();
    out[3 * p + 2] = rc->buffer[p].z();
  }
}

void ref_render_aov(void* scene, const float* cam, int W, int H, float near_,
                    float far_, float* normal, float* albedo, float* depth,
                    int threads) {
  (void)threads;
  RefScene* s = (RefScene*)scene;
  Ctx c(s, cam, W, H);
  if (normal) {
    NormalRenderer r(c.rc);
    r.Render();
    copy_buffer(c.rc, W, H, normal);
  }
  if (albedo) {
    AlbedoRenderer r(c.rc);
    r.Render();
    copy_buffer(c.rc, W, H, albedo);
  }
  if (depth) {
    DepthBufferRenderer r(c.rc, near_, far_);
    r.Render();
    copy_buffer(c.rc, W, H, depth);
  }
}

void ref_trace_paths(void* scene, const float* cam, int W, int H,
                     const int32_t* pixels, int npix, int first_sample,
                     int n_samples, int max_depth, uint64_t seed, float* out,
                     int threads) {
  RefScene* s = (RefScene*)scene;
  Ctx& c = path_context(s, cam, W, H);
  PathTracingRenderer r(c.rc, 1);
  rtx_ref_depth_cap = max_depth - 1;
  if (!pixels) npix = W * H;
  long total = (long)npix * n_samples;
#pragma omp parallel for num_threads(nthreads(threads)) schedule(dynamic, 16)
  for (long q = 0; q < total; ++q) {
    int si = (int)(q / npix);
    int pi = (int)(q % npix);
    int pix = pixels ? pixels[pi] : pi;
    int x = pix % W, y = pix / W;
    Ray ray = primary_ray(r, W, H, x, y);
    g_key.seed = seed;
    g_key.pixel = (uint32_t)pix;
    g_key.sample = (uint32_t)(first_sample + si);
    g_key.draw = 0;
    RayState state;
    Vector3f L = r.Radiance(ray, nullptr, state, 0, 0.0f);
    out[3 * q] = L.x();
    out[3 * q + 1] = L.y();
    out[3 * q + 2] = L.z();
  }
}

// PathTracingRenderer::Render itself (src/renderer.cpp:236-270): RenderToy's
// own OpenMP renderer, unmodified, on the scene's RenderContext -- the loop
// over samples and pixels with its shared-buffer accumulation.  Used to time
// the reference against the restatement; its image is not deterministic
// (renderer.cpp:247-261 races), so only the timing is meaningful.  The
// wrapped Random draws one stream per thread here (no per-path key).  The
// recursion cap is the build's: 4 in libref_orig, `max_depth - 1` in libref.
// Returns the seconds spent inside Render(), timed with steady_clock.
double ref_render_pt(void* scene, const float* cam, int W, int H, int spp, int max_depth,
                     int threads, float* out) {
  RefScene* s = (RefScene*)scene;
  Ctx c(s, cam, W, H);
  rtx_ref_depth_cap = max_depth - 1;
#ifdef _OPENMP
  const int saved = omp_get_max_threads();
  omp_set_num_threads(nthreads(threads));
#endif
  PathTracingRenderer r(c.rc, spp);
  auto t0 = std::chrono::steady_clock::now();
  r.Render();
  double sec = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
#ifdef _OPENMP
  omp_set_num_threads(saved);
#endif
  if (out) copy_buffer(c.rc, W, H, out);
  return sec;
}

void ref_bsdf_eval(const float* mat, float eta, const float* N, const float* V,
                   const float* L, float* f_out, float* pdf_out) {
  PrincipledBSDF b;
  b.base_color = Vector3f(mat[0], mat[1], mat[2]);
  b.emission = Vector3f(mat[3], mat[4], mat[5]);
  b.roughness = mat[6];
  b.metallic = mat[7];
  b.anisotropic = mat[8];
  b.subsurface = mat[9];
  b.specular_tint = mat[10];
  b.sheen = mat[11];
  b.sheen_tint = mat[12];
  b.clearcoat = mat[13];
  b.clearcoat_roughness = mat[14];
  b.spec_trans = mat[15];
  b.ior = mat[16];
  b.at_distance = mat[17];
  b.extinction = Vector3f(mat[18], mat[19], mat[20]);
  RayState st;
  st.eta = eta;
  st.ffnormal = Vector3f(N[0], N[1], N[2]);
  float pdf;
  Vector3f f = b.Eval(st, Vector3f(V[0], V[1], V[2]), Vector3f(N[0], N[1], N[2]),
                      Vector3f(L[0], L[1], L[2]), pdf);
  f_out[0] = f.x();
  f_out[1] = f.y();
  f_out[2] = f.z();
  *pdf_out = pdf;
}

int ref_bsdf_sample(const float* mat, float eta, const float* N,
                    const float* in_dir, uint64_t seed, uint32_t pixel,
                    uint32_t sample, float* out_dir, float* color,
                    float* pdf_out) {
  PrincipledBSDF b;
  b.base_color = Vector3f(mat[0], mat[1], mat[2]);
  b.emission = Vector3f(mat[3], mat[4], mat[5]);
  b.roughness = mat[6];
  b.metallic = mat[7];
  b.anisotropic = mat[8];
  b.subsurface = mat[9];
  b.specular_tint = mat[10];
  b.sheen = mat[11];
  b.sheen_tint = mat[12];
  b.clearcoat = mat[13];
  b.clearcoat_roughness = mat[14];
  b.spec_trans = mat[15];
  b.ior = mat[16];
  b.at_distance = mat[17];
  b.extinction = Vector3f(mat[18], mat[19], mat[20]);
  RayState st;
  st.eta = eta;
  st.ffnormal = Vector3f(N[0], N[1], N[2]);
  g_key.seed = seed;
  g_key.pixel = pixel;
  g_key.sample = sample;
  g_key.draw = 0;
  Vector3f od, c;
  float pdf;
  bool ok = b.Sample(Vector3f(in_dir[0], in_dir[1], in_dir[2]), od, c, pdf, st);
  out_dir[0] = od.x();
  out_dir[1] = od.y();
  out_dir[2] = od.z();
  color[0] = c.x();
  color[1] = c.y();
  color[2] = c.z();
  *pdf_out = pdf;
  return ok ? 1 : 0;
}

static Image* make_image(const float* in, int W, int H) {
  mallopt(M_MMAP_THRESHOLD, 1 << 30);
  Image* img = new Image(SizeN(W, H));
  Vector3f* b = img->GetBuffer();
  for (size_t p = 0; p < (size_t)W * H; ++p) b[p] = Vector3f(in[3 * p], in[3 * p + 1], in[3 * p + 2]);
  return img;
}
static void read_image(Image* img, int W, int H, float* out) {
  Vector3f* b = img->GetBuffer();
  for (size_t p = 0; p < (size_t)W * H; ++p) {
    out[3 * p] = b[p].x();
    out[3 * p + 1] = b[p].y();
    out[3 * p + 2] = b[p].z();
  }
}

void ref_convolve(const float* in, float* out, int W, int H, const float* k,
                  int kr, int kc, int normalize, int lengthf, int absval) {
  Image* img = make_image(in, W, H);
  IConvolutionKernel<float> ker(kr, kc);
  for (int i = 0; i < kr; ++i)
    for (int j = 0; j < kc; ++j) ker.kernel_mat[i][j] = k[i * kc + j];
  int mode = (normalize ? 4 : 0) | (lengthf ? 2 : 0) | (absval ? 1 : 0);
  switch (mode) {
    case 0: img->Convolute<false, false, false>(ker); break;
    case 1: img->Convolute<false, false, true>(ker); break;
    case 2: img->Convolute<false, true, false>(ker); break;
    case 3: img->Convolute<false, true, true>(ker); break;
    case 4: img->Convolute<true, false, false>(ker); break;
    case 5: img->Convolute<true, false, true>(ker); break;
    case 6: img->Convolute<true, true, false>(ker); break;
    default: img->Convolute<true, true, true>(ker); break;
  }
  read_image(img, W, H, out);
  delete img;
}

void ref_gaussian_weights(int size, float sigma, float* out) {
  UnitizedGaussianKernel<float, Orientation::X> gk(size, sigma);
  for (int j = 0; j < size; ++j) out[j] = gk.kernel_mat[0][j];
}

void ref_gaussian_blur(const float* in, float* out, int W, int H, int size,
                       float sigma) {
  Image* img = make_image(in, W, H);
  img->GaussianBlur(size, sigma);
  read_image(img, W, H, out);
  delete img;
}

void ref_edge_detect(const float* in, float* out, int W, int H) {
  Image* img = make_image(in, W, H);
  img->EdgeDetection<Orientation::All>();
  read_image(img, W, H, out);
  delete img;
}

void ref_bloom(const float* in, float* out, int W, int H, int size, float sigma,
               float threshold) {
  Image* img = make_image(in, W, H);
  img->Bloom(size, sigma, threshold);
  read_image(img, W, H, out);
  delete img;
}

// OBJModelImporter::Import (+ MTLImporter::Import) into a World, read back
// as flat arrays: triangles in World::triangles order (vert_w after
// UpdateCache, normals, uvs, mesh index), meshes (name, smooth, Mesh::tris as
// triangle indices), materials (24-float records).
struct RefObj {
  World w;
  std::vector<int32_t> mesh_tris, mesh_counts;
};

void* ref_obj_import(const char* obj, const char* mtl) {
  RefObj* o = new RefObj();
  OBJModelImporter::Import(o->w, obj);
  if (mtl) MTLImporter::Import(o->w, mtl);
  std::map<const Triangle*, int> id;
  for (size_t i = 0; i < o->w.triangles.size(); ++i) id[o->w.triangles[i]] = (int)i;
  for (Mesh* m : o->w.meshes) {
    o->mesh_counts.push_back((int32_t)m->tris.size());
    for (const Triangle* t : m->tris) o->mesh_tris.push_back(id.at(t));
  }
  return o;
}

void ref_obj_counts(void* h, int* n_tris, int* n_meshes, int* n_mats) {
  RefObj* o = (RefObj*)h;
  *n_tris = (int)o->w.triangles.size();
  *n_meshes = (int)o->w.meshes.size();
  *n_mats = (int)o->w.materials.size();
}

void ref_obj_arrays(void* h, float* verts, float* norms, float* uvs, int32_t* tri_mesh, uint8_t* smooth,
                    int32_t* mesh_counts, int32_t* mesh_tris, float* mats) {
  RefObj* o = (RefObj*)h;
  std::map<const Mesh*, int> mid;
  for (size_t i = 0; i < o->w.meshes.size(); ++i) mid[o->w.meshes[i]] = (int)i;
  for (size_t i = 0; i < o->w.triangles.size(); ++i) {
    Triangle* t = o->w.triangles[i];
    t->UpdateCache();
    for (int k = 0; k < 3; ++k)
      for (int c = 0; c < 3; ++c) {
        verts[9 * i + 3 * k + c] = t->vert_w[k][c];
        norms[9 * i + 3 * k + c] = t->norm[k][c];
      }
    for (int k = 0; k < 3; ++k)
      for (int c = 0; c < 2; ++c) uvs[6 * i + 2 * k + c] = t->uv[k][c];
    tri_mesh[i] = mid.at(t->parent);
  }
  for (size_t m = 0; m < o->w.meshes.size(); ++m) smooth[m] = o->w.meshes[m]->smooth ? 1 : 0;
  std::memcpy(mesh_counts, o->mesh_counts.data(), o->mesh_counts.size() * 4);
  std::memcpy(mesh_tris, o->mesh_tris.data(), o->mesh_tris.size() * 4);
  for (size_t i = 0; i < o->w.materials.size(); ++i) {
    const PrincipledBSDF* b = o->w.materials[i];
    float* r = mats + 24 * i;
    const float v[24] = {b->base_color[0], b->base_color[1], b->base_color[2], b->emission[0], b->emission[1],
                         b->emission[2], b->roughness, b->metallic, b->anisotropic, b->subsurface,
                         b->specular_tint, b->sheen, b->sheen_tint, b->clearcoat, b->clearcoat_roughness,
                         b->spec_trans, b->ior, b->at_distance, b->extinction[0], b->extinction[1],
                         b->extinction[2], 0, 0, 0};
    std::memcpy(r, v, sizeof v);
  }
}

const char* ref_obj_mesh_name(void* h, int i) { return ((RefObj*)h)->w.meshes[i]->name.c_str(); }
const char* ref_obj_mat_name(void* h, int i) { return ((RefObj*)h)->w.materials[i]->name.c_str(); }
void ref_obj_free(void* h) { delete (RefObj*)h; }

// Image::Tonemap<kITURBT709>(limit) then Image::GammaCorrection(gamma) of a
// W x H image (limit <= 0 / gamma <= 0 skip the step)
void ref_tonemap_gamma(const float* in, int W, int H, float limit, float gamma, float* out) {
  Image img(SizeN((std::size_t)W, (std::size_t)H));
  Vector3f* b = img.GetBuffer();
  for (size_t i = 0; i < (size_t)W * H; ++i) b[i] = Vector3f(in[3 * i], in[3 * i + 1], in[3 * i + 2]);
  if (limit > 0.0f) img.Tonemap(limit);
  if (gamma > 0.0f) img.GammaCorrection(gamma);
  for (size_t i = 0; i < (size_t)W * H; ++i)
    for (int k = 0; k < 3; ++k) out[3 * i + k] = b[i][k];
}

// BMPExporter / PPMExporter output of a W x H image into out (cap bytes);
// returns the size.  (BMP only for W % 4 == 0: the reference writes its row
// padding from a null pointer.)
long ref_encode(int bmp, const float* in, int W, int H, uint8_t* out, long cap) {
  Image img(SizeN((std::size_t)W, (std::size_t)H));
  Vector3f* b = img.GetBuffer();
  for (size_t i = 0; i < (size_t)W * H; ++i) b[i] = Vector3f(in[3 * i], in[3 * i + 1], in[3 * i + 2]);
  std::ostringstream os;
  if (bmp) {
    if (W % 4) return -1;
    BMPExporter(img).Export(os);
  } else {
    PPMExporter(img).Export(os);
  }
  std::string s = os.str();
  if ((long)s.size() <= cap) std::memcpy(out, s.data(), s.size());
  return (long)s.size();
}

// ProceduralTexture samplers (src/procedural.cpp:8-46) at n points;
// PerlinNoise as constructed (its constructor never reseeds: siv's default
// permutation) with `scale` = param
void ref_texture_sample(int kind, float param, const uint8_t* perm, int n, const float* uv, float* out) {
  (void)perm;
  ProceduralTexture::CheckerBoard cb((int)param);
  ProceduralTexture::Wave wv(param);
  ProceduralTexture::PerlinNoise pn(0);
  pn.scale = param;
  for (int i = 0; i < n; ++i) {
    Vector2f p(uv[2 * i], uv[2 * i + 1]);
    out[i] = kind == 1 ? cb.Sample(p) : kind == 2 ? wv.Sample(p) : kind == 3 ? pn.Sample(p) : 1.0f;
  }
}

// the permutation a default-constructed ProceduralTexture::PerlinNoise uses
void ref_perlin_table(uint8_t* out) {
  ProceduralTexture::PerlinNoise pn(0);
  for (int i = 0; i < 256; ++i) out[i] = pn.perlin_noise_generator.m_permutation[i];
}

void ref_rng_floats(uint64_t seed, uint32_t pixel, uint32_t sample, int n,
                    float* out) {
  g_key.seed = seed;
  g_key.pixel = pixel;
  g_key.sample = sample;
  g_key.draw = 0;
  for (int i = 0; i < n; ++i) out[i] = Random::Float();
}

}  // extern "C"
