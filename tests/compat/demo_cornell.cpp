// demo_cornell.cpp — a RenderToy application used as a drop-in test.
//
// The same source is compiled against RenderToy's own headers and sources
// (tests/golden/make_golden.py, for the golden outputs) and against the
// GB300 library's RenderToy-compatible headers (tests/test_compat.py).  It
// builds a World through the RenderToy API from a scene file, places the
// camera with SetO2W, runs the renderers and filters, and writes every buffer.
//
//   demo_cornell <scene.bin> <out.bin> <W> <H> <spp>
//
// scene.bin: int32 n_tris, n_meshes, n_mats; float32 verts[n*9], norms[n*9];
//            int32 tri_mesh[n], mesh_mat[m]; uint8 smooth[m]; float32
//            mats[k*24]; float32 camera[21]
// out.bin:   int32 W, H, count; then count images of W*H*3 float32
#include <RenderToy/rendertoy.h>

#include <array>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <vector>

using namespace RenderToy;

template <typename T>
static std::vector<T> read_n(FILE* f, size_t n) {
  std::vector<T> v(n);
  if (n && fread(v.data(), sizeof(T), n, f) != n) {
    fprintf(stderr, "short read\n");
    exit(2);
  }
  return v;
}

static void dump(FILE* f, const Vector3f* buf, size_t n) { fwrite(buf, sizeof(Vector3f), n, f); }

int main(int argc, char** argv) {
  if (argc < 6) {
    fprintf(stderr, "usage: %s scene.bin out.bin W H spp\n", argv[0]);
    return 1;
  }
  FILE* f = fopen(argv[1], "rb");
  if (!f) return 1;
  auto hdr = read_n<int32_t>(f, 3);
  int n = hdr[0], nm = hdr[1], nk = hdr[2];
  auto verts = read_n<float>(f, (size_t)n * 9);
  auto norms = read_n<float>(f, (size_t)n * 9);
  auto tri_mesh = read_n<int32_t>(f, n);
  auto mesh_mat = read_n<int32_t>(f, nm);
  auto smooth = read_n<uint8_t>(f, nm);
  auto mats = read_n<float>(f, (size_t)nk * 24);
  auto cam = read_n<float>(f, 21);
  fclose(f);
  int W = atoi(argv[3]), H = atoi(argv[4]), spp = atoi(argv[5]);

  World world;
  std::vector<PrincipledBSDF> bsdf(nk);
  for (int k = 0; k < nk; ++k) {
    const float* m = &mats[24 * (size_t)k];
    PrincipledBSDF b(Vector3f(m[0], m[1], m[2]), Vector3f(m[3], m[4], m[5]), m[6], m[7], m[15], m[16],
                     m[8], m[9], m[10], m[11], m[12], m[13], m[14], m[17], Vector3f(m[18], m[19], m[20]));
    bsdf[k] = b;
  }
  for (int i = 0; i < nm; ++i) {
    Mesh* mesh = new Mesh();
    mesh->tex = &bsdf[mesh_mat[i]];
    mesh->smooth = smooth[i] != 0;
    world.meshes.push_back(mesh);
  }
  for (int i = 0; i < n; ++i) {
    const float* p = &verts[9 * (size_t)i];
    const float* q = &norms[9 * (size_t)i];
    std::array<Vector3f, 3> v = {Vector3f(p[0], p[1], p[2]), Vector3f(p[3], p[4], p[5]), Vector3f(p[6], p[7], p[8])};
    std::array<Vector3f, 3> nn = {Vector3f(q[0], q[1], q[2]), Vector3f(q[3], q[4], q[5]), Vector3f(q[6], q[7], q[8])};
    std::array<Vector2f, 3> uv = {Vector2f::O, Vector2f::O, Vector2f::O};
    Mesh* mesh = world.meshes[tri_mesh[i]];
    Triangle* t = new Triangle(v, nn, uv, mesh);
    world.triangles.push_back(t);
    mesh->tris.push_back(t);
  }
  // move the first mesh with an affine transform, as an application would
  world.meshes[0]->SetO2W(AffineTransformation::Translation({0.0f, -2.0f, 0.0f}) *
                          AffineTransformation::RotationEulerXYZ({0.0f, Convert::DegreeToRadians(1), 0.0f}));
  world.PrepareDirectLightSampling();

  world.cameras.push_back(academy_format);
  Matrix4x4f m;
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) m[i][j] = cam[4 * i + j];
  world.cameras[0].SetO2W(m);
  world.cameras[0].focal_length = cam[16];
  world.cameras[0].gate_dimension = Vector2f(cam[17], cam[18]);

  RenderContext rc(&world, FormatSettings(SizeN(W, H), Vector2f(1.0f, 1.0f)));
  const size_t npix = (size_t)W * H;
  std::vector<std::vector<Vector3f>> out;
  auto keep = [&](const Vector3f* b) { out.emplace_back(b, b + npix); };

  NormalRenderer normal(&rc);
  normal.Render();
  keep(rc.buffer);
  Image nimg(&rc);
  AlbedoRenderer albedo(&rc);
  albedo.Render();
  keep(rc.buffer);
  DepthBufferRenderer depth(&rc, cam[19], cam[20]);
  depth.Render();
  keep(rc.buffer);
  IntersectTestRenderer hits(&rc);
  hits.Render();
  keep(rc.buffer);

  Image blur(nimg);
  blur.GaussianBlur(7, 1.5f);
  keep(blur.GetBuffer());
  Image edge(nimg);
  edge.EdgeDetection<Orientation::All>();
  keep(edge.GetBuffer());
  Image sob(nimg);
  sob.EdgeDetection<Orientation::X>();
  keep(sob.GetBuffer());
  Image bloom(nimg);
  bloom.Bloom(9, 2.0f, 0.5f);
  keep(bloom.GetBuffer());
  Image lap(nimg);
  UnitizedGaussianKernel<float> g3(5, 1.0f);
  lap.Convolute<false, false, true>(g3);
  keep(lap.GetBuffer());

  for (size_t p = 0; p < npix; ++p) rc.buffer[p] = Vector3f::O;
  PathTracingRenderer pt(&rc, spp);
  pt.Render();
  keep(rc.buffer);
  Image tm(&rc);
  tm.Tonemap();
  tm.GammaCorrection();
  keep(tm.GetBuffer());

  FILE* o = fopen(argv[2], "wb");
  int32_t h[3] = {W, H, (int32_t)out.size()};
  fwrite(h, 4, 3, o);
  for (auto& b : out) dump(o, b.data(), npix);
  fclose(o);
  printf("demo_cornell: %d triangles, %d emitters, %zu buffers\n", n, world.CountEmitters(), out.size());
  return 0;
}
