// demo_obj.cpp — a RenderToy application that loads its scene from OBJ / MTL
// files, used as a drop-in test of the importers and exporters.  Compiled
// against RenderToy's own sources (tests/golden/make_golden.py) and, unchanged,
// against the GB300 library's RenderToy-compatible headers (tests/test_compat.py).
//
//   demo_obj <scene.obj> <scene.mtl> <camera.bin> <out_prefix> <W> <H> <spp>
//
// Each mesh gets the material whose name equals the mesh name (RenderToy's
// importer ignores usemtl).  Writes <out_prefix>.bin (int32 W, H, count; then
// count W*H*3 float32 images: normal, albedo, depth, pt, pt tonemapped +
// gamma) and the normal pass as <out_prefix>_normal.bmp / .ppm.
#include <RenderToy/rendertoy.h>

#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <string>
#include <vector>

using namespace RenderToy;

int main(int argc, char** argv) {
  if (argc < 8) {
    fprintf(stderr, "usage: %s scene.obj scene.mtl camera.bin out_prefix W H spp\n", argv[0]);
    return 1;
  }
  World world;
  OBJModelImporter::Import(world, argv[1]);
  MTLImporter::Import(world, argv[2]);
  for (Mesh* m : world.meshes)
    for (PrincipledBSDF* b : world.materials)
      if (b->name == m->name) m->tex = b;
  world.PrepareDirectLightSampling();

  float cam[21];
  FILE* f = fopen(argv[3], "rb");
  if (!f || fread(cam, 4, 21, f) != 21) return 2;
  fclose(f);
  world.cameras.push_back(academy_format);
  Matrix4x4f m;
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) m[i][j] = cam[4 * i + j];
  world.cameras[0].SetO2W(m);
  world.cameras[0].focal_length = cam[16];
  world.cameras[0].gate_dimension = Vector2f(cam[17], cam[18]);

  int W = atoi(argv[5]), H = atoi(argv[6]), spp = atoi(argv[7]);
  RenderContext rc(&world, FormatSettings(SizeN(W, H), Vector2f(1.0f, 1.0f)));
  const size_t npix = (size_t)W * H;
  std::vector<std::vector<Vector3f>> out;
  auto keep = [&](const Vector3f* b) { out.emplace_back(b, b + npix); };

  NormalRenderer normal(&rc);
  normal.Render();
  keep(rc.buffer);
  Image nimg(&rc);
  std::string prefix = argv[4];
  {
    std::ofstream bmp(prefix + "_normal.bmp", std::ios::binary);
    BMPExporter(nimg).Export(bmp);
    std::ofstream ppm(prefix + "_normal.ppm", std::ios::binary);
    PPMExporter(nimg).Export(ppm);
  }
  AlbedoRenderer albedo(&rc);
  albedo.Render();
  keep(rc.buffer);
  DepthBufferRenderer depth(&rc, cam[19], cam[20]);
  depth.Render();
  keep(rc.buffer);
  for (size_t p = 0; p < npix; ++p) rc.buffer[p] = Vector3f::O;
  PathTracingRenderer pt(&rc, spp);
  pt.Render();
  keep(rc.buffer);
  Image tm(&rc);
  tm.Tonemap();
  tm.GammaCorrection();
  keep(tm.GetBuffer());

  FILE* o = fopen((prefix + ".bin").c_str(), "wb");
  int32_t h[3] = {W, H, (int32_t)out.size()};
  fwrite(h, 4, 3, o);
  for (auto& b : out) fwrite(b.data(), sizeof(Vector3f), npix, o);
  fclose(o);
  printf("demo_obj: %zu triangles, %zu meshes, %zu materials, %d emitters\n", world.triangles.size(),
         world.meshes.size(), world.materials.size(), world.CountEmitters());
  return 0;
}
