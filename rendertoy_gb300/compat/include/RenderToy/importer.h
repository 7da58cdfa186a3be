// RenderToy/importer.h — OBJ / MTL import into a World (RenderToy
// include/RenderToy/importer.h, src/importer.cpp:29-229), by the native
// importer of librtx (rtx_obj_import): the same meshes, triangles (fan
// triangulation, World::triangles order, Mesh::tris prepend order) and
// materials.  Failures throw Exception::DeviceException where RenderToy has
// undefined behaviour or ignores the error.
#ifndef RTX_COMPAT_IMPORTER_H
#define RTX_COMPAT_IMPORTER_H
#include <string>

#include "world.h"

namespace RenderToy {
class OBJModelImporter {
 public:
  OBJModelImporter() = delete;
  OBJModelImporter(const OBJModelImporter&) = delete;
  OBJModelImporter(const OBJModelImporter&&) = delete;
  static void Import(World& world, const std::string& path);
};

class MTLImporter {
 public:
  MTLImporter() = delete;
  static void Import(World& world, const std::string& path);
};

// (RenderToy: work in progress, no members)
class TARGAImporter {
 public:
  TARGAImporter() = delete;
  TARGAImporter(const TARGAImporter&) = delete;
  TARGAImporter(const TARGAImporter&&) = delete;
};
}  // namespace RenderToy
#endif
