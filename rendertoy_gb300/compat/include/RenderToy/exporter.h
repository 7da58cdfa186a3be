// RenderToy/exporter.h — image files (RenderToy include/RenderToy/exporter.h,
// src/exporter.cpp:8-95): the pixels are quantised on the GPU
// (rtx_encode_bmp / rtx_encode_ppm).  BMP rows are zero-padded (RenderToy
// writes the padding from a null pointer) and the header's file size counts
// the padding.
#ifndef RTX_COMPAT_EXPORTER_H
#define RTX_COMPAT_EXPORTER_H
#include <ostream>

#include "compositor.h"

namespace RenderToy {
struct IImageExporter {
  const Image& image;
  virtual void Export(std::ostream& os) = 0;
  IImageExporter(const Image& image_) : image(image_) {}
  virtual ~IImageExporter() = default;
};

struct PPMExporter : public IImageExporter {
  virtual void Export(std::ostream& os) override final;
  PPMExporter(const Image& image_) : IImageExporter(image_) {}
};

struct BMPExporter : public IImageExporter {
  virtual void Export(std::ostream& os) override final;
  BMPExporter(const Image& image_) : IImageExporter(image_) {}
};
}  // namespace RenderToy
#endif
