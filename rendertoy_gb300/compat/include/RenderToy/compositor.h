// RenderToy/compositor.h — Image and its filters (RenderToy
// include/RenderToy/compositor.h:18-292).  Convolute, GaussianBlur,
// EdgeDetection and Bloom run on the GPU (librtx); the per-pixel functor
// helpers (Extract, Transform and what is built on them), image arithmetic and
// drawing stay on the host.
#ifndef RTX_COMPAT_COMPOSITOR_H
#define RTX_COMPAT_COMPOSITOR_H
#include <functional>

#include "renderer.h"
#include "rtmath.h"

namespace RenderToy {
enum class EdgeMode { kReflect = 0, kBlackPadding = 1, kWhitePadding = 2 };

class Image {
  Vector3f* buffer;
  void Convolve(const IConvolutionKernel<float>& k, bool normalize, bool length, bool absval);

 public:
  enum class SampleMode { kNearestNeighbor = 0, kBilinearInterpolation = 1 };
  const SizeN resolution;

  Image(const SizeN& resolution_);
  Image(const RenderContext* const render_context_);
  Image(const Image& image);
  ~Image();

  Vector3f& operator()(const std::size_t x, const std::size_t y);
  const Vector3f& operator()(const std::size_t x, const std::size_t y) const;

  [[nodiscard]] const Image Extract(const std::function<bool(const Vector3f&)>& pixel_filter,
                                    const Vector3f& default_color = Vector3f::O);
  const void Transform(const std::function<void(Vector3f&)>& pixel_processor);

  template <bool _Normalize = false, bool _Length = false, bool _Abs = false>
  Image& Convolute(const IConvolutionKernel<float>& k) {
    Convolve(k, _Normalize, _Length, _Abs);
    return *this;
  }
  Image& GaussianBlur(const std::size_t size, const float sigma);
  template <Orientation _O>
  Image& EdgeDetection() {
    if constexpr (_O == Orientation::All) {
      EdgeDetectionAll();
    } else {
      SobelKernel<float, _O> sk;
      Convolute(sk);
    }
    return *this;
  }
  void EdgeDetectionAll();
  template <Convert::ColorStandard _CS>
  Image& GreyScale() {
    Transform([](Vector3f& p) { p = Convert::Luma<_CS>(p); });
    return *this;
  }
  template <Convert::ColorStandard _CS>
  Image& Binarize(const float threshold) {
    Transform([&threshold](Vector3f& p) { p = Convert::Luma<_CS>(p) > threshold ? 1.0f : 0.0f; });
    return *this;
  }
  template <Convert::ColorStandard _CS = Convert::ColorStandard::kITURBT709>
  Image& Tonemap(const float limit = 1.5f) {
    Transform([&limit](Vector3f& p) { p = Convert::Tonemap<_CS>(p, limit); });
    return *this;
  }
  Image& GammaCorrection(const float gamma = 2.2f);
  const Image operator+(const Image& img);
  const Image operator-(const Image& img);
  const Image operator*(const Image& img);
  const Image operator/(const Image& img);
  const void operator=(const Image& img);
  Image& Bloom(const std::size_t size, const float sigma, const float threshold);
  void DrawLine(PointN p1, PointN p2, const Vector3f& color = Vector3f::White);
  void Fill(PointN p1, PointN p2, const Vector3f& color = Vector3f::White);
  Vector3f*& GetBuffer();
  const Vector3f* const& GetBuffer() const;
};
}  // namespace RenderToy
#endif
