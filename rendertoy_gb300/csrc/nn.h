// nn.h — the denoiser's device operators (NHWC BF16 tensors, channel counts
// padded to multiples of 8; convolutions on the tcgen05 tensor cores).
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

namespace rtx {
namespace nn {

using bf16 = __nv_bfloat16;

// Network input and output records.
//   raw input, FP32 per pixel: radiance 3 (linear), albedo 3, normal 3 (as the
//   normal pass encodes it), depth 1, and the radiance's samples per pixel 1
//   (the same value over a frame; it tells the network how noisy the
//   radiance is).
//   prediction, FP32 per pixel: kKpTaps filter logits (padded to kPredCh).
//   The denoised radiance is the softmax of the logits applied to the
//   kKpWidth x kKpWidth neighbourhood of the input radiance (taps clamped to
//   the frame): a kernel-predicting output (Bako et al., SIGGRAPH 2017),
//   which can only average input pixels and so approaches its input as the
//   input's noise vanishes.
constexpr int kRawCh = 11;
constexpr int kKpWidth = 5;
constexpr int kKpTaps = kKpWidth * kKpWidth;
constexpr int kPredCh = 32;
// Loss: relative squared error with the prediction (not differentiated) in
// the denominator, (o - t)^2 / (o^2 + kRelEps): its minimiser over noisy
// targets is their mean, so unbiased targets of any noise level train it
// toward the clean image.
constexpr float kRelEps = 1e-2f;

// One input of a convolution: C channels; `up` = stored at half resolution
// and read upsampled (nearest) to the convolution's resolution.
struct Src {
  const bf16* ptr;
  int C;
  int up;
};

struct ConvFwd {
  Src s1, s2;        // s2.ptr == nullptr: single source
  int N, H, W;       // convolution (output) resolution
  int Cin;           // s1.C + s2.C
  int Cout;          // multiple of 16, <= 256
  const bf16* w;     // [Cout][9][Cin]
  const float* bias; // [Cout] or nullptr
  int relu;
  bf16* out;         // [P][Cout] or nullptr
  float* out_f32;    // [P][Cout] or nullptr
  int* err;
};

struct ConvDgrad {
  const bf16* dout;  // [P][Cout]
  int Cout;
  const bf16* wt;    // [Cin][9][Cout]
  int N, H, W, Cin;  // Cin multiple of 16
  Src s1, s2;        // the sources (read for the ReLU mask)
  int mask_relu;
  bf16* din;         // [P][Cin] (s1's channels upsampled when s1.up)
  int* err;
  int ctw = 256;     // row-tile kernel: input channels per tile (multiple of 16, <= 256)
};

struct ConvWgrad {
  const bf16* dout;  // [P][Cout]
  int Cout;
  Src s1, s2;
  int N, H, W, Cin;
  int pix_per_cta;   // pixels each CTA sums (multiple of 64)
  float* dw;         // [Cout][9][Cin], accumulated
  int* err;
  // set by conv_wgrad for the row-tile kernel: channels per CTA, tile width
  // in pixels, row tiles per CTA
  int cr, tw, tiles_per_cta;
};

cudaError_t conv_fwd(const ConvFwd& a, cudaStream_t st);
cudaError_t conv_dgrad(const ConvDgrad& a, cudaStream_t st);
cudaError_t conv_wgrad(const ConvWgrad& a, cudaStream_t st);
// pixels per weight-gradient CTA: enough CTAs for about eight per SM, each
// summing a multiple of 64 pixels
int wgrad_pixels_per_cta(long long P, int Cout, int Cin);

}  // namespace nn
}  // namespace rtx
