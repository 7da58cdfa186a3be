// noalloc.cu — a Gaussian blur entry point that allocates nothing.
//
// Some callers cannot allocate device memory when they call in: a plugin
// whose host application owns the whole device-memory budget and hands out
// no more, or a real-time frame loop where cudaMalloc / cudaFree would
// synchronise the device and stall the other streams.
// rtx_image_gaussian_blur_noalloc serves them: the
// caller passes device input and output images, and the intermediate image of
// the two separable passes lives in a fixed array in the library's device
// memory instead of in a buffer allocated per call.
//
// The array is a file-scope __device__ variable of kNoAllocMaxPixels pixels
// (24 MiB), resident on every GPU that loads the library until the process
// exits.  Host code cannot use its name as a device address, so the first call
// on a device looks the address up with cudaGetSymbolAddress (with that device
// current) and keeps it for the life of the process; make that first call
// before any stream capture, and do not use the entry point across a
// cudaDeviceReset (the kept address would no longer name the array).
// All calls share the array, so calls whose work overlaps on the GPU (other
// streams, other threads) race; serialise them.  Every pixel of the
// intermediate image is written by the first pass before the second pass reads
// it, so no part of the array needs clearing between calls.
#include <cmath>
#include <mutex>

#include "rtx_internal.h"

namespace rtx {
namespace {

constexpr int kNoAllocMaxPixels = 2097152;  // 24 MiB of float3 (2048 x 1024)
constexpr int kNoAllocMaxTaps = 255;
constexpr int kMaxRows = 65535;  // the row passes launch one block row per image row

static __device__ __align__(256) float g_noalloc_image[3 * (size_t)kNoAllocMaxPixels];
static __device__ __align__(256) float g_noalloc_weights[kNoAllocMaxTaps];

struct Taps {
  float w[kNoAllocMaxTaps];
};

// The weights travel as a kernel argument and are stored to device memory by
// the GPU itself, so no host-to-device copy call is needed either.
__global__ void k_store_taps(Taps t, int n, float* dst) {
  int i = threadIdx.x;
  if (i < n) dst[i] = t.w[i];
}

constexpr int kMaxDevices = 64;
std::mutex g_mu;
float* g_image_ptr[kMaxDevices] = {};
float* g_weights_ptr[kMaxDevices] = {};

void set_msg(char* msg, size_t len, const char* text) {
  if (!msg || len == 0) return;
  size_t i = 0;
  for (; text[i] && i + 1 < len; ++i) msg[i] = text[i];
  msg[i] = '\0';
}

}  // namespace
}  // namespace rtx

using namespace rtx;

extern "C" int rtx_image_gaussian_blur_noalloc(const float* d_in, float* d_out, int W, int H,
                                               int size, float sigma, void* stream, char* msg,
                                               size_t msg_len) {
  set_msg(msg, msg_len, "");
  if (!d_in || !d_out || W <= 0 || H <= 0) {
    set_msg(msg, msg_len, "invalid image or size");
    return RTX_ERR_INVALID;
  }
  if ((long long)W * H > kNoAllocMaxPixels) {
    set_msg(msg, msg_len, "image larger than the fixed scratch (2097152 pixels)");
    return RTX_ERR_INVALID;
  }
  if (H > kMaxRows) {
    set_msg(msg, msg_len, "image taller than 65535 rows");
    return RTX_ERR_INVALID;
  }
  if (size <= 0 || size > kNoAllocMaxTaps) {
    set_msg(msg, msg_len, "kernel size must be in [1, 255]");
    return RTX_ERR_INVALID;
  }
  // A launch error is read back through the thread's last-error slot, which
  // may already hold an error of the caller's own earlier work.  Leave such an
  // error where it is (the caller reads it) and do nothing, rather than
  // report it as this call's failure or clear it.
  cudaError_t pending = cudaPeekAtLastError();
  if (pending != cudaSuccess) {
    set_msg(msg, msg_len, "an earlier CUDA error is pending on this thread; nothing was enqueued");
    return RTX_ERR_CUDA;
  }
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    set_msg(msg, msg_len, "no current CUDA device");
    return RTX_ERR_CUDA;
  }
  float* img = nullptr;
  float* wts = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_image_ptr[dev]) {
      float *a = nullptr, *b = nullptr;
      if (cudaGetSymbolAddress((void**)&a, g_noalloc_image) != cudaSuccess ||
          cudaGetSymbolAddress((void**)&b, g_noalloc_weights) != cudaSuccess) {
        cudaGetLastError();
        set_msg(msg, msg_len, "cudaGetSymbolAddress failed for the scratch arrays");
        return RTX_ERR_CUDA;
      }
      g_image_ptr[dev] = a;
      g_weights_ptr[dev] = b;
    }
    img = g_image_ptr[dev];
    wts = g_weights_ptr[dev];
  }
  // UnitizedGaussianKernel weights (RenderToy include/RenderToy/rtmath.h:1019-1059),
  // computed on the host as in rtx_image_gaussian_blur
  Taps t;
  float mid = float(size >> 1);
  float sum = 0.0f;
  for (int j = 0; j < size; ++j) {
    float x2 = std::pow(float(j) - mid, 2.0f);
    float g = std::exp(-(x2) / (2.0f * sigma * sigma));
    sum += g;
    t.w[j] = g;
  }
  for (int j = 0; j < size; ++j) t.w[j] /= sum;
  cudaStream_t st = (cudaStream_t)stream;
  k_store_taps<<<1, kNoAllocMaxTaps + 1, 0, st>>>(t, size, wts);
  int launches = 0;
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess)
    e = launch_gaussian(d_in, img, nullptr, d_out, W, H, wts, size, 0, 0.0f, false, st, &launches);
  if (e != cudaSuccess) {
    set_msg(msg, msg_len, cudaGetErrorString(e));
    return RTX_ERR_CUDA;
  }
  return RTX_OK;
}
