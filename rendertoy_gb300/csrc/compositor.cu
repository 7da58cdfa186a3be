// compositor.cu — RenderToy's Image filters on the GPU
// (include/RenderToy/compositor.h:107-178, src/compositor.cpp:42-77).
//
// Every output pixel sums its taps in the reference's order (row of the
// kernel, then column; products rounded before each addition: the file is
// built with --fmad=false), so results equal the reference bit for bit.
// Edge taps use the reference's reflect mapping (compositor.h:25-39), in
// which index == size maps to itself; a tap whose linear index falls outside
// the image reads zero (the reference reads past its buffer there).
//
// Separable passes (GaussianBlur = 1 x size then size x 1) stage a row
// segment / column strip with its halo in shared memory, so each input pixel
// is read from HBM once per pass; bloom's extraction is fused into the first
// pass and its final addition into the second.
#include <algorithm>

#include "device_math.cuh"
#include "rtx_internal.h"

namespace rtx {

enum ConvFlags { kAbs = 1, kLength = 2, kNormalize = 4 };

RTX_DEV long long reflect_index(long long row, long long col, long long W, long long H) {
  if (row < 0) row = -row;
  if (col < 0) col = -col;
  if (col >= W) col = 2 * W - col;
  if (row >= H) row = 2 * H - row;
  long long idx = row * W + col;
  return (idx < 0 || idx >= W * H) ? -1 : idx;
}

RTX_DEV F3 load_px(const float* __restrict__ in, long long idx) {
  if (idx < 0) return f3s(0.0f);
  return f3(__ldg(in + 3 * idx), __ldg(in + 3 * idx + 1), __ldg(in + 3 * idx + 2));
}

// Image::Extract(Luma > threshold) (compositor.cpp:51-59, 69-71)
RTX_DEV F3 extract(F3 p, float thr) { return luma(p) > thr ? p : f3s(0.0f); }

// General kr x kc convolution, one pixel per thread (Image::Convolute)
__global__ void k_convolve(const float* __restrict__ in, float* __restrict__ out, int W, int H,
                           const float* __restrict__ k, int kr, int kc, int flags) {
  int x = blockIdx.x * blockDim.x + threadIdx.x;
  int y = blockIdx.y;
  if (x >= W) return;
  long long r2 = kr >> 1, c2 = kc >> 1;
  F3 acc = f3s(0.0f);
  for (int ii = 0; ii < kr; ++ii)
    for (int jj = 0; jj < kc; ++jj) {
      long long idx = reflect_index(y - r2 + ii, x - c2 + jj, W, H);
      acc = acc + load_px(in, idx) * __ldg(k + ii * kc + jj);
    }
  if (flags & kAbs) acc = f3(fabsf(acc.x), fabsf(acc.y), fabsf(acc.z));
  if (flags & kLength) acc = f3s(length(acc));
  if (flags & kNormalize) acc = normalized(acc);
  float* o = out + 3 * ((size_t)y * W + x);
  o[0] = acc.x;
  o[1] = acc.y;
  o[2] = acc.z;
}

// The same convolution from a shared-memory tile: a block fills its 32 x 8
// pixels plus the kernel's halo once (every element through reflect_index,
// so RenderToy's reflection, including its row wrap, is kept), then each
// thread sums its taps in the same order as k_convolve.
constexpr int kConvTX = 32, kConvTY = 8;

__global__ void __launch_bounds__(kConvTX * kConvTY) k_convolve_tiled(const float* __restrict__ in,
                                                                     float* __restrict__ out, int W, int H,
                                                                     const float* __restrict__ k, int kr,
                                                                     int kc, int flags) {
  extern __shared__ float sm[];
  float* wsm = sm;            // kr * kc weights
  float* tile = sm + kr * kc; // (kConvTY + kr - 1) x (kConvTX + kc - 1) pixels
  const int tid = threadIdx.x;
  const int x0 = blockIdx.x * kConvTX, y0 = blockIdx.y * kConvTY;
  const int r2 = kr >> 1, c2 = kc >> 1, tw = kConvTX + kc - 1, th = kConvTY + kr - 1;
  for (int i = tid; i < kr * kc; i += blockDim.x) wsm[i] = k[i];
  for (int i = tid; i < tw * th; i += blockDim.x) {
    const int ty = i / tw, tx = i - ty * tw;
    F3 p = load_px(in, reflect_index((long long)y0 - r2 + ty, (long long)x0 - c2 + tx, W, H));
    tile[3 * i] = p.x;
    tile[3 * i + 1] = p.y;
    tile[3 * i + 2] = p.z;
  }
  __syncthreads();
  const int lx = tid % kConvTX, ly = tid / kConvTX;
  const int x = x0 + lx, y = y0 + ly;
  if (x >= W || y >= H) return;
  F3 acc = f3s(0.0f);
  for (int ii = 0; ii < kr; ++ii)
    for (int jj = 0; jj < kc; ++jj) {
      const float* q = tile + 3 * ((ly + ii) * tw + lx + jj);
      acc = acc + f3(q[0], q[1], q[2]) * wsm[ii * kc + jj];
    }
  if (flags & kAbs) acc = f3(fabsf(acc.x), fabsf(acc.y), fabsf(acc.z));
  if (flags & kLength) acc = f3s(length(acc));
  if (flags & kNormalize) acc = normalized(acc);
  float* o = out + 3 * ((size_t)y * W + x);
  o[0] = acc.x;
  o[1] = acc.y;
  o[2] = acc.z;
}

// Horizontal pass (1 x size kernel): a block computes kTileX pixels of one row
// from a shared-memory copy of the row segment plus its halo.
constexpr int kTileX = 256;

__global__ void __launch_bounds__(kTileX) k_gauss_x(const float* __restrict__ in,
                                                    float* __restrict__ out, int W, int H,
                                                    const float* __restrict__ w, int size,
                                                    int extract_mode, float thr) {
  extern __shared__ float sm[];
  float* wsm = sm;                 // size weights
  float* tile = sm + size;         // (kTileX + size - 1) * 3
  int y = blockIdx.y;
  int x0 = blockIdx.x * kTileX;
  int r = size >> 1;
  for (int j = threadIdx.x; j < size; j += blockDim.x) wsm[j] = w[j];
  int span = kTileX + size - 1;
  for (int j = threadIdx.x; j < span; j += blockDim.x) {
    long long idx = reflect_index(y, (long long)x0 - r + j, W, H);
    F3 p = load_px(in, idx);
    if (extract_mode) p = extract(p, thr);
    tile[3 * j] = p.x;
    tile[3 * j + 1] = p.y;
    tile[3 * j + 2] = p.z;
  }
  __syncthreads();
  int x = x0 + threadIdx.x;
  if (x >= W) return;
  F3 acc = f3s(0.0f);
  const float* t = tile + 3 * threadIdx.x;
  for (int jj = 0; jj < size; ++jj)
    acc = acc + f3(t[3 * jj], t[3 * jj + 1], t[3 * jj + 2]) * wsm[jj];
  float* o = out + 3 * ((size_t)y * W + x);
  o[0] = acc.x;
  o[1] = acc.y;
  o[2] = acc.z;
}

// Vertical pass (size x 1 kernel): a block computes a kColsY x kRowsY tile
// from a shared-memory strip of (kRowsY + size - 1) rows.
constexpr int kColsY = 32, kRowsY = 32, kThreadsY = 256;

__global__ void __launch_bounds__(kThreadsY) k_gauss_y(const float* __restrict__ in,
                                                       const float* __restrict__ orig,
                                                       float* __restrict__ out, int W, int H,
                                                       const float* __restrict__ w, int size) {
  extern __shared__ float sm[];
  float* wsm = sm;
  float* strip = sm + size;  // rows (kRowsY + size - 1) x kColsY x 3
  int x0 = blockIdx.x * kColsY, y0 = blockIdx.y * kRowsY;
  int r = size >> 1;
  for (int j = threadIdx.x; j < size; j += blockDim.x) wsm[j] = w[j];
  int rows = kRowsY + size - 1;
  for (int e = threadIdx.x; e < rows * kColsY; e += blockDim.x) {
    int rr = e / kColsY, cc = e % kColsY;
    int x = x0 + cc;
    F3 p = f3s(0.0f);
    if (x < W) p = load_px(in, reflect_index((long long)y0 - r + rr, x, W, H));
    float* s = strip + 3 * (rr * kColsY + cc);
    s[0] = p.x;
    s[1] = p.y;
    s[2] = p.z;
  }
  __syncthreads();
  int cc = threadIdx.x % kColsY;
  int x = x0 + cc;
  if (x >= W) return;
  for (int ry = threadIdx.x / kColsY; ry < kRowsY; ry += kThreadsY / kColsY) {
    int y = y0 + ry;
    if (y >= H) break;
    F3 acc = f3s(0.0f);
    for (int ii = 0; ii < size; ++ii) {
      const float* s = strip + 3 * ((ry + ii) * kColsY + cc);
      acc = acc + f3(s[0], s[1], s[2]) * wsm[ii];
    }
    size_t p = (size_t)y * W + x;
    if (orig) acc = f3(__ldg(orig + 3 * p), __ldg(orig + 3 * p + 1), __ldg(orig + 3 * p + 2)) + acc;
    out[3 * p] = acc.x;
    out[3 * p + 1] = acc.y;
    out[3 * p + 2] = acc.z;
  }
}

// EdgeDetection<All> (compositor.h:153-178): Sobel-X and Sobel-Y sums of the
// 3 x 3 neighbourhood, each in the reference's tap order, then |gy + gx|.
__global__ void k_edge(const float* __restrict__ in, float* __restrict__ out, int W, int H) {
  int x = blockIdx.x * blockDim.x + threadIdx.x;
  int y = blockIdx.y;
  if (x >= W) return;
  const float sx[9] = {-1.f, 0.f, 1.f, -2.f, 0.f, 2.f, -1.f, 0.f, 1.f};
  const float sy[9] = {1.f, 2.f, 1.f, 0.f, 0.f, 0.f, -1.f, -2.f, -1.f};
  F3 gx = f3s(0.0f), gy = f3s(0.0f);
#pragma unroll
  for (int ii = 0; ii < 3; ++ii)
#pragma unroll
    for (int jj = 0; jj < 3; ++jj) {
      F3 p = load_px(in, reflect_index(y - 1 + ii, x - 1 + jj, W, H));
      gx = gx + p * sx[ii * 3 + jj];
      gy = gy + p * sy[ii * 3 + jj];
    }
  float l = length(gy + gx);
  float* o = out + 3 * ((size_t)y * W + x);
  o[0] = l;
  o[1] = l;
  o[2] = l;
}

__global__ void k_extract(const float* __restrict__ in, float* __restrict__ out, size_t n, float thr) {
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  F3 p = extract(f3(in[3 * i], in[3 * i + 1], in[3 * i + 2]), thr);
  out[3 * i] = p.x;
  out[3 * i + 1] = p.y;
  out[3 * i + 2] = p.z;
}

// Image::operator+ (compositor.cpp:102-115): out = a + b
__global__ void k_add(const float* __restrict__ a, const float* __restrict__ b,
                      float* __restrict__ out, size_t n) {
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  out[i] = a[i] + b[i];
}

cudaError_t launch_convolve(const float* in, float* out, int W, int H, const float* d_k, int kr,
                            int kc, int flags, cudaStream_t st, int* launches) {
  const size_t smem = sizeof(float) * ((size_t)kr * kc + 3 * (size_t)(kConvTY + kr - 1) * (kConvTX + kc - 1));
  if (smem <= 48 * 1024) {
    dim3 grid((W + kConvTX - 1) / kConvTX, (H + kConvTY - 1) / kConvTY);
    k_convolve_tiled<<<grid, kConvTX * kConvTY, smem, st>>>(in, out, W, H, d_k, kr, kc, flags);
  } else {
    dim3 grid((W + 127) / 128, H);
    k_convolve<<<grid, 128, 0, st>>>(in, out, W, H, d_k, kr, kc, flags);
  }
  ++*launches;
  return cudaGetLastError();
}

static size_t smem_x(int size) { return sizeof(float) * (size + 3 * (kTileX + size - 1)); }
static size_t smem_y(int size) { return sizeof(float) * (size + 3 * (kRowsY + size - 1) * kColsY); }

// GaussianBlur(size) on `in` (extract_mode: bloom's Extract fused into the
// first pass, and the second pass adds `in` back: Image::Bloom).
// Kernels too large for a shared-memory strip take the direct path, with
// extraction and the final addition as separate elementwise passes (tmp2 is
// then required).
cudaError_t launch_gaussian(const float* in, float* tmp, float* tmp2, float* out, int W, int H,
                            const float* d_w, int size, int extract_mode, float threshold,
                            cudaStream_t st, int* launches) {
  cudaError_t e;
  size_t sx = smem_x(size), sy = smem_y(size);
  const size_t kMaxSmem = 227 * 1024;
  size_t n = (size_t)W * H;
  if (extract_mode && (sx > kMaxSmem || sy > kMaxSmem)) {
    if (!tmp2) return cudaErrorInvalidValue;
    k_extract<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(in, tmp2, n, threshold);
    k_convolve<<<dim3((W + 127) / 128, H), 128, 0, st>>>(tmp2, tmp, W, H, d_w, 1, size, 0);
    k_convolve<<<dim3((W + 127) / 128, H), 128, 0, st>>>(tmp, tmp2, W, H, d_w, size, 1, 0);
    k_add<<<(unsigned)((3 * n + 255) / 256), 256, 0, st>>>(in, tmp2, out, 3 * n);
    *launches += 4;
    return cudaGetLastError();
  }
  if (sx <= kMaxSmem) {
    if (sx > 48 * 1024 &&
        (e = cudaFuncSetAttribute(k_gauss_x, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sx)))
      return e;
    k_gauss_x<<<dim3((W + kTileX - 1) / kTileX, H), kTileX, sx, st>>>(in, tmp, W, H, d_w, size,
                                                                     extract_mode, threshold);
  } else {
    k_convolve<<<dim3((W + 127) / 128, H), 128, 0, st>>>(in, tmp, W, H, d_w, 1, size, 0);
  }
  ++*launches;
  if (sy <= kMaxSmem) {
    if (sy > 48 * 1024 &&
        (e = cudaFuncSetAttribute(k_gauss_y, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sy)))
      return e;
    k_gauss_y<<<dim3((W + kColsY - 1) / kColsY, (H + kRowsY - 1) / kRowsY), kThreadsY, sy, st>>>(
        tmp, extract_mode ? in : nullptr, out, W, H, d_w, size);
  } else {
    k_convolve<<<dim3((W + 127) / 128, H), 128, 0, st>>>(tmp, out, W, H, d_w, size, 1, 0);
  }
  ++*launches;
  return cudaGetLastError();
}

cudaError_t launch_edge(const float* in, float* out, int W, int H, cudaStream_t st, int* launches) {
  k_edge<<<dim3((W + 127) / 128, H), 128, 0, st>>>(in, out, W, H);
  ++*launches;
  return cudaGetLastError();
}

}  // namespace rtx
