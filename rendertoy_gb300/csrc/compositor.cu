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
// segment / column strip with its halo in shared memory (cp.async, one wait
// per tile), so each input pixel is read from HBM once per pass; bloom's
// extraction is fused into the first pass and its final addition into the
// second.  The separable passes and the 3 x 3 / 5 x 5 convolutions are
// register-blocked (a thread computes 8 or 4 outputs along one axis and
// reuses every staged pixel for all of them) and run two outputs per packed
// FP32 instruction; each output's taps are still summed one by one in the
// reference's order with the same roundings.  They are FP32-issue bound: a
// size-49 pass is 49 x 3 multiplies and adds per pixel for 24 bytes of HBM.
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

// Stage pixel idx (or zeros for idx < 0) into shared memory at s with three
// 4-byte cp.async copies: a tile's fill issues all its loads before waiting
// once (cp_wait_all), instead of one DRAM round trip per loop iteration.
RTX_DEV void stage_px(float* s, const float* __restrict__ in, long long idx) {
  if (idx < 0) {
    s[0] = 0.0f;
    s[1] = 0.0f;
    s[2] = 0.0f;
    return;
  }
  const unsigned d = (unsigned)__cvta_generic_to_shared(s);
  const float* g = in + 3 * idx;
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(d), "l"(g) : "memory");
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(d + 4), "l"(g + 1) : "memory");
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(d + 8), "l"(g + 2) : "memory");
}
RTX_DEV void cp_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

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

// acc + p * w with the product rounded before the addition, exactly as the
// scalar multiply and add.  ptxas contracts a packed multiply followed by a
// packed add into one fused operation even under --fmad=false, so the
// product is formed as fma(p, w, nz) with nz = -0.0 passed in at run time
// (unknown to the compiler): that rounds p * w once, as a multiply does
// (x + -0 == x, also for x = +0 and -0), and leaves nothing to contract.
RTX_DEV f2_t f2_mul_add(f2_t acc, f2_t p, f2_t w, f2_t nz) { return f2_add(acc, f2_fma(p, w, nz)); }
// One tap into an accumulator pair: RenderToy's rounding (kFma = false) or one
// fused multiply-add per tap (kFma = true: RTX_OPT_COMPOSITOR_FMA), which
// halves the FP32 work of the register-blocked filters.
template <bool kFma>
RTX_DEV f2_t f2_tap(f2_t acc, f2_t p, f2_t w, f2_t nz) {
  return kFma ? f2_fma(p, w, acc) : f2_mul_add(acc, p, w, nz);
}
template <bool kFma>
RTX_DEV float f_tap(float acc, float p, float w) {
  return kFma ? __fmaf_rn(p, w, acc) : acc + p * w;
}
RTX_DEV float f3c(F3 p, int c) { return c == 0 ? p.x : (c == 1 ? p.y : p.z); }

// Small 2-D kernels (3 x 3, 5 x 5), register-blocked: a thread computes
// kConvR vertically adjacent outputs of one column, with the weights in
// registers.  It walks the staged rows of its window in order and output r
// takes staged row yy as kernel row yy - r, so each output still sums its
// taps row by row, column by column, as the reference does.
constexpr int kConvR = 4, kConvRegThreads = 256, kConvRegW = 32,
              kConvRegH = (kConvRegThreads / kConvRegW) * kConvR;

template <int KR, int KC, bool kFma>
__global__ void __launch_bounds__(kConvRegThreads, 4) k_convolve_reg(const float* __restrict__ in,
                                                                  float* __restrict__ out, int W, int H,
                                                                  const float* __restrict__ k, int flags,
                                                                  float negzero) {
  constexpr int tw = kConvRegW + KC - 1, th = kConvRegH + KR - 1;
  __shared__ float tile[3 * tw * th];
  const int tid = threadIdx.x;
  const int x0 = blockIdx.x * kConvRegW, y0 = blockIdx.y * kConvRegH;
  for (int i = tid; i < tw * th; i += kConvRegThreads) {
    const int ty = i / tw, tx = i - ty * tw;
    stage_px(tile + 3 * i, in, reflect_index((long long)y0 - KR / 2 + ty, (long long)x0 - KC / 2 + tx, W, H));
  }
  float wk[KR * KC];
#pragma unroll
  for (int i = 0; i < KR * KC; ++i) wk[i] = __ldg(k + i);
  cp_wait_all();
  __syncthreads();
  const int lx = tid % kConvRegW, g = tid / kConvRegW;
  const int x = x0 + lx, yb = y0 + kConvR * g;
  if (x >= W || yb >= H) return;
  const f2_t nz = f2_pack(negzero, negzero);
  f2_t acc[3][kConvR / 2];  // [channel][output pair (rows 2q, 2q + 1)]
#pragma unroll
  for (int c = 0; c < 3; ++c)
#pragma unroll
    for (int q = 0; q < kConvR / 2; ++q) acc[c][q] = f2_pack(0.0f, 0.0f);
#pragma unroll
  for (int yy = 0; yy < kConvR + KR - 1; ++yy)
#pragma unroll
    for (int jj = 0; jj < KC; ++jj) {
      const float* t = tile + 3 * ((kConvR * g + yy) * tw + lx + jj);
      const F3 p = f3(t[0], t[1], t[2]);
      const f2_t pp[3] = {f2_pack(p.x, p.x), f2_pack(p.y, p.y), f2_pack(p.z, p.z)};
#pragma unroll
      for (int q = 0; q < kConvR / 2; ++q) {
        const int i0 = yy - 2 * q, i1 = i0 - 1;  // kernel rows of outputs 2q, 2q + 1
        const bool v0 = i0 >= 0 && i0 < KR, v1 = i1 >= 0 && i1 < KR;
        if (v0 && v1) {
          const f2_t ww = f2_pack(wk[i0 * KC + jj], wk[i1 * KC + jj]);
#pragma unroll
          for (int c = 0; c < 3; ++c) acc[c][q] = f2_tap<kFma>(acc[c][q], pp[c], ww, nz);
        } else if (v0 || v1) {
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            float a, b;
            f2_unpack(acc[c][q], a, b);
            if (v0) a = f_tap<kFma>(a, f3c(p, c), wk[i0 * KC + jj]);
            if (v1) b = f_tap<kFma>(b, f3c(p, c), wk[i1 * KC + jj]);
            acc[c][q] = f2_pack(a, b);
          }
        }
      }
    }
#pragma unroll
  for (int r = 0; r < kConvR; ++r) {
    const int y = yb + r;
    if (y >= H) break;
    float lo[3], hi[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) f2_unpack(acc[c][r >> 1], lo[c], hi[c]);
    F3 v = (r & 1) ? f3(hi[0], hi[1], hi[2]) : f3(lo[0], lo[1], lo[2]);
    if (flags & kAbs) v = f3(fabsf(v.x), fabsf(v.y), fabsf(v.z));
    if (flags & kLength) v = f3s(length(v));
    if (flags & kNormalize) v = normalized(v);
    float* o = out + 3 * ((size_t)y * W + x);
    o[0] = v.x;
    o[1] = v.y;
    o[2] = v.z;
  }
}

// Separable passes, register-blocked: a thread computes kSepR consecutive
// outputs along the filter direction.  It walks its window of
// kSepR + size - 1 staged pixels once and adds each pixel into every output
// whose taps cover it (output o takes window pixel j as tap j - o).  j only
// grows, so each output still sums its taps in the order 0 .. size - 1 with
// the same roundings as one output per thread (products rounded, then
// added), while shared-memory loads drop kSepR-fold and every weight is
// loaded once per chunk of kSepR pixels.  Outputs 2q and 2q + 1 of a channel
// share one packed accumulator, so one f32x2 multiply and one f32x2 add
// serve two taps.
constexpr int kSepR = 8, kSepQ = kSepR / 2;

struct SepAcc {
  f2_t v[3][kSepQ];  // [channel][output pair]
  RTX_DEV F3 out(int o) const {
    float a[3], b[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) f2_unpack(v[c][o >> 1], a[c], b[c]);
    return (o & 1) ? f3(b[0], b[1], b[2]) : f3(a[0], a[1], a[2]);
  }
};

// Add window pixels j0 .. j0 + kSepR - 1 into the accumulators.  kAll: every
// (pixel, output) pair of the chunk is a tap (no range test, no early exit).
template <bool kAll, bool kFma, class Px>
RTX_DEV void sep_chunk(SepAcc& A, const float* __restrict__ wsm, int size, int j0, int nj, f2_t nz, Px px) {
  float wv[2 * kSepR - 1];  // wv[k]: weight of tap j0 - (kSepR - 1) + k
#pragma unroll
  for (int k = 0; k < 2 * kSepR - 1; ++k) {
    int ii = j0 - (kSepR - 1) + k;
    if (!kAll) ii = min(max(ii, 0), size - 1);
    wv[k] = wsm[ii];
  }
  f2_t wp[2 * kSepR - 1];  // wp[k] = (wv[k], wv[k - 1]): the taps of an output pair
#pragma unroll
  for (int k = 1; k < 2 * kSepR - 1; ++k) wp[k] = f2_pack(wv[k], wv[k - 1]);
#pragma unroll
  for (int s = 0; s < kSepR; ++s) {
    const int j = j0 + s;
    if (!kAll && j >= nj) break;
    const F3 p = px(j);
    const f2_t pp[3] = {f2_pack(p.x, p.x), f2_pack(p.y, p.y), f2_pack(p.z, p.z)};
#pragma unroll
    for (int q = 0; q < kSepQ; ++q) {
      const int o0 = 2 * q, o1 = 2 * q + 1, k0 = s - o0 + kSepR - 1;
      const bool v0 = kAll || (j - o0 >= 0 && j - o0 < size);
      const bool v1 = kAll || (j - o1 >= 0 && j - o1 < size);
      if (v0 && v1) {
#pragma unroll
        for (int c = 0; c < 3; ++c) A.v[c][q] = f2_tap<kFma>(A.v[c][q], pp[c], wp[k0], nz);
      } else if (v0 || v1) {
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          float a, b;
          f2_unpack(A.v[c][q], a, b);
          const float pc = f3c(p, c);
          if (v0) a = f_tap<kFma>(a, pc, wv[k0]);
          if (v1) b = f_tap<kFma>(b, pc, wv[k0 - 1]);
          A.v[c][q] = f2_pack(a, b);
        }
      }
    }
  }
}

template <bool kFma, class Px>
RTX_DEV void sep_window(SepAcc& A, const float* __restrict__ wsm, int size, float negzero, Px px) {
  const f2_t nz = f2_pack(negzero, negzero);
#pragma unroll
  for (int c = 0; c < 3; ++c)
#pragma unroll
    for (int q = 0; q < kSepQ; ++q) A.v[c][q] = f2_pack(0.0f, 0.0f);
  const int nj = size + kSepR - 1;
  for (int j0 = 0; j0 < nj; j0 += kSepR) {
    if (j0 >= kSepR - 1 && j0 + kSepR - 1 < size)
      sep_chunk<true, kFma>(A, wsm, size, j0, nj, nz, px);
    else
      sep_chunk<false, kFma>(A, wsm, size, j0, nj, nz, px);
  }
}

// Horizontal pass (1 x size kernel): a block computes kRowTile pixels of one
// row.  The row segment and its halo sit in shared memory as RGB triples with
// one spare triple after every kSepR pixels, so the kSepR-pixel strides of a
// warp's lanes (27 words apart) fall in distinct banks.
constexpr int kRowThreads = 128, kRowTile = kRowThreads * kSepR;
RTX_DEV int row_slot(int i) { return 3 * (i + i / kSepR); }

template <bool kFma>
__global__ void __launch_bounds__(kRowThreads, 8) k_gauss_x(const float* __restrict__ in,
                                                         float* __restrict__ out, int W, int H,
                                                         const float* __restrict__ w, int size,
                                                         int extract_mode, float thr, float negzero) {
  extern __shared__ float sm[];
  float* wsm = sm;                       // size weights
  float* tile = sm + ((size + 3) & ~3);  // row_slot(kRowTile + size - 1) floats
  const int y = blockIdx.y, x0 = blockIdx.x * kRowTile, r = size >> 1, tid = threadIdx.x;
  const int n_out = min(kRowTile, W - x0);
  const int span = n_out + size - 1, cap = kRowTile + size - 1;
  for (int j = tid; j < size; j += kRowThreads) wsm[j] = w[j];
  for (int j = tid; j < cap; j += kRowThreads)
    stage_px(tile + row_slot(j), in, j < span ? reflect_index(y, (long long)x0 - r + j, W, H) : -1);
  cp_wait_all();
  if (extract_mode) {  // bloom: Extract applied to the staged pixels
    for (int j = tid; j < span; j += kRowThreads) {
      float* s = tile + row_slot(j);
      const F3 p = extract(f3(s[0], s[1], s[2]), thr);
      s[0] = p.x;
      s[1] = p.y;
      s[2] = p.z;
    }
  }
  __syncthreads();
  SepAcc acc;
  const int b = kSepR * tid;
  if (b < n_out) {
    sep_window<kFma>(acc, wsm, size, negzero, [&](int j) {
      const float* s = tile + row_slot(b + j);
      return f3(s[0], s[1], s[2]);
    });
  }
  __syncthreads();  // the tile now holds the outputs, in the same slots
  if (b < n_out) {
#pragma unroll
    for (int o = 0; o < kSepR; ++o) {
      float* s = tile + row_slot(b + o);
      const F3 v = acc.out(o);
      s[0] = v.x;
      s[1] = v.y;
      s[2] = v.z;
    }
  }
  __syncthreads();
  float* orow = out + 3 * ((size_t)y * W + x0);
  for (int f = tid; f < 3 * n_out; f += kRowThreads) {
    const int q = f / 3;
    orow[f] = tile[row_slot(q) + (f - 3 * q)];
  }
}

// Vertical pass (size x 1 kernel): a block computes kColW columns x kColH
// rows; lanes take neighbouring columns, each thread kSepR consecutive rows,
// from a shared-memory strip of kColH + size - 1 rows.
constexpr int kColW = 32, kColThreads = 128, kColH = (kColThreads / kColW) * kSepR;

template <bool kFma>
__global__ void __launch_bounds__(kColThreads, 7) k_gauss_y(const float* __restrict__ in,
                                                         const float* __restrict__ orig,
                                                         float* __restrict__ out, int W, int H,
                                                         const float* __restrict__ w, int size,
                                                         float negzero) {
  extern __shared__ float sm[];
  float* wsm = sm;
  float* strip = sm + ((size + 3) & ~3);  // (kColH + size - 1) rows x kColW x 3
  const int x0 = blockIdx.x * kColW, y0 = blockIdx.y * kColH, r = size >> 1, tid = threadIdx.x;
  for (int j = tid; j < size; j += kColThreads) wsm[j] = w[j];
  const int rows = kColH + size - 1;
  for (int e = tid; e < rows * kColW; e += kColThreads) {
    const int rr = e / kColW, cc = e - rr * kColW;
    const int x = x0 + cc;
    stage_px(strip + 3 * e, in, x < W ? reflect_index((long long)y0 - r + rr, x, W, H) : -1);
  }
  cp_wait_all();
  __syncthreads();
  const int cc = tid % kColW, g = tid / kColW;
  const int x = x0 + cc, yb = y0 + kSepR * g;
  if (x >= W || yb >= H) return;
  SepAcc acc;
  sep_window<kFma>(acc, wsm, size, negzero, [&](int j) {
    const float* s = strip + 3 * ((kSepR * g + j) * kColW + cc);
    return f3(s[0], s[1], s[2]);
  });
#pragma unroll
  for (int o = 0; o < kSepR; ++o) {
    const int y = yb + o;
    if (y < H) {
      const size_t p = (size_t)y * W + x;
      F3 v = acc.out(o);
      if (orig) v = f3(__ldg(orig + 3 * p), __ldg(orig + 3 * p + 1), __ldg(orig + 3 * p + 2)) + v;
      out[3 * p] = v.x;
      out[3 * p + 1] = v.y;
      out[3 * p + 2] = v.z;
    }
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
                            int kc, int flags, bool fma, cudaStream_t st, int* launches) {
  const size_t smem = sizeof(float) * ((size_t)kr * kc + 3 * (size_t)(kConvTY + kr - 1) * (kConvTX + kc - 1));
  const dim3 rgrid((W + kConvRegW - 1) / kConvRegW, (H + kConvRegH - 1) / kConvRegH);
  if (kr == 5 && kc == 5) {
    if (fma)
      k_convolve_reg<5, 5, true><<<rgrid, kConvRegThreads, 0, st>>>(in, out, W, H, d_k, flags, -0.0f);
    else
      k_convolve_reg<5, 5, false><<<rgrid, kConvRegThreads, 0, st>>>(in, out, W, H, d_k, flags, -0.0f);
  } else if (kr == 3 && kc == 3) {
    if (fma)
      k_convolve_reg<3, 3, true><<<rgrid, kConvRegThreads, 0, st>>>(in, out, W, H, d_k, flags, -0.0f);
    else
      k_convolve_reg<3, 3, false><<<rgrid, kConvRegThreads, 0, st>>>(in, out, W, H, d_k, flags, -0.0f);
  } else if (smem <= 48 * 1024) {
    dim3 grid((W + kConvTX - 1) / kConvTX, (H + kConvTY - 1) / kConvTY);
    k_convolve_tiled<<<grid, kConvTX * kConvTY, smem, st>>>(in, out, W, H, d_k, kr, kc, flags);
  } else {
    dim3 grid((W + 127) / 128, H);
    k_convolve<<<grid, 128, 0, st>>>(in, out, W, H, d_k, kr, kc, flags);
  }
  ++*launches;
  return cudaGetLastError();
}

static size_t smem_x(int size) {
  const size_t cap = (size_t)kRowTile + size - 1;
  return sizeof(float) * (((size_t)size + 3 & ~(size_t)3) + 3 * (cap + cap / kSepR));
}
static size_t smem_y(int size) {
  return sizeof(float) * (((size_t)size + 3 & ~(size_t)3) + 3 * ((size_t)kColH + size - 1) * kColW);
}

// GaussianBlur(size) on `in` (extract_mode: bloom's Extract fused into the
// first pass, and the second pass adds `in` back: Image::Bloom).
// Kernels too large for a shared-memory strip take the direct path, with
// extraction and the final addition as separate elementwise passes (tmp2 is
// then required).
cudaError_t launch_gaussian(const float* in, float* tmp, float* tmp2, float* out, int W, int H,
                            const float* d_w, int size, int extract_mode, float threshold, bool fma,
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
    auto kx = fma ? k_gauss_x<true> : k_gauss_x<false>;
    if (sx > 48 * 1024 && (e = cudaFuncSetAttribute(kx, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sx)))
      return e;
    kx<<<dim3((W + kRowTile - 1) / kRowTile, H), kRowThreads, sx, st>>>(in, tmp, W, H, d_w, size, extract_mode,
                                                                       threshold, -0.0f);
  } else {
    k_convolve<<<dim3((W + 127) / 128, H), 128, 0, st>>>(in, tmp, W, H, d_w, 1, size, 0);
  }
  ++*launches;
  if (sy <= kMaxSmem) {
    auto ky = fma ? k_gauss_y<true> : k_gauss_y<false>;
    if (sy > 48 * 1024 && (e = cudaFuncSetAttribute(ky, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sy)))
      return e;
    ky<<<dim3((W + kColW - 1) / kColW, (H + kColH - 1) / kColH), kColThreads, sy, st>>>(
        tmp, extract_mode ? in : nullptr, out, W, H, d_w, size, -0.0f);
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
