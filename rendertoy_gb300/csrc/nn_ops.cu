// nn_ops.cu — the denoiser's memory-bound operators: input encoding, 2 x 2
// average pooling and its gradient, the gradient of nearest upsampling and of
// channel concatenation, the kernel-predicting output with its relative-L2
// loss, bias gradients, Adam and the BF16 weight layouts the convolutions
// read.  One thread per 8 channels of a pixel (16-byte BF16 accesses) unless
// noted.
#include <algorithm>

#include "nn.h"
#include "nn_ops.h"

namespace rtx {
namespace nn {

namespace {

__device__ __forceinline__ void ld8(const bf16* p, float* f) {
  uint4 u = *reinterpret_cast<const uint4*>(p);
  const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&u);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    float2 t = __bfloat1622float2(h[i]);
    f[2 * i] = t.x;
    f[2 * i + 1] = t.y;
  }
}

__device__ __forceinline__ void st8(bf16* p, const float* f) {
  uint4 u;
  __nv_bfloat162* h = reinterpret_cast<__nv_bfloat162*>(&u);
#pragma unroll
  for (int i = 0; i < 4; ++i) h[i] = __floats2bfloat162_rn(f[2 * i], f[2 * i + 1]);
  *reinterpret_cast<uint4*>(p) = u;
}

unsigned blocks(long long n, int t = 256) { return (unsigned)((n + t - 1) / t); }

// A radiance value made safe to filter and to learn from: NaN and negative
// values (the renderer's rare NaN pixels) read 0, +inf reads the BF16 range.
__device__ __forceinline__ float sane(float v) { return fminf(fmaxf(v, 0.0f), 65504.0f); }

// Pixel (n, y, x) of frames of Hs x Ws stored pixels, RGB of its raw record
__device__ __forceinline__ void raw_rgb(const float* raw, long long pix, float* c) {
  const float* r = raw + (long long)kRawCh * pix;
  c[0] = sane(r[0]);
  c[1] = sane(r[1]);
  c[2] = sane(r[2]);
}

// Softmax of the pixel's kKpTaps logits (max subtracted first); the logits
// are read as seven 16-byte loads (the record is kPredCh = 32 floats, 128-byte
// aligned).
__device__ __forceinline__ void kp_weights(const float* __restrict__ logits_g, float* w) {
  static_assert(kPredCh % 4 == 0 && kKpTaps <= 28 && kPredCh >= 28, "seven float4 of logits");
  float logits[28];
  const float4* l4 = reinterpret_cast<const float4*>(logits_g);
#pragma unroll
  for (int i = 0; i < 7; ++i) {
    const float4 v = __ldg(l4 + i);
    logits[4 * i] = v.x;
    logits[4 * i + 1] = v.y;
    logits[4 * i + 2] = v.z;
    logits[4 * i + 3] = v.w;
  }
  float m = logits[0];
#pragma unroll
  for (int k = 1; k < kKpTaps; ++k) m = fmaxf(m, logits[k]);
  float s = 0.0f;
#pragma unroll
  for (int k = 0; k < kKpTaps; ++k) {
    w[k] = expf(logits[k] - m);
    s += w[k];
  }
  const float inv = 1.0f / s;
#pragma unroll
  for (int k = 0; k < kKpTaps; ++k) w[k] *= inv;
}

// Tap k of pixel (x, y) of an Hc x Wc frame stored with row stride Ws:
// offset (k / kKpWidth - r, k % kKpWidth - r), clamped to the frame.
__device__ __forceinline__ long long kp_tap(long long frame0, int x, int y, int k, int Wc, int Hc, int Ws) {
  constexpr int r = kKpWidth / 2;
  const int ty = min(max(y + k / kKpWidth - r, 0), Hc - 1);
  const int tx = min(max(x + k % kKpWidth - r, 0), Wc - 1);
  return frame0 + (long long)ty * Ws + tx;
}

}  // namespace

// raw [P][kRawCh] -> [P][16] BF16: radiance as log(1 + x), albedo, normal and
// depth as they are, the samples per pixel as log2(spp) / 16, channels
// 11..15 zero
__global__ void k_encode_input(const float* __restrict__ raw, bf16* __restrict__ x, long long P) {
  long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (p >= P) return;
  const float* r = raw + (long long)kRawCh * p;
  float f[16];
#pragma unroll
  for (int i = 0; i < 16; ++i) f[i] = 0.0f;
  for (int i = 0; i < 3; ++i) f[i] = log1pf(sane(r[i]));
  for (int i = 3; i < 10; ++i) f[i] = r[i];
  f[10] = log2f(fmaxf(r[10], 1.0f)) * (1.0f / 16.0f);
  st8(x + 16 * p, f);
  st8(x + 16 * p + 8, f + 8);
}

__global__ void k_avgpool(const bf16* __restrict__ in, bf16* __restrict__ out, int N, int H, int W, int C) {
  int h = H >> 1, w = W >> 1, c8 = C >> 3;
  long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  long long total = (long long)N * h * w * c8;
  if (i >= total) return;
  int c = (int)(i % c8) * 8;
  long long q = i / c8;
  int x = (int)(q % w);
  long long r = q / w;
  int y = (int)(r % h);
  int n = (int)(r / h);
  float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0}, v[8];
  for (int dy = 0; dy < 2; ++dy)
    for (int dx = 0; dx < 2; ++dx) {
      ld8(in + (((size_t)n * H + 2 * y + dy) * W + 2 * x + dx) * C + c, v);
#pragma unroll
      for (int k = 0; k < 8; ++k) acc[k] += v[k];
    }
#pragma unroll
  for (int k = 0; k < 8; ++k) acc[k] *= 0.25f;
  st8(out + q * C + c, acc);
}

// d_low[n, y, x, c] = sum over the 2 x 2 block of dcat[.., c0 + c] (nearest
// upsampling's gradient), channels [c0, c0 + C) of a Ccat-channel tensor
__global__ void k_upsample_grad(const bf16* __restrict__ dcat, int Ccat, int c0, bf16* __restrict__ dlow,
                                int N, int H, int W, int C) {
  int h = H >> 1, w = W >> 1, c8 = C >> 3;
  long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  long long total = (long long)N * h * w * c8;
  if (i >= total) return;
  int c = (int)(i % c8) * 8;
  long long q = i / c8;
  int x = (int)(q % w);
  long long r = q / w;
  int y = (int)(r % h);
  int n = (int)(r / h);
  float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0}, v[8];
  for (int dy = 0; dy < 2; ++dy)
    for (int dx = 0; dx < 2; ++dx) {
      ld8(dcat + (((size_t)n * H + 2 * y + dy) * W + 2 * x + dx) * Ccat + c0 + c, v);
#pragma unroll
      for (int k = 0; k < 8; ++k) acc[k] += v[k];
    }
  st8(dlow + q * C + c, acc);
}

// dst[p, c] = dcat[p, c0 + c] (a skip connection's share of a concatenation)
__global__ void k_take_channels(const bf16* __restrict__ dcat, int Ccat, int c0, bf16* __restrict__ dst,
                                long long P, int C) {
  int c8 = C >> 3;
  long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= P * c8) return;
  long long p = i / c8;
  int c = (int)(i % c8) * 8;
  *reinterpret_cast<uint4*>(dst + p * C + c) = *reinterpret_cast<const uint4*>(dcat + p * Ccat + c0 + c);
}

// dskip[p, c] += (skip[p, c] > 0) * 0.25 * dpool[p / 2, c]: the pooled path's
// gradient reaching a ReLU output
__global__ void k_pool_grad_acc(const bf16* __restrict__ dpool, const bf16* __restrict__ skip,
                                bf16* __restrict__ dskip, int N, int H, int W, int C) {
  int c8 = C >> 3;
  long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  long long total = (long long)N * H * W * c8;
  if (i >= total) return;
  int c = (int)(i % c8) * 8;
  long long p = i / c8;
  int x = (int)(p % W);
  long long r = p / W;
  int y = (int)(r % H);
  int n = (int)(r / H);
  float d[8], s[8], g[8];
  ld8(dpool + (((size_t)n * (H >> 1) + (y >> 1)) * (W >> 1) + (x >> 1)) * C + c, d);
  ld8(skip + p * C + c, s);
  ld8(dskip + p * C + c, g);
#pragma unroll
  for (int k = 0; k < 8; ++k) g[k] += s[k] > 0.0f ? 0.25f * d[k] : 0.0f;
  st8(dskip + p * C + c, g);
}

// L1 on log(1 + target): pred [P][16] FP32 (channels 0..2), target [P][3];
// d_pred = sign(pred - log1p(target)) / (3P) as BF16 [P][16]; loss summed
// into *loss (FP64)
// The loss of the kernel-predicting output, per pixel p of N frames of H x W:
// o = sum_k w_k r(tap k), loss = sum_c (o_c - t_c)^2 / (o_c^2 + kRelEps),
// with the denominator held constant; the gradient of the mean over pixels
// and channels is taken through the filter and the softmax to the logits
// (dl_k = w_k (dw_k - sum_j w_j dw_j), dw_k = sum_c g_c r_c(tap k)), stored
// as BF16 [P][kPredCh] (zero beyond the taps).
// kTile (W a multiple of the 256-pixel block, so a block is one run of one
// image row): the block first stages the RGB of its kKpWidth clamped rows x
// (256 + kKpWidth - 1) clamped columns in shared memory, once, instead of
// every pixel reading its 25 taps twice through L1.
constexpr int kKpBlock = 256, kKpTileW = kKpBlock + kKpWidth - 1;

template <bool kTile>
__global__ void __launch_bounds__(kKpBlock) k_kp_loss(const float* __restrict__ pred, const float* __restrict__ raw,
                                                      const float* __restrict__ target, bf16* __restrict__ dpred,
                                                      int N, int H, int W, double* loss) {
  __shared__ float tile[kTile ? kKpWidth : 1][kTile ? kKpTileW : 1][3];
  const long long P = (long long)N * H * W;
  long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (kTile) {
    constexpr int r = kKpWidth / 2;
    const long long pb = blockIdx.x * (long long)blockDim.x;
    const int x0 = (int)(pb % W);
    const long long qb = pb / W;
    const int yb = (int)(qb % H);
    const long long fb = (qb / H) * (long long)H * W;
    for (int e = threadIdx.x; e < kKpWidth * kKpTileW; e += blockDim.x) {
      const int rr = e / kKpTileW, cc = e - rr * kKpTileW;
      const int ty = min(max(yb + rr - r, 0), H - 1), tx = min(max(x0 + cc - r, 0), W - 1);
      raw_rgb(raw, fb + (long long)ty * W + tx, tile[rr][cc]);
    }
    __syncthreads();
  }
  // tap k of this pixel: from the staged tile, or through kp_tap
  auto tap = [&](long long frame0, int x, int y, int k, float* c) {
    if (kTile) {
      const float* t = tile[k / kKpWidth][threadIdx.x + k % kKpWidth];
      c[0] = t[0];
      c[1] = t[1];
      c[2] = t[2];
    } else {
      raw_rgb(raw, kp_tap(frame0, x, y, k, W, H, W), c);
    }
  };
  float part = 0.0f;
  if (p < P) {
    const int x = (int)(p % W);
    const long long q = p / W;
    const int y = (int)(q % H);
    const long long frame0 = (q / H) * (long long)H * W;
    float w[kKpTaps];
    kp_weights(pred + (long long)kPredCh * p, w);
    float o[3] = {0.0f, 0.0f, 0.0f};
#pragma unroll
    for (int k = 0; k < kKpTaps; ++k) {
      float c[3];
      tap(frame0, x, y, k, c);
      o[0] += w[k] * c[0];
      o[1] += w[k] * c[1];
      o[2] += w[k] * c[2];
    }
    const float inv = 1.0f / (3.0f * (float)P);
    float g[3];
    for (int i = 0; i < 3; ++i) {
      const float d = o[i] - sane(target[3 * p + i]);
      const float den = o[i] * o[i] + kRelEps;
      part += d * d / den;
      g[i] = 2.0f * d / den * inv;
    }
    float dw[kKpTaps], s = 0.0f;
#pragma unroll
    for (int k = 0; k < kKpTaps; ++k) {
      float c[3];
      tap(frame0, x, y, k, c);
      dw[k] = g[0] * c[0] + g[1] * c[1] + g[2] * c[2];
      s += w[k] * dw[k];
    }
    float dl[kPredCh];
#pragma unroll
    for (int k = 0; k < kPredCh; ++k) dl[k] = k < kKpTaps ? w[k] * (dw[k] - s) : 0.0f;
#pragma unroll
    for (int k = 0; k < kPredCh; k += 8) st8(dpred + (long long)kPredCh * p + k, dl + k);
  }
  for (int o = 16; o > 0; o >>= 1) part += __shfl_down_sync(0xffffffffu, part, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss, (double)part);
}

// db[c] += sum_p dout[p, c].  Thread t of a 256-thread block owns the
// 8-channel group t % (C / 8) and walks pixels t / (C / 8), + 256 / (C / 8),
// ... of the block's range; the block then sums its partials in shared memory
// and adds one value per channel (C <= 256).
__device__ __forceinline__ void bias_grad_block(const bf16* __restrict__ dout, long long P, int C,
                                                long long per_block, int block, float* __restrict__ db) {
  __shared__ float part[256][9];
  const int groups = C >> 3, lanes = 256 / groups, tid = threadIdx.x;
  const int g = tid % groups, l = tid / groups;
  float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0}, v[8];
  if (l < lanes) {
    long long p0 = block * per_block, p1 = min(P, p0 + per_block);
    for (long long p = p0 + l; p < p1; p += lanes) {
      ld8(dout + p * C + 8 * g, v);
#pragma unroll
      for (int k = 0; k < 8; ++k) acc[k] += v[k];
    }
  }
#pragma unroll
  for (int k = 0; k < 8; ++k) part[tid][k] = acc[k];
  __syncthreads();
  if (tid < C) {
    int gg = tid >> 3, k = tid & 7;
    float s = 0.0f;
    for (int j = 0; j < lanes; ++j) s += part[j * groups + gg][k];
    atomicAdd(db + tid, s);
  }
}

__global__ void __launch_bounds__(256) k_bias_grad(const bf16* __restrict__ dout, long long P, int C,
                                                   long long per_block, float* __restrict__ db) {
  bias_grad_block(dout, P, C, per_block, blockIdx.x, db);
}

// Every layer's bias gradient in one launch: blockIdx.y picks the layer,
// blockIdx.x its pixel range (blocks past a layer's own count return).
__global__ void __launch_bounds__(256) k_bias_grads(BiasGrads j) {
  const int i = blockIdx.y;
  if ((long long)blockIdx.x * j.per_block[i] >= j.P[i]) return;
  bias_grad_block(j.dout[i], j.P[i], j.C[i], j.per_block[i], blockIdx.x, j.db[i]);
}

// Adam (Kingma & Ba) on the FP32 master parameters
__global__ void k_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, long long n, float lr, float b1, float b2, float eps,
                       float c1, float c2) {
  long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  float gi = g[i];
  float mi = b1 * m[i] + (1.0f - b1) * gi;
  float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

// master [Cout][9][Cin] FP32 -> w [Cout][9][Cin] and wt [Cin][9][Cout] BF16
__device__ __forceinline__ void weight_bf16(const float* __restrict__ master, bf16* __restrict__ w,
                                            bf16* __restrict__ wt, int Cout, int Cin, long long i) {
  long long n = (long long)Cout * 9 * Cin;
  if (i >= n) return;
  int c = (int)(i % Cin);
  long long r = i / Cin;
  int t = (int)(r % 9);
  int o = (int)(r / 9);
  bf16 b = __float2bfloat16_rn(master[i]);
  w[i] = b;
  if (wt) wt[((size_t)c * 9 + t) * Cout + o] = b;
}

__global__ void k_weights_bf16(const float* __restrict__ master, bf16* __restrict__ w, bf16* __restrict__ wt,
                               int Cout, int Cin) {
  weight_bf16(master, w, wt, Cout, Cin, blockIdx.x * (long long)blockDim.x + threadIdx.x);
}

// Every layer's BF16 weights and transposes in one launch (blockIdx.y = layer)
__global__ void k_weights_bf16_all(WeightLayouts j) {
  const int l = blockIdx.y;
  weight_bf16(j.master[l], j.w[l], j.wt[l], j.Cout[l], j.Cin[l], blockIdx.x * (long long)blockDim.x + threadIdx.x);
}

// The denoised radiance: the predicted filter applied to the input radiance,
// for N frames of Hc x Wc pixels stored as Hs x Ws (the frame is the top-left
// corner; taps are clamped to it); out [N][Hc][Wc][3].
__global__ void k_kp_apply(const float* __restrict__ pred, const float* __restrict__ raw, float* __restrict__ out,
                           int N, int Hc, int Wc, int Hs, int Ws) {
  const long long P = (long long)N * Hc * Wc;
  long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= P) return;
  const int x = (int)(i % Wc);
  const long long q = i / Wc;
  const int y = (int)(q % Hc);
  const long long frame0 = (q / Hc) * (long long)Hs * Ws;
  const long long p = frame0 + (long long)y * Ws + x;
  float w[kKpTaps];
  kp_weights(pred + (long long)kPredCh * p, w);
  float o[3] = {0.0f, 0.0f, 0.0f};
#pragma unroll
  for (int k = 0; k < kKpTaps; ++k) {
    float c[3];
    raw_rgb(raw, kp_tap(frame0, x, y, k, Wc, Hc, Ws), c);
    o[0] += w[k] * c[0];
    o[1] += w[k] * c[1];
    o[2] += w[k] * c[2];
  }
  out[3 * i] = o[0];
  out[3 * i + 1] = o[1];
  out[3 * i + 2] = o[2];
}

// the renderer's passes (W x H RGB FP32 each) + their samples per pixel ->
// raw [Hp][Wp][kRawCh], zero outside the W x H frame
__global__ void k_pack_passes(const float* __restrict__ rad, const float* __restrict__ alb,
                              const float* __restrict__ nrm, const float* __restrict__ dep, float spp,
                              float* __restrict__ raw, int W, int H, int Wp, int Hp) {
  long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= (long long)Wp * Hp) return;
  int x = (int)(i % Wp), y = (int)(i / Wp);
  float* r = raw + (long long)kRawCh * i;
  if (x >= W || y >= H) {
    for (int k = 0; k < kRawCh; ++k) r[k] = 0.0f;
    return;
  }
  long long s = ((long long)y * W + x) * 3;
  for (int k = 0; k < 3; ++k) {
    r[k] = rad[s + k];
    r[3 + k] = alb[s + k];
    r[6 + k] = nrm[s + k];
  }
  r[9] = dep[s];
  r[10] = spp;
}

// prediction [Hp][Wp][16] (log space) -> radiance W x H RGB
// ---- launchers ------------------------------------------------------------
cudaError_t encode_input(const float* raw, bf16* x, long long P, cudaStream_t st) {
  k_encode_input<<<blocks(P), 256, 0, st>>>(raw, x, P);
  return cudaGetLastError();
}
cudaError_t avgpool(const bf16* in, bf16* out, int N, int H, int W, int C, cudaStream_t st) {
  long long n = (long long)N * (H / 2) * (W / 2) * (C / 8);
  k_avgpool<<<blocks(n), 256, 0, st>>>(in, out, N, H, W, C);
  return cudaGetLastError();
}
cudaError_t upsample_grad(const bf16* dcat, int Ccat, int c0, bf16* dlow, int N, int H, int W, int C,
                          cudaStream_t st) {
  long long n = (long long)N * (H / 2) * (W / 2) * (C / 8);
  k_upsample_grad<<<blocks(n), 256, 0, st>>>(dcat, Ccat, c0, dlow, N, H, W, C);
  return cudaGetLastError();
}
cudaError_t take_channels(const bf16* dcat, int Ccat, int c0, bf16* dst, long long P, int C, cudaStream_t st) {
  k_take_channels<<<blocks(P * (C / 8)), 256, 0, st>>>(dcat, Ccat, c0, dst, P, C);
  return cudaGetLastError();
}
cudaError_t pool_grad_acc(const bf16* dpool, const bf16* skip, bf16* dskip, int N, int H, int W, int C,
                          cudaStream_t st) {
  long long n = (long long)N * H * W * (C / 8);
  k_pool_grad_acc<<<blocks(n), 256, 0, st>>>(dpool, skip, dskip, N, H, W, C);
  return cudaGetLastError();
}
cudaError_t kp_loss(const float* pred, const float* raw, const float* target, bf16* dpred, int N, int H,
                    int W, double* loss, cudaStream_t st) {
  if (W % kKpBlock == 0)
    k_kp_loss<true><<<blocks((long long)N * H * W), kKpBlock, 0, st>>>(pred, raw, target, dpred, N, H, W, loss);
  else
    k_kp_loss<false><<<blocks((long long)N * H * W), kKpBlock, 0, st>>>(pred, raw, target, dpred, N, H, W, loss);
  return cudaGetLastError();
}
cudaError_t bias_grad(const bf16* dout, long long P, int C, float* db, cudaStream_t st) {
  if (C % 8 || C > 256) return cudaErrorInvalidValue;
  long long nb = std::min<long long>(2 * 152, (P + 255) / 256);
  long long per = (P + nb - 1) / nb;
  k_bias_grad<<<(unsigned)nb, 256, 0, st>>>(dout, P, C, per, db);
  return cudaGetLastError();
}
cudaError_t bias_grads(BiasGrads j, cudaStream_t st) {
  if (j.n <= 0 || j.n > BiasGrads::kMax) return cudaErrorInvalidValue;
  long long nbmax = 1;
  for (int i = 0; i < j.n; ++i) {
    if (j.C[i] % 8 || j.C[i] > 256) return cudaErrorInvalidValue;
    const long long nb = std::min<long long>(2 * 152, (j.P[i] + 255) / 256);
    j.per_block[i] = (j.P[i] + nb - 1) / nb;
    nbmax = std::max(nbmax, nb);
  }
  k_bias_grads<<<dim3((unsigned)nbmax, (unsigned)j.n), 256, 0, st>>>(j);
  return cudaGetLastError();
}
cudaError_t adam(float* p, const float* g, float* m, float* v, long long n, float lr, int step,
                 cudaStream_t st) {
  const float b1 = 0.9f, b2 = 0.999f;
  float c1 = 1.0f - powf(b1, (float)step), c2 = 1.0f - powf(b2, (float)step);
  k_adam<<<blocks(n), 256, 0, st>>>(p, g, m, v, n, lr, b1, b2, 1e-8f, c1, c2);
  return cudaGetLastError();
}
cudaError_t weights_bf16(const float* master, bf16* w, bf16* wt, int Cout, int Cin, cudaStream_t st) {
  k_weights_bf16<<<blocks((long long)Cout * 9 * Cin), 256, 0, st>>>(master, w, wt, Cout, Cin);
  return cudaGetLastError();
}
cudaError_t weights_bf16_all(const WeightLayouts& j, cudaStream_t st) {
  if (j.n <= 0 || j.n > WeightLayouts::kMax) return cudaErrorInvalidValue;
  long long nmax = 1;
  for (int l = 0; l < j.n; ++l) nmax = std::max(nmax, (long long)j.Cout[l] * 9 * j.Cin[l]);
  k_weights_bf16_all<<<dim3(blocks(nmax), (unsigned)j.n), 256, 0, st>>>(j);
  return cudaGetLastError();
}
cudaError_t kp_apply(const float* pred, const float* raw, float* out, int N, int Hc, int Wc, int Hs, int Ws,
                     cudaStream_t st) {
  k_kp_apply<<<blocks((long long)N * Hc * Wc), 256, 0, st>>>(pred, raw, out, N, Hc, Wc, Hs, Ws);
  return cudaGetLastError();
}

cudaError_t pack_passes(const float* rad, const float* alb, const float* nrm, const float* dep, float spp,
                        float* raw, int W, int H, int Wp, int Hp, cudaStream_t st) {
  k_pack_passes<<<blocks((long long)Wp * Hp), 256, 0, st>>>(rad, alb, nrm, dep, spp, raw, W, H, Wp, Hp);
  return cudaGetLastError();
}

}  // namespace nn
}  // namespace rtx
