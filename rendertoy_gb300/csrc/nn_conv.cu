// nn_conv.cu — 3 x 3 convolutions of the denoiser as implicit GEMMs on the
// tcgen05 tensor cores (BF16 operands, FP32 accumulation in TMEM).
//
// Tensors are NHWC BF16 with channel counts padded to multiples of 8.  A
// convolution reads one or two sources: s1 (optionally at half resolution,
// upsampled by nearest neighbour on the fly) and s2 (a skip connection,
// concatenated after s1's channels); neither the upsampled nor the
// concatenated tensor is ever materialised.
//
//   forward : out[p, o]  = relu?(bias[o] + sum_{t, c} src[p + off(t), c] w[o, t, c])
//             GEMM M = pixels (128 per CTA), N = Cout (<= 256), K = 9 * Cin
//   dgrad   : din[p, c]  = mask(p, c) * sum_{t, o} dout[p - off(t), o] w[o, t, c]
//             GEMM M = pixels, N = Cin (tiles of <= 256), K = 9 * Cout, with
//             the weights re-laid out as wt[c, t, o]; mask = (src > 0) when
//             the source is a ReLU output
//   wgrad   : dw[o, t, c] += sum_p dout[p, o] src[p + off(t), c]
//             GEMM M = 9 * Cin (128 (t, c) rows per CTA), N = Cout (<= 256),
//             K = the CTA's range of pixels; both operands staged MN-major
//             (16-byte chunks = 8 channels of one pixel); FP32 atomics
//             combine the ranges
// off(t) = (t / 3 - 1, t % 3 - 1).  Out-of-image taps read zero ("same"
// zero padding).
#include <algorithm>

#include "nn.h"
#include "tc_core.cuh"

namespace rtx {
namespace nn {

namespace {

constexpr int kSlice = 64;  // K per shared-memory slice

struct Pix {
  int n, y, x;
};

__device__ __forceinline__ Pix pix_of(long long p, int H, int W) {
  Pix r;
  int hw = H * W;
  r.n = (int)(p / hw);
  int rem = (int)(p - (long long)r.n * hw);
  r.y = rem / W;
  r.x = rem - r.y * W;
  return r;
}

// 8 channels [c, c + 8) of the (virtually concatenated, upsampled) source at
// pixel (n, y, x) of the full-resolution grid; zero outside the image.
__device__ __forceinline__ uint4 src_chunk(const Src& s1, const Src& s2, int N, int H, int W, int n,
                                           int y, int x, int c) {
  uint4 v = make_uint4(0, 0, 0, 0);
  if (y < 0 || y >= H || x < 0 || x >= W) return v;
  if (c < s1.C) {
    if (s1.up) {
      size_t off = (((size_t)n * (H >> 1) + (y >> 1)) * (W >> 1) + (x >> 1)) * s1.C + c;
      v = *reinterpret_cast<const uint4*>(s1.ptr + off);
    } else {
      v = *reinterpret_cast<const uint4*>(s1.ptr + (((size_t)n * H + y) * W + x) * s1.C + c);
    }
  } else if (s2.ptr) {
    int cc = c - s1.C;
    v = *reinterpret_cast<const uint4*>(s2.ptr + (((size_t)n * H + y) * W + x) * s2.C + cc);
  }
  return v;
}

__device__ __forceinline__ void bf16x8_to_f32(uint4 u, float* f) {
  const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&u);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    float2 t = __bfloat1622float2(h[i]);
    f[2 * i] = t.x;
    f[2 * i + 1] = t.y;
  }
}

__device__ __forceinline__ uint4 f32_to_bf16x8(const float* f) {
  uint4 u;
  __nv_bfloat162* h = reinterpret_cast<__nv_bfloat162*>(&u);
#pragma unroll
  for (int i = 0; i < 4; ++i) h[i] = __floats2bfloat162_rn(f[2 * i], f[2 * i + 1]);
  return u;
}

// Shared set-up of a tensor-core CTA: TMEM columns and the MMA barrier.
struct TcCta {
  uint32_t tmem;
  uint32_t phase;
};

__device__ __forceinline__ void tc_begin(uint32_t* tmem_slot, uint64_t* bar, uint32_t ncols) {
  if ((threadIdx.x >> 5) == 0) tc::tmem_alloc(tmem_slot, ncols);
  if (threadIdx.x == 0) {
    tc::mbar_init(bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
}

__device__ __forceinline__ void tc_end(uint32_t tmem, uint32_t ncols) {
  tc::fence_before();
  __syncthreads();
  if ((threadIdx.x >> 5) == 0) tc::tmem_dealloc(tmem, ncols);
}

// Issue the slice's MMAs (K-major A and B tiles of kSlice K) and wait.
__device__ __forceinline__ bool tc_slice_kmajor(uint8_t* sa, uint8_t* sb, uint32_t tmem, uint32_t idesc,
                                                bool first, uint64_t* bar, uint32_t& phase, int* err) {
  tc::fence_proxy_async();
  __syncthreads();
  if (threadIdx.x == 0) {
    tc::fence_after();
    uint32_t a0 = tc::smem_u32(sa), b0 = tc::smem_u32(sb);
#pragma unroll
    for (int s = 0; s < kSlice / 16; ++s)
      tc::mma_bf16(tmem, tc::make_desc(a0 + s * 256, 128, kSlice * 16),
                   tc::make_desc(b0 + s * 256, 128, kSlice * 16), idesc, !first || s > 0);
    tc::mma_commit(bar);
  }
  bool ok = tc::mbar_wait(bar, phase);
  phase ^= 1;
  if (!ok && (threadIdx.x & 31) == 0) atomicOr(err, tc::kErrMbarTimeout);
  __syncthreads();
  return ok;
}

}  // namespace

// ---------------------------------------------------------------------------
// forward
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128) k_conv_fwd(ConvFwd a) {
  extern __shared__ __align__(1024) uint8_t smem[];
  uint8_t* sa = smem;                      // 128 x 64 K-major
  uint8_t* sb = smem + 128 * kSlice * 2;   // Cout x 64 K-major
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t tmem_slot;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const long long P = (long long)a.N * a.H * a.W;
  const long long m0 = (long long)blockIdx.x * 128;
  const uint32_t ncols = a.Cout <= 32 ? 32 : (a.Cout <= 64 ? 64 : (a.Cout <= 128 ? 128 : 256));
  tc_begin(&tmem_slot, &bar, ncols);
  const uint32_t tmem = tmem_slot;
  const uint32_t idesc = tc::make_idesc_bf16(128, a.Cout);
  uint32_t phase = 0;
  const int K = 9 * a.Cin;
  // this thread's 8 tile rows (tid >> 3) + 16 i and its chunk column tid & 7
  const int kc = tid & 7;
  Pix px[8];
  bool pv[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    long long p = m0 + (tid >> 3) + 16 * i;
    pv[i] = p < P;
    px[i] = pix_of(pv[i] ? p : 0, a.H, a.W);
  }
  bool ok = true;
  for (int k0 = 0; k0 < K && ok; k0 += kSlice) {
    int k = k0 + kc * 8;
    int t = k / a.Cin, c = k - t * a.Cin;
    int dy = t / 3 - 1, dx = t % 3 - 1;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      int row = (tid >> 3) + 16 * i;
      uint4 v = make_uint4(0, 0, 0, 0);
      if (pv[i] && k < K) v = src_chunk(a.s1, a.s2, a.N, a.H, a.W, px[i].n, px[i].y + dy, px[i].x + dx, c);
      *reinterpret_cast<uint4*>(sa + tc::tile_offset(row, kc * 8, kSlice)) = v;
    }
    for (int ch = tid; ch < a.Cout * 8; ch += 128) {
      int row = ch >> 3, kk = (ch & 7) * 8;
      uint4 v = make_uint4(0, 0, 0, 0);
      if (k0 + kk < K) v = *reinterpret_cast<const uint4*>(a.w + (size_t)row * K + k0 + kk);
      *reinterpret_cast<uint4*>(sb + tc::tile_offset(row, kk, kSlice)) = v;
    }
    ok = tc_slice_kmajor(sa, sb, tmem, idesc, k0 == 0, &bar, phase, a.err);
  }
  tc::fence_after();
  if (ok) {
    const long long p = m0 + warp * 32 + lane;
    const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16);
    for (int c0 = 0; c0 < a.Cout; c0 += 8) {
      float v[8];
      tc::tmem_ld8(taddr + c0, v);
      if (p < P) {
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          if (a.bias) v[i] += a.bias[c0 + i];
          if (a.relu) v[i] = fmaxf(v[i], 0.0f);
        }
        if (a.out) *reinterpret_cast<uint4*>(a.out + (size_t)p * a.Cout + c0) = f32_to_bf16x8(v);
        if (a.out_f32)
#pragma unroll
          for (int i = 0; i < 8; ++i) a.out_f32[(size_t)p * a.Cout + c0 + i] = v[i];
      }
    }
  }
  tc_end(tmem, ncols);
}

// ---------------------------------------------------------------------------
// data gradient
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128) k_conv_dgrad(ConvDgrad a) {
  extern __shared__ __align__(1024) uint8_t smem[];
  uint8_t* sa = smem;
  uint8_t* sb = smem + 128 * kSlice * 2;
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t tmem_slot;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const long long P = (long long)a.N * a.H * a.W;
  const long long m0 = (long long)blockIdx.x * 128;
  const int n0 = blockIdx.y * 256;
  const int NT = min(256, a.Cin - n0);  // output channels of this CTA
  const uint32_t ncols = NT <= 32 ? 32 : (NT <= 64 ? 64 : (NT <= 128 ? 128 : 256));
  tc_begin(&tmem_slot, &bar, ncols);
  const uint32_t tmem = tmem_slot;
  const uint32_t idesc = tc::make_idesc_bf16(128, NT);
  uint32_t phase = 0;
  const int K = 9 * a.Cout;
  const int kc = tid & 7;
  Pix px[8];
  bool pv[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    long long p = m0 + (tid >> 3) + 16 * i;
    pv[i] = p < P;
    px[i] = pix_of(pv[i] ? p : 0, a.H, a.W);
  }
  bool ok = true;
  for (int k0 = 0; k0 < K && ok; k0 += kSlice) {
    int k = k0 + kc * 8;
    int t = k / a.Cout, o = k - t * a.Cout;
    int dy = t / 3 - 1, dx = t % 3 - 1;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      int row = (tid >> 3) + 16 * i;
      uint4 v = make_uint4(0, 0, 0, 0);
      int yy = px[i].y - dy, xx = px[i].x - dx;
      if (pv[i] && k < K && yy >= 0 && yy < a.H && xx >= 0 && xx < a.W)
        v = *reinterpret_cast<const uint4*>(a.dout + (((size_t)px[i].n * a.H + yy) * a.W + xx) * a.Cout + o);
      *reinterpret_cast<uint4*>(sa + tc::tile_offset(row, kc * 8, kSlice)) = v;
    }
    for (int ch = tid; ch < NT * 8; ch += 128) {
      int row = ch >> 3, kk = (ch & 7) * 8;
      uint4 v = make_uint4(0, 0, 0, 0);
      if (k0 + kk < K) v = *reinterpret_cast<const uint4*>(a.wt + (size_t)(n0 + row) * K + k0 + kk);
      *reinterpret_cast<uint4*>(sb + tc::tile_offset(row, kk, kSlice)) = v;
    }
    ok = tc_slice_kmajor(sa, sb, tmem, idesc, k0 == 0, &bar, phase, a.err);
  }
  tc::fence_after();
  if (ok) {
    const long long p = m0 + warp * 32 + lane;
    const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16);
    Pix q = pix_of(p < P ? p : 0, a.H, a.W);
    for (int c0 = 0; c0 < NT; c0 += 8) {
      float v[8];
      tc::tmem_ld8(taddr + c0, v);
      if (p < P) {
        if (a.mask_relu) {
          float s[8];
          bf16x8_to_f32(src_chunk(a.s1, a.s2, a.N, a.H, a.W, q.n, q.y, q.x, n0 + c0), s);
#pragma unroll
          for (int i = 0; i < 8; ++i)
            if (!(s[i] > 0.0f)) v[i] = 0.0f;
        }
        *reinterpret_cast<uint4*>(a.din + (size_t)p * a.Cin + n0 + c0) = f32_to_bf16x8(v);
      }
    }
  }
  tc_end(tmem, ncols);
}

// ---------------------------------------------------------------------------
// weight gradient
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128) k_conv_wgrad(ConvWgrad a) {
  extern __shared__ __align__(1024) uint8_t smem[];
  uint8_t* sa = smem;                     // 128 (t, c) x 64 (pixels), MN-major
  uint8_t* sb = smem + 128 * kSlice * 2;  // Cout x 64 (pixels), MN-major
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t tmem_slot;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int P = a.N * a.H * a.W;  // < 2^31 (checked by the host)
  const int J = 9 * a.Cin;
  const int j0 = blockIdx.x * 128;
  const int pb = blockIdx.y * a.pix_per_cta;
  const int pe = min(P, pb + a.pix_per_cta);
  const uint32_t ncols = a.Cout <= 32 ? 32 : (a.Cout <= 64 ? 64 : (a.Cout <= 128 ? 128 : 256));
  tc_begin(&tmem_slot, &bar, ncols);
  const uint32_t tmem = tmem_slot;
  const uint32_t idesc = tc::make_idesc_bf16(128, a.Cout, true, true);
  uint32_t phase = 0;
  // this thread's 8 rows of the A tile: (tap, channel) j = j0 + 8 rg
  const int rg = tid & 15;
  const int j = j0 + rg * 8;
  const bool jv = j < J;
  const int t = jv ? j / a.Cin : 0, c = jv ? j - t * a.Cin : 0;
  const int dy = t / 3 - 1, dx = t % 3 - 1;
  const int HW = a.H * a.W;
  const int ng = a.Cout >> 3;
  bool ok = true;
  for (int q0 = pb; q0 < pe && ok; q0 += kSlice) {
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      int kp = (tid >> 4) + 8 * i;  // pixel within the slice
      int p = q0 + kp;
      uint4 v = make_uint4(0, 0, 0, 0);
      if (p < pe && jv) {
        int n = p / HW, rem = p - n * HW;
        int y = rem / a.W, x = rem - y * a.W;
        v = src_chunk(a.s1, a.s2, a.N, a.H, a.W, n, y + dy, x + dx, c);
      }
      *reinterpret_cast<uint4*>(sa + tc::tile_offset_mn(rg * 8, kp, 128)) = v;
    }
    for (int ch = tid; ch < ng * kSlice; ch += 128) {
      int og = ch % ng, kp = ch / ng;
      int p = q0 + kp;
      uint4 v = make_uint4(0, 0, 0, 0);
      if (p < pe) v = *reinterpret_cast<const uint4*>(a.dout + (size_t)p * a.Cout + og * 8);
      *reinterpret_cast<uint4*>(sb + tc::tile_offset_mn(og * 8, kp, a.Cout)) = v;
    }
    tc::fence_proxy_async();
    __syncthreads();
    if (tid == 0) {
      tc::fence_after();
      uint32_t a0 = tc::smem_u32(sa), b0 = tc::smem_u32(sb);
#pragma unroll
      for (int s = 0; s < kSlice / 16; ++s)
        tc::mma_bf16(tmem, tc::make_desc(a0 + s * 2 * 16 * 128, 16 * 128, 128),
                     tc::make_desc(b0 + s * 2 * 16 * a.Cout, 16 * a.Cout, 128), idesc, q0 > pb || s > 0);
      tc::mma_commit(&bar);
    }
    ok = tc::mbar_wait(&bar, phase);
    phase ^= 1;
    if (!ok && lane == 0) atomicOr(a.err, tc::kErrMbarTimeout);
    __syncthreads();
  }
  tc::fence_after();
  if (ok && pe > pb) {
    const int jj = j0 + warp * 32 + lane;  // this thread's accumulator row
    const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16);
    for (int c0 = 0; c0 < a.Cout; c0 += 8) {
      float v[8];
      tc::tmem_ld8(taddr + c0, v);
      if (jj < J)
#pragma unroll
        for (int i = 0; i < 8; ++i) atomicAdd(a.dw + (size_t)(c0 + i) * J + jj, v[i]);
    }
  }
  tc_end(tmem, ncols);
}

// ---------------------------------------------------------------------------
cudaError_t conv_fwd(const ConvFwd& a, cudaStream_t st) {
  long long P = (long long)a.N * a.H * a.W;
  size_t smem = 128 * kSlice * 2 + (size_t)a.Cout * kSlice * 2;
  cudaError_t e = cudaFuncSetAttribute(k_conv_fwd, cudaFuncAttributeMaxDynamicSharedMemorySize, 64 * 1024);
  if (e) return e;
  k_conv_fwd<<<(unsigned)((P + 127) / 128), 128, smem, st>>>(a);
  return cudaGetLastError();
}

cudaError_t conv_dgrad(const ConvDgrad& a, cudaStream_t st) {
  long long P = (long long)a.N * a.H * a.W;
  size_t smem = 128 * kSlice * 2 + 256 * kSlice * 2;
  cudaError_t e = cudaFuncSetAttribute(k_conv_dgrad, cudaFuncAttributeMaxDynamicSharedMemorySize, 64 * 1024);
  if (e) return e;
  dim3 grid((unsigned)((P + 127) / 128), (a.Cin + 255) / 256);
  k_conv_dgrad<<<grid, 128, smem, st>>>(a);
  return cudaGetLastError();
}

int wgrad_pixels_per_cta(long long P, int Cout, int Cin) {
  (void)Cout;
  int tiles = (9 * Cin + 127) / 128;
  long long ranges = std::max(1, 8 * 152 / tiles);
  long long per = (P + ranges - 1) / ranges;
  per = (per + 63) / 64 * 64;
  return (int)std::max(64LL, std::min(per, 1LL << 30));
}

cudaError_t conv_wgrad(const ConvWgrad& a, cudaStream_t st) {
  long long P = (long long)a.N * a.H * a.W;
  if (P >= (1LL << 31) || a.Cout % 16 || a.Cout > 256) return cudaErrorInvalidValue;
  size_t smem = 128 * kSlice * 2 + (size_t)a.Cout * kSlice * 2;
  cudaError_t e = cudaFuncSetAttribute(k_conv_wgrad, cudaFuncAttributeMaxDynamicSharedMemorySize, 64 * 1024);
  if (e) return e;
  dim3 grid((9 * a.Cin + 127) / 128, (unsigned)((P + a.pix_per_cta - 1) / a.pix_per_cta));
  k_conv_wgrad<<<grid, 128, smem, st>>>(a);
  return cudaGetLastError();
}

}  // namespace nn
}  // namespace rtx
