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
//
// Pipeline (all three): the K (or pixel) range is cut into slices of 64;
// every thread copies its 16-byte chunks of a slice straight into shared
// memory with cp.async (zero-filled where the tap falls outside the image),
// S - 1 slices ahead, into a ring of S stages.  Thread 0 issues the slice's
// MMAs and commits them to the stage's mbarrier; a stage is refilled once the
// MMAs that read it have completed.  The gathers of later slices therefore
// overlap the MMAs of earlier ones, and no thread stalls on its own loads.
#include <algorithm>

#include "nn.h"
#include "tc_core.cuh"

namespace rtx {
namespace nn {

namespace {

constexpr int kSlice = 64;    // K per shared-memory slice
constexpr int kThreads = 256;  // 8 warps: all gather, warps w and w + 4 share accumulator lanes

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

// Address of 8 channels [c, c + 8) of the (virtually concatenated,
// upsampled) source at pixel (n, y, x), or nullptr outside the image.
__device__ __forceinline__ const bf16* src_ptr(const Src& s1, const Src& s2, int H, int W, int n, int y, int x,
                                               int c) {
  if (y < 0 || y >= H || x < 0 || x >= W) return nullptr;
  if (c < s1.C) {
    if (s1.up) return s1.ptr + (((size_t)n * (H >> 1) + (y >> 1)) * (W >> 1) + (x >> 1)) * s1.C + c;
    return s1.ptr + (((size_t)n * H + y) * W + x) * s1.C + c;
  }
  if (s2.ptr) return s2.ptr + (((size_t)n * H + y) * W + x) * s2.C + (c - s1.C);
  return nullptr;
}

// 16 bytes from p into shared address dst, zeros when p is null (`base` is a
// valid address the zero-fill form names but does not read)
__device__ __forceinline__ void chunk_async(uint32_t dst, const void* p, const void* base) {
  tc::cp_async16(dst, p ? p : base, p ? 16u : 0u);
}

// Shared set-up of a tensor-core CTA: TMEM columns and S MMA barriers.
__device__ __forceinline__ void tc_begin(uint32_t* tmem_slot, uint64_t* bars, int nbar, uint32_t ncols) {
  if ((threadIdx.x >> 5) == 0) tc::tmem_alloc(tmem_slot, ncols);
  if (threadIdx.x == 0) {
    for (int i = 0; i < nbar; ++i) tc::mbar_init(&bars[i], 1);
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

// The S-stage ring over n slices (see the file comment).  load(slice, stage)
// issues this thread's copies of a slice (nothing for slice >= n); mma(stage,
// first) is run by thread 0.  Returns false, uniformly across the CTA, when
// an MMA barrier wait ran out (error flag set); copies are drained either way.
template <int S, class Load, class Mma>
__device__ __forceinline__ bool conv_pipeline(int n, uint64_t* bars, Load&& load, Mma&& mma, int* err) {
  uint32_t parity = 0;
#pragma unroll
  for (int s = 0; s < S - 1; ++s) {
    load(s, s);
    tc::cp_async_commit();
  }
  bool wok = true, ok = true;
  for (int it = 0; it < n; ++it) {
    const int st = it % S;
    tc::cp_async_wait<S - 2>();  // this thread's copies of slice `it` landed
    tc::fence_proxy_async();
    if (!__syncthreads_and(wok)) {
      ok = false;
      break;
    }
    if (threadIdx.x == 0) {
      tc::fence_after();
      mma(st, it == 0);
      tc::mma_commit(&bars[st]);
    }
    if (it > 0) {  // the previous slice's MMAs free its stage for slice it + S - 1
      const int ps = (it - 1) % S;
      wok = tc::mbar_wait(&bars[ps], (parity >> ps) & 1u);
      parity ^= 1u << ps;
    }
    load(it + S - 1, (it + S - 1) % S);
    tc::cp_async_commit();
  }
  if (ok && n > 0) {
    const int ls = (n - 1) % S;
    const bool w = wok && tc::mbar_wait(&bars[ls], (parity >> ls) & 1u);
    ok = __syncthreads_and(w);
  }
  if (!ok && (threadIdx.x & 31) == 0) atomicOr(err, tc::kErrMbarTimeout);
  tc::cp_async_wait_all();
  return ok;
}

}  // namespace

// ---------------------------------------------------------------------------
// forward
// ---------------------------------------------------------------------------
template <int S>
__global__ void __launch_bounds__(kThreads, 2) k_conv_fwd(ConvFwd a) {
  extern __shared__ __align__(1024) uint8_t smem[];
  __shared__ __align__(8) uint64_t bars[S];
  __shared__ uint32_t tmem_slot;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const long long P = (long long)a.N * a.H * a.W;
  const long long m0 = (long long)blockIdx.x * 128;
  const uint32_t ncols = a.Cout <= 32 ? 32 : (a.Cout <= 64 ? 64 : (a.Cout <= 128 ? 128 : 256));
  const uint32_t a_bytes = 128 * kSlice * 2, stage = a_bytes + (uint32_t)a.Cout * kSlice * 2;
  tc_begin(&tmem_slot, bars, S, ncols);
  const uint32_t tmem = tmem_slot;
  const uint32_t idesc = tc::make_idesc_bf16(128, a.Cout);
  const uint32_t s0 = tc::smem_u32(smem);
  const int K = 9 * a.Cin;
  const int n_slices = (K + kSlice - 1) / kSlice;
  // this thread's 4 tile rows (tid >> 3) + 32 i and its chunk column tid & 7
  const int kc = tid & 7;
  Pix px[4];
  bool pv[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    long long p = m0 + (tid >> 3) + 32 * i;
    pv[i] = p < P;
    px[i] = pix_of(pv[i] ? p : 0, a.H, a.W);
  }
  auto load = [&](int slice, int st) {
    if (slice >= n_slices) return;
    const uint32_t sa = s0 + st * stage, sb = sa + a_bytes;
    const int k0 = slice * kSlice, k = k0 + kc * 8;
    const bool kv = k < K;
    const int t = kv ? k / a.Cin : 0, c = k - t * a.Cin;
    const int dy = t / 3 - 1, dx = t % 3 - 1;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int row = (tid >> 3) + 32 * i;
      const bf16* p = (pv[i] && kv) ? src_ptr(a.s1, a.s2, a.H, a.W, px[i].n, px[i].y + dy, px[i].x + dx, c) : nullptr;
      chunk_async(sa + tc::tile_offset(row, kc * 8, kSlice), p, a.s1.ptr);
    }
    for (int ch = tid; ch < a.Cout * 8; ch += kThreads) {
      const int row = ch >> 3, kk = (ch & 7) * 8;
      const bf16* p = k0 + kk < K ? a.w + (size_t)row * K + k0 + kk : nullptr;
      chunk_async(sb + tc::tile_offset(row, kk, kSlice), p, a.w);
    }
  };
  auto mma = [&](int st, bool first) {
    const uint32_t a0 = s0 + st * stage, b0 = a0 + a_bytes;
#pragma unroll
    for (int s = 0; s < kSlice / 16; ++s)
      tc::mma_bf16(tmem, tc::make_desc(a0 + s * 256, 128, kSlice * 16), tc::make_desc(b0 + s * 256, 128, kSlice * 16),
                   idesc, !first || s > 0);
  };
  const bool ok = conv_pipeline<S>(n_slices, bars, load, mma, a.err);
  tc::fence_after();
  if (ok) {
    // warp w reads accumulator lanes 32 (w % 4) .. + 31, half w / 4 of the columns
    const int lw = warp & 3, half = a.Cout >> 1;
    const long long p = m0 + lw * 32 + lane;
    const uint32_t taddr = tmem + ((uint32_t)(lw * 32) << 16);
    for (int c0 = (warp >> 2) * half; c0 < (warp >> 2) * half + half; c0 += 8) {
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
// forward, row tiles: a CTA takes 128 consecutive pixels of one image row.
// Per slice of 16 input channels it copies the 3-row halo (pixels x0 - 1 ..
// x0 + 128, 2 chunks of 8 channels each) once; the nine taps are the same
// halo read through descriptors shifted by whole pixels (rows of the
// K-major layout are 16 B apart and the two channel chunks one halo row
// apart, so every shift is a legal start address).  One third of the gather
// traffic of k_conv_fwd, with one address per copied pixel chunk.
// ---------------------------------------------------------------------------
constexpr int kHalo = 130;                                  // pixels x0 - 1 .. x0 + 128
constexpr uint32_t kHaloBytes = 3 * 2 * kHalo * 16;          // rows x chunks x pixels x 16 B

template <int S>
__global__ void __launch_bounds__(kThreads, 2) k_conv_fwd_row(ConvFwd a) {
  extern __shared__ __align__(1024) uint8_t smem[];
  __shared__ __align__(8) uint64_t bars[S];
  __shared__ uint32_t tmem_slot;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int x0 = blockIdx.x * 128, y = blockIdx.y, n = blockIdx.z;
  const uint32_t ncols = a.Cout <= 32 ? 32 : (a.Cout <= 64 ? 64 : (a.Cout <= 128 ? 128 : 256));
  const uint32_t tap_bytes = (uint32_t)a.Cout * 32, stage = kHaloBytes + 9 * tap_bytes;
  tc_begin(&tmem_slot, bars, S, ncols);
  const uint32_t tmem = tmem_slot;
  const uint32_t idesc = tc::make_idesc_bf16(128, a.Cout);
  const uint32_t s0 = tc::smem_u32(smem);
  const int n_slices = a.Cin / 16;
  auto load = [&](int slice, int st) {
    if (slice >= n_slices) return;
    const uint32_t sh = s0 + st * stage, sb = sh + kHaloBytes;
    const int c0 = slice * 16;
    // chunk c of pixel h of halo row r: neighbouring threads take the two
    // chunks of one pixel (32 contiguous bytes)
    for (int i = tid; i < 3 * kHalo * 2; i += kThreads) {
      const int c = i & 1, h = (i >> 1) % kHalo, r = (i >> 1) / kHalo;
      const bf16* p = src_ptr(a.s1, a.s2, a.H, a.W, n, y + r - 1, x0 + h - 1, c0 + 8 * c);
      chunk_async(sh + ((r * 2 + c) * kHalo + h) * 16, p, a.s1.ptr);
    }
    // tap t: Cout x 16 K-major tile of w[o][t][c0 .. c0 + 15]
    for (int i = tid; i < 9 * a.Cout * 2; i += kThreads) {
      const int kc = i & 1, o = (i >> 1) % a.Cout, t = (i >> 1) / a.Cout;
      chunk_async(sb + t * tap_bytes + tc::tile_offset(o, 8 * kc, 16), a.w + ((size_t)o * 9 + t) * a.Cin + c0 + 8 * kc,
                  a.w);
    }
  };
  auto mma = [&](int st, bool first) {
    const uint32_t sh = s0 + st * stage, sb = sh + kHaloBytes;
#pragma unroll
    for (int t = 0; t < 9; ++t) {
      const int dy = t / 3 - 1, dx = t % 3 - 1;
      // A: pixel groups 128 B apart (SBO), channel chunks one halo row apart (LBO)
      const uint64_t ad = tc::make_desc(sh + ((dy + 1) * 2 * kHalo + 1 + dx) * 16, kHalo * 16, 128);
      const uint64_t bd = tc::make_desc(sb + t * tap_bytes, 128, 256);
      tc::mma_bf16(tmem, ad, bd, idesc, !first || t > 0);
    }
  };
  const bool ok = conv_pipeline<S>(n_slices, bars, load, mma, a.err);
  tc::fence_after();
  if (ok) {
    const int lw = warp & 3, half = a.Cout >> 1;
    const int x = x0 + lw * 32 + lane;
    const size_t p = ((size_t)n * a.H + y) * a.W + x;
    const uint32_t taddr = tmem + ((uint32_t)(lw * 32) << 16);
    for (int c0 = (warp >> 2) * half; c0 < (warp >> 2) * half + half; c0 += 8) {
      float v[8];
      tc::tmem_ld8(taddr + c0, v);
      if (x < a.W) {
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          if (a.bias) v[i] += a.bias[c0 + i];
          if (a.relu) v[i] = fmaxf(v[i], 0.0f);
        }
        if (a.out) *reinterpret_cast<uint4*>(a.out + p * a.Cout + c0) = f32_to_bf16x8(v);
        if (a.out_f32)
#pragma unroll
          for (int i = 0; i < 8; ++i) a.out_f32[p * a.Cout + c0 + i] = v[i];
      }
    }
  }
  tc_end(tmem, ncols);
}

// data gradient, row tiles: din[p] = sum_t dout[p - off(t)] wt_t, the same
// halo scheme over dout (slices of 16 of its channels, shifts negated)
template <int S>
__global__ void __launch_bounds__(kThreads, 2) k_conv_dgrad_row(ConvDgrad a) {
  extern __shared__ __align__(1024) uint8_t smem[];
  __shared__ __align__(8) uint64_t bars[S];
  __shared__ uint32_t tmem_slot;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int x0 = blockIdx.x * 128, y = blockIdx.y;
  const int n = blockIdx.z / ((a.Cin + 255) / 256);
  const int n0 = (blockIdx.z % ((a.Cin + 255) / 256)) * 256;
  const int NT = min(256, a.Cin - n0);
  const uint32_t ncols = NT <= 32 ? 32 : (NT <= 64 ? 64 : (NT <= 128 ? 128 : 256));
  const uint32_t tap_bytes = (uint32_t)min(256, a.Cin) * 32, stage = kHaloBytes + 9 * tap_bytes;
  tc_begin(&tmem_slot, bars, S, ncols);
  const uint32_t tmem = tmem_slot;
  const uint32_t idesc = tc::make_idesc_bf16(128, NT);
  const uint32_t s0 = tc::smem_u32(smem);
  const int n_slices = a.Cout / 16;
  auto load = [&](int slice, int st) {
    if (slice >= n_slices) return;
    const uint32_t sh = s0 + st * stage, sb = sh + kHaloBytes;
    const int o0 = slice * 16;
    for (int i = tid; i < 3 * kHalo * 2; i += kThreads) {
      const int c = i & 1, h = (i >> 1) % kHalo, r = (i >> 1) / kHalo;
      const int yy = y + r - 1, xx = x0 + h - 1;
      const bf16* p = (yy >= 0 && yy < a.H && xx >= 0 && xx < a.W)
                          ? a.dout + (((size_t)n * a.H + yy) * a.W + xx) * a.Cout + o0 + 8 * c
                          : nullptr;
      chunk_async(sh + ((r * 2 + c) * kHalo + h) * 16, p, a.dout);
    }
    for (int i = tid; i < 9 * NT * 2; i += kThreads) {
      const int kc = i & 1, row = (i >> 1) % NT, t = (i >> 1) / NT;
      chunk_async(sb + t * tap_bytes + tc::tile_offset(row, 8 * kc, 16),
                  a.wt + ((size_t)(n0 + row) * 9 + t) * a.Cout + o0 + 8 * kc, a.wt);
    }
  };
  auto mma = [&](int st, bool first) {
    const uint32_t sh = s0 + st * stage, sb = sh + kHaloBytes;
#pragma unroll
    for (int t = 0; t < 9; ++t) {
      const int dy = t / 3 - 1, dx = t % 3 - 1;
      const uint64_t ad = tc::make_desc(sh + ((1 - dy) * 2 * kHalo + 1 - dx) * 16, kHalo * 16, 128);
      const uint64_t bd = tc::make_desc(sb + t * tap_bytes, 128, 256);
      tc::mma_bf16(tmem, ad, bd, idesc, !first || t > 0);
    }
  };
  const bool ok = conv_pipeline<S>(n_slices, bars, load, mma, a.err);
  tc::fence_after();
  if (ok) {
    const int lw = warp & 3, half = NT >> 1;
    const int x = x0 + lw * 32 + lane;
    const size_t p = ((size_t)n * a.H + y) * a.W + x;
    const uint32_t taddr = tmem + ((uint32_t)(lw * 32) << 16);
    for (int c0 = (warp >> 2) * half; c0 < (warp >> 2) * half + half; c0 += 8) {
      float v[8];
      tc::tmem_ld8(taddr + c0, v);
      if (x < a.W) {
        if (a.mask_relu) {
          float sv[8];
          bf16x8_to_f32(src_chunk(a.s1, a.s2, a.N, a.H, a.W, n, y, x, n0 + c0), sv);
#pragma unroll
          for (int i = 0; i < 8; ++i)
            if (!(sv[i] > 0.0f)) v[i] = 0.0f;
        }
        *reinterpret_cast<uint4*>(a.din + p * a.Cin + n0 + c0) = f32_to_bf16x8(v);
      }
    }
  }
  tc_end(tmem, ncols);
}

// ---------------------------------------------------------------------------
// data gradient
// ---------------------------------------------------------------------------
template <int S>
__global__ void __launch_bounds__(kThreads, 2) k_conv_dgrad(ConvDgrad a) {
  extern __shared__ __align__(1024) uint8_t smem[];
  __shared__ __align__(8) uint64_t bars[S];
  __shared__ uint32_t tmem_slot;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const long long P = (long long)a.N * a.H * a.W;
  const long long m0 = (long long)blockIdx.x * 128;
  const int n0 = blockIdx.y * 256;
  const int NT = min(256, a.Cin - n0);  // output channels of this CTA
  const uint32_t ncols = NT <= 32 ? 32 : (NT <= 64 ? 64 : (NT <= 128 ? 128 : 256));
  const uint32_t a_bytes = 128 * kSlice * 2, stage = a_bytes + (uint32_t)min(256, a.Cin) * kSlice * 2;
  tc_begin(&tmem_slot, bars, S, ncols);
  const uint32_t tmem = tmem_slot;
  const uint32_t idesc = tc::make_idesc_bf16(128, NT);
  const uint32_t s0 = tc::smem_u32(smem);
  const int K = 9 * a.Cout;
  const int n_slices = (K + kSlice - 1) / kSlice;
  const int kc = tid & 7;
  Pix px[4];
  bool pv[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    long long p = m0 + (tid >> 3) + 32 * i;
    pv[i] = p < P;
    px[i] = pix_of(pv[i] ? p : 0, a.H, a.W);
  }
  auto load = [&](int slice, int st) {
    if (slice >= n_slices) return;
    const uint32_t sa = s0 + st * stage, sb = sa + a_bytes;
    const int k0 = slice * kSlice, k = k0 + kc * 8;
    const bool kv = k < K;
    const int t = kv ? k / a.Cout : 0, o = k - t * a.Cout;
    const int dy = t / 3 - 1, dx = t % 3 - 1;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int row = (tid >> 3) + 32 * i;
      const int yy = px[i].y - dy, xx = px[i].x - dx;
      const bf16* p = (pv[i] && kv && yy >= 0 && yy < a.H && xx >= 0 && xx < a.W)
                          ? a.dout + (((size_t)px[i].n * a.H + yy) * a.W + xx) * a.Cout + o
                          : nullptr;
      chunk_async(sa + tc::tile_offset(row, kc * 8, kSlice), p, a.dout);
    }
    for (int ch = tid; ch < NT * 8; ch += kThreads) {
      const int row = ch >> 3, kk = (ch & 7) * 8;
      const bf16* p = k0 + kk < K ? a.wt + (size_t)(n0 + row) * K + k0 + kk : nullptr;
      chunk_async(sb + tc::tile_offset(row, kk, kSlice), p, a.wt);
    }
  };
  auto mma = [&](int st, bool first) {
    const uint32_t a0 = s0 + st * stage, b0 = a0 + a_bytes;
#pragma unroll
    for (int s = 0; s < kSlice / 16; ++s)
      tc::mma_bf16(tmem, tc::make_desc(a0 + s * 256, 128, kSlice * 16), tc::make_desc(b0 + s * 256, 128, kSlice * 16),
                   idesc, !first || s > 0);
  };
  const bool ok = conv_pipeline<S>(n_slices, bars, load, mma, a.err);
  tc::fence_after();
  if (ok) {
    const int lw = warp & 3, half = NT >> 1;
    const long long p = m0 + lw * 32 + lane;
    const uint32_t taddr = tmem + ((uint32_t)(lw * 32) << 16);
    Pix q = pix_of(p < P ? p : 0, a.H, a.W);
    for (int c0 = (warp >> 2) * half; c0 < (warp >> 2) * half + half; c0 += 8) {
      float v[8];
      tc::tmem_ld8(taddr + c0, v);
      if (p < P) {
        if (a.mask_relu) {
          float sv[8];
          bf16x8_to_f32(src_chunk(a.s1, a.s2, a.N, a.H, a.W, q.n, q.y, q.x, n0 + c0), sv);
#pragma unroll
          for (int i = 0; i < 8; ++i)
            if (!(sv[i] > 0.0f)) v[i] = 0.0f;
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
template <int S>
__global__ void __launch_bounds__(kThreads, 2) k_conv_wgrad(ConvWgrad a) {
  extern __shared__ __align__(1024) uint8_t smem[];
  __shared__ __align__(8) uint64_t bars[S];
  __shared__ uint32_t tmem_slot;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int P = a.N * a.H * a.W;  // < 2^31 (checked by the host)
  const int J = 9 * a.Cin;
  const int j0 = blockIdx.x * 128;
  const int pb = blockIdx.y * a.pix_per_cta;
  const int pe = min(P, pb + a.pix_per_cta);
  const uint32_t ncols = a.Cout <= 32 ? 32 : (a.Cout <= 64 ? 64 : (a.Cout <= 128 ? 128 : 256));
  const uint32_t a_bytes = 128 * kSlice * 2, stage = a_bytes + (uint32_t)a.Cout * kSlice * 2;
  tc_begin(&tmem_slot, bars, S, ncols);
  const uint32_t tmem = tmem_slot;
  const uint32_t idesc = tc::make_idesc_bf16(128, a.Cout, true, true);
  const uint32_t s0 = tc::smem_u32(smem);
  const int n_slices = pe > pb ? (pe - pb + kSlice - 1) / kSlice : 0;
  // this thread's 8 rows of the A tile: (tap, channel) j = j0 + 8 rg
  const int rg = tid & 15;
  const int j = j0 + rg * 8;
  const bool jv = j < J;
  const int t = jv ? j / a.Cin : 0, c = jv ? j - t * a.Cin : 0;
  const int dy = t / 3 - 1, dx = t % 3 - 1;
  const int HW = a.H * a.W;
  const int ng = a.Cout >> 3;
  auto load = [&](int slice, int st) {
    if (slice >= n_slices) return;
    const uint32_t sa = s0 + st * stage, sb = sa + a_bytes;
    const int q0 = pb + slice * kSlice;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int kp = (tid >> 4) + 16 * i;  // pixel within the slice
      const int p = q0 + kp;
      const bf16* src = nullptr;
      if (p < pe && jv) {
        const int n = p / HW, rem = p - n * HW;
        const int y = rem / a.W, x = rem - y * a.W;
        src = src_ptr(a.s1, a.s2, a.H, a.W, n, y + dy, x + dx, c);
      }
      chunk_async(sa + tc::tile_offset_mn(rg * 8, kp, 128), src, a.s1.ptr);
    }
    for (int ch = tid; ch < ng * kSlice; ch += kThreads) {
      const int og = ch % ng, kp = ch / ng;
      const int p = q0 + kp;
      const bf16* src = p < pe ? a.dout + (size_t)p * a.Cout + og * 8 : nullptr;
      chunk_async(sb + tc::tile_offset_mn(og * 8, kp, a.Cout), src, a.dout);
    }
  };
  auto mma = [&](int st, bool first) {
    const uint32_t a0 = s0 + st * stage, b0 = a0 + a_bytes;
#pragma unroll
    for (int s = 0; s < kSlice / 16; ++s)
      tc::mma_bf16(tmem, tc::make_desc(a0 + s * 2 * 16 * 128, 16 * 128, 128),
                   tc::make_desc(b0 + s * 2 * 16 * a.Cout, 16 * a.Cout, 128), idesc, !first || s > 0);
  };
  const bool ok = conv_pipeline<S>(n_slices, bars, load, mma, a.err);
  tc::fence_after();
  if (ok && n_slices > 0) {
    const int lw = warp & 3, half = a.Cout >> 1;
    const int jj = j0 + lw * 32 + lane;  // this thread's accumulator row
    const uint32_t taddr = tmem + ((uint32_t)(lw * 32) << 16);
    for (int c0 = (warp >> 2) * half; c0 < (warp >> 2) * half + half; c0 += 8) {
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
// Stages of the ring for a B tile of nb rows: 3 stages up to 128 rows, 2
// beyond (72 KB per CTA for nb <= 64, at most 96 KB otherwise).
static int stages_for(int nb) { return nb <= 128 ? 3 : 2; }

template <class K4, class K3, class K2, class Args>
static cudaError_t launch_staged(K4 k4, K3 k3, K2 k2, int stages, dim3 grid, size_t stage_bytes, const Args& a,
                                 cudaStream_t st) {
  size_t smem = stage_bytes * stages;
  cudaError_t e;
  if (stages == 4) {
    if ((e = cudaFuncSetAttribute(k4, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem))) return e;
    k4<<<grid, kThreads, smem, st>>>(a);
  } else if (stages == 3) {
    if ((e = cudaFuncSetAttribute(k3, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem))) return e;
    k3<<<grid, kThreads, smem, st>>>(a);
  } else {
    if ((e = cudaFuncSetAttribute(k2, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem))) return e;
    k2<<<grid, kThreads, smem, st>>>(a);
  }
  return cudaGetLastError();
}

// Row tiles pay off once a row holds at least half a tile; they need input
// slices of 16 channels and a grid that fits the y / z limits.
static bool use_rows(int N, int H, int W, int Ck, int nz = 1) {
  return W >= 64 && Ck % 16 == 0 && H <= 65535 && (long long)N * nz <= 65535;
}

cudaError_t conv_fwd(const ConvFwd& a, cudaStream_t st) {
  long long P = (long long)a.N * a.H * a.W;
  if (a.Cout % 16 || a.Cout > 256 || a.Cin % 8) return cudaErrorInvalidValue;
  if (use_rows(a.N, a.H, a.W, a.Cin)) {
    size_t stage = kHaloBytes + (size_t)9 * a.Cout * 32;
    dim3 grid((a.W + 127) / 128, a.H, a.N);
    return launch_staged(k_conv_fwd_row<3>, k_conv_fwd_row<3>, k_conv_fwd_row<2>, stage <= 34 * 1024 ? 3 : 2,
                         grid, stage, a, st);
  }
  size_t stage = 128 * kSlice * 2 + (size_t)a.Cout * kSlice * 2;
  return launch_staged(k_conv_fwd<4>, k_conv_fwd<3>, k_conv_fwd<2>, stages_for(a.Cout),
                       dim3((unsigned)((P + 127) / 128)), stage, a, st);
}

cudaError_t conv_dgrad(const ConvDgrad& a, cudaStream_t st) {
  long long P = (long long)a.N * a.H * a.W;
  if (a.Cin % 16 || a.Cout % 8) return cudaErrorInvalidValue;
  const int nt = (a.Cin + 255) / 256;
  if (use_rows(a.N, a.H, a.W, a.Cout, nt)) {
    size_t stage = kHaloBytes + (size_t)9 * std::min(256, a.Cin) * 32;
    dim3 grid((a.W + 127) / 128, a.H, a.N * nt);
    return launch_staged(k_conv_dgrad_row<3>, k_conv_dgrad_row<3>, k_conv_dgrad_row<2>,
                         stage <= 34 * 1024 ? 3 : 2, grid, stage, a, st);
  }
  int nb = std::min(256, a.Cin);
  size_t stage = 128 * kSlice * 2 + (size_t)nb * kSlice * 2;
  return launch_staged(k_conv_dgrad<4>, k_conv_dgrad<3>, k_conv_dgrad<2>, stages_for(nb),
                       dim3((unsigned)((P + 127) / 128), (a.Cin + 255) / 256), stage, a, st);
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
  size_t stage = 128 * kSlice * 2 + (size_t)a.Cout * kSlice * 2;
  dim3 grid((9 * a.Cin + 127) / 128, (unsigned)((P + a.pix_per_cta - 1) / a.pix_per_cta));
  return launch_staged(k_conv_wgrad<4>, k_conv_wgrad<3>, k_conv_wgrad<2>, stages_for(a.Cout), grid, stage, a, st);
}

}  // namespace nn
}  // namespace rtx
