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
#include <cuda.h>
#include <cudaTypedefs.h>

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
// `done(it)` runs on every thread once slice it's MMAs (and all earlier
// ones) have completed, after the copies of slice it + S - 1 were issued and
// while slice it + 1's MMAs run: the persistent kernels read a finished
// accumulator there.
template <int S, class Load, class Mma, class Done>
__device__ __forceinline__ bool conv_ring(int n, uint64_t* bars, Load&& load, Mma&& mma, Done&& done, int* err) {
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
    tc::fence_before();  // order the previous done()'s TMEM reads before the barrier
    if (!__syncthreads_and(wok)) {
      ok = false;
      break;
    }
    if (threadIdx.x == 0) {
      tc::fence_after();
      mma(it, st, it == 0);
      tc::mma_commit(&bars[st]);
    }
    if (it > 0) {  // the previous slice's MMAs free its stage for slice it + S - 1
      const int ps = (it - 1) % S;
      wok = tc::mbar_wait(&bars[ps], (parity >> ps) & 1u);
      parity ^= 1u << ps;
    }
    load(it + S - 1, (it + S - 1) % S);
    tc::cp_async_commit();
    if (it > 0 && wok) {
      tc::fence_after();
      done(it - 1);
    }
  }
  if (ok && n > 0) {
    const int ls = (n - 1) % S;
    const bool w = wok && tc::mbar_wait(&bars[ls], (parity >> ls) & 1u);
    ok = __syncthreads_and(w);
    if (ok) {
      tc::fence_after();
      done(n - 1);
    }
  }
  if (!ok && (threadIdx.x & 31) == 0) atomicOr(err, tc::kErrMbarTimeout);
  tc::cp_async_wait_all();
  return ok;
}

// Warp-specialised rings (no CTA-wide barrier per slice).  Thread 0 issues
// the MMAs; producer warp 1 + p (p < S <= 7) owns ring stage p and copies
// units p, p + S, p + 2S, ...: it waits for the stage to be free (empty: the
// MMA commit of the unit S before), issues its 32 lanes' cp.async copies,
// waits for them, fences them to the async proxy and arrives on full (32
// arrivals).  Up to S units are in flight, each warp blocking only on its own
// copies; the MMA thread consumes units in order.  Because a warp's units on
// its stage are exactly one lap apart, every parity wait targets the
// barrier's current or next phase, never one two laps away.
// load(unit, stage, lane) copies with item stride kLoadStride.
constexpr int kProducerWarps = 7;
constexpr int kLoadStride = 32;
#ifndef RTX_CONV_TMA
#define RTX_CONV_TMA 1
#endif
constexpr bool kConvTma = RTX_CONV_TMA != 0;  // tensor copies where a source allows them

// pre(pw, lane) issues copies every MMA needs (resident weights, split over
// the producer warps); the warp waits for them and its 32 lanes arrive on
// wbar (kProducerWarps * 32 arrivals; null: none) before its first unit, so
// that arrival never waits on MMA progress.
template <int S, class Pre, class Load>
__device__ __forceinline__ bool produce(int n, uint64_t* full, uint64_t* empty, uint64_t* wbar, Pre&& pre,
                                        Load&& load) {
  static_assert(S >= 1 && S <= kProducerWarps, "one producer warp per stage");
  const int pw = (threadIdx.x >> 5) - 1, lane = threadIdx.x & 31;
  if (wbar) {
    pre(pw, lane);
    tc::cp_async_commit();
    tc::cp_async_wait<0>();
    tc::fence_proxy_async();
    tc::mbar_arrive(wbar);
  }
  if (pw >= S) return true;
  for (int u = pw; u < n; u += S) {
    if (u >= S && !tc::mbar_wait(&empty[pw], (uint32_t)(u / S - 1) & 1u)) return false;
    load(u, pw, lane);
    tc::cp_async_commit();
    tc::cp_async_wait<0>();
    tc::fence_proxy_async();
    tc::mbar_arrive(&full[pw]);
  }
  return true;
}

// produce() for units that arrive as tensor copies: the producer warps
// still copy what every MMA needs (pre, then wbar), then thread 32 alone
// issues each unit's copies (issue(unit, stage, bar)) into its stage once
// the stage is free, with one arrival carrying the unit's `tx` bytes.
// `issued` counts the units it issued.
template <int S, class Pre, class Issue>
__device__ __forceinline__ bool produce_tma(int n, uint64_t* full, uint64_t* empty, uint64_t* wbar, uint32_t tx,
                                            Pre&& pre, Issue&& issue, int& issued) {
  const int pw = (threadIdx.x >> 5) - 1, lane = threadIdx.x & 31;
  issued = 0;
  if (wbar) {
    pre(pw, lane);
    tc::cp_async_commit();
    tc::cp_async_wait<0>();
    tc::fence_proxy_async();
    tc::mbar_arrive(wbar);
  }
  if (threadIdx.x != 32) return true;
  for (int u = 0; u < n; ++u) {
    const int st = u % S;
    if (u >= S && !tc::mbar_wait(&empty[st], (uint32_t)(u / S - 1) & 1u)) return false;
    tc::mbar_arrive_expect_tx(&full[st], tx);
    issue(u, st, &full[st]);
    issued = u + 1;
  }
  return true;
}

// After a timed-out wait: thread 32 waits (bounded) for the tensor copies it
// issued last on each stage, so that none lands after the CTA has left.
template <int S>
__device__ __forceinline__ void drain_tma(uint64_t* full, int issued) {
  if (threadIdx.x != 32) return;
  for (int u = max(0, issued - S); u < issued; ++u) tc::mbar_wait(&full[u % S], (uint32_t)(u / S) & 1u);
}

// One accumulation over n slices (the weight gradient).  Returns true,
// uniformly, once every MMA has completed; false (error flag set) when a
// bounded wait ran out.
template <int S, class Load, class Mma>
__device__ __forceinline__ bool ws_ring(int n, uint64_t* full, uint64_t* empty, Load&& load, Mma&& mma, int* err) {
  const int tid = threadIdx.x;
  bool ok = true;
  if (tid < 32) {
    if (tid == 0) {
      for (int it = 0; it < n; ++it) {
        const int st = it % S;
        if (!tc::mbar_wait(&full[st], (uint32_t)(it / S) & 1u)) {
          ok = false;
          break;
        }
        tc::fence_after();
        mma(it, st);
        tc::mma_commit(&empty[st]);
      }
    }
  } else {
    ok = produce<S>(n, full, empty, nullptr, [](int, int) {}, load);
  }
  // the last commit covers every MMA (waited after a plain barrier, so the
  // producers do not spin while the MMAs drain)
  bool fin = __syncthreads_and(ok);
  if (fin && n > 0) fin = tc::mbar_wait(&empty[(n - 1) % S], (uint32_t)((n - 1) / S) & 1u);
  fin = __syncthreads_and(fin);
  if (!fin && (tid & 31) == 0) atomicOr(err, tc::kErrMbarTimeout);
  tc::fence_after();
  return fin;
}

// The same accumulation fed by tensor copies (TMA): thread 32 issues unit
// it's copies into stage it % S once the MMAs of unit it - S have released
// it (one arrival carrying the unit's byte count, `tx`), thread 0 issues the
// MMAs.  On a timed-out wait the issuing thread waits (bounded) for the
// copies it issued last on each stage before the CTA leaves, so that none
// lands in released shared memory.
template <int S, class Issue, class Mma>
__device__ __forceinline__ bool tma_ring(int n, uint64_t* full, uint64_t* empty, uint32_t tx, Issue&& issue,
                                         Mma&& mma, int* err) {
  const int tid = threadIdx.x;
  bool ok = true;
  int issued = 0;
  if (tid == 0) {
    for (int it = 0; it < n; ++it) {
      const int st = it % S;
      if (!tc::mbar_wait(&full[st], (uint32_t)(it / S) & 1u)) {
        ok = false;
        break;
      }
      tc::fence_after();
      mma(it, st);
      tc::mma_commit(&empty[st]);
    }
  } else if (tid == 32) {
    for (int it = 0; it < n; ++it) {
      const int st = it % S;
      if (it >= S && !tc::mbar_wait(&empty[st], (uint32_t)(it / S - 1) & 1u)) {
        ok = false;
        break;
      }
      tc::mbar_arrive_expect_tx(&full[st], tx);
      issue(it, st, &full[st]);
      issued = it + 1;
    }
  }
  bool fin = __syncthreads_and(ok);
  if (fin && n > 0) fin = tc::mbar_wait(&empty[(n - 1) % S], (uint32_t)((n - 1) / S) & 1u);
  fin = __syncthreads_and(fin);
  if (!fin) {
    if (tid == 32)
      for (int it = max(0, issued - S); it < issued; ++it) tc::mbar_wait(&full[it % S], (uint32_t)(it / S) & 1u);
    if ((tid & 31) == 0) atomicOr(err, tc::kErrMbarTimeout);
  }
  tc::fence_after();
  return fin;
}

// Persistent tiles (kTileThreads = 12 warps): thread 0 issues MMAs, warps
// 1 .. 7 produce, warps 8 .. 11 run the epilogue, warp 8 + q reading
// accumulator lanes 32 q .. 32 q + 31.  A CTA walks n_tiles output tiles of
// nsl slices each; tile i accumulates in TMEM buffer i & 1, so tile i's
// epilogue overlaps tile i + 1's copies and MMAs.  accf[b]: MMA commit after
// a tile's last slice (buffer b complete); acce[b]: the 128 epilogue threads'
// arrivals once they have read buffer b.  mma(unit, stage, buffer, slice)
// and epi(tile, buffer) are the kernel's.
constexpr int kTileThreads = 384;
constexpr int kEpilogue = 128;
constexpr int kMaxStages = 8;

struct TileBars {
  uint64_t full[kMaxStages], empty[kMaxStages], accf[2], acce[2], wbar;
};

template <int S>
__device__ __forceinline__ void tile_bars_init(TileBars& b, uint32_t full_count = kLoadStride) {
  if (threadIdx.x == 0) {
    for (int i = 0; i < S; ++i) {
      tc::mbar_init(&b.full[i], full_count);
      tc::mbar_init(&b.empty[i], 1);
    }
    for (int i = 0; i < 2; ++i) {
      tc::mbar_init(&b.accf[i], 1);
      tc::mbar_init(&b.acce[i], kEpilogue);
    }
    tc::mbar_init(&b.wbar, kProducerWarps * 32);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
}

template <int S, bool kTma = false, class Pre, class Load, class Mma, class Epi, class Issue>
__device__ __forceinline__ bool ws_tiles(int n_tiles, int nsl, TileBars& b, Pre&& pre, Load&& load, Mma&& mma,
                                         Epi&& epi, int* err, Issue&& issue, uint32_t tx) {
  const int tid = threadIdx.x, warp = tid >> 5;
  const int n = n_tiles * nsl;
  bool ok = true;
  int issued = 0;
  if (warp == 0) {
    if (tid == 0) {
      if (n > 0) ok = tc::mbar_wait(&b.wbar, 0u);
      for (int u = 0; u < n && ok; ++u) {
        const int i = u / nsl, s = u - i * nsl, st = u % S, buf = i & 1;
        if (s == 0 && i >= 2) ok = tc::mbar_wait(&b.acce[buf], (uint32_t)((i >> 1) - 1) & 1u);
        if (ok) ok = tc::mbar_wait(&b.full[st], (uint32_t)(u / S) & 1u);
        if (!ok) break;
        tc::fence_after();
        mma(u, st, buf, s);
        tc::mma_commit(&b.empty[st]);
        if (s == nsl - 1) tc::mma_commit(&b.accf[buf]);
      }
    }
  } else if (warp <= kProducerWarps) {
    if constexpr (kTma)
      ok = produce_tma<S>(n, b.full, b.empty, &b.wbar, tx, pre, issue, issued);
    else
      ok = produce<S>(n, b.full, b.empty, &b.wbar, pre, load);
  } else {
    for (int i = 0; i < n_tiles; ++i) {
      const int buf = i & 1;
      if (!tc::mbar_wait(&b.accf[buf], (uint32_t)(i >> 1) & 1u)) {
        ok = false;
        break;
      }
      tc::fence_after();
      epi(i, buf);
      tc::fence_before();
      tc::mbar_arrive(&b.acce[buf]);
    }
  }
  ok = __syncthreads_and(ok);
  if (!ok) {
    if constexpr (kTma) drain_tma<S>(b.full, issued);
    if ((tid & 31) == 0) atomicOr(err, tc::kErrMbarTimeout);
  }
  return ok;
}

template <int S, class Load, class Mma>
__device__ __forceinline__ bool conv_pipeline(int n, uint64_t* bars, Load&& load, Mma&& mma, int* err) {
  return conv_ring<S>(
      n, bars, load, [&](int, int st, bool first) { mma(st, first); }, [](int) {}, err);
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
    // consecutive K steps are 256 B apart: +16 in the descriptors' address field
    const uint64_t ad = tc::make_desc(a0, 128, kSlice * 16), bd = tc::make_desc(b0, 128, kSlice * 16);
#pragma unroll
    for (int s = 0; s < kSlice / 16; ++s) tc::mma_bf16(tmem, ad + 16 * s, bd + 16 * s, idesc, !first || s > 0);
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
// forward, row tiles: a tile is 128 consecutive pixels of one image row.  Per
// slice of 16 input channels the producers copy the tile's 3-row halo (pixels
// x0 - 1 .. x0 + 128, 2 chunks of 8 channels each) once; the nine taps are
// the same halo read through descriptors shifted by whole pixels (rows of the
// K-major layout are 16 B apart and the two channel chunks one halo row
// apart, so every shift is a legal start address): one third of the gather
// traffic of k_conv_fwd, one address per copied pixel chunk.  Persistent and
// warp-specialised (ws_tiles): a CTA walks tiles blockIdx.x, + gridDim.x, ...;
// with kRes the whole weight tensor stays in shared memory ([slice][tap]
// tiles of Cout x 16, K-major), otherwise each stage carries its slice's nine
// weight tiles.
// ---------------------------------------------------------------------------
constexpr int kHalo = 130;                                  // pixels x0 - 1 .. x0 + 128
constexpr uint32_t kHaloBytes = 3 * 2 * kHalo * 16;          // rows x chunks x pixels x 16 B
constexpr uint32_t kHaloStage = (kHaloBytes + 1023) & ~1023u;  // 1 KB aligned for tensor copies

// smem byte offset of chunk c (of 2) of halo pixel h in halo row r
__device__ __forceinline__ uint32_t halo_off(int r, int c, int h) { return ((r * 2 + c) * kHalo + h) * 16; }

template <int S, bool kRes, bool kTma = false>
__global__ void __launch_bounds__(kTileThreads, 1)
    k_conv_fwd_rows(ConvFwd a, const __grid_constant__ CUtensorMap tm_halo,
                    const __grid_constant__ CUtensorMap tm_w) {
  extern __shared__ __align__(1024) uint8_t smem[];
  __shared__ __align__(8) TileBars bars;
  __shared__ uint32_t tmem_slot;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int TR = (a.W + 127) / 128;  // tiles per image row
  const int T = a.N * a.H * TR;
  const int n_tiles = (int)blockIdx.x < T ? (T - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
  const int nsl = a.Cin / 16;
  const uint32_t ncols = a.Cout <= 32 ? 32 : (a.Cout <= 64 ? 64 : (a.Cout <= 128 ? 128 : 256));
  const uint32_t tap_bytes = (uint32_t)a.Cout * 32;
  // tensor copies: the halo, then (streamed weights) the slice's nine weight
  // tiles from the next 1 KB boundary
  const uint32_t stage = kTma ? kHaloStage + (kRes ? 0u : (9 * tap_bytes + 1023u) & ~1023u)
                              : (kRes ? kHaloBytes : kHaloBytes + 9 * tap_bytes);
  const uint32_t w_off = kTma ? kHaloStage : kHaloBytes;  // weights within a streamed stage
  if (warp == 0) tc::tmem_alloc(&tmem_slot, 2 * ncols);
  tile_bars_init<S>(bars, kTma ? 1 : kLoadStride);
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t tmem = tmem_slot;
  const uint32_t idesc = tc::make_idesc_bf16(128, a.Cout);
  const uint32_t s0 = tc::smem_u32(smem), sw = s0 + S * stage;  // sw: resident weights
  auto tile_of = [&](int i, int& n, int& y, int& x0) {
    const int j = (int)blockIdx.x + i * (int)gridDim.x;
    const int row = j / TR;
    x0 = (j - row * TR) * 128;
    n = row / a.H;
    y = row - n * a.H;
  };
  auto weight_tile = [&](uint32_t dst, int q) {  // chunk q of one [slice][tap] tile set
    const int kc = q & 1, o = (q >> 1) % a.Cout, st = (q >> 1) / a.Cout, sl = st / 9, t = st - sl * 9;
    chunk_async(dst + st * tap_bytes + tc::tile_offset(o, 8 * kc, 16),
                a.w + ((size_t)o * 9 + t) * a.Cin + sl * 16 + 8 * kc, a.w);
  };
  auto pre = [&](int pw, int lane) {
    if (kRes)
      for (int q = pw * 32 + lane; q < nsl * 9 * a.Cout * 2; q += kProducerWarps * 32) weight_tile(sw, q);
  };
  auto load = [&](int u, int st, int lane) {
    const int i = u / nsl, s = u - i * nsl;
    int n, y, x0;
    tile_of(i, n, y, x0);
    const uint32_t sh = s0 + st * stage;
    const int c0 = s * 16;
    // neighbouring lanes take the two chunks of one pixel (32 B)
    for (int q = lane; q < 3 * kHalo * 2; q += kLoadStride) {
      const int c = q & 1, h = (q >> 1) % kHalo, r = (q >> 1) / kHalo;
      chunk_async(sh + halo_off(r, c, h), src_ptr(a.s1, a.s2, a.H, a.W, n, y + r - 1, x0 + h - 1, c0 + 8 * c),
                  a.s1.ptr);
    }
    if (!kRes)  // slice s's nine tiles: q -> (tap, row, chunk) with the slice fixed
      for (int q = lane; q < 9 * a.Cout * 2; q += kLoadStride) {
        const int kc = q & 1, o = (q >> 1) % a.Cout, t = (q >> 1) / a.Cout;
        chunk_async(sh + kHaloBytes + t * tap_bytes + tc::tile_offset(o, 8 * kc, 16),
                    a.w + ((size_t)o * 9 + t) * a.Cin + c0 + 8 * kc, a.w);
      }
  };
  auto mma = [&](int, int st, int buf, int s) {
    const uint32_t sh = s0 + st * stage;
    const uint32_t sb = kRes ? sw + (uint32_t)s * 9 * tap_bytes : sh + w_off;
    // A: pixel groups 128 B apart (SBO), channel chunks one halo row apart
    // (LBO); tap t starts (dy + 1) halo rows and 1 + dx pixels in (offsets in
    // the descriptors' 16-byte address units)
    const uint64_t ah = tc::make_desc(sh, kHalo * 16, 128), bw = tc::make_desc(sb, 128, 256);
    const uint32_t d = tmem + buf * ncols;
#pragma unroll
    for (int t = 0; t < 9; ++t) {
      const int dy = t / 3 - 1, dx = t % 3 - 1;
      tc::mma_bf16(d, ah + ((dy + 1) * 2 * kHalo + 1 + dx), bw + t * (tap_bytes >> 4), idesc, s > 0 || t > 0);
    }
  };
  auto epi = [&](int i, int buf) {
    const int q = warp & 3;  // accumulator lanes 32 q .. 32 q + 31 = pixels
    int n, y, x0;
    tile_of(i, n, y, x0);
    const int x = x0 + q * 32 + lane;
    const size_t p = ((size_t)n * a.H + y) * a.W + x;
    const uint32_t taddr = tmem + buf * ncols + ((uint32_t)(q * 32) << 16);
    for (int c0 = 0; c0 < a.Cout; c0 += 8) {
      float v[8];
      tc::tmem_ld8(taddr + c0, v);
      if (x < a.W) {
#pragma unroll
        for (int k = 0; k < 8; ++k) {
          if (a.bias) v[k] += a.bias[c0 + k];
          if (a.relu) v[k] = fmaxf(v[k], 0.0f);
        }
        if (a.out) *reinterpret_cast<uint4*>(a.out + p * a.Cout + c0) = f32_to_bf16x8(v);
        if (a.out_f32)
#pragma unroll
          for (int k = 0; k < 8; ++k) a.out_f32[p * a.Cout + c0 + k] = v[k];
      }
    }
  };
  // tensor-copy form: the unit's halo slice as one box of the source map
  auto issue = [&](int u, int st, uint64_t* bar) {
    const int i = u / nsl, s = u - i * nsl;
    int n, y, x0;
    tile_of(i, n, y, x0);
    tc::tma_load_5d(s0 + st * stage, &tm_halo, 0, x0 - 1, 2 * s, y - 1, n, bar);
    // the slice's nine [Cout x 16] weight tiles, tap-major
    if (!kRes) tc::tma_load_5d(s0 + st * stage + w_off, &tm_w, 0, 0, 2 * s, 0, 0, bar);
  };
  ws_tiles<S, kTma>(n_tiles, nsl, bars, pre, load, mma, epi, a.err, issue, kHaloBytes + (kRes ? 0u : 9 * tap_bytes));
  tc_end(tmem, 2 * ncols);
}

// data gradient, row tiles: din[p] = sum_t dout[p - off(t)] wt_t, the same
// halo scheme over dout (slices of 16 of its channels, shifts negated).  A
// tile is (image row, 128 pixels, 256 input channels); the channel tile
// varies fastest, so neighbouring CTAs read the same dout halo.  Resident
// weights: [channel tile][slice][tap] tiles of NTmax x 16.
template <int S, bool kRes, bool kTma = false>
__global__ void __launch_bounds__(kTileThreads, 1)
    k_conv_dgrad_rows(ConvDgrad a, const __grid_constant__ CUtensorMap tm_halo,
                      const __grid_constant__ CUtensorMap tm_w) {
  extern __shared__ __align__(1024) uint8_t smem[];
  __shared__ __align__(8) TileBars bars;
  __shared__ uint32_t tmem_slot;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int TR = (a.W + 127) / 128, nt = (a.Cin + a.ctw - 1) / a.ctw;
  const int T = a.N * a.H * TR * nt;
  const int n_tiles = (int)blockIdx.x < T ? (T - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
  const int nsl = a.Cout / 16;
  const int ntm = min(a.ctw, a.Cin);  // widest channel tile
  const uint32_t ncols = ntm <= 32 ? 32 : (ntm <= 64 ? 64 : (ntm <= 128 ? 128 : 256));
  const uint32_t tap_bytes = (uint32_t)ntm * 32;
  const uint32_t stage = kTma ? kHaloStage + (kRes ? 0u : (9 * tap_bytes + 1023u) & ~1023u)
                              : (kRes ? kHaloBytes : kHaloBytes + 9 * tap_bytes);
  const uint32_t w_off = kTma ? kHaloStage : kHaloBytes;  // weights within a streamed stage
  if (warp == 0) tc::tmem_alloc(&tmem_slot, 2 * ncols);
  tile_bars_init<S>(bars, kTma ? 1 : kLoadStride);
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t tmem = tmem_slot;
  const uint32_t s0 = tc::smem_u32(smem), sw = s0 + S * stage;
  auto tile_of = [&](int i, int& n, int& y, int& x0, int& ct) {
    const int j = (int)blockIdx.x + i * (int)gridDim.x;
    const int rx = j / nt;
    ct = j - rx * nt;
    const int row = rx / TR;
    x0 = (rx - row * TR) * 128;
    n = row / a.H;
    y = row - n * a.H;
  };
  auto pre = [&](int pw, int lane) {
    if (kRes)  // q -> (channel tile, slice, tap, row, chunk)
      for (int q = pw * 32 + lane; q < nt * nsl * 9 * ntm * 2; q += kProducerWarps * 32) {
        const int kc = q & 1, row = (q >> 1) % ntm, set = (q >> 1) / ntm;  // set = (ct * nsl + sl) * 9 + t
        const int t = set % 9, cs = set / 9, sl = cs % nsl, c = cs / nsl;
        const int ch = c * a.ctw + row;
        chunk_async(sw + set * tap_bytes + tc::tile_offset(row, 8 * kc, 16),
                    ch < a.Cin ? a.wt + ((size_t)ch * 9 + t) * a.Cout + sl * 16 + 8 * kc : nullptr, a.wt);
      }
  };
  auto load = [&](int u, int st, int lane) {
    const int i = u / nsl, s = u - i * nsl;
    int n, y, x0, ct;
    tile_of(i, n, y, x0, ct);
    const uint32_t sh = s0 + st * stage;
    const int o0 = s * 16;
    for (int q = lane; q < 3 * kHalo * 2; q += kLoadStride) {
      const int c = q & 1, h = (q >> 1) % kHalo, r = (q >> 1) / kHalo;
      const int yy = y + r - 1, xx = x0 + h - 1;
      const bf16* p = (yy >= 0 && yy < a.H && xx >= 0 && xx < a.W)
                          ? a.dout + (((size_t)n * a.H + yy) * a.W + xx) * a.Cout + o0 + 8 * c
                          : nullptr;
      chunk_async(sh + halo_off(r, c, h), p, a.dout);
    }
    if (!kRes) {
      const int n0 = ct * a.ctw, NT = min(a.ctw, a.Cin - n0);
      for (int q = lane; q < 9 * NT * 2; q += kLoadStride) {
        const int kc = q & 1, row = (q >> 1) % NT, t = (q >> 1) / NT;
        chunk_async(sh + kHaloBytes + t * tap_bytes + tc::tile_offset(row, 8 * kc, 16),
                    a.wt + ((size_t)(n0 + row) * 9 + t) * a.Cout + o0 + 8 * kc, a.wt);
      }
    }
  };
  auto mma = [&](int u, int st, int buf, int s) {
    int n, y, x0, ct;
    tile_of(u / nsl, n, y, x0, ct);
    const int NT = min(a.ctw, a.Cin - ct * a.ctw);
    const uint32_t idesc = tc::make_idesc_bf16(128, NT);
    const uint32_t sh = s0 + st * stage;
    const uint32_t sb = kRes ? sw + (uint32_t)(ct * nsl + s) * 9 * tap_bytes : sh + w_off;
    const uint64_t ah = tc::make_desc(sh, kHalo * 16, 128), bw = tc::make_desc(sb, 128, 256);
    const uint32_t d = tmem + buf * ncols;
#pragma unroll
    for (int t = 0; t < 9; ++t) {
      const int dy = t / 3 - 1, dx = t % 3 - 1;
      tc::mma_bf16(d, ah + ((1 - dy) * 2 * kHalo + 1 - dx), bw + t * (tap_bytes >> 4), idesc, s > 0 || t > 0);
    }
  };
  auto epi = [&](int i, int buf) {
    const int q = warp & 3;
    int n, y, x0, ct;
    tile_of(i, n, y, x0, ct);
    const int n0 = ct * a.ctw, NT = min(a.ctw, a.Cin - n0);
    const int x = x0 + q * 32 + lane;
    const size_t p = ((size_t)n * a.H + y) * a.W + x;
    const uint32_t taddr = tmem + buf * ncols + ((uint32_t)(q * 32) << 16);
    for (int c0 = 0; c0 < NT; c0 += 8) {
      float v[8];
      tc::tmem_ld8(taddr + c0, v);
      if (x < a.W) {
        if (a.mask_relu) {
          float sv[8];
          bf16x8_to_f32(src_chunk(a.s1, a.s2, a.N, a.H, a.W, n, y, x, n0 + c0), sv);
#pragma unroll
          for (int k = 0; k < 8; ++k)
            if (!(sv[k] > 0.0f)) v[k] = 0.0f;
        }
        *reinterpret_cast<uint4*>(a.din + p * a.Cin + n0 + c0) = f32_to_bf16x8(v);
      }
    }
  };
  // tensor-copy form: the unit's dout halo slice as one box of dout's map
  auto issue = [&](int u, int st, uint64_t* bar) {
    const int i = u / nsl, s = u - i * nsl;
    int n, y, x0, ct;
    tile_of(i, n, y, x0, ct);
    tc::tma_load_5d(s0 + st * stage, &tm_halo, 0, x0 - 1, 2 * s, y - 1, n, bar);
    // the slice's nine [ntm x 16] tiles of the channel tile (rows past Cin
    // read zeros), tap-major
    if (!kRes) tc::tma_load_5d(s0 + st * stage + w_off, &tm_w, 0, 0, 2 * s, (ct * a.ctw) >> 3, 0, bar);
  };
  ws_tiles<S, kTma>(n_tiles, nsl, bars, pre, load, mma, epi, a.err, issue, kHaloBytes + (kRes ? 0u : 9 * tap_bytes));
  tc_end(tmem, 2 * ncols);
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
    // consecutive K steps are 256 B apart: +16 in the descriptors' address field
    const uint64_t ad = tc::make_desc(a0, 128, kSlice * 16), bd = tc::make_desc(b0, 128, kSlice * 16);
#pragma unroll
    for (int s = 0; s < kSlice / 16; ++s) tc::mma_bf16(tmem, ad + 16 * s, bd + 16 * s, idesc, !first || s > 0);
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
    const uint64_t ad = tc::make_desc(a0, 16 * 128, 128), bd = tc::make_desc(b0, 16 * a.Cout, 128);
#pragma unroll
    for (int s = 0; s < kSlice / 16; ++s)
      tc::mma_bf16(tmem, ad + s * 2 * 128, bd + s * 2 * a.Cout, idesc, !first || s > 0);
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
// weight gradient, row tiles: a CTA owns source channels [c0, c0 + CR)
// (CR <= 48) for all nine taps and sums over a run of row tiles (TW pixels
// of one image row, TW = 64 or 128).  GEMM M = output channels (the 128
// accumulator lanes; lanes >= Cout are never read), N = CR per tap, K = the
// tile's pixels, both operands MN-major:
//   A = the dout tile, chunk g of pixel k at (g * TW + k) * 16
//   B = the 3-row source halo, chunk ch of pixel h of row r at
//       ((r * CR / 8 + ch) * (TW + 2) + h) * 16
// Tap t = (dy, dx) reads halo row dy + 1 shifted by dx pixels (any 16-byte
// shift of an MN-major operand whose K neighbours are 16 B apart is a legal
// start address) into accumulator columns [t * CR, t * CR + CR).  Per tile a
// CTA copies the dout tile and the halo once, so the source is read about
// three times and dout Cin / CR times, against nine and 9 Cin / 128 times in
// k_conv_wgrad.  The accumulator lives in TMEM across all of the CTA's tiles;
// one set of FP32 atomics per CTA combines the runs.
//
// kSwap (narrow outputs, Cout <= 56, and Cin >= 64): the operands trade
// places.  M = the CTA's source channels (up to 128 accumulator lanes; the
// MMA reads 128 rows of the halo, and rows past CR land in lanes that are
// never read), N = Cout, A = the halo read at each tap's shift, B = the dout
// tile; tap t accumulates in columns [t * Cout, t * Cout + Cout), 9 Cout <=
// 512.  With M = Cout = 32 three quarters of every MMA would be padding; with
// M = 96 source channels one quarter is, and one CTA covers all channels, so
// dout is read once per tile.
//
// kTma (single, full-resolution source; Cin a multiple of the CTA's
// channels): each unit's halo and dout tile arrive as two tensor copies
// into the same layouts.  The source map is NHWC viewed as 5-D (8 channels,
// x, channel chunk, y, image), so a box of (8, TW + 2, CR / 8, 3, 1) lands
// row, chunk, pixel major -- the layout above -- with zeros outside the
// image; dout's map is the same view of [rows][W][Cout] with a box of
// (8, TW, Cout / 8, 1, 1).  Stages are 1 KB aligned for the copies.
// ---------------------------------------------------------------------------
template <int S, bool kSwap, bool kTma>
__global__ void __launch_bounds__(kThreads, 1)
    k_conv_wgrad_row(ConvWgrad a, const __grid_constant__ CUtensorMap tm_src,
                     const __grid_constant__ CUtensorMap tm_dout) {
  extern __shared__ __align__(1024) uint8_t smem[];
  __shared__ __align__(8) uint64_t full[S], empty[S];
  __shared__ uint32_t tmem_slot;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int TW = a.tw, TW2 = a.tw + 2;
  const int c0 = blockIdx.x * a.cr;
  const int CR = min(a.cr, a.Cin - c0);  // this CTA's channels (multiple of 16)
  const int nch = CR >> 3, nco = a.Cout >> 3;
  const int TR = (a.W + TW - 1) / TW;  // tiles per image row
  const int T = a.N * a.H * TR;
  const int tb = blockIdx.y * a.tiles_per_cta;
  const int n_tiles = max(0, min(a.tiles_per_cta, T - tb));
  const uint32_t ncols = (!kSwap && 9 * a.cr <= 256) ? 256 : 512;
  const uint32_t dout_bytes = (uint32_t)a.Cout * TW * 2;
  const uint32_t tx = dout_bytes + 3u * (a.cr >> 3) * TW2 * 16;  // one unit's bytes
  const uint32_t stage = kTma ? (tx + 1023u) & ~1023u : tx;
  if (warp == 0) tc::tmem_alloc(&tmem_slot, ncols);
  if (tid == 0) {
    for (int i = 0; i < S; ++i) {
      tc::mbar_init(&full[i], kTma ? 1 : kLoadStride);
      tc::mbar_init(&empty[i], 1);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t tmem = tmem_slot;
  const uint32_t idesc = tc::make_idesc_bf16(128, kSwap ? a.Cout : CR, true, true);
  const uint32_t s0 = tc::smem_u32(smem);
  // a producer's starting item and the per-iteration step of the two copy
  // loops (items: dout = (pixel k, chunk g), g fastest; halo = (row r, pixel
  // h, chunk ch), ch fastest, so neighbouring threads read contiguous bytes)
  const int pt = lane;
  const int d_g0 = pt % nco, d_k0 = pt / nco, d_dg = kLoadStride % nco, d_dk = kLoadStride / nco;
  const int h_c0 = pt % nch, h_p0 = pt / nch, h_dc = kLoadStride % nch, h_dp = kLoadStride / nch;
  auto load = [&](int slice, int st, int ptid) {
    const uint32_t sd = s0 + st * stage, sh = sd + dout_bytes;
    const int j = tb + slice;
    const int row = j / TR, x0 = (j - row * TR) * TW;  // row = n * H + y
    const int n = row / a.H, y = row - n * a.H;
    const bf16* drow = a.dout + (size_t)row * a.W * a.Cout;
    for (int i = ptid, g = d_g0, k = d_k0; i < TW * nco; i += kLoadStride) {
      const bf16* p = x0 + k < a.W ? drow + (size_t)(x0 + k) * a.Cout + g * 8 : nullptr;
      chunk_async(sd + (g * TW + k) * 16, p, a.dout);
      g += d_dg;
      k += d_dk;
      if (g >= nco) {
        g -= nco;
        ++k;
      }
    }
    int r = 0, h = h_p0;
    while (h >= TW2) {
      h -= TW2;
      ++r;
    }
    for (int i = ptid, ch = h_c0; i < 3 * TW2 * nch; i += kLoadStride) {
      const bf16* p = src_ptr(a.s1, a.s2, a.H, a.W, n, y + r - 1, x0 + h - 1, c0 + 8 * ch);
      chunk_async(sh + ((r * nch + ch) * TW2 + h) * 16, p, a.s1.ptr);
      ch += h_dc;
      h += h_dp;
      if (ch >= nch) {
        ch -= nch;
        ++h;
      }
      while (h >= TW2) {
        h -= TW2;
        ++r;
      }
    }
  };
  auto mma = [&](int it, int st) {
    const bool first = it == 0;
    const uint32_t sd = s0 + st * stage, sh = sd + dout_bytes;
    // descriptors built once; a K step (16 pixels) is +256 B = +16 in the
    // address field, tap t's B starts (dy + 1) halo rows and 1 + dx pixels in
    const uint64_t ad0 = tc::make_desc(sd, 128, TW * 16), bh = tc::make_desc(sh, 128, TW2 * 16);
    const int nks = TW / 16;
#pragma unroll 1
    for (int t = 0; t < 9; ++t) {
      const int dy = t / 3 - 1, dx = t % 3 - 1;
      const uint64_t hd = bh + ((dy + 1) * nch * TW2 + 1 + dx);
      if (kSwap) {  // A = the shifted halo (M = channels), B = the dout tile
        const uint32_t d = tmem + t * a.Cout;
        tc::mma_bf16(d, hd, ad0, idesc, !first);
#pragma unroll 8
        for (int ks = 1; ks < nks; ++ks) tc::mma_bf16(d, hd + 16 * ks, ad0 + 16 * ks, idesc, true);
      } else {
        const uint32_t d = tmem + t * CR;
        tc::mma_bf16(d, ad0, hd, idesc, !first);
#pragma unroll 8
        for (int ks = 1; ks < nks; ++ks) tc::mma_bf16(d, ad0 + 16 * ks, hd + 16 * ks, idesc, true);
      }
    }
  };
  // the tensor-copy form: unit `slice` of this CTA (its row tile) as two boxes
  auto issue = [&](int slice, int st, uint64_t* bar) {
    const uint32_t sd = s0 + st * stage, sh = sd + dout_bytes;
    const int j = tb + slice;
    const int row = j / TR, x0 = (j - row * TR) * TW;  // row = n * H + y
    const int n = row / a.H, y = row - n * a.H;
    tc::tma_load_5d(sh, &tm_src, 0, x0 - 1, c0 >> 3, y - 1, n, bar);
    tc::tma_load_5d(sd, &tm_dout, 0, x0, 0, row, 0, bar);
  };
  bool ok;
  if constexpr (kTma)
    ok = tma_ring<S>(n_tiles, full, empty, tx, issue, mma, a.err);
  else
    ok = ws_ring<S>(n_tiles, full, empty, load, mma, a.err);
  const int lw = warp & 3;
  if (kSwap) {
    // warp w reads lanes 32 (w % 4) .. + 31 (source channel c0 + ch), half
    // w / 4 of the 9 Cout / 8 column chunks (tap t, output channels o0 ..)
    const int ch = lw * 32 + lane;
    const uint32_t taddr = tmem + ((uint32_t)(lw * 32) << 16);
    const int nq = 9 * nco, q0 = (warp >> 2) * (nq >> 1), q1 = (warp >> 2) ? nq : (nq >> 1);
    if (ok && n_tiles > 0 && lw * 32 < CR) {
      for (int q = q0; q < q1; ++q) {
        float v[8];
        tc::tmem_ld8(taddr + q * 8, v);  // warp-wide: every lane loads, valid lanes add
        if (ch < CR) {
          const int t = q / nco, o0 = (q - t * nco) * 8;
#pragma unroll
          for (int k = 0; k < 8; ++k) atomicAdd(a.dw + ((size_t)(o0 + k) * 9 + t) * a.Cin + c0 + ch, v[k]);
        }
      }
    }
    tc_end(tmem, ncols);
    return;
  }
  if (ok && n_tiles > 0 && lw * 32 < a.Cout) {
    // warp w reads lanes 32 (w % 4) .. + 31 (output channel o), half w / 4 of
    // the 9 CR / 8 column chunks
    const int o = lw * 32 + lane;
    const uint32_t taddr = tmem + ((uint32_t)(lw * 32) << 16);
    const int nq = 9 * nch, q0 = (warp >> 2) * (nq >> 1), q1 = (warp >> 2) ? nq : (nq >> 1);
    const bool vec = ((reinterpret_cast<uintptr_t>(a.dw) & 15) == 0);
    for (int q = q0; q < q1; ++q) {
      float v[8];
      tc::tmem_ld8(taddr + q * 8, v);
      if (o < a.Cout) {
        const int t = q / nch, cl = (q - t * nch) * 8;
        float* d = a.dw + ((size_t)o * 9 + t) * a.Cin + c0 + cl;
        if (vec) {
          atomicAdd(reinterpret_cast<float4*>(d), make_float4(v[0], v[1], v[2], v[3]));
          atomicAdd(reinterpret_cast<float4*>(d + 4), make_float4(v[4], v[5], v[6], v[7]));
        } else {
#pragma unroll
          for (int i = 0; i < 8; ++i) atomicAdd(d + i, v[i]);
        }
      }
    }
  }
  tc_end(tmem, ncols);
}

// ---------------------------------------------------------------------------
// Stages of the ring for a B tile of nb rows: 3 stages up to 128 rows, 2
// beyond (72 KB per CTA for nb <= 64, at most 96 KB otherwise).
static int stages_for(int nb) { return nb <= 128 ? 3 : 2; }

// Ring depth of a gather kernel: stages_for(nb), except that a grid of
// fewer CTAs than SMs (the 16- and 32-pixel-wide levels at small batches)
// whose stages are too large for three gets four (one CTA per SM), so that
// more slices' copies are in flight along each CTA's K loop: 160 output
// channels at 16^2 x 8, 44.8 -> 35.4 us (forward) and 64.6 -> 45.8 us (data
// gradient); three -> six stages measured no faster.
static int gather_stages(int nb, dim3 grid, size_t stage_bytes);

template <class K4, class K3, class K2, class Args>
static cudaError_t launch_staged(K4 k4, K3 k3, K2 k2, int stages, dim3 grid, size_t stage_bytes, const Args& a,
                                 cudaStream_t st, size_t extra = 0) {
  size_t smem = stage_bytes * stages + extra;
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

static int sm_count() {
  static int n = 0;
  if (!n) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0)
      n = 148;
  }
  return n;
}

static int gather_stages(int nb, dim3 grid, size_t stage_bytes) {
  const int base = stages_for(nb);
  const long long ctas = (long long)grid.x * grid.y * grid.z;
  return (base == 2 && ctas < sm_count() && 4 * stage_bytes <= 200 * 1024) ? 4 : base;
}

// Row tiles pay off once a row holds at least half a tile; they need input
// slices of 16 channels.
static bool use_rows(int W, int Ck) { return W >= 64 && Ck % 16 == 0; }

// Persistent tile kernels (ws_tiles): one CTA per SM, shared memory padded
// past half the SM so that a second CTA never waits on the first one's TMEM
// columns.  Resident weights take a 7-stage halo ring; streamed weights the
// deepest ring (6, 4 or 2 stages) that fits 200 KB.
template <class KR, class K6, class K4, class K2, class Args>
static cudaError_t launch_tiles(KR kr, K6 k6, K4 k4, K2 k2, bool res, size_t stage, size_t res_bytes, long long T,
                                const Args& a, const CUtensorMap& tm, const CUtensorMap& tw, cudaStream_t st) {
  if (T <= 0) return cudaSuccess;
  int S = 7;
  size_t smem = 7 * stage + res_bytes;
  if (!res) {
    S = 6 * stage <= 200 * 1024 ? 6 : (4 * stage <= 200 * 1024 ? 4 : 2);
    smem = S * stage;
  }
  smem = std::max(smem, (size_t)116 * 1024);
  const unsigned grid = (unsigned)std::min<long long>(T, sm_count());
  cudaError_t e;
#define RTX_LAUNCH_TILES(K)                                                                          \
  if ((e = cudaFuncSetAttribute(K, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem))) return e; \
  K<<<grid, kTileThreads, smem, st>>>(a, tm, tw);
  if (res) {
    RTX_LAUNCH_TILES(kr)
  } else if (S == 6) {
    RTX_LAUNCH_TILES(k6)
  } else if (S == 4) {
    RTX_LAUNCH_TILES(k4)
  } else {
    RTX_LAUNCH_TILES(k2)
  }
#undef RTX_LAUNCH_TILES
  return cudaGetLastError();
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (null if
// the driver does not provide it)
static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      p = nullptr;
    return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }();
  return fn;
}

// Tensor map of an [imgs][H][W][C] BF16 tensor (C a multiple of 8) viewed as
// 5-D (8 channels, x, channel chunk, y, image), with a box of (8, box_w,
// box_chunks, box_rows, 1): the box lands in shared memory row, chunk,
// pixel major, 16 bytes per (pixel, chunk).  False if it cannot be encoded.
static bool chunk_major_map(CUtensorMap* m, const void* base, int imgs, int H, int W, int C, int box_w,
                            int box_chunks, int box_rows) {
  const PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
  if (!enc || (reinterpret_cast<uintptr_t>(base) & 15) || C % 8 || box_w > 256 || box_chunks > 256 ||
      box_rows > 256)
    return false;
  const cuuint64_t dims[5] = {8, (cuuint64_t)W, (cuuint64_t)(C / 8), (cuuint64_t)H, (cuuint64_t)imgs};
  const cuuint64_t strides[4] = {(cuuint64_t)C * 2, 16, (cuuint64_t)W * C * 2, (cuuint64_t)H * W * C * 2};
  const cuuint32_t box[5] = {8, (cuuint32_t)box_w, (cuuint32_t)box_chunks, (cuuint32_t)box_rows, 1};
  const cuuint32_t es[5] = {1, 1, 1, 1, 1};
  return enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<void*>(base), dims, strides, box, es,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Tensor map of a [rows][9][K] BF16 weight array (rows, K multiples of 16)
// viewed as 5-D (8 of K, row % 8, K chunk, row / 8, tap) with a box of (8, 8,
// 2, box_rows / 8, 9): a slice's nine K-major [box_rows x 16] tiles land
// tap-major in the no-swizzle core-matrix layout (tc::tile_offset).  False
// if it cannot be encoded.
static bool weight_map(CUtensorMap* m, const void* base, int rows, int K, int box_rows) {
  const PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
  if (!enc || (reinterpret_cast<uintptr_t>(base) & 15) || rows % 8 || K % 16 || box_rows % 8 || box_rows > 2048)
    return false;
  const cuuint64_t dims[5] = {8, 8, (cuuint64_t)(K / 8), (cuuint64_t)(rows / 8), 9};
  const cuuint64_t strides[4] = {(cuuint64_t)9 * K * 2, 16, (cuuint64_t)8 * 9 * K * 2, (cuuint64_t)K * 2};
  const cuuint32_t box[5] = {8, 8, 2, (cuuint32_t)(box_rows / 8), 9};
  const cuuint32_t es[5] = {1, 1, 1, 1, 1};
  return enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<void*>(base), dims, strides, box, es,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// weights kept in shared memory by the persistent kernels up to this size
// (128 KB: with 1 KB-aligned tensor-copy halo stages, 7 x 13 KB + 128 KB
// fits the 227 KB of a CTA; measured 0.75 % faster per training step than 96)
constexpr size_t kResidentWeights = 128 * 1024;

cudaError_t conv_fwd(const ConvFwd& a, cudaStream_t st) {
  long long P = (long long)a.N * a.H * a.W;
  if (a.Cout % 16 || a.Cout > 256 || a.Cin % 8) return cudaErrorInvalidValue;
  if (use_rows(a.W, a.Cin)) {
    const size_t wbytes = (size_t)9 * a.Cin * a.Cout * 2;
    const bool res = wbytes <= kResidentWeights;
    // one full-resolution source: halo slices (and streamed weight tiles)
    // arrive as tensor copies, if the maps encode
    CUtensorMap tm{}, tw{};
    const bool tma = kConvTma && !a.s2.ptr && !a.s1.up && a.s1.C == a.Cin &&
                     chunk_major_map(&tm, a.s1.ptr, a.N, a.H, a.W, a.Cin, kHalo, 2, 3) &&
                     (res || weight_map(&tw, a.w, a.Cout, a.Cin, a.Cout));
    const size_t wtiles = (size_t)9 * a.Cout * 32;
    const size_t stage = tma ? kHaloStage + (res ? 0 : (wtiles + 1023) / 1024 * 1024)
                             : (res ? kHaloBytes : kHaloBytes + wtiles);
    const long long T = (long long)a.N * a.H * ((a.W + 127) / 128);
    if (tma)
      return launch_tiles(k_conv_fwd_rows<7, true, true>, k_conv_fwd_rows<6, false, true>,
                          k_conv_fwd_rows<4, false, true>, k_conv_fwd_rows<2, false, true>, res, stage,
                          res ? wbytes : 0, T, a, tm, tw, st);
    return launch_tiles(k_conv_fwd_rows<7, true>, k_conv_fwd_rows<6, false>, k_conv_fwd_rows<4, false>,
                        k_conv_fwd_rows<2, false>, res, stage, res ? wbytes : 0, T, a, tm, tw, st);
  }
  size_t stage = 128 * kSlice * 2 + (size_t)a.Cout * kSlice * 2;
  const dim3 grid((unsigned)((P + 127) / 128));
  return launch_staged(k_conv_fwd<4>, k_conv_fwd<3>, k_conv_fwd<2>, gather_stages(a.Cout, grid, stage), grid,
                       stage, a, st);
}

cudaError_t conv_dgrad(const ConvDgrad& a, cudaStream_t st) {
  long long P = (long long)a.N * a.H * a.W;
  if (a.Cin % 16 || a.Cout % 8) return cudaErrorInvalidValue;
  const int nt = (a.Cin + 255) / 256;
  if (use_rows(a.W, a.Cout)) {
    ConvDgrad b = a;
    b.ctw = std::min(256, a.Cin);
    const size_t wbytes = (size_t)nt * b.ctw * 9 * a.Cout * 2;
    const bool res = wbytes <= kResidentWeights;
    if (!res) {
      // streamed weights: split the channels into the fewest equal tiles
      // (multiples of 16) whose stage lets at least four stages fit
      for (int k = 1; k <= 16; ++k) {
        const int w = ((a.Cin + k - 1) / k + 15) / 16 * 16;
        if (w > 256) continue;
        b.ctw = w;
        if (4 * (kHaloBytes + (size_t)9 * w * 32) <= 200 * 1024) break;
      }
    }
    const int ntb = (a.Cin + b.ctw - 1) / b.ctw;
    // dout's halo slices (and streamed weight tiles) arrive as tensor
    // copies, if the maps encode
    CUtensorMap tm{}, tw{};
    const int ntm = std::min(b.ctw, a.Cin);  // rows of the widest channel tile
    const bool tma = kConvTma && a.Cout % 16 == 0 &&
                     chunk_major_map(&tm, a.dout, a.N, a.H, a.W, a.Cout, kHalo, 2, 3) &&
                     (res || weight_map(&tw, a.wt, a.Cin, a.Cout, ntm));
    const size_t wtiles = (size_t)9 * ntm * 32;
    const size_t stage = tma ? kHaloStage + (res ? 0 : (wtiles + 1023) / 1024 * 1024)
                             : (res ? kHaloBytes : kHaloBytes + (size_t)9 * b.ctw * 32);
    const long long T = (long long)a.N * a.H * ((a.W + 127) / 128) * ntb;
    if (tma)
      return launch_tiles(k_conv_dgrad_rows<7, true, true>, k_conv_dgrad_rows<6, false, true>,
                          k_conv_dgrad_rows<4, false, true>, k_conv_dgrad_rows<2, false, true>, res, stage,
                          res ? wbytes : 0, T, b, tm, tw, st);
    return launch_tiles(k_conv_dgrad_rows<7, true>, k_conv_dgrad_rows<6, false>, k_conv_dgrad_rows<4, false>,
                        k_conv_dgrad_rows<2, false>, res, stage, res ? wbytes : 0, T, b, tm, tw, st);
  }
  int nb = std::min(256, a.Cin);
  size_t stage = 128 * kSlice * 2 + (size_t)nb * kSlice * 2;
  const dim3 grid((unsigned)((P + 127) / 128), (a.Cin + 255) / 256);
  return launch_staged(k_conv_dgrad<4>, k_conv_dgrad<3>, k_conv_dgrad<2>, gather_stages(nb, grid, stage), grid,
                       stage, a, st);
}

int wgrad_pixels_per_cta(long long P, int Cout, int Cin) {
  (void)Cout;
  int tiles = (9 * Cin + 127) / 128;
  long long ranges = std::max(1, 8 * 152 / tiles);
  long long per = (P + ranges - 1) / ranges;
  per = (per + 63) / 64 * 64;
  return (int)std::max(64LL, std::min(per, 1LL << 30));
}

// Channels per CTA of the row-tile weight gradient (16, 32 or 48; the last
// range may be narrower): fewest ranges, weighing each range's fixed dout
// copy against its width.
static int wgrad_row_channels(int Cin, int Cout) {
  int best = 16;
  long long best_cost = -1;
  for (int cr : {48, 32, 16}) {
    if (cr > Cin) continue;
    long long cost = (long long)((Cin + cr - 1) / cr) * (cr + Cout / 4 + 8);
    if (best_cost < 0 || cost < best_cost) best = cr, best_cost = cost;
  }
  return best;
}

// The row-tile weight gradient with S ring stages (2..7): each stage has its
// own producer warp, so a deeper ring is also more warps copying at once
// (tensor-copy form: one issuing thread for all stages).
template <bool kSwap, bool kTma>
static cudaError_t launch_wgrad_row(int S, dim3 grid, size_t smem, const ConvWgrad& a, const CUtensorMap& ms,
                                    const CUtensorMap& md, cudaStream_t st) {
  auto go = [&](auto kern) -> cudaError_t {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e) return e;
    kern<<<grid, kThreads, smem, st>>>(a, ms, md);
    return cudaGetLastError();
  };
  switch (S) {
    case 7: return go(k_conv_wgrad_row<7, kSwap, kTma>);
    case 6: return go(k_conv_wgrad_row<6, kSwap, kTma>);
    case 5: return go(k_conv_wgrad_row<5, kSwap, kTma>);
    case 4: return go(k_conv_wgrad_row<4, kSwap, kTma>);
    case 3: return go(k_conv_wgrad_row<3, kSwap, kTma>);
    default: return go(k_conv_wgrad_row<2, kSwap, kTma>);
  }
}

cudaError_t conv_wgrad(const ConvWgrad& a0, cudaStream_t st) {
  long long P = (long long)a0.N * a0.H * a0.W;
  if (P >= (1LL << 31) || a0.Cout % 16 || a0.Cout > 256) return cudaErrorInvalidValue;
  constexpr size_t kRing = 190 * 1024;  // shared memory for the ring
  auto stages = [&](size_t stage) { return (int)std::min<size_t>(kProducerWarps, kRing / stage); };
  if (use_rows(a0.W, a0.Cin) && 9 * a0.Cout <= 512 && a0.Cin >= 64) {
    // narrow outputs: source channels on the accumulator lanes (kSwap)
    ConvWgrad a = a0;
    const int nr = (a.Cin + 127) / 128;
    a.cr = (a.Cin + nr - 1) / nr;
    a.cr = (a.cr + 15) / 16 * 16;
    const int nch = a.cr / 8;
    auto stage_of = [&](int tw) { return (size_t)a.Cout * tw * 2 + (size_t)3 * nch * (tw + 2) * 16; };
    // the tile width whose ring is deepest (ties: the wider tile)
    a.tw = stages(stage_of(32)) > stages(stage_of(64)) ? 32 : 64;
    const size_t stage = stage_of(a.tw);
    const int S = std::max(2, stages(stage));
    const long long T = (long long)a.N * a.H * ((a.W + a.tw - 1) / a.tw);
    const int TW2 = a.tw + 2;
    // the MMA's A operand spans 128 channel rows of a halo row: at the last
    // stage's last halo row that reaches past the halo by this much
    const size_t a_over = ((size_t)(16 - std::min(nch, 16)) * TW2 + a.tw + 2) * 16;
    const long long ctas = (long long)sm_count();  // 512 TMEM columns: one CTA per SM
    const long long npg = std::max(1LL, ctas / nr);
    a.tiles_per_cta = (int)((T + npg - 1) / npg);
    const unsigned gy = (unsigned)((T + a.tiles_per_cta - 1) / a.tiles_per_cta);
    const CUtensorMap none{};
    return launch_wgrad_row<true, false>(S, dim3(nr, gy), S * stage + a_over, a, none, none, st);
  }
  if (use_rows(a0.W, a0.Cin) && a0.Cout <= 128) {
    ConvWgrad a = a0;
    a.cr = wgrad_row_channels(a.Cin, a.Cout);
    const int nr = (a.Cin + a.cr - 1) / a.cr;
    a.tw = a.W >= 128 ? 128 : 64;
    // a single full-resolution source whose channels split evenly over the
    // CTAs: the tensor-copy form, if both maps encode
    CUtensorMap ms{}, md{};
    const bool tma = kConvTma && !a.s2.ptr && !a.s1.up && a.Cin % a.cr == 0 &&
                     chunk_major_map(&ms, a.s1.ptr, a.N, a.H, a.W, a.Cin, a.tw + 2, a.cr / 8, 3) &&
                     chunk_major_map(&md, a.dout, 1, a.N * a.H, a.W, a.Cout, a.tw, a.Cout / 8, 1);
    const size_t tx = (size_t)a.Cout * a.tw * 2 + (size_t)3 * (a.cr / 8) * (a.tw + 2) * 16;
    const size_t stage = tma ? (tx + 1023) / 1024 * 1024 : tx;
    // the MMA's A operand spans 128 rows of TW pixels; rows past Cout are
    // read (and their accumulator lanes ignored), so they must lie inside the
    // allocation
    const size_t a_span = (size_t)256 * a.tw;
    size_t extra = a_span > stage ? a_span - stage : 0;
    // at most 4 stages with producer warps: deeper rings (narrower tiles, or
    // more stages of the same tile) measured 0-10 % slower on these layers.
    // Tensor copies: as deep as fits, but not so deep that it costs the
    // second CTA per SM that a 256-column accumulator allows.
    int S = std::max(2, tma ? stages(stage) : std::min(4, stages(stage)));
    if (tma && 9 * a.cr <= 256 && 2 * stage + extra <= 110 * 1024)
      S = std::min(S, (int)((110 * 1024 - extra) / stage));
    const int per_sm = (9 * a.cr <= 256 && S * stage + extra <= 110 * 1024) ? 2 : 1;
    // one CTA per SM when it takes all 512 TMEM columns: a second CTA on the
    // SM would wait in its allocation for the first to finish
    if (per_sm == 1 && S * stage + extra < 116 * 1024) extra = 116 * 1024 - S * stage;
    const long long T = (long long)a.N * a.H * ((a.W + a.tw - 1) / a.tw);
    const long long ctas = (long long)sm_count() * per_sm;
    const long long npg = std::max(1LL, ctas / nr);
    a.tiles_per_cta = (int)((T + npg - 1) / npg);
    const unsigned gy = (unsigned)((T + a.tiles_per_cta - 1) / a.tiles_per_cta);
    if (tma) return launch_wgrad_row<false, true>(S, dim3(nr, gy), S * stage + extra, a, ms, md, st);
    return launch_wgrad_row<false, false>(S, dim3(nr, gy), S * stage + extra, a, ms, md, st);
  }
  const ConvWgrad& a = a0;
  size_t stage = 128 * kSlice * 2 + (size_t)a.Cout * kSlice * 2;
  dim3 grid((9 * a.Cin + 127) / 128, (unsigned)((P + a.pix_per_cta - 1) / a.pix_per_cta));
  return launch_staged(k_conv_wgrad<4>, k_conv_wgrad<3>, k_conv_wgrad<2>, stages_for(a.Cout), grid, stage, a, st);
}

}  // namespace nn
}  // namespace rtx
