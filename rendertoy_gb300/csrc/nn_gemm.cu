// nn_gemm.cu — BF16 GEMM on tcgen05 tensor cores (FP32 accumulation in
// TMEM): C[M x N] = A[M x K] * B[N x K]^T, A and B row-major (K contiguous).
//
// a_mn / b_mn: the operand is stored K x M (K x N), M (N) contiguous, and is
// staged in the MN-major canonical layout.
//
// One CTA of 128 threads owns a 128 x 128 tile of C.  For each 64-wide slice
// of K, all threads stage the A and B slices in shared memory in the
// canonical K-major layout (tc_core.cuh), one thread issues four
// 128 x 128 x 16 MMAs and commits them to an mbarrier, and the CTA waits for
// it before reusing the buffers.  The epilogue reads the accumulator from
// TMEM (each warp its 32 lanes = rows) and writes FP32.
//
// This is the denoiser's GEMM engine in its plainest form and the entry point
// its layout and descriptor conventions are validated through.
#include "tc_core.cuh"

namespace rtx {

constexpr int kGemmTile = 128;  // rows of A / B per CTA
constexpr int kGemmK = 64;      // K per shared-memory slice

// 16 bytes of operand X for tile row `row`, K index k (8 elements along K
// for a K-major operand, along the rows for an MN-major one).
__device__ __forceinline__ uint4 load_chunk(const __nv_bfloat16* X, bool mn, int rows_total, int K,
                                            int row, int k) {
  uint4 v = make_uint4(0, 0, 0, 0);
  if (!mn) {
    if (row < rows_total && k < K) v = *reinterpret_cast<const uint4*>(X + (size_t)row * K + k);
  } else {
    if (row < rows_total && k < K) v = *reinterpret_cast<const uint4*>(X + (size_t)k * rows_total + row);
  }
  return v;
}

__global__ void __launch_bounds__(128) k_gemm_bf16(const __nv_bfloat16* __restrict__ A,
                                                   const __nv_bfloat16* __restrict__ B,
                                                   float* __restrict__ C, int M, int N, int K,
                                                   int a_mn, int b_mn, int* err) {
  extern __shared__ __align__(1024) uint8_t smem[];
  uint8_t* sa = smem;
  uint8_t* sb = smem + kGemmTile * kGemmK * 2;
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t tmem_slot;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.x * kGemmTile, n0 = blockIdx.y * kGemmTile;

  if (warp == 0) tc::tmem_alloc(&tmem_slot, 128);
  if (tid == 0) {
    tc::mbar_init(&bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t tmem = tmem_slot;
  const uint32_t idesc = tc::make_idesc_bf16(128, 128, a_mn != 0, b_mn != 0);
  uint32_t phase = 0;
  bool ok = true;

  for (int k0 = 0; k0 < K && ok; k0 += kGemmK) {
    // 16-byte chunks: 1024 per operand (128 rows x 64 K)
    for (int c = tid; c < kGemmTile * (kGemmK / 8); c += 128) {
      // K-major chunk: row c >> 3, K 8 (c & 7); MN-major chunk: rows 8 (c & 15), K c >> 4
      int rk = c >> 3, kk = (c & 7) * 8;
      int rm = (c & 15) * 8, km = c >> 4;
      if (!a_mn)
        *reinterpret_cast<uint4*>(sa + tc::tile_offset(rk, kk, kGemmK)) =
            load_chunk(A, false, M, K, m0 + rk, k0 + kk);
      else
        *reinterpret_cast<uint4*>(sa + tc::tile_offset_mn(rm, km, kGemmTile)) =
            load_chunk(A, true, M, K, m0 + rm, k0 + km);
      if (!b_mn)
        *reinterpret_cast<uint4*>(sb + tc::tile_offset(rk, kk, kGemmK)) =
            load_chunk(B, false, N, K, n0 + rk, k0 + kk);
      else
        *reinterpret_cast<uint4*>(sb + tc::tile_offset_mn(rm, km, kGemmTile)) =
            load_chunk(B, true, N, K, n0 + rm, k0 + km);
    }
    tc::fence_proxy_async();
    __syncthreads();
    if (tid == 0) {
      tc::fence_after();
      uint32_t a0 = tc::smem_u32(sa), b0 = tc::smem_u32(sb);
#pragma unroll
      for (int s = 0; s < kGemmK / 16; ++s) {
        // K-major: 16 K = two core matrices along K (256 B); MN-major: two
        // 8-step K groups (2 x 16 * rows B)
        uint64_t ad = a_mn ? tc::make_desc(a0 + s * 2 * 16 * kGemmTile, 16 * kGemmTile, 128)
                           : tc::make_desc(a0 + s * 256, 128, (kGemmK / 8) * 128);
        uint64_t bd = b_mn ? tc::make_desc(b0 + s * 2 * 16 * kGemmTile, 16 * kGemmTile, 128)
                           : tc::make_desc(b0 + s * 256, 128, (kGemmK / 8) * 128);
        tc::mma_bf16(tmem, ad, bd, idesc, k0 > 0 || s > 0);
      }
      tc::mma_commit(&bar);
    }
    if (!tc::mbar_wait(&bar, phase)) {
      if (lane == 0) atomicOr(err, tc::kErrMbarTimeout);
      ok = false;
    }
    phase ^= 1;
    __syncthreads();
  }

  tc::fence_after();
  if (ok) {
    const int row = warp * 32 + lane;
    const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16);
    for (int c = 0; c < kGemmTile; c += 8) {
      float v[8];
      tc::tmem_ld8(taddr + c, v);
      if (m0 + row < M)
        for (int i = 0; i < 8; ++i)
          if (n0 + c + i < N) C[(size_t)(m0 + row) * N + n0 + c + i] = v[i];
    }
  }
  tc::fence_before();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, 128);
}

cudaError_t launch_gemm_bf16(const void* A, const void* B, float* C, int M, int N, int K, int a_mn,
                             int b_mn, int* err, cudaStream_t st) {
  dim3 grid((M + kGemmTile - 1) / kGemmTile, (N + kGemmTile - 1) / kGemmTile);
  // two 16 KB operand tiles; the allocation is 64 KB so that every address the
  // descriptors can form (either reading of LBO / SBO) stays inside it
  size_t smem = 64 * 1024;
  cudaError_t e = cudaFuncSetAttribute(k_gemm_bf16, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  k_gemm_bf16<<<grid, 128, smem, st>>>((const __nv_bfloat16*)A, (const __nv_bfloat16*)B, C, M, N, K,
                                       a_mn, b_mn, err);
  return cudaGetLastError();
}

}  // namespace rtx
