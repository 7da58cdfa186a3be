// nn_gemm.cu — BF16 GEMM on tcgen05 tensor cores (FP32 accumulation in
// TMEM): C[M x N] = A[M x K] * B[N x K]^T, A and B row-major (K contiguous).
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

__global__ void __launch_bounds__(128) k_gemm_bf16(const __nv_bfloat16* __restrict__ A,
                                                   const __nv_bfloat16* __restrict__ B,
                                                   float* __restrict__ C, int M, int N, int K,
                                                   int* err) {
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
  const uint32_t idesc = tc::make_idesc_bf16(128, 128);
  uint32_t phase = 0;
  bool ok = true;

  for (int k0 = 0; k0 < K && ok; k0 += kGemmK) {
    // 16-byte chunks: 128 rows x 8 chunks per operand
    for (int c = tid; c < kGemmTile * (kGemmK / 8); c += 128) {
      int row = c >> 3, kc = c & 7;
      int k = k0 + kc * 8;
      uint4 va = make_uint4(0, 0, 0, 0), vb = make_uint4(0, 0, 0, 0);
      if (m0 + row < M && k < K) va = *reinterpret_cast<const uint4*>(A + (size_t)(m0 + row) * K + k);
      if (n0 + row < N && k < K) vb = *reinterpret_cast<const uint4*>(B + (size_t)(n0 + row) * K + k);
      *reinterpret_cast<uint4*>(sa + tc::tile_offset(row, kc * 8, kGemmK)) = va;
      *reinterpret_cast<uint4*>(sb + tc::tile_offset(row, kc * 8, kGemmK)) = vb;
    }
    tc::fence_proxy_async();
    __syncthreads();
    if (tid == 0) {
      tc::fence_after();
      uint32_t a0 = tc::smem_u32(sa), b0 = tc::smem_u32(sb);
#pragma unroll
      for (int s = 0; s < kGemmK / 16; ++s) {
        uint64_t ad = tc::make_desc(a0 + s * 256, 128, (kGemmK / 8) * 128);
        uint64_t bd = tc::make_desc(b0 + s * 256, 128, (kGemmK / 8) * 128);
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

cudaError_t launch_gemm_bf16(const void* A, const void* B, float* C, int M, int N, int K, int* err,
                             cudaStream_t st) {
  dim3 grid((M + kGemmTile - 1) / kGemmTile, (N + kGemmTile - 1) / kGemmTile);
  size_t smem = 2 * kGemmTile * kGemmK * 2;
  k_gemm_bf16<<<grid, 128, smem, st>>>((const __nv_bfloat16*)A, (const __nv_bfloat16*)B, C, M, N, K, err);
  return cudaGetLastError();
}

}  // namespace rtx
