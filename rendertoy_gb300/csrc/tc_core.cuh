// tc_core.cuh — 5th-generation tensor-core (tcgen05) building blocks for the
// denoiser's GEMM-shaped work: TMEM allocation, shared-memory matrix
// descriptors, BF16 MMA with FP32 accumulation in TMEM, commit to an
// mbarrier, bounded waits, and the TMEM -> register epilogue load.
//
// Operand tiles are staged in shared memory in the canonical K-major layout
// without swizzle: 8 x 16-byte "core matrices" (8 rows x 8 BF16); core matrix
// (i, j) of a tile (rows 8i.., K elements 8j..) lives at i * SBO + j * LBO.
// Tiles here use LBO = 128 B (K neighbours adjacent) and SBO = 128 B * (K/8).
#pragma once
#include <cuda_bf16.h>
#include <cstdint>

#include "rtx_internal.h"

namespace rtx {
namespace tc {

constexpr int kWaitLimit = 1 << 22;  // bounded spin on an mbarrier (far above any legitimate wait)
enum TcError : int { kErrMbarTimeout = 8 };

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// Shared-memory matrix descriptor (tcgen05): start address, leading- and
// stride-dimension byte offsets (all >> 4), descriptor version 1 (bit 46),
// no swizzle.
__device__ __forceinline__ uint64_t make_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// Instruction descriptor for kind::f16: FP32 accumulator, BF16 A and B,
// shape M x N (x 16); a_mn / b_mn select MN-major instead of K-major operands.
__host__ __device__ constexpr uint32_t make_idesc_bf16(int M, int N, bool a_mn = false,
                                                       bool b_mn = false) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((a_mn ? 1u : 0u) << 15) | ((b_mn ? 1u : 0u) << 16) |
         ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void tmem_alloc(uint32_t* smem_slot, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(smem_slot)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// generic-proxy shared-memory writes -> visible to the tensor core's reads
__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// 16-byte asynchronous copy global -> shared; src_bytes 0 zero-fills the
// destination without reading (src must still be a valid address)
__device__ __forceinline__ void cp_async16(uint32_t dst, const void* src, uint32_t src_bytes) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src), "r"(src_bytes) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// One arrival on the barrier (release: this thread's earlier writes are
// visible to a thread that observes the phase complete).
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.release.cta.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// Wait for phase `parity` of the barrier; false after `limit` polls.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, int limit) {
  uint32_t a = smem_u32(bar);
  for (int i = 0; i < limit; ++i) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  return mbar_wait_bounded(bar, parity, kWaitLimit);
}

// Arrive on the barrier and add `bytes` to the transaction count its phase
// waits for (the bytes of the tensor copies that complete on it).
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.release.cta.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

// Tensor copy (TMA) of one box of a 5-D tensor map into shared memory at
// dst, completing its bytes on `bar`.  The map is a __grid_constant__ kernel
// parameter; c0 is the innermost coordinate (kept 16-byte aligned: 0 here).
// Coordinates outside the tensor read zeros.
__device__ __forceinline__ void tma_load_5d(uint32_t dst, const void* tmap, int c0, int c1, int c2, int c3, int c4,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4, %5, %6}], [%7];" ::"r"(dst),
      "l"(tmap), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(c4), "r"(smem_u32(bar))
      : "memory");
}

// D (TMEM) [+]= A (smem desc) * B (smem desc)^T, one M x N x 16 step.
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         bool accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"((uint32_t)accumulate)
      : "memory");
}

// Arrive on `bar` when every MMA issued so far by this thread has completed.
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   smem_u32(bar))
               : "memory");
}

// 8 consecutive FP32 columns of this thread's TMEM lane (warp w of a
// warpgroup reads lanes 32w .. 32w + 31).
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float* v) {
  uint32_t r[8];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                 "=r"(r[7])
               : "r"(taddr)
               : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}

// Byte offset of element (row, k) in a K-major no-swizzle tile whose rows
// hold kdim elements (kdim a multiple of 8): LBO = 128, SBO = 16 * kdim.
__host__ __device__ constexpr uint32_t tile_offset(int row, int k, int kdim) {
  return (uint32_t)(((row >> 3) * (kdim >> 3) + (k >> 3)) * 128 + (row & 7) * 16 + (k & 7) * 2);
}

// Byte offset of element (row, k) in an MN-major no-swizzle tile of `rows`
// rows (a multiple of 8): a core matrix holds 8 K-steps x 8 consecutive rows;
// SBO (next 8 rows) = 128, LBO (next 8 K-steps) = 16 * rows.
__host__ __device__ constexpr uint32_t tile_offset_mn(int row, int k, int rows) {
  return (uint32_t)(((k >> 3) * (rows >> 3) + (row >> 3)) * 128 + (k & 7) * 16 + (row & 7) * 2);
}

}  // namespace tc
}  // namespace rtx
