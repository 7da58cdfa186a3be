// probe_kernels.cu — a plain streaming read of one device buffer: the read
// bandwidth a kernel can draw from L2 when the buffer fits in it (or from HBM
// when it does not).  It is the denominator of the traversal kernels' L2
// roofline: the BVH and triangles of a scene of about a million triangles fit
// the 129 MB L2, so their fetches are bounded by L2, not HBM, bandwidth.
//
// Every thread reads 16-byte vectors with ld.global.cg (cached in L2 only,
// so L1 hits cannot inflate the figure), four independent loads in flight per
// iteration, over a grid-stride walk of the whole buffer, `passes` times in
// one launch.  The loaded words are folded with XOR (no floating point) into
// one word per thread, written only if it equals an impossible value, so the
// loads cannot be removed.
#include "rtx_internal.h"
#include "tc_core.cuh"

namespace rtx {

namespace {

__device__ __forceinline__ uint4 ld_cg(const uint4* p) {
  uint4 v;
  asm volatile("ld.global.cg.v4.u32 {%0, %1, %2, %3}, [%4];"
               : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
               : "l"(p));
  return v;
}

__global__ void __launch_bounds__(256) k_read_probe(const uint4* __restrict__ p, size_t n16,
                                                    int passes, uint32_t* __restrict__ sink) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  const size_t t0 = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t acc = 0;
  for (int r = 0; r < passes; ++r) {
    size_t i = t0;
    for (; i + 3 * stride < n16; i += 4 * stride) {
      const uint4 a = ld_cg(p + i), b = ld_cg(p + i + stride), c = ld_cg(p + i + 2 * stride),
                  d = ld_cg(p + i + 3 * stride);
      acc ^= a.x ^ a.y ^ a.z ^ a.w ^ b.x ^ b.y ^ b.z ^ b.w ^ c.x ^ c.y ^ c.z ^ c.w ^ d.x ^ d.y ^
             d.z ^ d.w;
    }
    for (; i < n16; i += stride) {
      const uint4 a = ld_cg(p + i);
      acc ^= a.x ^ a.y ^ a.z ^ a.w;
    }
    acc = (acc << 1) | (acc >> 31);  // keep the passes distinct
  }
  if (acc == 0x9E3779B9u) sink[t0 & 255] = acc;
}

// The bounded mbarrier wait of the tensor-core kernels, on a barrier that
// nothing arrives on: every thread gives up after `polls` polls and warp
// leaders report the timeout through the error word, as the convolution
// kernels do.  No copy or MMA is in flight, so returning is all that is left.
__global__ void k_wait_timeout(int polls, int* err) {
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) tc::mbar_init(&bar, 1);
  __syncthreads();
  const bool ok = tc::mbar_wait_bounded(&bar, 0, polls);
  if (!ok && (threadIdx.x & 31) == 0) atomicOr(err, tc::kErrMbarTimeout);
}

}  // namespace

cudaError_t launch_wait_timeout(int polls, int* err, cudaStream_t st) {
  k_wait_timeout<<<1, 64, 0, st>>>(polls, err);
  return cudaGetLastError();
}

cudaError_t launch_read_probe(const void* buf, size_t bytes, int passes, uint32_t* sink, int sms,
                              cudaStream_t st) {
  const int blocks = sms * 8;  // 2,048 threads per SM, 4 loads of 16 B in flight each
  k_read_probe<<<blocks, 256, 0, st>>>((const uint4*)buf, bytes / 16, passes, sink);
  return cudaGetLastError();
}

}  // namespace rtx
