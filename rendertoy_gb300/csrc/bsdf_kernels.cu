// bsdf_kernels.cu — the device principled BSDF (device_math.cuh) applied to
// arrays of independent cases: PrincipledBSDF::Eval (RenderToy
// src/material.cpp:143-204) and PrincipledBSDF::Sample (material.cpp:206-295).
// These run the very functions the shading kernel inlines, so that the BSDF
// can be checked lobe by lobe on its own instead of only through whole paths.
#include "device_math.cuh"
#include "rtx_internal.h"

namespace rtx {

namespace {

RTX_DEV F3 ld3(const float* p, int i) { return f3(p[3 * i], p[3 * i + 1], p[3 * i + 2]); }
RTX_DEV void st3(float* p, int i, F3 v) {
  p[3 * i] = v.x;
  p[3 * i + 1] = v.y;
  p[3 * i + 2] = v.z;
}

__global__ void k_bsdf_eval(int n, const float* __restrict__ mats, const float* __restrict__ eta,
                            const float* __restrict__ N, const float* __restrict__ V,
                            const float* __restrict__ L, float* __restrict__ f_out,
                            float* __restrict__ pdf_out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const Mat m = load_mat(mats + 24 * (size_t)i);
  float pdf;
  const F3 f = BsdfEval(m, eta[i], ld3(V, i), ld3(N, i), ld3(L, i), pdf);
  st3(f_out, i, f);
  pdf_out[i] = pdf;
}

// Case i draws its two numbers as path (pixel i, sample `sample`) draws 0
// and 1 of the Philox stream: the order of material.cpp:214-215.
__global__ void k_bsdf_sample(int n, const float* __restrict__ mats, const float* __restrict__ eta,
                              const float* __restrict__ N, const float* __restrict__ in_dir,
                              uint32_t k0, uint32_t k1, uint32_t sample, int* __restrict__ ok_out,
                              float* __restrict__ dir_out, float* __restrict__ color_out,
                              float* __restrict__ pdf_out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const Mat m = load_mat(mats + 24 * (size_t)i);
  Rng rng{k0, k1, (uint32_t)i, sample, 0u};
  const float r1 = rng.uniform();
  const float r2 = rng.uniform();
  F3 od = f3s(0.0f), col = f3s(0.0f);
  float pdf = 0.0f;
  const bool ok = BsdfSample(m, eta[i], ld3(N, i), ld3(in_dir, i), r1, r2, od, col, pdf);
  ok_out[i] = ok ? 1 : 0;
  st3(dir_out, i, od);
  st3(color_out, i, col);
  pdf_out[i] = pdf;
}

}  // namespace

cudaError_t launch_bsdf_eval(int n, const float* mats, const float* eta, const float* N,
                             const float* V, const float* L, float* f, float* pdf, cudaStream_t st) {
  k_bsdf_eval<<<(n + 127) / 128, 128, 0, st>>>(n, mats, eta, N, V, L, f, pdf);
  return cudaGetLastError();
}

cudaError_t launch_bsdf_sample(int n, const float* mats, const float* eta, const float* N,
                               const float* in_dir, uint64_t seed, int sample, int* ok, float* dir,
                               float* color, float* pdf, cudaStream_t st) {
  k_bsdf_sample<<<(n + 127) / 128, 128, 0, st>>>(n, mats, eta, N, in_dir, (uint32_t)seed,
                                                 (uint32_t)(seed >> 32), (uint32_t)sample, ok, dir,
                                                 color, pdf);
  return cudaGetLastError();
}

}  // namespace rtx
