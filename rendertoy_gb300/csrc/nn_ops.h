// nn_ops.h — launchers of the denoiser's memory-bound operators (nn_ops.cu).
#pragma once
#include "nn.h"

namespace rtx {
namespace nn {

cudaError_t encode_input(const float* raw, bf16* x, long long P, cudaStream_t st);
cudaError_t avgpool(const bf16* in, bf16* out, int N, int H, int W, int C, cudaStream_t st);
cudaError_t upsample_grad(const bf16* dcat, int Ccat, int c0, bf16* dlow, int N, int H, int W, int C,
                          cudaStream_t st);
cudaError_t take_channels(const bf16* dcat, int Ccat, int c0, bf16* dst, long long P, int C, cudaStream_t st);
cudaError_t pool_grad_acc(const bf16* dpool, const bf16* skip, bf16* dskip, int N, int H, int W, int C,
                          cudaStream_t st);
// loss of the kernel-predicting output of N frames of H x W (see nn.h);
// adds the summed per-pixel, per-channel loss to *loss
cudaError_t kp_loss(const float* pred, const float* raw, const float* target, bf16* dpred, int N, int H,
                    int W, double* loss, cudaStream_t st);
cudaError_t bias_grad(const bf16* dout, long long P, int C, float* db, cudaStream_t st);
// Several layers' bias gradients (db_i[c] += sum_p dout_i[p, c]) in one launch
struct BiasGrads {
  static constexpr int kMax = 16;
  int n = 0;
  const bf16* dout[kMax];
  long long P[kMax];
  int C[kMax];
  long long per_block[kMax];  // set by bias_grads
  float* db[kMax];
};
cudaError_t bias_grads(BiasGrads jobs, cudaStream_t st);
cudaError_t adam(float* p, const float* g, float* m, float* v, long long n, float lr, int step,
                 cudaStream_t st);
cudaError_t weights_bf16(const float* master, bf16* w, bf16* wt, int Cout, int Cin, cudaStream_t st);
// Several layers' BF16 weights w [Cout][9][Cin] and transposes wt [Cin][9][Cout]
// from their FP32 masters in one launch
struct WeightLayouts {
  static constexpr int kMax = 16;
  int n = 0;
  const float* master[kMax];
  bf16* w[kMax];
  bf16* wt[kMax];
  int Cout[kMax], Cin[kMax];
};
cudaError_t weights_bf16_all(const WeightLayouts& layers, cudaStream_t st);
// out [N][Hc][Wc][3] = the predicted filters applied to the input radiance of
// frames stored as Hs x Ws pixels (pred and raw share that layout)
cudaError_t kp_apply(const float* pred, const float* raw, float* out, int N, int Hc, int Wc, int Hs, int Ws,
                     cudaStream_t st);
cudaError_t pack_passes(const float* rad, const float* alb, const float* nrm, const float* dep, float spp,
                        float* raw, int W, int H, int Wp, int Hp, cudaStream_t st);

}  // namespace nn
}  // namespace rtx
