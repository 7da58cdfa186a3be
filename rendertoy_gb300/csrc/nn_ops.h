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
cudaError_t l1log_loss(const float* pred, const float* target, bf16* dpred, long long P, double* loss,
                       cudaStream_t st);
cudaError_t bias_grad(const bf16* dout, long long P, int C, float* db, cudaStream_t st);
cudaError_t adam(float* p, const float* g, float* m, float* v, long long n, float lr, int step,
                 cudaStream_t st);
cudaError_t weights_bf16(const float* master, bf16* w, bf16* wt, int Cout, int Cin, cudaStream_t st);
cudaError_t decode_output(const float* pred, float* out, long long P, cudaStream_t st);
cudaError_t pack_passes(const float* rad, const float* alb, const float* nrm, const float* dep, float* raw,
                        int W, int H, int Wp, int Hp, cudaStream_t st);
cudaError_t decode_crop(const float* pred, float* out, int W, int H, int Wp, cudaStream_t st);

}  // namespace nn
}  // namespace rtx
