// nn_unet.h — the learned denoiser (nn_unet.cu): a 5-level U-Net trained
// and run on the tcgen05 convolutions.  Inputs are device pointers; H and W
// must be multiples of 16 (four 2 x 2 poolings).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

namespace rtx {
namespace nn {

class UNet {
 public:
  UNet();
  ~UNet();
  UNet(const UNet&) = delete;
  UNet& operator=(const UNet&) = delete;

  // He-normal weights from `seed`, zero biases, Adam state cleared
  cudaError_t init(uint64_t seed, cudaStream_t st);
  int64_t num_params() const;       // FP32 entries of the padded parameter array
  int64_t num_real_params() const;  // parameters of the network proper
  int step() const;                 // Adam steps taken
  static int num_layers();
  int last_launches() const;  // kernels launched by the last forward / step
  // cout_pad, cout, cin_pad, cin, c1_pad, up1, relu, level, w_off, b_off, s1
  void layer_info(int layer, int64_t* info) const;

  cudaError_t set_params(const float* host, cudaStream_t st);
  cudaError_t get_params(float* host, cudaStream_t st) const;
  cudaError_t get_grads(float* host, cudaStream_t st) const;
  cudaError_t get_state(float* host_m, float* host_v, cudaStream_t st) const;
  cudaError_t set_state(const float* host_m, const float* host_v, int step, cudaStream_t st);

  // raw [N*H*W][kRawCh] = radiance 3, albedo 3, normal 3, depth 1, spp 1 (FP32)
  cudaError_t forward(const float* d_raw, int N, int H, int W, int* err, cudaStream_t st);
  // gradients of the loss of the last forward (d_pred set by the loss)
  cudaError_t backward(int N, int H, int W, int* err, cudaStream_t st);
  // forward + loss against target [N*H*W][3] + backward (no update)
  cudaError_t loss_and_grads(const float* d_raw, const float* d_target, int N, int H, int W,
                             double* loss, int* err, cudaStream_t st);
  // forward + loss + backward + Adam + BF16 weight refresh
  cudaError_t train_step(const float* d_raw, const float* d_target, int N, int H, int W, float lr,
                         double* loss, int* err, cudaStream_t st);
  // out [N][Hc][Wc][3] = the last forward's predicted filters applied to the
  // radiance of d_raw (the same input), frames stored as Hs x Ws pixels
  cudaError_t decode(const float* d_raw, float* d_out, int N, int Hc, int Wc, int Hs, int Ws,
                     cudaStream_t st) const;

  cudaError_t reserve(long long P0);  // activation buffers for P0 pixels
  float* scratch_raw();               // [P0][kRawCh] staging for host inputs
  float* scratch_target();            // [P0][3]
  const float* prediction() const;    // [P0][kPredCh] FP32 filter logits

 private:
  cudaError_t refresh_weights(cudaStream_t st);
  struct Impl;
  Impl* p_;
};

}  // namespace nn
}  // namespace rtx
