// nn_unet.cu — the learned denoiser: a 5-level U-Net over the renderer's
// low-spp radiance, its albedo / normal / depth passes and its samples per
// pixel, trained and run with the tcgen05 convolutions of nn_conv.cu.
// RenderToy has no counterpart (its demos call Intel OIDN, an external
// binary).
//
// Layers (3 x 3 convolutions, ReLU except the last; pooling 2 x 2 average,
// upsampling nearest; channels 32 / 64 / 96 / 128 / 160):
//   level 0: e0a 11->32, e0b 32->32 = S0         (H   x W)
//   level 1: e1a 32->64, e1b 64->64 = S1         (H/2)
//   level 2: e2a 64->96, e2b 96->96 = S2         (H/4)
//   level 3: e3a 96->128, e3b 128->128 = S3      (H/8)
//   level 4: bottleneck 128->160 = B             (H/16)
//   decoder: d3 [up(B), S3] 288->128, d2 [up, S2] 224->96,
//            d1 [up, S1] 160->64, d0 [up, S0] 96->32, out 32->25 (linear)
// The output is a 5 x 5 filter per pixel (softmax of 25 logits) applied to the
// input radiance; the loss is the relative squared error of the filtered
// radiance against the target (nn.h).
// Parameters live as FP32 masters in one flat array in the padded layout the
// kernels read (w [Cout][9][Cin] then b [Cout] per layer, padding zero and
// kept zero by construction); BF16 copies (and transposes for the data
// gradient) are refreshed after every Adam step.
#include <algorithm>
#include <cmath>
#include <random>
#include <vector>

#include "nn.h"
#include "nn_ops.h"
#include "nn_unet.h"

namespace rtx {
namespace nn {

namespace {

enum T {
  tX, tA0a, tS0, tP1, tA1a, tS1, tP2, tA2a, tS2, tP3, tA3a, tS3, tP4, tB, tU3, tU2, tU1, tU0, kTensors
};
// channels (padded) and level of every activation tensor
const int kTC[kTensors] = {16, 32, 32, 32, 64, 64, 64, 96, 96, 96, 128, 128, 128, 160, 128, 96, 64, 32};
const int kTL[kTensors] = {0, 0, 0, 1, 1, 1, 2, 2, 2, 3, 3, 3, 4, 4, 3, 2, 1, 0};

struct LayerDef {
  int s1, s1_up, s2;  // source tensors (s2 = -1: none)
  int out;            // output tensor (-1: the FP32 prediction)
  int cout_pad, cout_real, cin_real, relu;
};
const LayerDef kLayers[] = {
    {tX, 0, -1, tA0a, 32, 32, kRawCh, 1}, {tA0a, 0, -1, tS0, 32, 32, 32, 1},
    {tP1, 0, -1, tA1a, 64, 64, 32, 1},   {tA1a, 0, -1, tS1, 64, 64, 64, 1},
    {tP2, 0, -1, tA2a, 96, 96, 64, 1},   {tA2a, 0, -1, tS2, 96, 96, 96, 1},
    {tP3, 0, -1, tA3a, 128, 128, 96, 1}, {tA3a, 0, -1, tS3, 128, 128, 128, 1},
    {tP4, 0, -1, tB, 160, 160, 128, 1},  {tB, 1, tS3, tU3, 128, 128, 288, 1},
    {tU3, 1, tS2, tU2, 96, 96, 224, 1},  {tU2, 1, tS1, tU1, 64, 64, 160, 1},
    {tU1, 1, tS0, tU0, 32, 32, 96, 1},   {tU0, 0, -1, -1, kPredCh, kKpTaps, 32, 0},
};
constexpr int kNumLayers = 14;

size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

}  // namespace

struct UNet::Impl {
  struct Layer {
    LayerDef d;
    int cin_pad;
    size_t w_off, b_off;     // in the FP32 master array (floats)
    size_t wb_off, wt_off;   // in the BF16 weight buffer (elements)
  };
  Layer L[kNumLayers];
  size_t n_params = 0, n_real = 0, n_wbf16 = 0;
  float *master = nullptr, *grad = nullptr, *m = nullptr, *v = nullptr;
  bf16* wbf = nullptr;
  int step = 0;
  int launches = 0;  // kernels launched by the last forward / step
  // activations and gradients, sized for cap pixels at level 0
  long long cap = 0;
  bf16* act[kTensors] = {};
  bf16* dact[kTensors] = {};
  bf16* dcat = nullptr;
  float* pred = nullptr;     // filter logits [P][kPredCh]
  bf16* dpred = nullptr;
  float* raw = nullptr;     // staged input [P][kRawCh]
  float* target = nullptr;  // staged target [P][3]
  double* loss = nullptr;

  ~Impl() { release(); }

  void release_acts() {
    for (int t = 0; t < kTensors; ++t) {
      if (act[t]) cudaFree(act[t]);
      if (dact[t]) cudaFree(dact[t]);
      act[t] = dact[t] = nullptr;
    }
    void* ps[] = {dcat, pred, dpred, raw, target};
    for (void* p : ps)
      if (p) cudaFree(p);
    dcat = nullptr;
    pred = nullptr;
    dpred = nullptr;
    raw = nullptr;
    target = nullptr;
    cap = 0;
  }
  void release() {
    release_acts();
    void* ps[] = {master, grad, m, v, wbf, loss};
    for (void* p : ps)
      if (p) cudaFree(p);
    master = grad = m = v = nullptr;
    wbf = nullptr;
    loss = nullptr;
  }

  cudaError_t ensure(long long P0) {
    if (P0 <= cap) return cudaSuccess;
    release_acts();
    cudaError_t e;
    for (int t = 0; t < kTensors; ++t) {
      size_t n = (size_t)(P0 >> (2 * kTL[t])) * kTC[t];
      if ((e = cudaMalloc(&act[t], n * sizeof(bf16)))) return e;
      if ((e = cudaMalloc(&dact[t], n * sizeof(bf16)))) return e;
    }
    size_t ncat = std::max({(size_t)P0 * 96, (size_t)(P0 >> 2) * 160, (size_t)(P0 >> 4) * 224,
                            (size_t)(P0 >> 6) * 288});
    if ((e = cudaMalloc(&dcat, ncat * sizeof(bf16)))) return e;
    if ((e = cudaMalloc(&pred, (size_t)P0 * kPredCh * sizeof(float)))) return e;
    if ((e = cudaMalloc(&dpred, (size_t)P0 * kPredCh * sizeof(bf16)))) return e;
    if ((e = cudaMalloc(&raw, (size_t)P0 * kRawCh * sizeof(float)))) return e;
    if ((e = cudaMalloc(&target, (size_t)P0 * 3 * sizeof(float)))) return e;
    cap = P0;
    return cudaSuccess;
  }

  Src src(int t, int up) const { return Src{act[t], kTC[t], up}; }
};

UNet::UNet() : p_(new Impl()) {}
UNet::~UNet() { delete p_; }

int64_t UNet::num_params() const { return (int64_t)p_->n_params; }
int64_t UNet::num_real_params() const { return (int64_t)p_->n_real; }
int UNet::step() const { return p_->step; }
int UNet::num_layers() { return kNumLayers; }
int UNet::last_launches() const { return p_->launches; }

void UNet::layer_info(int i, int64_t* info) const {
  const Impl::Layer& l = p_->L[i];
  int64_t v[11] = {l.d.cout_pad, l.d.cout_real, l.cin_pad, l.d.cin_real, kTC[l.d.s1], l.d.s1_up,
                   l.d.relu, kTL[l.d.out >= 0 ? l.d.out : tU0], (int64_t)l.w_off, (int64_t)l.b_off,
                   l.d.s1};
  for (int k = 0; k < 11; ++k) info[k] = v[k];
}

cudaError_t UNet::init(uint64_t seed, cudaStream_t st) {
  Impl& I = *p_;
  size_t off = 0, woff = 0;
  for (int i = 0; i < kNumLayers; ++i) {
    Impl::Layer& l = I.L[i];
    l.d = kLayers[i];
    l.cin_pad = kTC[l.d.s1] + (l.d.s2 >= 0 ? kTC[l.d.s2] : 0);
    l.w_off = off;
    off = align_up(off + (size_t)l.d.cout_pad * 9 * l.cin_pad, 4);
    l.b_off = off;
    off = align_up(off + l.d.cout_pad, 4);
    l.wb_off = woff;
    woff = align_up(woff + (size_t)l.d.cout_pad * 9 * l.cin_pad, 128);
    l.wt_off = woff;
    woff = align_up(woff + (size_t)l.d.cout_pad * 9 * l.cin_pad, 128);
    I.n_real += (size_t)l.d.cout_real * 9 * l.d.cin_real + l.d.cout_real;
  }
  I.n_params = off;
  I.n_wbf16 = woff;
  // He-normal weights on the real entries, zero padding and biases
  std::vector<float> h(I.n_params, 0.0f);
  std::mt19937_64 rng(seed);
  for (int i = 0; i < kNumLayers; ++i) {
    const Impl::Layer& l = I.L[i];
    std::normal_distribution<float> nd(0.0f, std::sqrt(2.0f / (9.0f * l.d.cin_real)));
    int c1 = kTC[l.d.s1];
    for (int o = 0; o < l.d.cout_real; ++o)
      for (int t = 0; t < 9; ++t)
        for (int c = 0; c < l.cin_pad; ++c) {
          // real input channels: the first cin of s1 (its real count) then s2
          bool real;
          if (l.d.s2 < 0)
            real = c < l.d.cin_real;
          else
            real = c < c1 || (c - c1) < kTC[l.d.s2];
          if (real) h[l.w_off + ((size_t)o * 9 + t) * l.cin_pad + c] = nd(rng);
        }
  }
  cudaError_t e;
  if ((e = cudaMalloc(&I.master, I.n_params * 4))) return e;
  if ((e = cudaMalloc(&I.grad, I.n_params * 4))) return e;
  if ((e = cudaMalloc(&I.m, I.n_params * 4))) return e;
  if ((e = cudaMalloc(&I.v, I.n_params * 4))) return e;
  if ((e = cudaMalloc(&I.wbf, I.n_wbf16 * sizeof(bf16)))) return e;
  if ((e = cudaMalloc(&I.loss, sizeof(double)))) return e;
  if ((e = cudaMemcpyAsync(I.master, h.data(), I.n_params * 4, cudaMemcpyHostToDevice, st))) return e;
  if ((e = cudaMemsetAsync(I.m, 0, I.n_params * 4, st))) return e;
  if ((e = cudaMemsetAsync(I.v, 0, I.n_params * 4, st))) return e;
  if ((e = cudaMemsetAsync(I.grad, 0, I.n_params * 4, st))) return e;
  if ((e = cudaStreamSynchronize(st))) return e;
  I.step = 0;
  return refresh_weights(st);
}

cudaError_t UNet::refresh_weights(cudaStream_t st) {
  Impl& I = *p_;
  WeightLayouts j;
  for (int i = 0; i < kNumLayers; ++i) {
    const Impl::Layer& l = I.L[i];
    j.master[i] = I.master + l.w_off;
    j.w[i] = I.wbf + l.wb_off;
    j.wt[i] = I.wbf + l.wt_off;
    j.Cout[i] = l.d.cout_pad;
    j.Cin[i] = l.cin_pad;
  }
  j.n = kNumLayers;
  return weights_bf16_all(j, st);
}

cudaError_t UNet::set_params(const float* host, cudaStream_t st) {
  cudaError_t e = cudaMemcpyAsync(p_->master, host, p_->n_params * 4, cudaMemcpyHostToDevice, st);
  if (e) return e;
  return refresh_weights(st);
}
cudaError_t UNet::get_params(float* host, cudaStream_t st) const {
  return cudaMemcpyAsync(host, p_->master, p_->n_params * 4, cudaMemcpyDeviceToHost, st);
}
cudaError_t UNet::get_grads(float* host, cudaStream_t st) const {
  return cudaMemcpyAsync(host, p_->grad, p_->n_params * 4, cudaMemcpyDeviceToHost, st);
}
cudaError_t UNet::get_state(float* host_m, float* host_v, cudaStream_t st) const {
  cudaError_t e = cudaMemcpyAsync(host_m, p_->m, p_->n_params * 4, cudaMemcpyDeviceToHost, st);
  if (e) return e;
  return cudaMemcpyAsync(host_v, p_->v, p_->n_params * 4, cudaMemcpyDeviceToHost, st);
}
cudaError_t UNet::set_state(const float* host_m, const float* host_v, int step, cudaStream_t st) {
  cudaError_t e = cudaMemcpyAsync(p_->m, host_m, p_->n_params * 4, cudaMemcpyHostToDevice, st);
  if (e) return e;
  p_->step = step;
  return cudaMemcpyAsync(p_->v, host_v, p_->n_params * 4, cudaMemcpyHostToDevice, st);
}

cudaError_t UNet::forward(const float* d_raw, int N, int H, int W, int* err, cudaStream_t st) {
  Impl& I = *p_;
  long long P0 = (long long)N * H * W;
  cudaError_t e;
  if ((e = I.ensure(P0))) return e;
  I.launches = 0;
  if ((e = encode_input(d_raw, I.act[tX], P0, st))) return e;
  ++I.launches;
  for (int i = 0; i < kNumLayers; ++i) {
    const Impl::Layer& l = I.L[i];
    int lev = kTL[l.d.out >= 0 ? l.d.out : tU0];
    // pooled inputs are produced just before their consumer
    if (l.d.s1 == tP1 || l.d.s1 == tP2 || l.d.s1 == tP3 || l.d.s1 == tP4) {
      int from = l.d.s1 - 1;  // S0 -> P1, S1 -> P2, ...
      if ((e = avgpool(I.act[from], I.act[l.d.s1], N, H >> (lev - 1), W >> (lev - 1), kTC[from], st))) return e;
      ++I.launches;
    }
    ConvFwd c;
    c.s1 = I.src(l.d.s1, l.d.s1_up);
    c.s2 = l.d.s2 >= 0 ? I.src(l.d.s2, 0) : Src{nullptr, 0, 0};
    c.N = N;
    c.H = H >> lev;
    c.W = W >> lev;
    c.Cin = l.cin_pad;
    c.Cout = l.d.cout_pad;
    c.w = I.wbf + l.wb_off;
    c.bias = I.master + l.b_off;
    c.relu = l.d.relu;
    c.out = l.d.out >= 0 ? I.act[l.d.out] : nullptr;
    c.out_f32 = l.d.out >= 0 ? nullptr : I.pred;
    c.err = err;
    if ((e = conv_fwd(c, st))) return e;
    ++I.launches;
  }
  return cudaSuccess;
}

cudaError_t UNet::backward(int N, int H, int W, int* err, cudaStream_t st) {
  Impl& I = *p_;
  cudaError_t e;
  if ((e = cudaMemsetAsync(I.grad, 0, I.n_params * 4, st))) return e;
  I.launches = 0;
  // Bias gradients are summed for all layers in one launch at the end: each
  // layer's output gradient holds its final value once its own step is done
  // (later steps write only the gradients of earlier layers' outputs).
  BiasGrads bias;
  for (int i = kNumLayers - 1; i >= 0; --i) {
    const Impl::Layer& l = I.L[i];
    int lev = kTL[l.d.out >= 0 ? l.d.out : tU0];
    int h = H >> lev, w = W >> lev;
    long long P = (long long)N * h * w;
    const bf16* dout = l.d.out >= 0 ? I.dact[l.d.out] : I.dpred;
    Src s1 = I.src(l.d.s1, l.d.s1_up);
    Src s2 = l.d.s2 >= 0 ? I.src(l.d.s2, 0) : Src{nullptr, 0, 0};
    // weight and bias gradients
    ConvWgrad g;
    g.dout = dout;
    g.Cout = l.d.cout_pad;
    g.s1 = s1;
    g.s2 = s2;
    g.N = N;
    g.H = h;
    g.W = w;
    g.Cin = l.cin_pad;
    g.pix_per_cta = wgrad_pixels_per_cta(P, l.d.cout_pad, l.cin_pad);
    g.dw = I.grad + l.w_off;
    g.err = err;
    if ((e = conv_wgrad(g, st))) return e;
    bias.dout[bias.n] = dout;
    bias.P[bias.n] = P;
    bias.C[bias.n] = l.d.cout_pad;
    bias.db[bias.n] = I.grad + l.b_off;
    ++bias.n;
    ++I.launches;
    if (i == 0) break;  // the input needs no gradient
    // data gradient into the sources
    bool pooled = l.d.s1 == tP1 || l.d.s1 == tP2 || l.d.s1 == tP3 || l.d.s1 == tP4;
    ConvDgrad d;
    d.dout = dout;
    d.Cout = l.d.cout_pad;
    d.wt = I.wbf + l.wt_off;
    d.N = N;
    d.H = h;
    d.W = w;
    d.Cin = l.cin_pad;
    d.s1 = s1;
    d.s2 = s2;
    d.mask_relu = pooled ? 0 : 1;  // pooled inputs are not ReLU outputs
    d.err = err;
    if (l.d.s2 >= 0) {
      d.din = I.dcat;
      if ((e = conv_dgrad(d, st))) return e;
      int c1 = kTC[l.d.s1], c2 = kTC[l.d.s2];
      if ((e = upsample_grad(I.dcat, l.cin_pad, 0, I.dact[l.d.s1], N, h, w, c1, st))) return e;
      if ((e = take_channels(I.dcat, l.cin_pad, c1, I.dact[l.d.s2], P, c2, st))) return e;
      I.launches += 3;
    } else {
      d.din = I.dact[l.d.s1];
      if ((e = conv_dgrad(d, st))) return e;
      ++I.launches;
      if (pooled) {
        ++I.launches;
        int skip = l.d.s1 - 1;
        if ((e = pool_grad_acc(I.dact[l.d.s1], I.act[skip], I.dact[skip], N, h * 2, w * 2, kTC[skip], st)))
          return e;
      }
    }
  }
  if ((e = bias_grads(bias, st))) return e;
  ++I.launches;
  return cudaSuccess;
}

cudaError_t UNet::train_step(const float* d_raw, const float* d_target, int N, int H, int W, float lr,
                             double* loss_out, int* err, cudaStream_t st) {
  Impl& I = *p_;
  cudaError_t e;
  long long P0 = (long long)N * H * W;
  if ((e = forward(d_raw, N, H, W, err, st))) return e;
  if ((e = cudaMemsetAsync(I.loss, 0, sizeof(double), st))) return e;
  if ((e = kp_loss(I.pred, d_raw, d_target, I.dpred, N, H, W, I.loss, st))) return e;
  int fwd = I.launches;
  if ((e = backward(N, H, W, err, st))) return e;
  ++I.step;
  if ((e = adam(I.master, I.grad, I.m, I.v, (long long)I.n_params, lr, I.step, st))) return e;
  if ((e = refresh_weights(st))) return e;
  I.launches += fwd + 3;  // loss, Adam, weight refresh
  if (loss_out) {
    double s = 0.0;
    if ((e = cudaMemcpyAsync(&s, I.loss, sizeof(double), cudaMemcpyDeviceToHost, st))) return e;
    if ((e = cudaStreamSynchronize(st))) return e;
    *loss_out = s / (3.0 * (double)P0);
  }
  return cudaSuccess;
}

cudaError_t UNet::loss_and_grads(const float* d_raw, const float* d_target, int N, int H, int W,
                                 double* loss_out, int* err, cudaStream_t st) {
  Impl& I = *p_;
  cudaError_t e;
  long long P0 = (long long)N * H * W;
  if ((e = forward(d_raw, N, H, W, err, st))) return e;
  if ((e = cudaMemsetAsync(I.loss, 0, sizeof(double), st))) return e;
  if ((e = kp_loss(I.pred, d_raw, d_target, I.dpred, N, H, W, I.loss, st))) return e;
  int fwd = I.launches;
  if ((e = backward(N, H, W, err, st))) return e;
  I.launches += fwd + 1;
  double s = 0.0;
  if ((e = cudaMemcpyAsync(&s, I.loss, sizeof(double), cudaMemcpyDeviceToHost, st))) return e;
  if ((e = cudaStreamSynchronize(st))) return e;
  if (loss_out) *loss_out = s / (3.0 * (double)P0);
  return cudaSuccess;
}

float* UNet::scratch_raw() { return p_->raw; }
float* UNet::scratch_target() { return p_->target; }
const float* UNet::prediction() const { return p_->pred; }
cudaError_t UNet::reserve(long long P0) { return p_->ensure(P0); }

cudaError_t UNet::decode(const float* d_raw, float* d_out, int N, int Hc, int Wc, int Hs, int Ws,
                         cudaStream_t st) const {
  return kp_apply(p_->pred, d_raw, d_out, N, Hc, Wc, Hs, Ws, st);
}

}  // namespace nn
}  // namespace rtx
