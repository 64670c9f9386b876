// Fused Adam step over every parameter tensor of an optimiser in one launch
// (the optimiser of both inversion loops, torch.optim.Adam in
// Parameter_inversion/Inversion_adam.py:421-447 and
// Damage_inversion/Inversion_adam.py:477-514).  Per element, with t the
// step count after this step:
//   g  = grad + weight_decay * p
//   m  = m + (1 - beta1) (g - m)
//   v  = beta2 v + (1 - beta2) g^2
//   p  = p - lr / (1 - beta1^t) * m / (sqrt(v) / sqrt(1 - beta2^t) + eps)
// the update of torch.optim.Adam (no amsgrad), in FP32 with the bias
// corrections formed in FP64.  The step count lives in device memory, so a
// CUDA graph that captured the launch advances it on every replay: every
// block reads count, the last block to finish (a ticket counter, reset by
// that block) stores count + 1.
#include <cmath>
#include <cstdint>

#include "ernn.h"
#include "ernn_launch.h"

namespace ernn {
namespace {

constexpr int kAdamThreads = 256;
constexpr int kAdamMaxBlocksX = 1024;

__global__ void __launch_bounds__(kAdamThreads)
    adam_kernel(const ErnnAdamTensor* __restrict__ tensors, ErnnAdamHyper h, int32_t* __restrict__ state) {
  const ErnnAdamTensor T = tensors[blockIdx.y];
  const int32_t t = state[0] + 1;
  // bias corrections in FP64 by one thread (the FP64 pipe is narrow), shared
  __shared__ float corr[2];
  if (threadIdx.x == 0) {
    const double bc1 = 1.0 - pow(h.beta1, (double)t);
    const double bc2 = 1.0 - pow(h.beta2, (double)t);
    corr[0] = (float)(h.lr / bc1);
    corr[1] = (float)sqrt(bc2);
  }
  __syncthreads();
  const float step_size = corr[0], sqrt_bc2 = corr[1];
  const float b1 = (float)h.beta1, b2 = (float)h.beta2, eps = (float)h.eps, wd = (float)h.weight_decay;
  for (int64_t e = (int64_t)blockIdx.x * kAdamThreads + threadIdx.x; e < T.n;
       e += (int64_t)gridDim.x * kAdamThreads) {
    float g = T.grad[e];
    float p = T.param[e];
    if (wd != 0.f) g += wd * p;
    const float m = T.exp_avg[e] + (1.f - b1) * (g - T.exp_avg[e]);
    const float v = b2 * T.exp_avg_sq[e] + (1.f - b2) * g * g;
    T.exp_avg[e] = m;
    T.exp_avg_sq[e] = v;
    T.param[e] = p + (-step_size) * (m / (sqrtf(v) / sqrt_bc2 + eps));
  }
  // the last block stores the new count and resets the ticket
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    const unsigned total = gridDim.x * gridDim.y;
    const unsigned ticket = atomicAdd(reinterpret_cast<unsigned*>(&state[1]), 1u);
    if (ticket == total - 1) {
      state[0] = t;
      state[1] = 0;
    }
  }
}

}  // namespace
}  // namespace ernn

using namespace ernn;

extern "C" {

int ernn_adam_step(const ErnnAdamTensor* tensors, int32_t ntensors, int64_t max_numel,
                   const ErnnAdamHyper* h, int32_t* state, void* stream) {
  if (tensors == nullptr || h == nullptr || state == nullptr || ntensors < 1 || ntensors > 65535 ||
      max_numel < 1)
    return ERNN_ERR_INVALID;
  if (!(h->lr >= 0.0) || !(h->beta1 >= 0.0 && h->beta1 < 1.0) || !(h->beta2 >= 0.0 && h->beta2 < 1.0) ||
      !(h->eps >= 0.0) || !(h->weight_decay >= 0.0))
    return ERNN_ERR_INVALID;
  cudaStream_t st = (cudaStream_t)stream;
  int64_t bx = (max_numel + kAdamThreads - 1) / kAdamThreads;
  if (bx > kAdamMaxBlocksX) bx = kAdamMaxBlocksX;
  const dim3 grid((unsigned)bx, (unsigned)ntensors, 1);
  const ErnnAdamHyper hv = *h;
  if (tracked_launch(kProfOther, st, [&] { adam_kernel<<<grid, kAdamThreads, 0, st>>>(tensors, hv, state); }) !=
      cudaSuccess)
    return ERNN_ERR_CUDA;
  return ERNN_OK;
}

}  // extern "C"
