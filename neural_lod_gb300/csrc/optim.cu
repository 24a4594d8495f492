// Optimizer, weight-conversion and initialisation kernels.
//
// Adam restates tiny-cuda-nn's adam_step (rptr/ext/tiny-cuda-nn/include/tiny-cuda-nn/optimizers/adam.h:47-119):
// gradients are divided by the loss scale; non-matrix (encoding) parameters whose gradient is
// exactly zero are skipped (no moment update, no step increment); L2 regularisation applies to
// matrix parameters only; every parameter has its own step counter for the bias correction;
// AdaBound-style clamping of the effective learning rate; relative/absolute weight decay.
// The EMA wrapper (optimizers/ema.h:45-124) is fused: after the Adam update every parameter's
// exponential moving average is refreshed with the debiasing factors computed on the host.
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "kernels.h"

namespace nlod {

namespace {

__global__ void k_adam_step(const __grid_constant__ AdamStepArgs a) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n_params) return;
    const bool matrix = i < a.n_matrix;
    float w = a.params[i];
    float gradient = a.grads[i] / a.loss_scale;
    bool skip = matrix ? !a.hp.optimize_matrix : (!a.hp.optimize_non_matrix || gradient == 0.f);
    if (!skip) {
        if (matrix) gradient += a.hp.l2_reg * w;
        const float g2 = gradient * gradient;
        const float m1 = a.m1[i] = a.hp.beta1 * a.m1[i] + (1.f - a.hp.beta1) * gradient;
        const float m2 = a.m2[i] = a.hp.beta2 * a.m2[i] + (1.f - a.hp.beta2) * g2;
        float lr = a.learning_rate;
        if (!matrix) lr *= a.hp.non_matrix_lr_factor;
        const uint32_t step = ++a.steps[i];
        lr *= sqrtf(1.f - powf(a.hp.beta2, (float)step)) / (1.f - powf(a.hp.beta1, (float)step));
        const float eff = fminf(fmaxf(lr / (sqrtf(m2) + a.hp.epsilon), a.lower_lr_bound), a.upper_lr_bound);
        const float rel = a.hp.relative_decay * lr, absd = a.hp.absolute_decay * lr;
        const float decayed = (1.f - rel) * w - copysignf(absd, w);
        float nw = decayed - eff * m1;
        if (a.hp.weight_clipping != 0.f) nw = fminf(fmaxf(nw, -a.hp.weight_clipping), a.hp.weight_clipping);
        a.params[i] = nw;
        w = nw;
    }
    if (a.ema) {
        a.ema[i] = (a.ema[i] * a.ema_decay * a.ema_debias_old + w * (1.f - a.ema_decay)) * a.ema_debias_new;
    }
}

__global__ void k_convert_f16(const float* __restrict__ src, __half* __restrict__ dst, uint32_t n) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = __float2half_rn(src[i]);
}

__global__ void k_convert_bf16(const float* __restrict__ src, __nv_bfloat16* __restrict__ dst, uint32_t n) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = __float2bfloat16_rn(src[i]);
}

// SplitMix64 finaliser (Steele, Lea, Flood 2014) as a counter-based generator.
__device__ __forceinline__ uint64_t splitmix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

__global__ void k_init_uniform(float* __restrict__ p, uint32_t n, uint64_t seed, uint64_t stream_id, float lo, float hi) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint64_t r = splitmix64(seed ^ splitmix64(stream_id * 0x100000001B3ull + i));
    const float u = (float)(r >> 40) * (1.0f / 16777216.0f);  // 24 random bits in [0,1)
    p[i] = lo + (hi - lo) * u;
}

}  // namespace

cudaError_t launch_adam_step(const AdamStepArgs& a, cudaStream_t s) {
    if (a.n_params == 0) return cudaSuccess;
    k_adam_step<<<(a.n_params + 255) / 256, 256, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_convert_weights(const float* src, void* dst, uint32_t n, int kind, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    if (kind == 1) k_convert_f16<<<(n + 255) / 256, 256, 0, s>>>(src, (__half*)dst, n);
    else k_convert_bf16<<<(n + 255) / 256, 256, 0, s>>>(src, (__nv_bfloat16*)dst, n);
    return cudaGetLastError();
}

cudaError_t launch_init_uniform(float* p, uint32_t n, uint64_t seed, uint64_t stream_id, float lo, float hi, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    k_init_uniform<<<(n + 255) / 256, 256, 0, s>>>(p, n, seed, stream_id, lo, hi);
    return cudaGetLastError();
}

}  // namespace nlod
