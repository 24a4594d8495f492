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

__device__ __forceinline__ float adam_one(const AdamStepArgs& a, uint32_t i, float w, float grad_scaled, float& m1, float& m2,
                                          uint32_t& step, bool& changed) {
    const bool matrix = i < a.n_matrix;
    float gradient = grad_scaled / a.loss_scale;
    const bool skip = matrix ? !a.hp.optimize_matrix : (!a.hp.optimize_non_matrix || gradient == 0.f);
    changed = !skip;
    if (skip) return w;
    if (matrix) gradient += a.hp.l2_reg * w;
    const float g2 = gradient * gradient;
    m1 = a.hp.beta1 * m1 + (1.f - a.hp.beta1) * gradient;
    m2 = a.hp.beta2 * m2 + (1.f - a.hp.beta2) * g2;
    float lr = a.learning_rate;
    if (!matrix) lr *= a.hp.non_matrix_lr_factor;
    ++step;
    // beta^step as exp2(step * log2(beta)) (log2 of the betas computed once on the host)
    const float b2t = exp2f((float)step * a.log2_beta2), b1t = exp2f((float)step * a.log2_beta1);
    lr *= sqrtf(1.f - b2t) / (1.f - b1t);
    const float eff = fminf(fmaxf(lr / (sqrtf(m2) + a.hp.epsilon), a.lower_lr_bound), a.upper_lr_bound);
    const float rel = a.hp.relative_decay * lr, absd = a.hp.absolute_decay * lr;
    const float decayed = (1.f - rel) * w - copysignf(absd, w);
    float nw = decayed - eff * m1;
    if (a.hp.weight_clipping != 0.f) nw = fminf(fmaxf(nw, -a.hp.weight_clipping), a.hp.weight_clipping);
    return nw;
}

// Operand-type (FP16 / BF16) copies of four / one matrix parameters.
__device__ __forceinline__ void store_op4(void* dst, uint32_t q, float4 v, int kind) {
    uint2 pk;
    if (kind == 1) {
        const __half2 lo = __floats2half2_rn(v.x, v.y), hi = __floats2half2_rn(v.z, v.w);
        pk.x = *reinterpret_cast<const uint32_t*>(&lo);
        pk.y = *reinterpret_cast<const uint32_t*>(&hi);
    } else {
        const __nv_bfloat162 lo = __floats2bfloat162_rn(v.x, v.y), hi = __floats2bfloat162_rn(v.z, v.w);
        pk.x = *reinterpret_cast<const uint32_t*>(&lo);
        pk.y = *reinterpret_cast<const uint32_t*>(&hi);
    }
    reinterpret_cast<uint2*>(dst)[q] = pk;
}
__device__ __forceinline__ void store_op1(void* dst, uint32_t i, float v, int kind) {
    if (kind == 1) reinterpret_cast<__half*>(dst)[i] = __float2half_rn(v);
    else reinterpret_cast<__nv_bfloat16*>(dst)[i] = __float2bfloat16_rn(v);
}

// Four parameters per thread with 16-byte loads and stores; moments and step counters are only
// written for parameters that were updated.
__global__ void __launch_bounds__(256) k_adam_step(const __grid_constant__ AdamStepArgs a) {
    const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t i0 = 4u * q;
    if (q == 0 && a.cells_stale) *a.cells_stale = 1u;
    if (i0 >= a.n_params) return;
    if (i0 + 4u <= a.n_params) {
        float4 w = reinterpret_cast<const float4*>(a.params)[q];
        const float4 g = reinterpret_cast<const float4*>(a.grads)[q];
        float4 m1 = reinterpret_cast<const float4*>(a.m1)[q];
        float4 m2 = reinterpret_cast<const float4*>(a.m2)[q];
        uint4 st = reinterpret_cast<const uint4*>(a.steps)[q];
        bool c0, c1, c2, c3;
        w.x = adam_one(a, i0, w.x, g.x, m1.x, m2.x, st.x, c0);
        w.y = adam_one(a, i0 + 1, w.y, g.y, m1.y, m2.y, st.y, c1);
        w.z = adam_one(a, i0 + 2, w.z, g.z, m1.z, m2.z, st.z, c2);
        w.w = adam_one(a, i0 + 3, w.w, g.w, m1.w, m2.w, st.w, c3);
        if (c0 | c1 | c2 | c3) {
            reinterpret_cast<float4*>(a.params)[q] = w;
            reinterpret_cast<float4*>(a.m1)[q] = m1;
            reinterpret_cast<float4*>(a.m2)[q] = m2;
            reinterpret_cast<uint4*>(a.steps)[q] = st;
        }
        if (a.w_op && i0 < a.n_matrix && (c0 | c1 | c2 | c3)) store_op4(a.w_op, q, w, a.op_kind);
        float4 inf = w;
        if (a.ema) {
            float4 e = reinterpret_cast<const float4*>(a.ema)[q];
            const float k0 = a.ema_decay * a.ema_debias_old, k1 = 1.f - a.ema_decay;
            e.x = (e.x * k0 + w.x * k1) * a.ema_debias_new;
            e.y = (e.y * k0 + w.y * k1) * a.ema_debias_new;
            e.z = (e.z * k0 + w.z * k1) * a.ema_debias_new;
            e.w = (e.w * k0 + w.w * k1) * a.ema_debias_new;
            reinterpret_cast<float4*>(a.ema)[q] = e;
            inf = e;
        }
        // n_matrix is a multiple of 256: a group of four is all matrix or all grid parameters
        if (a.w_op_inf && a.w_op_inf != a.w_op && i0 < a.n_matrix) store_op4(a.w_op_inf, q, inf, a.op_kind);
        if (a.grid_h && i0 >= a.n_matrix && (a.ema || c0 | c1 | c2 | c3)) {
            const __half2 lo = __floats2half2_rn(inf.x, inf.y), hi = __floats2half2_rn(inf.z, inf.w);
            uint2 pk;
            pk.x = *reinterpret_cast<const uint32_t*>(&lo);
            pk.y = *reinterpret_cast<const uint32_t*>(&hi);
            reinterpret_cast<uint2*>(a.grid_h)[q] = pk;
        }
        if (a.grid_h_train && i0 >= a.n_matrix && (c0 | c1 | c2 | c3)) {
            const __half2 lo = __floats2half2_rn(w.x, w.y), hi = __floats2half2_rn(w.z, w.w);
            uint2 pk;
            pk.x = *reinterpret_cast<const uint32_t*>(&lo);
            pk.y = *reinterpret_cast<const uint32_t*>(&hi);
            reinterpret_cast<uint2*>(a.grid_h_train)[q] = pk;
        }
        if (a.grid_b_train && i0 >= a.n_matrix && (c0 | c1 | c2 | c3)) {
            const __nv_bfloat162 lo = __floats2bfloat162_rn(w.x, w.y), hi = __floats2bfloat162_rn(w.z, w.w);
            uint2 pk;
            pk.x = *reinterpret_cast<const uint32_t*>(&lo);
            pk.y = *reinterpret_cast<const uint32_t*>(&hi);
            reinterpret_cast<uint2*>(a.grid_b_train)[q] = pk;
        }
        return;
    }
    for (uint32_t i = i0; i < a.n_params; ++i) {
        float m1 = a.m1[i], m2 = a.m2[i];
        uint32_t st = a.steps[i];
        bool c;
        const float w = adam_one(a, i, a.params[i], a.grads[i], m1, m2, st, c);
        if (c) {
            a.params[i] = w;
            a.m1[i] = m1;
            a.m2[i] = m2;
            a.steps[i] = st;
        }
        float inf = w;
        if (a.ema) {
            a.ema[i] = (a.ema[i] * a.ema_decay * a.ema_debias_old + w * (1.f - a.ema_decay)) * a.ema_debias_new;
            inf = a.ema[i];
        }
        if (a.grid_h && i >= a.n_matrix) a.grid_h[i] = __float2half_rn(inf);
        if (a.grid_h_train && i >= a.n_matrix && c) a.grid_h_train[i] = __float2half_rn(w);
        if (a.grid_b_train && i >= a.n_matrix && c) a.grid_b_train[i] = __float2bfloat16_rn(w);
        if (i < a.n_matrix) {
            if (a.w_op && c) store_op1(a.w_op, i, w, a.op_kind);
            if (a.w_op_inf && a.w_op_inf != a.w_op) store_op1(a.w_op_inf, i, inf, a.op_kind);
        }
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
    const uint32_t threads = (a.n_params + 3u) / 4u;
    k_adam_step<<<(threads + 255) / 256, 256, 0, s>>>(a);
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
