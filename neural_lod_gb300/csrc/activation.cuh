// Activations of the fully fused MLP and the derivative of the output activation from its output
// value (tiny-cuda-nn include/tiny-cuda-nn/common_device.h:68-230 and :341-352), shared by the
// plain FP32 kernels and the tensor-core kernels.
//
// Hidden-layer loops take the activation through ReluOrNone, a flag tested per element, not through
// a switch on the activation code: in the tensor-core query one 128-row tile's 64-column hidden
// epilogue took 3.8 us with the per-element switch against 0.4 us with the flag.
#pragma once

#include <cstdint>

#include "desc.h"

namespace nlod {

__device__ __forceinline__ float act_fwd(int32_t act, float v) {
    switch (act) {
        case ACT_RELU: return v > 0.f ? v : 0.f;
        case ACT_SIGMOID: return 1.0f / (1.0f + expf(-v));
        case ACT_EXP: return expf(v);
        default: return v;
    }
}

// d act / d x expressed through the activation's output y.
__device__ __forceinline__ float act_grad_from_output(int32_t act, float y) {
    switch (act) {
        case ACT_RELU: return y > 0.f ? 1.f : 0.f;
        case ACT_SIGMOID: return y * (1.f - y);
        case ACT_EXP: return y;
        default: return 1.f;
    }
}

// The hidden activation (ReLU or identity, the two that model descriptions accept) chosen by a
// flag: exactly act_fwd's two cases, NaN included, in one compiled copy of the loop (a loop copy
// per activation made the tensor-core kernels spill registers).
struct ReluOrNone {
    bool relu;
    __device__ __forceinline__ float operator()(float v) const { return (relu && !(v > 0.f)) ? 0.f : v; }
};

}  // namespace nlod
