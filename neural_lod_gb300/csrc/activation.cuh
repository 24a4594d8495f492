// Activations of the fully fused MLP and the derivative of the output activation from its output
// value (tiny-cuda-nn include/tiny-cuda-nn/common_device.h:68-230 and :341-352), shared by the
// plain FP32 kernels and the tensor-core kernels.
//
// Element loops take the activation through with_act(), which branches once on the activation
// code and runs the loop body with the activation fixed at compile time.  A switch on the code
// inside the loop measured about ten times slower than the fixed form: one 128-row tile's
// 64-column hidden epilogue in the tensor-core query took 3.8 us with the per-element switch
// against 0.4 us with the activation fixed.
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

// One activation as a compile-time constant (act_fwd folds to its case).
template <int32_t A>
struct FixedAct {
    static constexpr int32_t kind = A;
    __device__ __forceinline__ float operator()(float v) const { return act_fwd(A, v); }
    __device__ __forceinline__ float grad_from_output(float y) const { return act_grad_from_output(A, y); }
};

// body(FixedAct<act>{}) for the runtime activation code act (uniform over the caller's threads).
template <typename Body>
__device__ __forceinline__ void with_act(int32_t act, Body&& body) {
    switch (act) {
        case ACT_RELU: body(FixedAct<ACT_RELU>{}); break;
        case ACT_SIGMOID: body(FixedAct<ACT_SIGMOID>{}); break;
        case ACT_EXP: body(FixedAct<ACT_EXP>{}); break;
        default: body(FixedAct<ACT_NONE>{}); break;
    }
}

// The hidden activation (ReLU or identity, the two that model descriptions accept) chosen by a
// flag: exactly act_fwd's two cases, NaN included, in one compiled copy of the loop (a copy per
// activation spilled registers in the tensor-core kernels).
struct ReluOrNone {
    bool relu;
    __device__ __forceinline__ float operator()(float v) const { return (relu && !(v > 0.f)) ? 0.f : v; }
};

}  // namespace nlod
