// Launcher of the persistent render kernel (render_pk.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "desc.h"
#include "render_common.cuh"

namespace nlod {

// One network's inference operands for the persistent kernel.
struct PkNet {
    const void* weights_op;   // inference weights, operand type, row-major [out][in] per layer
    const void* table;        // parameter vector whose grid part the encoding gathers: the FP16
                              // copy (FP16 form) or the FP32 inference parameters (BF16 form)
    float max_level;          // grid max-level fraction for every query of this network
};

struct PkArgs {
    render::RenderConsts C;
    PkNet vis, thr;
    float* image;             // [n_rays][3]
    uint32_t* ray_stats;      // [n_rays][2] visibility / throughput queries per ray
    render::Control* ctl;     // cnt[0] is the ray queue; totals as in the wavefront form
    uint32_t* status;         // 2: DDA step budget, 4: frame time bound, 8: MMA wait timed out
};

// Organisations of the persistent kernel: 4 or 6 = that many tile pipelines per CTA, each marching
// its own rays; kWsForm16 / kWsForm8 = the warp-specialized form with 16 marcher warps (2 ray slots
// per lane) or 8 (4 per lane) feeding two tensor-core groups.
constexpr int kWsForm16 = 16;
constexpr int kWsForm8 = 8;

// Whether the persistent kernel can run these two networks in the given organisation.
bool render_pk_supported(const ModelDesc& dv, const ModelDesc& dt, int groups);
// Resets the frame's control words and launches one persistent frame (kind 1 = FP16, 2 = BF16).
cudaError_t launch_render_pk(const ModelDesc& dv, const ModelDesc& dt, const PkArgs& a, int kind, int groups, cudaStream_t s);

}  // namespace nlod
