// Tensor-core form of the fused neural-LoD query: the C++ entry points over the kernel
// organisations of tc_forward.cuh (tile pipelines per CTA, grid levels per gather batch,
// shared-memory staging of coarse levels, threads per tile row), whose instantiations live in one
// unit per operand type and width.
#include "tc_forward.cuh"

namespace nlod {

cudaError_t launch_tc_f16_w64(const ModelDesc& d, const ForwardArgs& a, int variant, uint32_t* status, cudaStream_t s);
cudaError_t launch_tc_bf16_w64(const ModelDesc& d, const ForwardArgs& a, int variant, uint32_t* status, cudaStream_t s);
cudaError_t launch_tc_f16_w128(const ModelDesc& d, const ForwardArgs& a, int variant, uint32_t* status, cudaStream_t s);
cudaError_t launch_tc_bf16_w128(const ModelDesc& d, const ForwardArgs& a, int variant, uint32_t* status, cudaStream_t s);

int tc_num_variants() { return kNumVariants; }

bool tc_variant_ok(const ModelDesc& d, int variant, int kind) {
    if (variant < 0 || variant >= kNumVariants) return false;
    if (kVariants[variant].stage_levels && kind != 1) return false;
    int per_sm = 0;
    const size_t bytes = tc_smem_bytes(d, kVariants[variant].G, kVariants[variant].stage_levels, &per_sm);
    if (kVariants[variant].stage_levels && tc_layout(d, kVariants[variant].G, true).tab_levels == 0) return false;
    return bytes <= 227u * 1024u && per_sm >= 1 && (uint32_t)kVariants[variant].G * d.width <= 512u &&
           kVariants[variant].G * kGroupThreads * kVariants[variant].tpr <= 1024 && d.width % (32u * kVariants[variant].tpr) == 0;
}

int tc_default_variant(const ModelDesc& d) {
    for (int v = 0; v < kNumVariants; ++v)
        if (tc_variant_ok(d, v)) return v;
    return -1;
}

bool tc_supported(const ModelDesc& d) {
    if (d.width != 64 && d.width != 128) return false;
    if (d.enc_width % 16 != 0 || d.enc_width > 256) return false;
    return tc_default_variant(d) >= 0;
}

cudaError_t launch_forward_tc(const ModelDesc& d, const ForwardArgs& a, int kind, int variant, uint32_t* status, cudaStream_t s) {
    if (!tc_variant_ok(d, variant, kind)) return cudaErrorInvalidValue;
    if (kind == 1 && d.n_grids > 0 && !a.grid_h) return cudaErrorInvalidValue;   // the FP16 form reads the FP16 grid copy
    if (d.width == 64 && kind == 1) return launch_tc_f16_w64(d, a, variant, status, s);
    if (d.width == 64 && kind == 2) return launch_tc_bf16_w64(d, a, variant, status, s);
    if (d.width == 128 && kind == 1) return launch_tc_f16_w128(d, a, variant, status, s);
    if (d.width == 128 && kind == 2) return launch_tc_bf16_w128(d, a, variant, status, s);
    return cudaErrorInvalidValue;
}

}  // namespace nlod
