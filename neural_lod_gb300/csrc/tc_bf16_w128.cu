// Instantiations of the tensor-core query kernel for __nv_bfloat16 operands and 128-wide hidden layers
// (every organisation of tc_forward.cuh's variant table).
#include "tc_forward.cuh"

namespace nlod {

cudaError_t launch_tc_bf16_w128(const ModelDesc& d, const ForwardArgs& a, int variant, uint32_t* status, cudaStream_t s) {
    return launch_typed<128, __nv_bfloat16>(d, a, variant, status, s);
}

}  // namespace nlod
