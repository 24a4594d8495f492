// Instantiations of the tensor-core query kernel for __half operands and 64-wide hidden layers
// (every organisation of tc_forward.cuh's variant table).
#include "tc_forward.cuh"

namespace nlod {

cudaError_t launch_tc_f16_w64(const ModelDesc& d, const ForwardArgs& a, int variant, uint32_t* status, cudaStream_t s) {
    return launch_typed<64, __half>(d, a, variant, status, s);
}

}  // namespace nlod
