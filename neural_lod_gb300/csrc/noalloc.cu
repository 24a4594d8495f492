// Fixed device scratch for the training step entry point that allocates nothing
// (nlod_training_step_noalloc).
//
// Some callers cannot allocate device memory at the moment they train: an online learner that
// takes one training step inside a real-time frame loop with a no-allocation budget, or code that
// runs while another component owns the allocator.  For them the step's intermediates
// (encoded rows, hidden activations, outputs, output gradients, per-layer deltas, encoding
// gradients, loss partial sums) live in this file-scope array instead of a cudaMalloc'ed
// workspace.  Every GPU that loads this part of the library holds the array until the process
// exits.  All calls share it, so calls that overlap on the GPU (two streams, two threads) race on
// its contents; each call clears the parts that must start at zero.
#include <cuda_runtime.h>

#include <cstddef>

#include "kernels.h"

namespace nlod {

namespace {

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

}  // namespace

// Device address of the scratch in the current device's context.  The host-side name of the array
// is only a stand-in, so the address is looked up with cudaGetSymbolAddress, with that device
// current, on every call: once the array is loaded the lookup is a table read, and a context
// created again after cudaDeviceReset gets its own array and address rather than a stale one.
// Under CUDA's lazy module loading the first lookup in a context loads this file's module, which
// is when the array takes its device memory.
cudaError_t noalloc_scratch(void** ptr, size_t* bytes) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    *ptr = p;
    *bytes = kNoAllocScratchBytes;
    return cudaSuccess;
}

}  // namespace nlod
