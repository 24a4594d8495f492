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
#include <mutex>

#include "kernels.h"

namespace nlod {

namespace {

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_addr[kMaxDevices] = {};

}  // namespace

// Device address of the scratch on the current device.  The host-side name of the array is only a
// stand-in, so the address is looked up with cudaGetSymbolAddress once per device (with that
// device current) and cached.
cudaError_t noalloc_scratch(void** ptr, size_t* bytes) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_addr[dev] = p;
    }
    *ptr = g_addr[dev];
    *bytes = kNoAllocScratchBytes;
    return cudaSuccess;
}

}  // namespace nlod
