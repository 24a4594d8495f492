// Helpers shared by the C ABI translation units: status-code errors, CUDA checks, device
// allocation and the exception guard that turns every failure into a status + message.
#pragma once

#include <cuda_runtime.h>

#include <new>
#include <stdexcept>
#include <string>

#include "nlod.h"

namespace nlod {

// Message of the last failure on the calling thread (defined in api.cu).
std::string& last_error();

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

inline void cuda_check(cudaError_t e, const char* what) {
    if (e != cudaSuccess) {
        cudaGetLastError();  // clear non-sticky errors
        throw Error(e == cudaErrorMemoryAllocation ? NLOD_ERR_ALLOC : NLOD_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
    }
}

template <typename T>
T* dev_alloc(size_t count) {
    if (count == 0) return nullptr;
    void* p = nullptr;
    cuda_check(cudaMalloc(&p, count * sizeof(T)), "cudaMalloc");
    return static_cast<T*>(p);
}

inline void dev_free(void* p) {
    if (p) cudaFree(p);
}

template <typename F>
int guarded(F&& f) {
    try {
        f();
        last_error().clear();
        return NLOD_OK;
    } catch (const Error& e) {
        last_error() = e.what();
        return e.code;
    } catch (const std::bad_alloc&) {
        last_error() = "host allocation failed";
        return NLOD_ERR_ALLOC;
    } catch (const std::exception& e) {
        last_error() = e.what();
        return NLOD_ERR_INVALID;
    }
}

}  // namespace nlod
