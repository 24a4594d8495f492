// Helpers shared by the tensor-core kernels (query and training): per-group named barriers,
// and the store of encoded features into a K-major operand tile.
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <cstdint>

#include "activation.cuh"
#include "desc.h"
#include "tc_common.cuh"

namespace nlod {

// Named barrier over the N threads of one group (id 1 + group; id 0 is __syncthreads).
template <uint32_t N = 128>
__device__ __forceinline__ void group_sync(uint32_t id) {
    asm volatile("bar.sync %0, %1;" ::"r"(id), "n"(N) : "memory");
}

// Group barrier that also ORs a predicate over the group's N threads.
template <uint32_t N = 128>
__device__ __forceinline__ bool group_sync_or(uint32_t id, bool v) {
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\t"
        "setp.ne.u32 p, %1, 0;\n\t"
        "bar.red.or.pred q, %2, %3, p;\n\t"
        "selp.u32 %0, 1, 0, q;\n\t}"
        : "=r"(r)
        : "r"((uint32_t)v), "r"(id), "n"(N)
        : "memory");
    return r != 0;
}

// Encoded features as FP16/BF16 into the K-major core-matrix A operand.
template <typename T>
struct TcStore {
    uint8_t* tile;
    uint32_t sbo;
    template <int M>
    __device__ __forceinline__ void run(uint32_t r, uint32_t col, const float (&f)[M], uint32_t n) {
        using Op = tc::OpType<T>;
        if (M % 8 == 0 && n == (uint32_t)M && (col & 7u) == 0) {
#pragma unroll
            for (int i = 0; i < M; i += 8) {
                uint4 pk;
                pk.x = Op::pack2(f[i + 0], f[i + 1]);
                pk.y = Op::pack2(f[i + 2], f[i + 3]);
                pk.z = Op::pack2(f[i + 4], f[i + 5]);
                pk.w = Op::pack2(f[i + 6], f[i + 7]);
                *reinterpret_cast<uint4*>(tile + tc::kmajor_offset(r, col + i, sbo)) = pk;
            }
        } else if (M == 4 && n == 4 && (col & 3u) == 0) {
            uint2 pk;
            pk.x = Op::pack2(f[0], f[1]);
            pk.y = Op::pack2(f[2 % M], f[3 % M]);
            *reinterpret_cast<uint2*>(tile + tc::kmajor_offset(r, col, sbo)) = pk;
        } else {
#pragma unroll
            for (uint32_t i = 0; i < (uint32_t)M / 2; ++i)
                if (2 * i < n) *reinterpret_cast<uint32_t*>(tile + tc::kmajor_offset(r, col + 2 * i, sbo)) = Op::pack2(f[2 * i], f[2 * i + 1]);
        }
    }
    __device__ __forceinline__ void one(uint32_t r, uint32_t col, float v) {
        *reinterpret_cast<uint16_t*>(tile + tc::kmajor_offset(r, col, sbo)) = tc::OpType<T>::pack1(v);
    }
};


}  // namespace nlod
