// LoD occupancy pyramid and the first-active-voxel ray search on the GPU.
//
// Pyramid: level k holds voxel (x, y, z) >> k of every active level-0 voxel (the OR-downsampling
// of rptr/cuda/neural-lod/neural_lod_learning_init.cu:238-248), stored as one bit per voxel
// (bit x + y*res + z*res^2, most significant bit first per 32-bit word: the cuda_voxelizer layout)
// plus the existence flags of the 8^3 leaf and 128^3 lower nodes a NanoVDB tree built from those
// voxels would have, and the tight bounding box of the active voxels.
//
// Search: one thread per ray restates, operation for operation, NanoVDB's TreeMarcher over leaf
// nodes (rptr/ext/nanovdb/nanovdb/util/HDDA.h:370-450) with its HDDA (:27-188, forward stepping
// on), the unit DDA inside each leaf span (:190-307), getDim of the sparse tree
// (NanoVDB.h:3358-3369, 3745-3757, 4442-4448), and the search loop + slab test of
// first_active_voxel_intersection (rptr/cuda/neural-lod/neural_lod_learning_common.cuh:567-606,
// 783-832).  Every float expression is written with explicit round-to-nearest intrinsics so no
// multiply-add is contracted (the ray itself is evaluated with fmaf, as nanovdb::Ray does); the
// result is the voxel, t_near and t_far of NanoVDB's DDA evaluated in IEEE single precision.
// Loops are bounded: a ray that exceeds the step budget reports no hit and sets the status word.
#include <cuda_runtime.h>

#include <cfloat>
#include <cstdint>

#include "lod.h"
#include "lod_dda.cuh"

namespace nlod {

using dda::test_bit;
using dda::first_active_voxel;

namespace {


// ---- pyramid construction -------------------------------------------------------------------

// Level k from level k-1: one thread per output voxel, words assembled with a warp ballot.
__global__ void k_downsample(const uint32_t* __restrict__ src, int32_t src_res, uint32_t* __restrict__ dst, int32_t dst_res) {
    const uint64_t n = (uint64_t)dst_res * dst_res * dst_res;
    const uint64_t word_base = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) & ~uint64_t(31);
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    bool on = false;
    if (i < n) {
        const int32_t x = (int32_t)(i % dst_res), y = (int32_t)((i / dst_res) % dst_res), z = (int32_t)(i / ((uint64_t)dst_res * dst_res));
#pragma unroll
        for (int c = 0; c < 8; ++c) {
            const uint64_t s = (uint64_t)(2 * x + (c & 1)) + (uint64_t)src_res * ((uint64_t)(2 * y + ((c >> 1) & 1)) + (uint64_t)src_res * (2 * z + ((c >> 2) & 1)));
            on |= test_bit(src, s);
        }
    }
    const uint32_t ballot = __ballot_sync(0xffffffffu, on);
    if ((threadIdx.x & 31) == 0 && word_base < n) dst[word_base >> 5] = __brev(ballot);
}

// Leaf flags + active count + bounding box: one thread per 8^3 block.
__global__ void k_leaf_flags(const uint32_t* __restrict__ bits, int32_t res, uint8_t* __restrict__ leaf, int32_t* __restrict__ stats) {
    const int32_t nb = (res + 7) / 8;
    const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= (int64_t)nb * nb * nb) return;
    const int32_t bx = (int32_t)(b % nb), by = (int32_t)((b / nb) % nb), bz = (int32_t)(b / ((int64_t)nb * nb));
    int32_t count = 0;
    int32_t mn[3] = {INT32_MAX, INT32_MAX, INT32_MAX}, mx[3] = {-1, -1, -1};
    for (int32_t z = bz * 8; z < min(res, bz * 8 + 8); ++z)
        for (int32_t y = by * 8; y < min(res, by * 8 + 8); ++y)
            for (int32_t x = bx * 8; x < min(res, bx * 8 + 8); ++x) {
                if (!test_bit(bits, (uint64_t)x + (uint64_t)res * ((uint64_t)y + (uint64_t)res * z))) continue;
                ++count;
                mn[0] = min(mn[0], x); mn[1] = min(mn[1], y); mn[2] = min(mn[2], z);
                mx[0] = max(mx[0], x); mx[1] = max(mx[1], y); mx[2] = max(mx[2], z);
            }
    leaf[b] = count ? 1 : 0;
    if (count) {
        atomicAdd(&stats[0], count);
        for (int k = 0; k < 3; ++k) {
            atomicMin(&stats[1 + k], mn[k]);
            atomicMax(&stats[4 + k], mx[k]);
        }
    }
}

// Lower-node flags from leaf flags: one thread per 128^3 block.
__global__ void k_lower_flags(const uint8_t* __restrict__ leaf, int32_t res, uint8_t* __restrict__ lower) {
    const int32_t nb = (res + 7) / 8, nl = (res + 127) / 128;
    const int32_t b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nl * nl * nl) return;
    const int32_t lx = b % nl, ly = (b / nl) % nl, lz = b / (nl * nl);
    uint8_t any = 0;
    for (int32_t z = lz * 16; z < min(nb, lz * 16 + 16) && !any; ++z)
        for (int32_t y = ly * 16; y < min(nb, ly * 16 + 16) && !any; ++y)
            for (int32_t x = lx * 16; x < min(nb, lx * 16 + 16); ++x)
                if (leaf[x + nb * (y + nb * z)]) { any = 1; break; }
    lower[b] = any;
}

__global__ void k_first_active_voxel(const __grid_constant__ LodLevelDev L, uint32_t n, const float* __restrict__ eye,
                                     const float* __restrict__ dir, const float* __restrict__ t_min, const int32_t* __restrict__ prev,
                                     int32_t* __restrict__ hit, int32_t* __restrict__ ijk, float* __restrict__ t_near,
                                     float* __restrict__ t_far, uint32_t budget, uint32_t* __restrict__ status) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float E[3] = {eye[3 * i], eye[3 * i + 1], eye[3 * i + 2]};
    const float D[3] = {dir[3 * i], dir[3 * i + 1], dir[3 * i + 2]};
    const int32_t pv[3] = {prev ? prev[3 * i] : -1, prev ? prev[3 * i + 1] : -1, prev ? prev[3 * i + 2] : -1};
    int32_t v[3] = {0, 0, 0};
    float tn = 0.f, tf = 0.f;
    const int r = first_active_voxel(L, E, D, t_min ? t_min[i] : 0.f, pv, v, tn, tf, budget);
    if (r < 0) atomicOr(status, 2u);
    const bool h = r == 1;
    hit[i] = h ? 1 : 0;
    ijk[3 * i] = h ? v[0] : 0;
    ijk[3 * i + 1] = h ? v[1] : 0;
    ijk[3 * i + 2] = h ? v[2] : 0;
    t_near[i] = h ? tn : 0.f;
    t_far[i] = h ? tf : 0.f;
}

}  // namespace

cudaError_t launch_downsample(const uint32_t* src, int32_t src_res, uint32_t* dst, int32_t dst_res, cudaStream_t s) {
    const uint64_t n = (uint64_t)dst_res * dst_res * dst_res;
    const uint64_t threads = (n + 31) / 32 * 32;
    if (!threads) return cudaSuccess;
    k_downsample<<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(src, src_res, dst, dst_res);
    return cudaGetLastError();
}

cudaError_t launch_level_flags(const uint32_t* bits, int32_t res, uint8_t* leaf, uint8_t* lower, int32_t* stats, cudaStream_t s) {
    const int32_t nb = (res + 7) / 8, nl = (res + 127) / 128;
    const int64_t nleaf = (int64_t)nb * nb * nb;
    k_leaf_flags<<<(unsigned)((nleaf + 127) / 128), 128, 0, s>>>(bits, res, leaf, stats);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_lower_flags<<<(nl * nl * nl + 63) / 64, 64, 0, s>>>(leaf, res, lower);
    return cudaGetLastError();
}

cudaError_t launch_first_active_voxel(const LodLevelDev& L, uint32_t n, const float* eye, const float* dir, const float* t_min,
                                      const int32_t* prev, int32_t* hit, int32_t* ijk, float* t_near, float* t_far,
                                      uint32_t* status, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    // Each leaf span costs at most 3*8 voxel steps and the tree walk at most 3*res/8 node steps
    // plus level changes; the budget is far above what any ray through the grid needs.
    const uint32_t budget = 64u * (uint32_t)L.res + 4096u;
    k_first_active_voxel<<<(n + 127) / 128, 128, 0, s>>>(L, n, eye, dir, t_min, prev, hit, ijk, t_near, t_far, budget, status);
    return cudaGetLastError();
}

}  // namespace nlod
