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

namespace nlod {

namespace {

__device__ __forceinline__ bool test_bit(const uint32_t* __restrict__ bits, uint64_t idx) {
    return (__ldg(bits + (idx >> 5)) >> (31u - (uint32_t)(idx & 31u))) & 1u;
}

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

// ---- search -----------------------------------------------------------------------------------

struct Hdda {
    int32_t dim;
    float t0, t1;
    int32_t voxel[3], step[3];
    float delta[3], next[3];
};

__device__ __forceinline__ void ray_at(const float (&E)[3], const float (&D)[3], float t, float (&p)[3]) {
#pragma unroll
    for (int k = 0; k < 3; ++k) p[k] = fmaf(t, D[k], E[k]);
}

__device__ __forceinline__ int32_t floor_i(float x) { return (int32_t)floorf(x); }

__device__ __forceinline__ int get_dim(const LodLevelDev& L, const int32_t (&ijk)[3]) {
    if (L.n_active == 0) return 4096;
#pragma unroll
    for (int k = 0; k < 3; ++k)
        if (ijk[k] < 0 || ijk[k] >= 4096) return 4096;
    const int32_t nl = (L.res + 127) / 128, nb = (L.res + 7) / 8;
    const int32_t lx = ijk[0] >> 7, ly = ijk[1] >> 7, lz = ijk[2] >> 7;
    if (lx >= nl || ly >= nl || lz >= nl || !L.lower[lx + nl * (ly + nl * lz)]) return 128;
    const int32_t bx = ijk[0] >> 3, by = ijk[1] >> 3, bz = ijk[2] >> 3;
    if (bx >= nb || by >= nb || bz >= nb || !L.leaf[bx + nb * (by + nb * bz)]) return 8;
    return 1;
}

__device__ __forceinline__ void hdda_init(Hdda& h, const float (&E)[3], const float (&D)[3], const float (&inv)[3], float t0, float t1,
                                          int32_t dim) {
    h.dim = dim;
    h.t0 = t0;
    h.t1 = t1;
    float pos[3];
    ray_at(E, D, t0, pos);
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        h.voxel[a] = floor_i(pos[a]) & ~(dim - 1);
        h.delta[a] = 0.f;
        if (D[a] == 0.f) {
            h.next[a] = FLT_MAX;
            h.step[a] = 0;
        } else if (inv[a] > 0.f) {
            h.step[a] = 1;
            h.next[a] = __fadd_rn(t0, __fmul_rn(__fsub_rn((float)(h.voxel[a] + dim), pos[a]), inv[a]));
            h.delta[a] = inv[a];
        } else {
            h.step[a] = -1;
            h.next[a] = __fadd_rn(t0, __fmul_rn(__fsub_rn((float)h.voxel[a], pos[a]), inv[a]));
            h.delta[a] = -inv[a];
        }
    }
}

__device__ __forceinline__ void hdda_update(Hdda& h, const float (&E)[3], const float (&D)[3], const float (&inv)[3], int32_t dim) {
    if (h.dim == dim) return;
    h.dim = dim;
    float pos[3];
    ray_at(E, D, h.t0, pos);
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        h.voxel[a] = floor_i(pos[a]) & ~(dim - 1);
        if (h.step[a] == 0) continue;
        h.next[a] = __fadd_rn(h.t0, __fmul_rn(__fsub_rn((float)h.voxel[a], pos[a]), inv[a]));
        if (h.step[a] > 0) h.next[a] = __fadd_rn(h.next[a], __fmul_rn((float)dim, inv[a]));
    }
}

__device__ __forceinline__ bool hdda_step(Hdda& h) {
    const int a = (h.next[0] < h.next[1] && h.next[0] < h.next[2]) ? 0 : (h.next[1] < h.next[2] ? 1 : 2);
    float na = h.next[a];
    if (na <= h.t0) na = __fadd_rn(na, __fadd_rn(__fsub_rn(h.t0, __fmul_rn(0.999999f, na)), 1.0e-6f));
    h.t0 = na;
    h.next[a] = __fadd_rn(na, __fmul_rn((float)h.dim, h.delta[a]));
    h.voxel[a] += h.dim * h.step[a];
    return h.t0 <= h.t1;
}

__device__ __forceinline__ bool slab(const float (&o)[3], const float (&d)[3], const int32_t (&ijk)[3], float& near_t, float& far_t) {
    near_t = -1e20f;
    far_t = 1e20f;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const float inv = __fdiv_rn(1.f, d[i]);
        const float lo = (float)ijk[i], hi = __fadd_rn(lo, 1.0f);
        if (d[i] == 0.f) {
            if (o[i] < lo || o[i] > hi) return false;
        } else {
            float t1 = __fmul_rn(__fsub_rn(lo, o[i]), inv), t2 = __fmul_rn(__fsub_rn(hi, o[i]), inv);
            if (t1 > t2) { const float t = t1; t1 = t2; t2 = t; }
            near_t = (t1 < near_t) ? near_t : t1;
            far_t = (far_t < t2) ? far_t : t2;
            if (!(near_t < far_t) || far_t < 0.0f) return false;
        }
    }
    return true;
}

// Returns 1 on a hit, 0 on a miss, -1 when the step budget ran out.
__device__ int first_active_voxel(const LodLevelDev& L, const float (&E)[3], const float (&D)[3], float t_min, const int32_t (&prev)[3],
                                  int32_t (&out)[3], float& t_near, float& t_far, uint32_t budget) {
    if (L.n_active == 0) return 0;
    const float inv[3] = {__fdiv_rn(1.f, D[0]), __fdiv_rn(1.f, D[1]), __fdiv_rn(1.f, D[2])};
    float t0 = t_min, t1 = FLT_MAX;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        float a = (float)L.bbox_min[i], b = (float)(L.bbox_max[i] + 1);
        if (a >= b) return 0;
        a = __fmul_rn(__fsub_rn(a, E[i]), inv[i]);
        b = __fmul_rn(__fsub_rn(b, E[i]), inv[i]);
        if (a > b) { const float t = a; a = b; b = t; }
        if (a > t0) t0 = a;
        if (b < t1) t1 = b;
        if (t0 > t1) return 0;
    }
    const float ta = __fadd_rn(t0, 0.000001f), tb = __fsub_rn(t1, 0.000001f);
    if (ta > tb) return 0;
    int32_t ijk[3], leaf[3] = {0, 0, 0};
    bool have_leaf = false;
    float p[3];
    ray_at(E, D, ta, p);
#pragma unroll
    for (int k = 0; k < 3; ++k) ijk[k] = floor_i(p[k]);
    const int dim = get_dim(L, ijk);
    if (dim == 1) {
        have_leaf = true;
#pragma unroll
        for (int k = 0; k < 3; ++k) leaf[k] = ijk[k] >> 3;
    }
    Hdda h;
    hdda_init(h, E, D, inv, ta, tb, dim > 8 ? dim : 8);
    float mt0 = dim <= 1 ? h.t0 : -1.f;
    const float tmax = tb;
    bool valid;
    uint32_t steps = 0;
    do {
        if (++steps > budget) return -1;
        const float s0 = mt0;
        const bool cur_have = have_leaf;
        const int32_t cur[3] = {leaf[0], leaf[1], leaf[2]};
        valid = hdda_step(h);
        ray_at(E, D, __fadd_rn(h.t0, 0.01f), p);
        int32_t nxt[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) nxt[k] = floor_i(p[k]);
        const int nd = get_dim(L, nxt);
        if (nd == 1) {
            have_leaf = true;
#pragma unroll
            for (int k = 0; k < 3; ++k) leaf[k] = nxt[k] >> 3;
        }
        hdda_update(h, E, D, inv, nd > 8 ? nd : 8);
        mt0 = nd <= 1 ? h.t0 : -1.f;
        if (s0 >= 0.f) {
            const float s1 = (tmax < h.t0) ? tmax : h.t0;
            if (s0 >= s1 || !cur_have) continue;
            Hdda dda;
            hdda_init(dda, E, D, inv, s0, s1, 1);
            do {
                if (++steps > budget) return -1;
                const int32_t v[3] = {dda.voxel[0], dda.voxel[1], dda.voxel[2]};
                const int32_t lx = v[0] - cur[0] * 8, ly = v[1] - cur[1] * 8, lz = v[2] - cur[2] * 8;
                if (lx < 0 || ly < 0 || lz < 0 || lx >= 8 || ly >= 8 || lz >= 8) continue;
                if (v[0] >= L.res || v[1] >= L.res || v[2] >= L.res) continue;
                if (!test_bit(L.bits, (uint64_t)v[0] + (uint64_t)L.res * ((uint64_t)v[1] + (uint64_t)L.res * v[2]))) continue;
                if (v[0] == prev[0] && v[1] == prev[1] && v[2] == prev[2]) continue;
                if (slab(E, D, v, t_near, t_far)) {
#pragma unroll
                    for (int k = 0; k < 3; ++k) out[k] = v[k];
                    return 1;
                }
            } while (hdda_step(dda));
        }
    } while (valid);
    return 0;
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
