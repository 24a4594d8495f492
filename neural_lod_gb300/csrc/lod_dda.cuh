// First-active-voxel search of one ray through one level of the LoD pyramid (device code shared
// by the search kernel of lod.cu and the wavefront renderer).  It restates, operation for
// operation, NanoVDB's TreeMarcher over leaf nodes (rptr/ext/nanovdb/nanovdb/util/HDDA.h:370-450)
// with its HDDA (:27-188, forward stepping on), the unit DDA inside each leaf span (:190-307),
// getDim of the sparse tree (NanoVDB.h:3358-3369, 3745-3757, 4442-4448), and the search loop +
// slab test of first_active_voxel_intersection (rptr/cuda/neural-lod/neural_lod_learning_common.cuh:
// 567-606, 783-832), with explicit round-to-nearest intrinsics (no contracted multiply-add).
#pragma once

#include <cuda_runtime.h>

#include <cfloat>
#include <cstdint>

#include "lod.h"

namespace nlod {
namespace dda {

__device__ __forceinline__ bool test_bit(const uint32_t* __restrict__ bits, uint64_t idx) {
    return (__ldg(bits + (idx >> 5)) >> (31u - (uint32_t)(idx & 31u))) & 1u;
}

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

// One step along the axis with the nearest crossing.  The axis is applied through selects rather
// than an index, so that the state stays in registers (an indexed array lives in local memory).
__device__ __forceinline__ bool hdda_step(Hdda& h) {
    const bool x = h.next[0] < h.next[1] && h.next[0] < h.next[2];
    const bool y = !x && h.next[1] < h.next[2];
    const bool z = !x && !y;
    float na = x ? h.next[0] : (y ? h.next[1] : h.next[2]);
    if (na <= h.t0) na = __fadd_rn(na, __fadd_rn(__fsub_rn(h.t0, __fmul_rn(0.999999f, na)), 1.0e-6f));
    h.t0 = na;
    const float delta = x ? h.delta[0] : (y ? h.delta[1] : h.delta[2]);
    const int32_t step = x ? h.step[0] : (y ? h.step[1] : h.step[2]);
    const float nn = __fadd_rn(na, __fmul_rn((float)h.dim, delta));
    const int32_t dv = h.dim * step;
    h.next[0] = x ? nn : h.next[0];
    h.next[1] = y ? nn : h.next[1];
    h.next[2] = z ? nn : h.next[2];
    h.voxel[0] += x ? dv : 0;
    h.voxel[1] += y ? dv : 0;
    h.voxel[2] += z ? dv : 0;
    return h.t0 <= h.t1;
}

__device__ __forceinline__ bool slab(const float (&o)[3], const float (&d)[3], const int32_t (&ijk)[3], float& near_t, float& far_t) {
    near_t = -1e20f;
    far_t = 1e20f;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const float inv = __frcp_rn(d[i]);   // 1 / d, correctly rounded (the same value as 1.f / d)
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

// Returns 1 on a hit, 0 on a miss, -1 when the step budget ran out.  The search covers ray
// parameters [t_min, t_max] (t_max = FLT_MAX: up to the grid's active bbox).
__device__ __forceinline__ int first_active_voxel(const LodLevelDev& L, const float (&E)[3], const float (&D)[3], float t_min, const int32_t (&prev)[3],
                                  int32_t (&out)[3], float& t_near, float& t_far, uint32_t budget, float t_max = FLT_MAX) {
    if (L.n_active == 0) return 0;
    // 1 / D correctly rounded (__frcp_rn: the value of the IEEE division 1.f / D)
    const float inv[3] = {__frcp_rn(D[0]), __frcp_rn(D[1]), __frcp_rn(D[2])};
    float t0 = t_min, t1 = t_max;
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

}  // namespace dda
}  // namespace nlod
