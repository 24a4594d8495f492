// Device-side input encodings: multiresolution hash/dense grid, spherical harmonics,
// identity and one-hot.  Semantics follow tiny-cuda-nn (paths relative to
// rptr/ext/tiny-cuda-nn/include/tiny-cuda-nn/):
//   grid index / hashes       encodings/grid.h:111-187
//   pos_fract (+0.5 offset)   common_device.h:437-464
//   forward interpolation     encodings/grid.h:220-392
//   backward scatter          encodings/grid.h:394-517
//   max-level masking         encodings/grid.h:242-265, 413-424
//   spherical harmonics       encodings/spherical_harmonics.h:46-151 (input mapped by 2x-1,
//                             padding written first as 1.0)
//   identity                  encodings/identity.h:45-66 (padding written last as 1.0)
//
// Work decomposition of a tile: grid slots are evaluated as (row, group of 4 levels) units so one
// thread has 32 independent table gathers in flight and writes 8 adjacent features at once; the
// other slots are evaluated as (row, slot) units.  A Store policy (shared-memory layout of the
// consuming kernel) receives the features.
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <cstdint>
#include <type_traits>

#include "desc.h"

namespace nlod {

// ---- hashing and table index (grid.h:111-187) -----------------------------------------------

__device__ __forceinline__ uint32_t grid_hash3(int32_t kind, uint32_t x, uint32_t y, uint32_t z) {
    // XOR of coordinate * prime; the coherent variant keeps x unscrambled (prime 1).
    if (kind == HASH_COHERENT_PRIME) return x ^ (y * 2654435761u) ^ (z * 805459861u);
    if (kind == HASH_PRIME) return (x * 1958374283u) ^ (y * 2654435761u) ^ (z * 805459861u);
    return (x * 2165219737u) ^ (y * 1434869437u) ^ (z * 2097192037u);  // reversed primes
}

// Table entry of integer grid vertex (x, y, z) within one level: the dense row-major index over the
// dims whose running stride fits the level's table, replaced by the spatial hash on hashed levels,
// taken modulo the level size.  uint32 wrap-around is part of the definition.
__device__ __forceinline__ uint32_t level_entry(int32_t hash_kind, const GridLevel& L, uint32_t x, uint32_t y, uint32_t z) {
    const uint32_t f = L.res_flags;
    const uint32_t res = f & kLevelResMask;
    uint32_t idx;
    if (f & kLevelHashed) {
        idx = grid_hash3(hash_kind, x, y, z);
    } else {
        const uint32_t dims = f >> kLevelDimsShift;
        idx = x;
        if (dims > 1) idx += y * res;
        if (dims > 2) idx += z * (res * res);
    }
    if (f & kLevelPow2) return idx & (L.size - 1u);
    if (idx < L.size) return idx;
    const uint32_t t = idx - L.size;   // one wrap covers every vertex of inputs in [0,1]
    return t < L.size ? t : idx % L.size;
}

// pos_fract: p = x * scale + 0.5 (a single fused multiply-add), cell = floor(p), frac = p - cell.
__device__ __forceinline__ void grid_pos_fract(float x, float scale, float& frac, uint32_t& cell) {
    const float p = fmaf(x, scale, 0.5f);
    const float fl = floorf(p);
    cell = (uint32_t)(int)fl;
    frac = p - fl;
}

__device__ __forceinline__ float interp_weight_fun(int32_t interp, float t) {
    return interp == INTERP_SMOOTHSTEP ? t * t * (3.0f - 2.0f * t) : t;
}

// Whether `level` of a grid is masked for this element in the forward pass (grid.h:242-265:
// levels at or above max_level + 1e-3 are zeroed).  max_level_frac is the per-element fraction
// in [0,1] (or the scalar default 1000).
__device__ __forceinline__ bool grid_level_masked(uint32_t level, float max_level_frac, uint32_t n_levels) {
    const float max_level = (max_level_frac * (float)(n_levels * 2u)) / 2.0f;
    return (float)level >= max_level + 1e-3f;
}

// The backward pass skips a level only when it lies strictly above max_level + 1e-3 (grid.h:422).
__device__ __forceinline__ bool grid_level_skipped_backward(uint32_t level, float max_level_frac, uint32_t n_levels) {
    const float max_level = (max_level_frac * (float)(n_levels * 2u)) / 2.0f;
    return (float)level > max_level + 1e-3f;
}

__device__ __forceinline__ void hash_primes(int32_t kind, uint32_t& p0, uint32_t& p1, uint32_t& p2) {
    if (kind == HASH_COHERENT_PRIME) { p0 = 1u; p1 = 2654435761u; p2 = 805459861u; }
    else if (kind == HASH_PRIME) { p0 = 1958374283u; p1 = 2654435761u; p2 = 805459861u; }
    else { p0 = 2165219737u; p1 = 1434869437u; p2 = 2097192037u; }
}

// Reduces a dense index modulo a non power-of-two level size (one subtraction covers inputs in
// [0,1]; anything else takes the division).
__device__ __forceinline__ uint32_t dense_mod(uint32_t idx, uint32_t size) {
    if (idx < size) return idx;
    const uint32_t t = idx - size;
    return t < size ? t : idx % size;
}

// Table entries of the 8 corners of the cell (cx, cy, cz) at one level: corner c takes
// (cx + (c&1), cy + (c>>1 & 1), cz + (c>>2 & 1)).  The per-axis terms of the index (dense
// strides or hash products) are formed once and combined per corner, which is exactly
// level_entry() for each corner.
__device__ __forceinline__ void level_corner_entries(const GridLevel& L, uint32_t p0, uint32_t p1, uint32_t p2, uint32_t cx,
                                                     uint32_t cy, uint32_t cz, uint32_t (&e)[8]) {
    const uint32_t f = L.res_flags;
    if (f & kLevelHashed) {
        // hashed levels always have a power-of-two size
        const uint32_t m = L.size - 1u;
        const uint32_t x0 = cx * p0, x1 = (cx + 1u) * p0;
        const uint32_t y0 = cy * p1, y1 = (cy + 1u) * p1;
        const uint32_t z0 = cz * p2, z1 = (cz + 1u) * p2;
#pragma unroll
        for (int c = 0; c < 8; ++c) e[c] = ((c & 1) ? x1 : x0) ^ ((c & 2) ? y1 : y0) ^ ((c & 4) ? z1 : z0);
#pragma unroll
        for (int c = 0; c < 8; ++c) e[c] &= m;
    } else {
        const uint32_t dims = f >> kLevelDimsShift;
        const uint32_t res = f & kLevelResMask;
        const uint32_t sy = dims > 1 ? res : 0u, sz = dims > 2 ? res * res : 0u;
        const uint32_t y0 = cy * sy, y1 = (cy + 1u) * sy;
        const uint32_t z0 = cz * sz, z1 = (cz + 1u) * sz;
#pragma unroll
        for (int c = 0; c < 8; ++c) e[c] = ((c & 1) ? cx + 1u : cx) + ((c & 2) ? y1 : y0) + ((c & 4) ? z1 : z0);
        if (f & kLevelPow2) {
#pragma unroll
            for (int c = 0; c < 8; ++c) e[c] &= L.size - 1u;
        } else {
#pragma unroll
            for (int c = 0; c < 8; ++c) e[c] = dense_mod(e[c], L.size);
        }
    }
}

// One grid entry (F = 2 features) of a table stored as FP32 pairs or as FP16 pairs (the half
// copy the FP16 query kernels read, tiny-cuda-nn's half-precision parameters), and the 16- / 8-byte
// load of the aligned entry pair {2m, 2m+1}.
__device__ __forceinline__ float2 table_entry(const float* t, uint32_t e) { return __ldg(reinterpret_cast<const float2*>(t) + e); }
__device__ __forceinline__ float2 table_entry(const __half* t, uint32_t e) {
    const uint32_t w = __ldg(reinterpret_cast<const unsigned int*>(t) + e);
    return __half22float2(*reinterpret_cast<const __half2*>(&w));
}
__device__ __forceinline__ void table_pair(const float* t, uint32_t even, float2& lo, float2& hi) {
    const float4 q = __ldg(reinterpret_cast<const float4*>(t) + (even >> 1));
    lo = make_float2(q.x, q.y);
    hi = make_float2(q.z, q.w);
}
__device__ __forceinline__ void table_pair(const __half* t, uint32_t even, float2& lo, float2& hi) {
    const uint2 q = __ldg(reinterpret_cast<const uint2*>(t) + (even >> 1));
    lo = __half22float2(*reinterpret_cast<const __half2*>(&q.x));
    hi = __half22float2(*reinterpret_cast<const __half2*>(&q.y));
}
__device__ __forceinline__ float2 table_entry(const __nv_bfloat16* t, uint32_t e) {
    const uint32_t w = __ldg(reinterpret_cast<const unsigned int*>(t) + e);
    return __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&w));
}
__device__ __forceinline__ void table_pair(const __nv_bfloat16* t, uint32_t even, float2& lo, float2& hi) {
    const uint2 q = __ldg(reinterpret_cast<const uint2*>(t) + (even >> 1));
    lo = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&q.x));
    hi = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&q.y));
}
// Entries a and b of one aligned block of four BF16 entries {4m .. 4m+3} with one 16-byte load.
__device__ __forceinline__ void table_quad(const __nv_bfloat16* t, uint32_t a, uint32_t b, float2& va, float2& vb) {
    const uint4 q = __ldg(reinterpret_cast<const uint4*>(t) + (a >> 2));
    const uint32_t wa = (a & 2u) ? ((a & 1u) ? q.w : q.z) : ((a & 1u) ? q.y : q.x);
    const uint32_t wb = (b & 2u) ? ((b & 1u) ? q.w : q.z) : ((b & 1u) ? q.y : q.x);
    va = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&wa));
    vb = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&wb));
}
// Entries a and b of one aligned block of four FP16 entries {4m .. 4m+3} with one 16-byte load.
__device__ __forceinline__ void table_quad(const __half* t, uint32_t a, uint32_t b, float2& va, float2& vb) {
    const uint4 q = __ldg(reinterpret_cast<const uint4*>(t) + (a >> 2));
    const uint32_t wa = (a & 2u) ? ((a & 1u) ? q.w : q.z) : ((a & 1u) ? q.y : q.x);
    const uint32_t wb = (b & 2u) ? ((b & 1u) ? q.w : q.z) : ((b & 1u) ? q.y : q.x);
    va = __half22float2(*reinterpret_cast<const __half2*>(&wa));
    vb = __half22float2(*reinterpret_cast<const __half2*>(&wb));
}

// Features of levels [l0, l0 + nl) (nl <= NL) of one grid for one element: f[2i], f[2i+1] are
// the two features of level l0 + i.  All gathers of the group are issued before any is used.
// `levels` is the grid's level table (the kernel parameter copy or a shared-memory copy); `table`
// the grid's parameters (TT = float, or __half for the FP16 copy).
// Cell table of the first grid's leading levels (FP16 tables; cells.cu): for every cell
// (cx, cy, cz) < res of level l < levels, the FP16 pairs of its eight corner entries in one 32-byte
// record at record base[l] + cx + res (cy + res cz).  rec == nullptr: no table.
struct CellTable {
    const uint4* rec;
    const uint32_t* base;
    uint32_t levels;
};

// `ct` (FP16 tables only): a level the cell table covers reads a cell's eight corners with two
// 16-byte loads of one sector instead of four to eight gathers; cells outside [0, res)^3 take the
// gathers.
template <int NL, typename TT = float>
__device__ __forceinline__ void grid_group_forward(const GridDesc& g, const GridLevel* __restrict__ levels, uint32_t l0, uint32_t nl,
                                                   const TT* __restrict__ table, float px, float py, float pz, float ml_frac,
                                                   float (&f)[2 * NL], const uint32_t* smem_tab = nullptr, uint32_t smem_levels = 0,
                                                   CellTable ct = {}) {
    uint32_t p0, p1, p2;
    hash_primes(g.hash, p0, p1, p2);
    float2 v[NL][8];
    float w3[NL][3];
    bool on[NL];
#pragma unroll
    for (int i = 0; i < NL; ++i) {
        const uint32_t l = l0 + i;
        on[i] = (uint32_t)i < nl && !grid_level_masked(l, ml_frac, g.n_levels);
        if (on[i]) {
            const GridLevel L = levels[l];
            float fx, fy, fz;
            uint32_t cx, cy, cz;
            grid_pos_fract(px, L.scale, fx, cx);
            grid_pos_fract(py, L.scale, fy, cy);
            grid_pos_fract(pz, L.scale, fz, cz);
            w3[i][0] = interp_weight_fun(g.interp, fx);
            w3[i][1] = interp_weight_fun(g.interp, fy);
            w3[i][2] = interp_weight_fun(g.interp, fz);
            const TT* lv = table + 2u * L.offset;
            bool from_cells = false;
            if constexpr (std::is_same<TT, __half>::value) {
                const uint32_t res = L.res_flags & kLevelResMask;
                if (ct.rec != nullptr && l < ct.levels && cx < res && cy < res && cz < res) {
                    const uint4* cp = ct.rec + 2u * (ct.base[l] + cx + res * (cy + res * cz));
                    const uint4 q0 = __ldg(cp), q1 = __ldg(cp + 1);
                    const uint32_t w[8] = {q0.x, q0.y, q0.z, q0.w, q1.x, q1.y, q1.z, q1.w};
#pragma unroll
                    for (int c = 0; c < 8; ++c) v[i][c] = __half22float2(*reinterpret_cast<const __half2*>(&w[c]));
                    from_cells = true;
                }
            }
            if (from_cells) {
            } else if (g.interp == INTERP_NEAREST) {
                v[i][0] = table_entry(lv, level_entry(g.hash, L, cx, cy, cz));
            } else {
                uint32_t e[8];
                level_corner_entries(L, p0, p1, p2, cx, cy, cz, e);
                // x-adjacent corners whose entries lie in one aligned block come in one load:
                // a pair {2m, 2m+1} of FP32 entries in 16 bytes, a block {4m .. 4m+3} of 16-bit
                // (FP16 or BF16) entries in 16 bytes (3 in 4 x-pairs of the coherent-prime hash and of dense
                // levels, against 1 in 2 for 8-byte pairs; measured -8 % in the gathers).  Every
                // level starts on a multiple of 8 entries.
#pragma unroll
                for (int c = 0; c < 8; c += 2) {
                    const uint32_t ea = e[c], eb = e[c + 1];
                    if constexpr (sizeof(TT) == 2) {
                        if (std::is_same<TT, __half>::value && l < smem_levels) {
                            // a level staged in shared memory: one FP16 pair per 32-bit word
                            const uint32_t* sl = smem_tab + L.offset;
                            const uint32_t wa = sl[ea], wb = sl[eb];
                            v[i][c] = __half22float2(*reinterpret_cast<const __half2*>(&wa));
                            v[i][c + 1] = __half22float2(*reinterpret_cast<const __half2*>(&wb));
                            continue;
                        }
                        if ((ea >> 2) == (eb >> 2)) {
                            table_quad(lv, ea, eb, v[i][c], v[i][c + 1]);
                        } else {
                            v[i][c] = table_entry(lv, ea);
                            v[i][c + 1] = table_entry(lv, eb);
                        }
                        continue;
                    }
                    if ((ea ^ eb) == 1u) {
                        float2 lo, hi;
                        table_pair(lv, ea & ~1u, lo, hi);
                        v[i][c] = (ea & 1u) ? hi : lo;
                        v[i][c + 1] = (ea & 1u) ? lo : hi;
                    } else {
                        v[i][c] = table_entry(lv, ea);
                        v[i][c + 1] = table_entry(lv, eb);
                    }
                }
            }
        }
    }
#pragma unroll
    for (int i = 0; i < NL; ++i) {
        float a = 0.f, b = 0.f;
        if (on[i]) {
            if (g.interp == INTERP_NEAREST) {
                a = v[i][0].x;
                b = v[i][0].y;
            } else {
                const float wx0 = 1.0f - w3[i][0], wx1 = w3[i][0];
                const float wy0 = 1.0f - w3[i][1], wy1 = w3[i][1];
                const float wz0 = 1.0f - w3[i][2], wz1 = w3[i][2];
#pragma unroll
                for (int c = 0; c < 8; ++c) {
                    const float w = ((c & 1) ? wx1 : wx0) * ((c & 2) ? wy1 : wy0) * ((c & 4) ? wz1 : wz0);
                    a = fmaf(w, v[i][c].x, a);
                    b = fmaf(w, v[i][c].y, b);
                }
            }
        }
        f[2 * i] = a;
        f[2 * i + 1] = b;
    }
}

// Scatter dL/d(features) of one level into the FP32 gradient table (grid.h:394-517).
// Lanes of a warp that hit the same entry are merged before the atomic (warp aggregation),
// which matters on the coarse levels where whole warps share a handful of vertices.
// Must be called by all lanes of the warp (inactive lanes pass active = false).
__device__ __forceinline__ void grid_level_backward(const GridDesc& g, uint32_t level, float* __restrict__ grad_table,
                                                    float px, float py, float pz, float2 dy, bool active) {
    const GridLevel L = g.levels[level];
    float2* lv = reinterpret_cast<float2*>(grad_table) + L.offset;
    float fx, fy, fz;
    uint32_t cx, cy, cz;
    grid_pos_fract(px, L.scale, fx, cx);
    grid_pos_fract(py, L.scale, fy, cy);
    grid_pos_fract(pz, L.scale, fz, cz);
    const unsigned full = __activemask();
    const int lane = threadIdx.x & 31;
    const int ncorners = g.interp == INTERP_NEAREST ? 1 : 8;
    fx = interp_weight_fun(g.interp, fx);
    fy = interp_weight_fun(g.interp, fy);
    fz = interp_weight_fun(g.interp, fz);
    const float wx[2] = {1.0f - fx, fx};
    const float wy[2] = {1.0f - fy, fy};
    const float wz[2] = {1.0f - fz, fz};
    for (int c = 0; c < ncorners; ++c) {
        const float w = ncorners == 1 ? 1.0f : wx[c & 1] * wy[(c >> 1) & 1] * wz[(c >> 2) & 1];
        const uint32_t e = active ? level_entry(g.hash, L, cx + (c & 1), cy + ((c >> 1) & 1), cz + ((c >> 2) & 1)) : 0xFFFFFFFFu;
        float2 v = make_float2(active ? w * dy.x : 0.f, active ? w * dy.y : 0.f);
        // Lanes with equal entries form a group; the lowest lane of a group sums the group.
        const unsigned peers = __match_any_sync(full, e);
        const int leader = __ffs(peers) - 1;
        if (__popc(peers) > 1) {
            float sx = 0.f, sy = 0.f;
            unsigned m = peers;
            while (m) {
                const int src = __ffs(m) - 1;
                m &= m - 1;
                sx += __shfl_sync(peers, v.x, src);
                sy += __shfl_sync(peers, v.y, src);
            }
            v = make_float2(sx, sy);
        }
        if (active && lane == leader) atomicAdd(lv + e, v);
    }
}

// Scatter of one linear / smoothstep-interpolated level for one element with the 8 corner
// entries formed at once, so that the 8 atomics (and, with AGG, the 8 warp matches) are
// independent.  The gradient table must start on a 16-byte boundary and each level's offset be
// even (tiny-cuda-nn aligns level offsets to 8 entries; the network part before the tables is a
// multiple of 256 floats).  AGG merges the lanes of a warp that hit the same entry before the atomic (pays
// when a warp's elements are spatially coherent); without it every corner is one FP32x2 atomic,
// as in tiny-cuda-nn's kernel_grid_backward.  Must be called by all lanes of the warp.
template <bool AGG>
__device__ __forceinline__ void grid_level_scatter8(const GridDesc& g, const GridLevel& L, float* __restrict__ grad_table, uint32_t p0,
                                                    uint32_t p1, uint32_t p2, float px, float py, float pz, float2 dy, bool active) {
    float2* lv = reinterpret_cast<float2*>(grad_table) + L.offset;
    float fx, fy, fz;
    uint32_t cx, cy, cz;
    grid_pos_fract(px, L.scale, fx, cx);
    grid_pos_fract(py, L.scale, fy, cy);
    grid_pos_fract(pz, L.scale, fz, cz);
    fx = interp_weight_fun(g.interp, fx);
    fy = interp_weight_fun(g.interp, fy);
    fz = interp_weight_fun(g.interp, fz);
    uint32_t e[8];
    level_corner_entries(L, p0, p1, p2, cx, cy, cz, e);
    const float wx[2] = {1.0f - fx, fx};
    const float wy[2] = {1.0f - fy, fy};
    const float wz[2] = {1.0f - fz, fz};
    float2 v[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        const float w = wx[c & 1] * wy[(c >> 1) & 1] * wz[(c >> 2) & 1];
        v[c] = make_float2(w * dy.x, w * dy.y);
    }
    if (!AGG) {
        if (active) {
            // Corners c and c+1 differ only in x.  When their entries form an aligned pair
            // {2m, 2m+1} (half of the pairs for the coherent prime hash and for dense levels) one
            // 16-byte reduction covers both: fewer reductions on the L2, same sums.
#pragma unroll
            for (int c = 0; c < 8; c += 2) {
                const uint32_t a = e[c], b = e[c + 1];
                if ((a ^ b) == 1u) {
                    const float2 lo = (a & 1u) ? v[c + 1] : v[c];
                    const float2 hi = (a & 1u) ? v[c] : v[c + 1];
                    atomicAdd(reinterpret_cast<float4*>(lv + (a & ~1u)), make_float4(lo.x, lo.y, hi.x, hi.y));
                } else {
                    atomicAdd(lv + a, v[c]);
                    atomicAdd(lv + b, v[c + 1]);
                }
            }
        }
        return;
    }
    const unsigned full = __activemask();
    unsigned peers[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) peers[c] = __match_any_sync(full, active ? e[c] : 0xFFFFFFFFu);
    bool dup = false;
#pragma unroll
    for (int c = 0; c < 8; ++c) dup |= (peers[c] & (peers[c] - 1u)) != 0u;
    if (!__any_sync(full, dup)) {
        if (active) {
#pragma unroll
            for (int c = 0; c < 8; ++c) atomicAdd(lv + e[c], v[c]);
        }
        return;
    }
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        float2 s = v[c];
        if (__popc(peers[c]) > 1) {
            float sx = 0.f, sy = 0.f;
            unsigned m = peers[c];
            while (m) {
                const int src = __ffs(m) - 1;
                m &= m - 1;
                sx += __shfl_sync(peers[c], v[c].x, src);
                sy += __shfl_sync(peers[c], v[c].y, src);
            }
            s = make_float2(sx, sy);
        }
        if (active && lane == __ffs(peers[c]) - 1) atomicAdd(lv + e[c], s);
    }
}

// ---- spherical harmonics -------------------------------------------------------------------

#include "sh_basis.inc"

// Writes degree^2 SH values of direction d (given in [0,1]^3, mapped by 2x-1) through OUT.
template <typename Writer>
__device__ __forceinline__ void sh_forward(uint32_t degree, float dx01, float dy01, float dz01, Writer&& out) {
    const float x = dx01 * 2.f - 1.f;
    const float y = dy01 * 2.f - 1.f;
    const float z = dz01 * 2.f - 1.f;
#define NLOD_SH_OUT(i, v) out((i), (v))
    SH_BASIS(NLOD_SH_OUT, x, y, z, degree);
#undef NLOD_SH_OUT
}

// Evaluates one non-grid slot (or the padding of a grid slot) for one element through put(col, v).
template <typename Put>
__device__ __forceinline__ void encode_slot_scalar(const Slot& s, const ModelDesc& d, const float* __restrict__ row, Put&& put) {
    switch (s.type) {
        case SLOT_GRID: {
            const uint32_t nf = d.grids[s.grid].n_levels * 2u;
            for (uint32_t p = 0; p < s.n_pad; ++p) put(s.out_begin + nf + p, 0.0f);
            break;
        }
        case SLOT_SH: {
            for (uint32_t p = 0; p < s.n_pad; ++p) put(s.out_begin + p, 1.0f);
            const uint32_t base = s.out_begin + s.n_pad;
            sh_forward(s.degree, row[s.in_begin], row[s.in_begin + 1], row[s.in_begin + 2],
                       [&](uint32_t i, float v) { put(base + i, v); });
            break;
        }
        case SLOT_IDENTITY: {
            for (uint32_t j = 0; j < s.n_in; ++j) put(s.out_begin + j, fmaf(row[s.in_begin + j], s.scale, s.offset));
            for (uint32_t p = 0; p < s.n_pad; ++p) put(s.out_begin + s.n_in + p, 1.0f);
            break;
        }
        case SLOT_ONEHOT: {
            const float v = row[s.in_begin];
            int bin = (int)floorf(v * (float)s.n_bins);
            bin = bin < 0 ? 0 : (bin >= (int)s.n_bins ? (int)s.n_bins - 1 : bin);
            for (uint32_t j = 0; j < s.n_bins; ++j) put(s.out_begin + j, j == (uint32_t)bin ? 1.0f : 0.0f);
            for (uint32_t p = 0; p < s.n_pad; ++p) put(s.out_begin + s.n_bins + p, 0.0f);
            break;
        }
        default: break;
    }
}

// Row-per-thread encoding of a tile: thread t encodes rows t, t + nthreads, ...  The position and
// max level of a row are read once; grid levels go NL at a time (NL * 8 gathers in flight) with
// the level parameters read from `level_tables` (kMaxLevels entries per grid, shared memory).
template <int NL, typename Store, typename TT = float>
__device__ __forceinline__ void encode_tile_rows(const ModelDesc& d, const GridLevel* level_tables, const TT* __restrict__ params,
                                                 const float* in_s, uint32_t in_ld, const float* __restrict__ ml_gpu, float ml_scalar,
                                                 uint32_t row0, uint32_t rows, uint32_t tid, uint32_t nthreads, Store& st,
                                                 const uint32_t* smem_tab = nullptr, uint32_t smem_levels = 0, CellTable ct = {}) {
    for (uint32_t r = tid; r < rows; r += nthreads) {
        const float* row = in_s + r * in_ld;
        const float ml = ml_gpu ? __ldg(ml_gpu + row0 + r) : ml_scalar;
        for (uint32_t si = 0; si < d.n_slots; ++si) {
            const Slot& s = d.slots[si];
            if (s.type == SLOT_GRID) {
                const float px = row[s.in_begin], py = row[s.in_begin + 1], pz = row[s.in_begin + 2];
                const GridDesc& g = d.grids[s.grid];
                const uint32_t nlev = g.n_levels;
                const TT* table = params + g.param_offset;
                const GridLevel* lv = level_tables + s.grid * kMaxLevels;
#pragma unroll 1
                for (uint32_t l0 = 0; l0 < nlev; l0 += NL) {
                    float f[2 * NL];
                    const uint32_t nl = min((uint32_t)NL, nlev - l0);
                    // the staged levels and the cell table belong to the first grid
                    grid_group_forward<NL, TT>(g, lv, l0, nl, table, px, py, pz, ml, f, smem_tab, s.grid == 0 ? smem_levels : 0u,
                                               s.grid == 0 ? ct : CellTable{});
                    st.run(r, s.out_begin + 2u * l0, f, 2u * nl);
                }
                if (s.n_pad) encode_slot_scalar(s, d, row, [&](uint32_t col, float v) { st.one(r, col, v); });
            } else if (s.type == SLOT_SH && s.degree == 4 && s.n_pad == 0 && (s.out_begin & 1u) == 0) {
                float v[16];
                sh_forward(4u, row[s.in_begin], row[s.in_begin + 1], row[s.in_begin + 2], [&](uint32_t i, float x) { v[i] = x; });
                st.run(r, s.out_begin, v, 16u);
            } else if (s.type == SLOT_ONEHOT && s.out_width <= 16u && (s.out_width & 1u) == 0 && (s.out_begin & 1u) == 0) {
                float v[16];
                int bin = (int)floorf(row[s.in_begin] * (float)s.n_bins);
                bin = bin < 0 ? 0 : (bin >= (int)s.n_bins ? (int)s.n_bins - 1 : bin);
#pragma unroll
                for (int j = 0; j < 16; ++j) v[j] = j == bin ? 1.0f : 0.0f;
                st.run(r, s.out_begin, v, s.out_width);
            } else {
                encode_slot_scalar(s, d, row, [&](uint32_t col, float v) { st.one(r, col, v); });
            }
        }
    }
}

// One part of one row's encoding, for tiles that TPR threads encode per row: part p takes grid
// levels [p * per, (p + 1) * per) of every grid slot (per = the grid's levels / TPR, rounded up
// to NL), and the last part also the other slots and the grids' padding.  Every column is
// computed exactly as encode_tile_rows computes it.
// The split counts each spherical-harmonics slot, which the last part evaluates, as two grid
// levels (one-hot and identity slots cost next to nothing): the throughput network's 16 levels go
// 10 / 6 between the two threads of a row (its two SH slots on the second), the visibility
// network's 8 levels 5 / 3.
// Measured on the throughput query (2^21, variant 12, one box): 0.630 ms with an even split,
// 0.623 ms.
__host__ __device__ __forceinline__ uint32_t row_part_levels(const ModelDesc& d, uint32_t nlev, int tpr, int nl) {
    uint32_t extra = 0;
    if (tpr > 1)
        for (uint32_t si = 0; si < d.n_slots; ++si)
            if (d.slots[si].type == SLOT_SH) extra += 2u;
    const uint32_t per = (nlev + extra + (uint32_t)tpr - 1) / (uint32_t)tpr;
    const uint32_t r = (per + (uint32_t)nl - 1) / (uint32_t)nl * (uint32_t)nl;
    return r < nlev ? r : nlev;
}

template <int NL, int TPR, typename Store, typename TT>
__device__ __forceinline__ void encode_row_part(const ModelDesc& d, const GridLevel* level_tables, const TT* __restrict__ params,
                                                const float* in_s, uint32_t in_ld, const float* __restrict__ ml_gpu, float ml_scalar,
                                                uint32_t row0, uint32_t r, uint32_t part, Store& st, const uint32_t* smem_tab = nullptr,
                                                uint32_t smem_levels = 0, CellTable ct = {}) {
    const float* row = in_s + r * in_ld;
    const float ml = ml_gpu ? __ldg(ml_gpu + row0 + r) : ml_scalar;
    const bool last = part == (uint32_t)(TPR - 1);
    for (uint32_t si = 0; si < d.n_slots; ++si) {
        const Slot& s = d.slots[si];
        if (s.type == SLOT_GRID) {
            const float px = row[s.in_begin], py = row[s.in_begin + 1], pz = row[s.in_begin + 2];
            const GridDesc& g = d.grids[s.grid];
            const uint32_t nlev = g.n_levels;
            const uint32_t per = row_part_levels(d, nlev, TPR, NL);
            const uint32_t lb = part * per, le = min(nlev, lb + per);
            const TT* table = params + g.param_offset;
            const GridLevel* lv = level_tables + s.grid * kMaxLevels;
#pragma unroll 1
            for (uint32_t l0 = lb; l0 < le; l0 += NL) {
                float f[2 * NL];
                const uint32_t nl = min((uint32_t)NL, le - l0);
                grid_group_forward<NL, TT>(g, lv, l0, nl, table, px, py, pz, ml, f, smem_tab, s.grid == 0 ? smem_levels : 0u,
                                           s.grid == 0 ? ct : CellTable{});
                st.run(r, s.out_begin + 2u * l0, f, 2u * nl);
            }
            if (last && s.n_pad) encode_slot_scalar(s, d, row, [&](uint32_t col, float v) { st.one(r, col, v); });
        } else if (!last) {
            continue;
        } else if (s.type == SLOT_SH && s.degree == 4 && s.n_pad == 0 && (s.out_begin & 1u) == 0) {
            float v[16];
            sh_forward(4u, row[s.in_begin], row[s.in_begin + 1], row[s.in_begin + 2], [&](uint32_t i, float x) { v[i] = x; });
            st.run(r, s.out_begin, v, 16u);
        } else if (s.type == SLOT_ONEHOT && s.out_width <= 16u && (s.out_width & 1u) == 0 && (s.out_begin & 1u) == 0) {
            float v[16];
            int bin = (int)floorf(row[s.in_begin] * (float)s.n_bins);
            bin = bin < 0 ? 0 : (bin >= (int)s.n_bins ? (int)s.n_bins - 1 : bin);
#pragma unroll
            for (int j = 0; j < 16; ++j) v[j] = j == bin ? 1.0f : 0.0f;
            st.run(r, s.out_begin, v, s.out_width);
        } else {
            encode_slot_scalar(s, d, row, [&](uint32_t col, float v) { st.one(r, col, v); });
        }
    }
}

// Encodes `rows` staged input rows (in_s, row stride in_ld) into the consumer's tile; each grid
// unit covers NL levels (NL = 2 or 4).
// Store must provide: run(r, col, const float (&f)[2*NL], n) storing f[0..n) at columns
// col..col+n (col even, n even) and one(r, col, v).
template <int NL, typename Store>
__device__ __forceinline__ void encode_tile(const ModelDesc& d, const float* __restrict__ params, const float* in_s, uint32_t in_ld,
                                            const float* __restrict__ ml_gpu, float ml_scalar, uint32_t row0, uint32_t rows,
                                            uint32_t tid, uint32_t nthreads, Store& st) {
    for (uint32_t si = 0; si < d.n_slots; ++si) {
        const Slot& s = d.slots[si];
        if (s.type != SLOT_GRID) continue;
        const GridDesc& g = d.grids[s.grid];
        const uint32_t ngroups = (g.n_levels + NL - 1u) / NL;
        const float* table = params + g.param_offset;
        for (uint32_t u = tid; u < rows * ngroups; u += nthreads) {
            const uint32_t r = u % rows, grp = u / rows;
            const float* row = in_s + r * in_ld + s.in_begin;
            const float ml = ml_gpu ? __ldg(ml_gpu + row0 + r) : ml_scalar;
            const uint32_t l0 = grp * NL;
            const uint32_t nl = min((uint32_t)NL, g.n_levels - l0);
            float f[2 * NL];
            grid_group_forward<NL>(g, g.levels, l0, nl, table, row[0], row[1], row[2], ml, f);
            st.run(r, s.out_begin + 2u * l0, f, 2u * nl);
        }
    }
    for (uint32_t u = tid; u < rows * d.n_slots; u += nthreads) {
        const uint32_t r = u % rows, si = u / rows;
        const Slot& s = d.slots[si];
        if (s.type == SLOT_GRID && s.n_pad == 0) continue;
        const float* row = in_s + r * in_ld;
        if (s.type == SLOT_SH && s.degree == 4 && s.n_pad == 0 && (s.out_begin & 1u) == 0) {
            // 16 values in registers, stored as whole runs
            float v[16];
            sh_forward(4u, row[s.in_begin], row[s.in_begin + 1], row[s.in_begin + 2], [&](uint32_t i, float x) { v[i] = x; });
            st.run(r, s.out_begin, v, 16u);
            continue;
        }
        if (s.type == SLOT_ONEHOT && s.out_width <= 16u && (s.out_width & 1u) == 0 && (s.out_begin & 1u) == 0) {
            // one-hot bins followed by zero padding, stored as one run
            float v[16];
            int bin = (int)floorf(row[s.in_begin] * (float)s.n_bins);
            bin = bin < 0 ? 0 : (bin >= (int)s.n_bins ? (int)s.n_bins - 1 : bin);
#pragma unroll
            for (int j = 0; j < 16; ++j) v[j] = j == bin ? 1.0f : 0.0f;
            st.run(r, s.out_begin, v, s.out_width);
            continue;
        }
        encode_slot_scalar(s, d, row, [&](uint32_t col, float v) { st.one(r, col, v); });
    }
}

}  // namespace nlod
