// Device-side input encodings: multiresolution hash/dense grid, spherical harmonics,
// identity and one-hot, evaluated per (element, encoding part).  Semantics follow
// tiny-cuda-nn (paths relative to rptr/ext/tiny-cuda-nn/include/tiny-cuda-nn/):
//   grid index / hashes       encodings/grid.h:111-187
//   pos_fract (+0.5 offset)   common_device.h:437-464
//   forward interpolation     encodings/grid.h:220-392
//   backward scatter          encodings/grid.h:394-517
//   max-level masking         encodings/grid.h:242-265, 413-424
//   spherical harmonics       encodings/spherical_harmonics.h:46-151 (input mapped by 2x-1,
//                             padding written first as 1.0)
//   identity                  encodings/identity.h:45-66 (padding written last as 1.0)
#pragma once

#include <cstdint>

#include "desc.h"

namespace nlod {

// ---- hashing (grid.h:111-187) --------------------------------------------------------------

__device__ __forceinline__ uint32_t grid_hash3(int32_t kind, uint32_t x, uint32_t y, uint32_t z) {
    // XOR of coordinate * prime; the coherent variant keeps x unscrambled (prime 1).
    if (kind == HASH_COHERENT_PRIME) return x ^ (y * 2654435761u) ^ (z * 805459861u);
    if (kind == HASH_PRIME) return (x * 1958374283u) ^ (y * 2654435761u) ^ (z * 805459861u);
    return (x * 2165219737u) ^ (y * 1434869437u) ^ (z * 2097192037u);  // reversed primes
}

// Table entry of integer grid vertex (x, y, z) within one level: dense row-major index while the
// running stride fits the level's table, else the spatial hash; always taken modulo the level
// size.  uint32 wrap-around is part of the definition.
__device__ __forceinline__ uint32_t grid_entry(const GridDesc& g, const GridLevel& L, uint32_t x, uint32_t y, uint32_t z) {
    const uint32_t size = L.size;
    uint32_t stride = 1, index = 0;
    // dims 0..2, stopping once the stride exceeds the table (avoids overflow at fine levels)
    if (stride <= size) { index += x * stride; stride *= L.res; }
    if (stride <= size) { index += y * stride; stride *= L.res; }
    if (stride <= size) { index += z * stride; stride *= L.res; }
    if (g.kind == GRID_HASH && size < stride) index = grid_hash3(g.hash, x, y, z);
    return (size & (size - 1)) == 0 ? (index & (size - 1)) : (index % size);
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

// Trilinear (or nearest) interpolation of the two features of one level.
// table points at the grid's first float; returns the 2 interpolated features.
__device__ __forceinline__ float2 grid_level_forward(const GridDesc& g, uint32_t level, const float* __restrict__ table,
                                                     float px, float py, float pz) {
    const GridLevel L = g.levels[level];
    const float2* __restrict__ lv = reinterpret_cast<const float2*>(table) + L.offset;
    float fx, fy, fz;
    uint32_t cx, cy, cz;
    grid_pos_fract(px, L.scale, fx, cx);
    grid_pos_fract(py, L.scale, fy, cy);
    grid_pos_fract(pz, L.scale, fz, cz);
    if (g.interp == INTERP_NEAREST) {
        return __ldg(lv + grid_entry(g, L, cx, cy, cz));
    }
    fx = interp_weight_fun(g.interp, fx);
    fy = interp_weight_fun(g.interp, fy);
    fz = interp_weight_fun(g.interp, fz);
    // Issue all 8 gathers before using any of them.
    float2 v[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        v[c] = __ldg(lv + grid_entry(g, L, cx + (c & 1), cy + ((c >> 1) & 1), cz + ((c >> 2) & 1)));
    }
    float2 r = make_float2(0.f, 0.f);
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        float w = 1.0f;
        w *= (c & 1) ? fx : 1.0f - fx;
        w *= (c & 2) ? fy : 1.0f - fy;
        w *= (c & 4) ? fz : 1.0f - fz;
        r.x = fmaf(w, v[c].x, r.x);
        r.y = fmaf(w, v[c].y, r.y);
    }
    return r;
}

// Scatter dL/d(features) of one level into the FP32 gradient table (grid.h:394-517).
// Adjacent lanes that hit the same entry are merged before the atomic (warp aggregation),
// which matters on the coarse levels where whole warps share a handful of vertices.
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
    if (g.interp == INTERP_NEAREST) {
        if (active) {
            uint32_t e = grid_entry(g, L, cx, cy, cz);
            atomicAdd(reinterpret_cast<float2*>(lv + e), dy);
        }
        return;
    }
    fx = interp_weight_fun(g.interp, fx);
    fy = interp_weight_fun(g.interp, fy);
    fz = interp_weight_fun(g.interp, fz);
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        float w = 1.0f;
        w *= (c & 1) ? fx : 1.0f - fx;
        w *= (c & 2) ? fy : 1.0f - fy;
        w *= (c & 4) ? fz : 1.0f - fz;
        const uint32_t e = active ? grid_entry(g, L, cx + (c & 1), cy + ((c >> 1) & 1), cz + ((c >> 2) & 1)) : 0xFFFFFFFFu;
        float2 v = make_float2(active ? w * dy.x : 0.f, active ? w * dy.y : 0.f);
        // Lanes with equal entries form a group; the lowest lane of a group sums the group.
        const unsigned peers = __match_any_sync(full, e);
        const int lane = threadIdx.x & 31;
        const int leader = __ffs(peers) - 1;
        if (__popc(peers) > 1) {
            // Sum within the group by walking its members (groups are small except on coarse levels).
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
        if (active && lane == leader) atomicAdd(reinterpret_cast<float2*>(lv + e), v);
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

// ---- encoding parts ------------------------------------------------------------------------
// The encoded row is produced as a list of "parts": one per grid level and one per non-grid
// slot.  A part writes a fixed set of columns, so parts can be spread over threads.

// Evaluates one part for one element.  `row` is the element's input row, `put(col, value)` stores
// one encoded feature.  Padding columns of the slot are written by the part of its first level
// (or by the slot's single part).
template <typename Put>
__device__ __forceinline__ void encode_part(const ModelDesc& d, const float* __restrict__ params, uint32_t slot_idx,
                                            uint32_t level, const float* __restrict__ row, float max_level_frac, Put&& put) {
    const Slot& s = d.slots[slot_idx];
    switch (s.type) {
        case SLOT_GRID: {
            const GridDesc& g = d.grids[s.grid];
            const uint32_t nf = g.n_levels * 2u;
            if (level == 0) {
                for (uint32_t p = 0; p < s.n_pad; ++p) put(s.out_begin + nf + p, 0.0f);
            }
            float2 r = make_float2(0.f, 0.f);
            if (!grid_level_masked(level, max_level_frac, g.n_levels)) {
                r = grid_level_forward(g, level, params + g.param_offset, row[s.in_begin], row[s.in_begin + 1], row[s.in_begin + 2]);
            }
            put(s.out_begin + 2 * level, r.x);
            put(s.out_begin + 2 * level + 1, r.y);
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

}  // namespace nlod
