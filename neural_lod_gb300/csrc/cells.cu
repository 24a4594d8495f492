// Cell table of the FP16 grid tables' leading levels (dense or hashed): for every cell
// (cx, cy, cz) in [0, res)^3 of such a level, the FP16 feature pairs of its eight corner entries
// (corner c = x + 2y + 4z, entries exactly as level_corner_entries forms them: the dense index
// with its wrap-around, or the spatial hash) in one 32-byte record at record
// base[l] + cx + res (cy + res cz).  grid_group_forward reads a cell's corners with two 16-byte
// loads of one sector instead of four to eight gathers, and gets bit-identical features.  Rebuilt whenever the FP16 copy changes (parameter upload, optimizer
// step), so that captured inference reads current records.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "desc.h"
#include "encoding.cuh"
#include "kernels.h"

namespace nlod {
namespace {

// Cell records the table may hold per level, and in all: a level of res^3 cells costs 32 res^3
// bytes (up to res = 128); the table holds the leading levels that fit both.
constexpr uint64_t kMaxLevelRecords = 2u << 20;
constexpr uint64_t kMaxRecords = 3u << 20;

struct CellBases {
    uint32_t base[kMaxLevels + 1];
};

__global__ void __launch_bounds__(256) k_build_cells(const __grid_constant__ GridDesc g, const __grid_constant__ CellBases cb,
                                                     const uint32_t* __restrict__ grid_h_words, uint4* __restrict__ cells,
                                                     uint32_t n_levels) {
    uint32_t p0, p1, p2;
    hash_primes(g.hash, p0, p1, p2);
    const uint32_t n_records = cb.base[n_levels];
    for (uint32_t rec = blockIdx.x * blockDim.x + threadIdx.x; rec < n_records; rec += gridDim.x * blockDim.x) {
        uint32_t l = 0;
        while (l + 1 < n_levels && rec >= cb.base[l + 1]) ++l;
        const GridLevel& L = g.levels[l];
        const uint32_t res = L.res_flags & kLevelResMask;
        const uint32_t c = rec - cb.base[l];
        const uint32_t cx = c % res, cy = (c / res) % res, cz = c / (res * res);
        uint32_t e[8];
        level_corner_entries(L, p0, p1, p2, cx, cy, cz, e);
        const uint32_t* t = grid_h_words + L.offset;
        uint32_t w[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) w[k] = __ldg(t + e[k]);
        cells[2u * rec] = make_uint4(w[0], w[1], w[2], w[3]);
        cells[2u * rec + 1u] = make_uint4(w[4], w[5], w[6], w[7]);
    }
}

}  // namespace

uint32_t cells_levels_of(const ModelDesc& d, uint32_t (&base)[kMaxLevels + 1]) {
    for (uint32_t& b : base) b = 0;
    if (d.n_grids == 0) return 0;
    const GridDesc& g = d.grids[0];
    if (g.n_features != 2 || g.interp == INTERP_NEAREST) return 0;
    uint32_t n = 0;
    uint64_t total = 0;
    while (n < g.n_levels) {
        const uint32_t f = g.levels[n].res_flags;
        if (!(f & kLevelHashed) && (f >> kLevelDimsShift) != 3u) break;   // a dense level of fewer dims
        const uint64_t res = f & kLevelResMask;
        const uint64_t recs = res * res * res;
        if (recs > kMaxLevelRecords || total + recs > kMaxRecords) break;
        total += recs;
        ++n;
        base[n] = (uint32_t)total;
    }
    return n;
}

cudaError_t launch_build_cells(const ModelDesc& d, const void* grid_h, uint32_t levels, const uint32_t (&base)[kMaxLevels + 1], void* cells,
                               cudaStream_t s) {
    if (levels == 0 || base[levels] == 0) return cudaSuccess;
    CellBases cb;
    for (uint32_t i = 0; i <= kMaxLevels; ++i) cb.base[i] = base[i];
    const uint32_t n = base[levels];
    const uint32_t blocks = (n + 255) / 256 < 152u * 8u ? (n + 255) / 256 : 152u * 8u;
    const GridDesc& g = d.grids[0];
    k_build_cells<<<blocks, 256, 0, s>>>(g, cb, reinterpret_cast<const uint32_t*>(static_cast<const __half*>(grid_h) + g.param_offset),
                                         static_cast<uint4*>(cells), levels);
    return cudaGetLastError();
}

}  // namespace nlod
