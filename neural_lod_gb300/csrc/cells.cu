// Cell table of the FP16 grid tables' dense levels: for every cell (cx, cy, cz) in [0, res)^3 of
// such a level, the FP16 feature pairs of its eight corner entries (corner c = x + 2y + 4z,
// entries exactly as level_corner_entries forms them, wrap-around of the last cells included) in
// one 32-byte record at record L.offset + cx + res (cy + res cz).  grid_group_forward reads a
// cell's corners with two 16-byte loads of one sector instead of four to eight gathers, and gets
// bit-identical features.  Rebuilt whenever the FP16 copy changes (parameter upload, optimizer
// step), so that captured inference reads current records.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "desc.h"
#include "encoding.cuh"
#include "kernels.h"

namespace nlod {
namespace {

__global__ void __launch_bounds__(256) k_build_cells(const __grid_constant__ GridDesc g, const uint32_t* __restrict__ grid_h_words,
                                                     uint4* __restrict__ cells, uint32_t n_levels, uint32_t n_records) {
    for (uint32_t rec = blockIdx.x * blockDim.x + threadIdx.x; rec < n_records; rec += gridDim.x * blockDim.x) {
        // the level whose records hold `rec` (levels are contiguous from record 0)
        uint32_t l = 0;
        while (l + 1 < n_levels && rec >= g.levels[l + 1].offset) ++l;
        const GridLevel& L = g.levels[l];
        const uint32_t res = L.res_flags & kLevelResMask;
        const uint32_t c = rec - L.offset;
        if (c >= res * res * res) continue;   // the level's padding past res^3 records
        const uint32_t cx = c % res, cy = (c / res) % res, cz = c / (res * res);
        uint32_t e[8];
        level_corner_entries(L, 0u, 0u, 0u, cx, cy, cz, e);
        const uint32_t* t = grid_h_words + L.offset;
        uint32_t w[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) w[k] = __ldg(t + e[k]);
        cells[2u * rec] = make_uint4(w[0], w[1], w[2], w[3]);
        cells[2u * rec + 1u] = make_uint4(w[4], w[5], w[6], w[7]);
    }
}

}  // namespace

uint32_t cells_levels_of(const ModelDesc& d) {
    if (d.n_grids == 0) return 0;
    const GridDesc& g = d.grids[0];
    if (g.n_features != 2 || g.interp == INTERP_NEAREST) return 0;
    uint32_t n = 0;
    while (n < g.n_levels) {
        const uint32_t f = g.levels[n].res_flags;
        if ((f & kLevelHashed) || (f >> kLevelDimsShift) != 3u || g.levels[n].offset != (n ? g.levels[n - 1].offset + g.levels[n - 1].size : 0u))
            break;
        const uint64_t res = f & kLevelResMask;
        if (res * res * res > g.levels[n].size) break;
        ++n;
    }
    return n;
}

size_t cells_records(const ModelDesc& d, uint32_t levels) {
    if (levels == 0) return 0;
    const GridLevel& L = d.grids[0].levels[levels - 1];
    return (size_t)L.offset + L.size;
}

cudaError_t launch_build_cells(const ModelDesc& d, const void* grid_h, uint32_t levels, void* cells, cudaStream_t s) {
    const size_t n = cells_records(d, levels);
    if (n == 0) return cudaSuccess;
    const uint32_t blocks = (uint32_t)((n + 255) / 256 < 152u * 8u ? (n + 255) / 256 : 152u * 8u);
    const GridDesc& g = d.grids[0];
    k_build_cells<<<blocks, 256, 0, s>>>(g, reinterpret_cast<const uint32_t*>(static_cast<const __half*>(grid_h) + g.param_offset),
                                         static_cast<uint4*>(cells), levels, (uint32_t)n);
    return cudaGetLastError();
}

}  // namespace nlod
