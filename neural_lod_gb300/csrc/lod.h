// LoD occupancy pyramid + first-active-voxel search (lod.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

namespace nlod {

constexpr int kMaxLodLevels = 12;

// One pyramid level as the search kernel sees it (device pointers).
struct LodLevelDev {
    int32_t res;                 // voxels per axis
    int32_t n_active;
    int32_t bbox_min[3];         // tight inclusive bbox of active voxels
    int32_t bbox_max[3];
    const uint32_t* bits;        // occupancy, bit x + y*res + z*res^2, MSB first per word
    const uint8_t* leaf;         // [ceil(res/8)]^3 leaf-node flags
    const uint8_t* lower;        // [ceil(res/128)]^3 lower-node flags
};

cudaError_t launch_downsample(const uint32_t* src, int32_t src_res, uint32_t* dst, int32_t dst_res, cudaStream_t s);
// stats: [count, min x, min y, min z, max x, max y, max z] (initialised by the caller to 0, INT_MAX x3, -1 x3)
cudaError_t launch_level_flags(const uint32_t* bits, int32_t res, uint8_t* leaf, uint8_t* lower, int32_t* stats, cudaStream_t s);
cudaError_t launch_first_active_voxel(const LodLevelDev& L, uint32_t n, const float* eye, const float* dir, const float* t_min,
                                      const int32_t* prev, int32_t* hit, int32_t* ijk, float* t_near, float* t_far,
                                      uint32_t* status, cudaStream_t s);

}  // namespace nlod

// The C ABI's pyramid object (include/nlod.h): one LodLevelDev per level plus owned buffers.
struct nlod_lod_grid {
    uint32_t n_levels = 0;
    int32_t res0 = 0;
    nlod::LodLevelDev levels[nlod::kMaxLodLevels]{};
    uint32_t n_leaves[nlod::kMaxLodLevels]{};
    std::vector<void*> owned;
    uint32_t* status = nullptr;
};
