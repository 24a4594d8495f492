// Conservative surface voxelization and mesh bounds (voxelize.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace nlod {

// Voxel frame of one voxelization: cube bbox minimum, voxel size per axis, voxels per axis.
struct VoxFrame {
    float bmin[3];
    float unit[3];
    uint32_t grid;
};

// Triangles whose candidate box holds more voxels than this are tested by a whole warp.
constexpr uint32_t kVoxSmallDefault = 24;

// ORs the conservative surface voxels of n triangles (9 floats each) into bits (grid^3 bits,
// bit x + y*grid + z*grid^2, most significant bit first per word).
cudaError_t launch_voxelize(const float* tris, uint64_t n, const VoxFrame& f, uint32_t* bits, uint32_t small_limit, cudaStream_t s);

// Per-axis min / max over all triangle vertices, as order-preserving uint32 keys in
// keys[0..2] (min, initialised to 0xFFFFFFFF) and keys[3..5] (max, initialised to 0).
cudaError_t launch_mesh_bounds(const float* tris, uint64_t n, uint32_t* keys, cudaStream_t s);

// Host inverse of the order-preserving key.
inline float bounds_key_to_float(uint32_t k) {
    const uint32_t u = (k & 0x80000000u) ? (k & 0x7FFFFFFFu) : ~k;
    float f;
    __builtin_memcpy(&f, &u, sizeof f);
    return f;
}

}  // namespace nlod
