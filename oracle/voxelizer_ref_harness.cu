// TEST INFRASTRUCTURE ONLY -- never linked into libnlod.so.
//
// Runs the reference voxelizer kernel itself: cuda_voxelizer's voxelize_triangle
// (neural_lod/cuda_voxelizer/src/voxelize.cu:58-190), compiled from its own source as staged by
// oracle/build_ref.py, with the GLM it needs supplied by oracle/glm_shim.  The launch is the one
// voxelize() makes (voxelize.cu:214-228): one thread per triangle, block size from the occupancy
// calculator, the non-Morton bit order.  oracle/build_ref.py builds it twice, with nvcc's default
// contraction of multiply-adds into FMAs (as the reference builds it) and with -fmad=false.
#include "voxelize.cu"

#include <cstdint>

extern "C" {

// voxinfo's unit for a bounding box and grid (util.h:58-63).
void vref_unit(const float bbox_min[3], const float bbox_max[3], uint32_t grid, float unit[3]) {
    AABox<glm::vec3> box(glm::vec3(bbox_min[0], bbox_min[1], bbox_min[2]), glm::vec3(bbox_max[0], bbox_max[1], bbox_max[2]));
    voxinfo info(box, glm::uvec3(grid, grid, grid), 0);
    unit[0] = info.unit.x;
    unit[1] = info.unit.y;
    unit[2] = info.unit.z;
}

// ORs the voxels of n triangles (device float [n][9]) into the device bit grid `table`
// (grid^3 bits, most significant bit first).  Returns a cudaError_t.
int vref_voxelize(const float* triangles, uint64_t n, uint32_t grid, const float bbox_min[3], const float bbox_max[3],
                  uint32_t* table, void* stream) {
    AABox<glm::vec3> box(glm::vec3(bbox_min[0], bbox_min[1], bbox_min[2]), glm::vec3(bbox_max[0], bbox_max[1], bbox_max[2]));
    voxinfo info(box, glm::uvec3(grid, grid, grid), (size_t)n);
    int block = 0, min_grid = 0;
    cudaError_t e = cudaOccupancyMaxPotentialBlockSize(&min_grid, &block, voxelize_triangle, 0, 0);
    if (e != cudaSuccess) return (int)e;
    if (n == 0) return 0;
    const int blocks = (int)((n + block - 1) / block);
    voxelize_triangle<<<blocks, block, 0, (cudaStream_t)stream>>>(info, const_cast<float*>(triangles), table, false);
    return (int)cudaGetLastError();
}

}  // extern "C"
