// C ABI of the conservative surface voxelizer (include/nlod.h).
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>

#include "abi_util.h"
#include "nlod.h"
#include "vox.h"

using namespace nlod;

namespace {

float fmax_glm(float a, float b) { return (a < b) ? b : a; }

void check_grid(uint32_t grid) {
    if (grid == 0 || grid > 4096) throw Error(NLOD_ERR_INVALID, "grid must be in [1, 4096] voxels per axis");
}

}  // namespace

extern "C" {

int nlod_mesh_frame(const float mesh_min[3], const float mesh_max[3], uint32_t grid, float epsilon_padding, float bbox_min[3],
                    float bbox_max[3], float unit[3]) {
    return guarded([&] {
        if (!mesh_min || !mesh_max || !bbox_min || !bbox_max || !unit) throw Error(NLOD_ERR_INVALID, "pointers must not be NULL");
        check_grid(grid);
        // createMeshBBCube (cuda_voxelizer/src/util.h:87-112)
        float len[3], mn[3], mx[3];
        for (int i = 0; i < 3; ++i) {
            len[i] = mesh_max[i] - mesh_min[i];
            mn[i] = mesh_min[i];
            mx[i] = mesh_max[i];
        }
        const float max_len = fmax_glm(len[0], fmax_glm(len[1], len[2]));
        for (int i = 0; i < 3; ++i) {
            if (max_len == len[i]) continue;
            const float delta = max_len - len[i];
            mn[i] = mesh_min[i] - delta / 2.0f;
            mx[i] = mesh_max[i] + delta / 2.0f;
        }
        if (epsilon_padding != 0.f) {
            float e[3];
            for (int i = 0; i < 3; ++i) e[i] = (mx[i] - mn[i]) * epsilon_padding;
            for (int i = 0; i < 3; ++i) {
                mn[i] -= e[i];
                mx[i] += e[i];
            }
        }
        // voxinfo (util.h:58-63)
        for (int i = 0; i < 3; ++i) {
            bbox_min[i] = mn[i];
            bbox_max[i] = mx[i];
            unit[i] = (mx[i] - mn[i]) / (float)grid;
        }
        if (!(unit[0] > 0.f && unit[1] > 0.f && unit[2] > 0.f)) throw Error(NLOD_ERR_INVALID, "the mesh has zero extent");
    });
}

int nlod_mesh_bounds(const float* triangles, uint64_t n_triangles, void* stream, float mesh_min[3], float mesh_max[3]) {
    return guarded([&] {
        if (!triangles || !mesh_min || !mesh_max) throw Error(NLOD_ERR_INVALID, "pointers must not be NULL");
        if (n_triangles == 0) throw Error(NLOD_ERR_INVALID, "the mesh has no triangles");
        cudaStream_t s = (cudaStream_t)stream;
        uint32_t init[6] = {0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0u, 0u, 0u}, keys[6];
        uint32_t* d = dev_alloc<uint32_t>(6);
        try {
            cuda_check(cudaMemcpyAsync(d, init, sizeof init, cudaMemcpyHostToDevice, s), "copy");
            cuda_check(launch_mesh_bounds(triangles, n_triangles, d, s), "mesh bounds");
            cuda_check(cudaMemcpyAsync(keys, d, sizeof keys, cudaMemcpyDeviceToHost, s), "copy");
            cuda_check(cudaStreamSynchronize(s), "mesh bounds");
        } catch (...) {
            dev_free(d);
            throw;
        }
        dev_free(d);
        for (int i = 0; i < 3; ++i) {
            mesh_min[i] = bounds_key_to_float(keys[i]);
            mesh_max[i] = bounds_key_to_float(keys[3 + i]);
        }
    });
}

int nlod_voxelize(const float* triangles, uint64_t n_triangles, uint32_t grid, const float bbox_min[3], const float unit[3],
                  uint32_t* bits, void* stream) {
    return guarded([&] {
        if (!bbox_min || !unit) throw Error(NLOD_ERR_INVALID, "bbox_min and unit must not be NULL");
        check_grid(grid);
        if (n_triangles == 0) return;
        if (!triangles || !bits) throw Error(NLOD_ERR_INVALID, "triangle and bit buffers must not be NULL");
        if (n_triangles > (UINT64_MAX / 36)) throw Error(NLOD_ERR_INVALID, "too many triangles");
        VoxFrame f;
        for (int i = 0; i < 3; ++i) {
            if (!(unit[i] > 0.f)) throw Error(NLOD_ERR_INVALID, "voxel size must be positive");
            f.bmin[i] = bbox_min[i];
            f.unit[i] = unit[i];
        }
        f.grid = grid;
        cuda_check(launch_voxelize(triangles, n_triangles, f, bits, kVoxSmallDefault, (cudaStream_t)stream), "voxelize");
    });
}

}  // extern "C"
