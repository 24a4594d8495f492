// C ABI of the LoD occupancy pyramid and the first-active-voxel search (include/nlod.h).
#include <cuda_runtime.h>

#include <climits>
#include <cstdint>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "abi_util.h"
#include "lod.h"
#include "nlod.h"

using namespace nlod;

extern "C" {

void nlod_lod_grid_destroy(nlod_lod_grid* g) {
    if (!g) return;
    cudaDeviceSynchronize();
    for (void* p : g->owned) dev_free(p);
    dev_free(g->status);
    delete g;
}

int nlod_lod_grid_create(const uint32_t* level0_bits, uint32_t res, uint32_t n_levels, void* stream, nlod_lod_grid** out) {
    return guarded([&] {
        if (!out) throw Error(NLOD_ERR_INVALID, "out must not be NULL");
        *out = nullptr;
        if (!level0_bits) throw Error(NLOD_ERR_INVALID, "level-0 occupancy must not be NULL");
        if (res == 0 || res > 4096 || (res & (res - 1)) != 0) throw Error(NLOD_ERR_INVALID, "resolution must be a power of two in [1, 4096]");
        if (n_levels == 0 || n_levels > (uint32_t)kMaxLodLevels || (res >> (n_levels - 1)) == 0)
            throw Error(NLOD_ERR_INVALID, "n_levels must be in [1, 12] and keep at least one voxel per axis");
        cudaStream_t s = (cudaStream_t)stream;
        std::unique_ptr<nlod_lod_grid> g(new nlod_lod_grid());
        try {
            g->n_levels = n_levels;
            g->res0 = (int32_t)res;
            g->status = dev_alloc<uint32_t>(1);
            cuda_check(cudaMemsetAsync(g->status, 0, sizeof(uint32_t), s), "memset");
            std::vector<int32_t*> stats(n_levels);
            int32_t* stat_buf = dev_alloc<int32_t>(7 * (size_t)n_levels);
            g->owned.push_back(stat_buf);
            const int32_t init[7] = {0, INT_MAX, INT_MAX, INT_MAX, -1, -1, -1};
            std::vector<int32_t> host_init(7 * (size_t)n_levels);
            for (uint32_t l = 0; l < n_levels; ++l) std::memcpy(&host_init[7 * l], init, sizeof init);
            cuda_check(cudaMemcpyAsync(stat_buf, host_init.data(), sizeof(int32_t) * host_init.size(), cudaMemcpyHostToDevice, s), "copy");
            for (uint32_t l = 0; l < n_levels; ++l) {
                const int32_t r = (int32_t)(res >> l);
                const uint64_t nbits = (uint64_t)r * r * r;
                const int32_t nb = (r + 7) / 8, nl = (r + 127) / 128;
                uint32_t* bits = dev_alloc<uint32_t>((size_t)((nbits + 31) / 32));
                g->owned.push_back(bits);
                uint8_t* leaf = dev_alloc<uint8_t>((size_t)nb * nb * nb);
                g->owned.push_back(leaf);
                uint8_t* lower = dev_alloc<uint8_t>((size_t)nl * nl * nl);
                g->owned.push_back(lower);
                if (l == 0) {
                    cuda_check(cudaMemcpyAsync(bits, level0_bits, sizeof(uint32_t) * (size_t)((nbits + 31) / 32), cudaMemcpyDeviceToDevice, s), "copy");
                } else {
                    cuda_check(launch_downsample(g->levels[l - 1].bits, g->levels[l - 1].res, bits, r, s), "downsample");
                }
                cuda_check(launch_level_flags(bits, r, leaf, lower, stat_buf + 7 * l, s), "level flags");
                LodLevelDev& L = g->levels[l];
                L.res = r;
                L.bits = bits;
                L.leaf = leaf;
                L.lower = lower;
            }
            std::vector<int32_t> st(7 * (size_t)n_levels);
            cuda_check(cudaMemcpyAsync(st.data(), stat_buf, sizeof(int32_t) * st.size(), cudaMemcpyDeviceToHost, s), "copy");
            cuda_check(cudaStreamSynchronize(s), "pyramid build");
            for (uint32_t l = 0; l < n_levels; ++l) {
                LodLevelDev& L = g->levels[l];
                L.n_active = st[7 * l];
                for (int k = 0; k < 3; ++k) {
                    L.bbox_min[k] = L.n_active ? st[7 * l + 1 + k] : 0;
                    L.bbox_max[k] = L.n_active ? st[7 * l + 4 + k] : -1;
                }
                // leaf count
                const int32_t nb = (L.res + 7) / 8;
                std::vector<uint8_t> lf((size_t)nb * nb * nb);
                cuda_check(cudaMemcpy(lf.data(), L.leaf, lf.size(), cudaMemcpyDeviceToHost), "copy");
                uint32_t c = 0;
                for (uint8_t v : lf) c += v;
                g->n_leaves[l] = c;
            }
        } catch (...) {
            nlod_lod_grid_destroy(g.release());
            throw;
        }
        *out = g.release();
    });
}

int nlod_lod_grid_level_info(const nlod_lod_grid* g, uint32_t level, int32_t* res, int32_t* n_active, int32_t* bbox6, uint32_t* n_leaves) {
    return guarded([&] {
        if (!g) throw Error(NLOD_ERR_INVALID, "grid is NULL");
        if (level >= g->n_levels) throw Error(NLOD_ERR_INVALID, "level out of range");
        const LodLevelDev& L = g->levels[level];
        if (res) *res = L.res;
        if (n_active) *n_active = L.n_active;
        if (bbox6) {
            for (int k = 0; k < 3; ++k) {
                bbox6[k] = L.bbox_min[k];
                bbox6[3 + k] = L.bbox_max[k];
            }
        }
        if (n_leaves) *n_leaves = g->n_leaves[level];
    });
}

const uint32_t* nlod_lod_grid_level_bits(const nlod_lod_grid* g, uint32_t level) {
    if (!g || level >= g->n_levels) return nullptr;
    return g->levels[level].bits;
}

int nlod_lod_grid_copy_bits(const nlod_lod_grid* g, uint32_t level, uint32_t* host_dst) {
    return guarded([&] {
        if (!g || !host_dst) throw Error(NLOD_ERR_INVALID, "grid and destination must not be NULL");
        if (level >= g->n_levels) throw Error(NLOD_ERR_INVALID, "level out of range");
        const uint64_t r = (uint64_t)g->levels[level].res;
        cuda_check(cudaDeviceSynchronize(), "synchronize");
        cuda_check(cudaMemcpy(host_dst, g->levels[level].bits, sizeof(uint32_t) * (size_t)((r * r * r + 31) / 32), cudaMemcpyDeviceToHost),
                   "copy bits");
    });
}

int nlod_first_active_voxel(const nlod_lod_grid* g, uint32_t level, void* stream, uint32_t n, const float* origin, const float* dir,
                            const float* t_min, const int32_t* prev, int32_t* hit, int32_t* ijk, float* t_near, float* t_far) {
    return guarded([&] {
        if (!g) throw Error(NLOD_ERR_INVALID, "grid is NULL");
        if (level >= g->n_levels) throw Error(NLOD_ERR_INVALID, "level out of range");
        if (n == 0) return;
        if (!origin || !dir || !hit || !ijk || !t_near || !t_far) throw Error(NLOD_ERR_INVALID, "ray and result buffers must not be NULL");
        cuda_check(launch_first_active_voxel(g->levels[level], n, origin, dir, t_min, prev, hit, ijk, t_near, t_far, g->status,
                                             (cudaStream_t)stream), "first active voxel");
    });
}

int nlod_lod_grid_sync_status(nlod_lod_grid* g, void* stream) {
    return guarded([&] {
        if (!g) throw Error(NLOD_ERR_INVALID, "grid is NULL");
        uint32_t st = 0;
        cuda_check(cudaStreamSynchronize((cudaStream_t)stream), "synchronize");
        cuda_check(cudaMemcpy(&st, g->status, sizeof st, cudaMemcpyDeviceToHost), "status");
        if (st) {
            cuda_check(cudaMemset(g->status, 0, sizeof st), "status");
            throw Error(NLOD_ERR_TIMEOUT, "a ray exceeded its traversal step budget");
        }
    });
}

}  // extern "C"
