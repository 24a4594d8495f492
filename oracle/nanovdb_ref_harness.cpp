// Harness that runs the reference's first-active-voxel search on the reference's own NanoVDB
// grids -- TEST INFRASTRUCTURE ONLY (built by oracle/build_ref.py into oracle/_ref/, used by
// tests/golden/make_dda_golden.py to produce golden vectors).
//
// Grids are built exactly as rptr/cuda/neural-lod/neural_lod_learning_init.cu:194-267 builds the LoD
// pyramid: nanovdb::GridBuilder<float>(0, VoxelVolume), setValue((x,y,z) >> lod, 0.5) for every
// active level-0 voxel, getHandle<AbsDiff>.  The search is the loop of
// first_active_voxel_intersection (rptr/cuda/neural-lod/neural_lod_learning_common.cuh:783-832):
// nanovdb::TreeMarcher over leaf nodes, nanovdb::DDA inside each leaf span, voxels outside the leaf
// skipped, first active voxel other than the previous one accepted after an AABB slab test
// (neural_lod_learning_common.cuh:567-606), restated here without glm.  The index-space ray is
// nanovdb::Ray(eye, dir, t_min) as raymarch_impl builds it (rptr/cuda/wavefront_neural_pt.cuh:111-118).
//
// Input file (little endian): uint32 res, n_levels, n_rays; uint32 level-0 occupancy words
// (bit x + y*res + z*res*res, most significant bit first); per ray int32 lod, float eye[3],
// float dir[3], float t_min, int32 prev[3].
// Output file: per level int32 bbox_min[3], bbox_max[3], uint32 n_leaves, n_active; per ray
// int32 hit, ijk[3], float t_near, t_far.
#include <nanovdb/NanoVDB.h>
#include <nanovdb/util/GridBuilder.h>
#include <nanovdb/util/HDDA.h>
#include <nanovdb/util/Ray.h>

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <vector>

namespace {

bool slab_test(const nanovdb::Vec3f& o, const nanovdb::Vec3f& d, const nanovdb::Coord& ijk, float& near_t, float& far_t) {
    near_t = -1e20f;
    far_t = 1e20f;
    for (int i = 0; i < 3; ++i) {
        const float inv = 1.f / d[i];
        const float lo = (float)ijk[i];
        const float hi = lo + 1.0f;
        if (d[i] == 0) {
            if (o[i] < lo || o[i] > hi) return false;
        } else {
            float t1 = (lo - o[i]) * inv;
            float t2 = (hi - o[i]) * inv;
            if (t1 > t2) { float tmp = t1; t1 = t2; t2 = tmp; }
            near_t = (t1 < near_t) ? near_t : t1;   // std::max(t1, near_t)
            far_t = (far_t < t2) ? far_t : t2;      // std::min(t2, far_t)
            if (!(near_t < far_t) || far_t < 0.0) return false;
        }
    }
    return true;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc != 3) {
        std::fprintf(stderr, "usage: %s input.bin output.bin\n", argv[0]);
        return 2;
    }
    FILE* f = std::fopen(argv[1], "rb");
    if (!f) return 3;
    uint32_t hdr[3];
    if (std::fread(hdr, 4, 3, f) != 3) return 4;
    const uint32_t res = hdr[0], n_levels = hdr[1], n_rays = hdr[2];
    const uint64_t n_bits = (uint64_t)res * res * res;
    std::vector<uint32_t> bits((n_bits + 31) / 32);
    if (std::fread(bits.data(), 4, bits.size(), f) != bits.size()) return 5;
    struct RayIn { int32_t lod; float eye[3], dir[3], tmin; int32_t prev[3]; };
    std::vector<RayIn> rays(n_rays);
    if (n_rays && std::fread(rays.data(), sizeof(RayIn), n_rays, f) != n_rays) return 6;
    std::fclose(f);

    using GridT = nanovdb::FloatGrid;
    std::vector<nanovdb::GridHandle<nanovdb::HostBuffer>> handles;
    std::vector<uint32_t> counts(n_levels, 0);
    for (uint32_t lod = 0; lod < n_levels; ++lod) {
        nanovdb::GridBuilder<float> builder(0.0f, nanovdb::GridClass::VoxelVolume);
        auto acc = builder.getAccessor();
        for (uint64_t idx = 0; idx < n_bits; ++idx) {
            if (!((bits[idx >> 5] >> (31 - (idx & 31))) & 1u)) continue;
            const uint32_t x = idx % res, y = (idx / res) % res, z = idx / ((uint64_t)res * res);
            acc.setValue(nanovdb::Coord(x >> lod, y >> lod, z >> lod), 0.5f);
        }
        handles.push_back(builder.getHandle<nanovdb::AbsDiff>(1.0, nanovdb::Vec3d(0.0)));
    }

    FILE* o = std::fopen(argv[2], "wb");
    if (!o) return 7;
    for (uint32_t lod = 0; lod < n_levels; ++lod) {
        const GridT* grid = handles[lod].grid<float>();
        const auto bb = grid->tree().root().bbox();
        const int32_t b[6] = {bb.min()[0], bb.min()[1], bb.min()[2], bb.max()[0], bb.max()[1], bb.max()[2]};
        const uint32_t c[2] = {(uint32_t)grid->tree().nodeCount(0), (uint32_t)grid->activeVoxelCount()};
        std::fwrite(b, 4, 6, o);
        std::fwrite(c, 4, 2, o);
    }
    for (const RayIn& r : rays) {
        const GridT* grid = handles[r.lod].grid<float>();
        auto acc = grid->tree().getAccessor();
        using RayT = nanovdb::Ray<float>;
        RayT ray(nanovdb::Vec3f(r.eye[0], r.eye[1], r.eye[2]), nanovdb::Vec3f(r.dir[0], r.dir[1], r.dir[2]), 0.0f);
        if (r.tmin != 0.0f) ray.setMinTime(r.tmin);
        const nanovdb::Coord prev(r.prev[0], r.prev[1], r.prev[2]);
        int32_t out_i[4] = {0, 0, 0, 0};
        float out_t[2] = {0.f, 0.f};
        nanovdb::TreeMarcher<GridT::TreeType::LeafNodeType, RayT, decltype(acc)> marcher(acc);
        bool done = false;
        if (marcher.init(ray)) {
            const GridT::TreeType::LeafNodeType* node = nullptr;
            float t0 = 0, t1 = 0;
            while (!done && marcher.step(&node, t0, t1)) {
                nanovdb::DDA<RayT> dda;
                dda.init(marcher.ray(), t0, t1);
                do {
                    const nanovdb::Coord ijk = dda.voxel();
                    const auto local = ijk - node->origin();
                    if (local[0] < 0 || local[1] < 0 || local[2] < 0 || local[0] >= 8 || local[1] >= 8 || local[2] >= 8) continue;
                    if (node->isActive(node->CoordToOffset(ijk)) && ijk != prev) {
                        float tn, tf;
                        if (slab_test(marcher.ray().eye(), marcher.ray().dir(), ijk, tn, tf)) {
                            out_i[0] = 1;
                            out_i[1] = ijk[0];
                            out_i[2] = ijk[1];
                            out_i[3] = ijk[2];
                            out_t[0] = tn;
                            out_t[1] = tf;
                            done = true;
                            break;
                        }
                    }
                } while (dda.step());
            }
        }
        std::fwrite(out_i, 4, 4, o);
        std::fwrite(out_t, 4, 2, o);
    }
    std::fclose(o);
    return 0;
}
