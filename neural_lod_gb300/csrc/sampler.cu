// Training-sample generation on the GPU: the reference's sampler restated, with exact-DDA
// stand-ins for its Vulkan ray queries.
//
//   nlod_morton_voxels      sorted Morton codes of the set voxels of a bit grid: the reference's
//                           morton_sparse_voxel_idx_mapping (std::set of encode_morton3 codes,
//                           sorted; rptr/cuda/neural-lod/neural_lod_learning_init.cu:201-294)
//   nlod_sample_visibility  fill_ray_queries_visibility (neural_lod_learning_kernels.cuh:364-569):
//                           voxel + LoD (sample_voxel, sample_discrete_lods with
//                           shifted_square_pdf, :29-98), direction wi, dilated-cube rejection
//                           sampling of the chord (pi, po), optional boundary-density rejection,
//                           the deterministic pi/po order (neural_lod_learning_common.cuh:255-308);
//                           per-voxel mode of the threshold optimisation (:392-421)
//   nlod_sample_throughput  fill_ray_queries_throughput (:100-238)
//   nlod_trace_visibility   stand-in for main_visibility_optimisation (rptr/vulkan/raygen.rgen:
//                           695-730): the query ray's first occupied level-0 voxel, occluded (1)
//                           when its entry point lies inside the query box, else 0
//   nlod_trace_throughput   stand-in for the throughput ray query (raygen.rgen:505-687) and
//                           record_ray_query_results_throughput_optim (kernels.cuh:240-278): the
//                           query ray must hit an occupied voxel inside the box (else the sample
//                           is invalid: every input and target -1); wi uniform on the sphere;
//                           target = per-voxel albedo x (1 if the ray from the hit point along wi
//                           leaves the box unoccluded, else 0)
//   nlod_compact_samples    copy_valid_results_throughput_optim (:280-318) in a stable order, with
//                           the reference's count rule (next multiple of 128 below the count)
//
// Every loop the reference leaves unbounded (rejection sampling) is bounded by max_attempts; a
// sample that exhausts it is marked invalid (t_max = -1 in its query, inputs -1).  This unit is
// built with -fmad=false: its float and double expressions are the uncontracted, correctly
// rounded operations of the host restatement, which therefore draws identical samples.
#include <cuda_runtime.h>

#include <cfloat>
#include <cmath>
#include <cstdint>

#include "abi_util.h"
#include "lod.h"
#include "lod_dda.cuh"
#include "nlod.h"

namespace nlod {
namespace {

constexpr uint32_t kBlock = 256;
constexpr uint32_t kItemsPerThread = 16;
constexpr uint32_t kItemsPerBlock = kBlock * kItemsPerThread;
constexpr uint32_t kDdaBudget = 1u << 16;
constexpr uint32_t kMaxLods = 16;

// ---- Morton codes (encode_morton3 / decode_morton3, neural_lod_learning.h:519-580) ----------

__device__ inline uint32_t compact1by2(uint32_t x) {
    x &= 0x09249249u;
    x = (x ^ (x >> 2)) & 0x030c30c3u;
    x = (x ^ (x >> 4)) & 0x0300f00fu;
    x = (x ^ (x >> 8)) & 0xff0000ffu;
    x = (x ^ (x >> 16)) & 0x000003ffu;
    return x;
}

__device__ inline bool bit_set(const uint32_t* bits, uint32_t res, uint32_t x, uint32_t y, uint32_t z) {
    const uint64_t idx = (uint64_t)x + (uint64_t)res * ((uint64_t)y + (uint64_t)res * z);
    return (bits[idx >> 5] >> (31u - (uint32_t)(idx & 31u))) & 1u;
}

// ---- RNG: LCG seeded by MurmurHash3 mixing (rptr/rendering/pointsets/lcg_rng.glsl, hashing.glsl) --

__device__ inline uint32_t murmur_mix(uint32_t h, uint32_t k) {
    k *= 0xcc9e2d51u;
    k = (k << 15) | (k >> 17);
    k *= 0x1b873593u;
    h ^= k;
    h = ((h << 13) | (h >> 19)) * 5u + 0xe6546b64u;
    return h;
}
__device__ inline uint32_t murmur_fin(uint32_t h) {
    h ^= h >> 16;
    h *= 0x85ebca6bu;
    h ^= h >> 13;
    h *= 0xc2b2ae35u;
    h ^= h >> 16;
    return h;
}
struct Lcg {
    uint32_t s;
    __device__ float next() {
        s = s * 1664525u + 1013904223u;
        return __uint2float_rn(s) * 2.3283064365386962890625e-10f;   // ldexp(float(s), -32)
    }
};
__device__ inline Lcg lcg_rng(uint32_t index, uint32_t frame, uint32_t linear) {
    uint32_t s = murmur_mix(frame, linear);
    s = murmur_mix(s, index);
    return Lcg{murmur_fin(s)};
}

// ---- cos and sin of a float angle in [0, 2pi]: reduction by the nearest multiple of pi/2 and
// the Taylor series of sin and cos about 0 (nested form, terms to r^17 / r^16; truncation below
// 1e-17 for |r| <= pi/4), evaluated in double and rounded to float once.

__device__ inline void cos_sin(float phi, float& c_out, float& s_out) {
    const double d = (double)phi;
    const double q = floor(d * 0.63661977236758134 + 0.5);
    const double r = d - q * 1.5707963267948966;
    const double r2 = r * r;
    // (reciprocals folded at compile time: multiplications only, FP64 division is slow here)
    double t = 1.0 - r2 * (1.0 / 272.0);
    t = 1.0 - r2 * (1.0 / 210.0) * t;
    t = 1.0 - r2 * (1.0 / 156.0) * t;
    t = 1.0 - r2 * (1.0 / 110.0) * t;
    t = 1.0 - r2 * (1.0 / 72.0) * t;
    t = 1.0 - r2 * (1.0 / 42.0) * t;
    t = 1.0 - r2 * (1.0 / 20.0) * t;
    const double sr = r * (1.0 - r2 * (1.0 / 6.0) * t);
    double u = 1.0 - r2 * (1.0 / 240.0);
    u = 1.0 - r2 * (1.0 / 182.0) * u;
    u = 1.0 - r2 * (1.0 / 132.0) * u;
    u = 1.0 - r2 * (1.0 / 90.0) * u;
    u = 1.0 - r2 * (1.0 / 56.0) * u;
    u = 1.0 - r2 * (1.0 / 30.0) * u;
    u = 1.0 - r2 * (1.0 / 12.0) * u;
    const double cr = 1.0 - r2 * 0.5 * u;
    const int m = ((int)q) & 3;
    const double c = m == 0 ? cr : m == 1 ? -sr : m == 2 ? -cr : sr;
    const double s = m == 0 ? sr : m == 1 ? cr : m == 2 ? -sr : -cr;
    c_out = (float)c;
    s_out = (float)s;
}

// square_to_uniform_sphere (neural_lod_learning_common.cuh:48-54)
__device__ inline void uniform_sphere(float u1, float u2, float (&w)[3]) {
    const float phi = (float)(6.283185307179586 * (double)u1);   // 2.0f * M_PI * rng.x
    const float cos_theta = u2 * 2.0f - 1.0f;
    const float sin_theta = sqrtf(1.0f - cos_theta * cos_theta);
    float c, s;
    cos_sin(phi, c, s);
    w[0] = sin_theta * c;
    w[1] = sin_theta * s;
    w[2] = cos_theta;
}

__device__ inline float min3(float a, float b, float c) {
    const float m = b < a ? b : a;   // glm::min(a, b) = b < a ? b : a
    return c < m ? c : m;
}

// intersect_aabb(_min_max) (neural_lod_learning_common.cuh:567-619), box centred at 0.
__device__ inline bool intersect_box0(const float (&o)[3], const float (&d)[3], float extent, float& near_t, float& far_t) {
    const float h = 0.5f * extent;
    const float lo = 0.0f - h, hi = 0.0f + h;
    near_t = -1e20f;
    far_t = 1e20f;
    for (int i = 0; i < 3; ++i) {
        const float inv = 1.f / d[i];
        if (d[i] == 0.f) {
            if (o[i] < lo || o[i] > hi) return false;
        } else {
            float t1 = (lo - o[i]) * inv, t2 = (hi - o[i]) * inv;
            if (t1 > t2) { const float t = t1; t1 = t2; t2 = t; }
            near_t = t1 < near_t ? near_t : t1;   // std::max(t1, near)
            far_t = far_t < t2 ? far_t : t2;      // std::min(t2, far)
            if (!(near_t < far_t) || (double)far_t < 0.0) return false;
        }
    }
    return true;
}

// sample_discrete_lods with shifted_square_pdf (kernels.cuh:33-70): the first LoD whose
// normalised CDF (double) exceeds the float sample; a sample no entry exceeds (sample == 1) takes
// the last LoD.  The host turns each CDF entry c into the smallest float >= c, so that
// `sample < c` is the float comparison `sample < bound` (LodBounds).
struct LodBounds {
    float b[kMaxLods];
};
__device__ inline uint32_t sample_lod(float sample, const LodBounds& lb, uint32_t n_lods) {
    for (uint32_t l = 0; l < n_lods; ++l)
        if (sample < lb.b[l]) return l;
    return n_lods - 1;
}

LodBounds lod_bounds(const nlod_sampler_params& p) {
    double cdf[kMaxLods];
    for (uint32_t l = 0; l < p.n_lods; ++l) {
        const float x = (float)l / (float)p.n_lods + p.pdf_shift - 0.5f + 0.0625f;
        const float pdf = (float)(1.0 + (double)(p.pdf_strength * x * x));
        cdf[l] = l == 0 ? (double)pdf : cdf[l - 1] + (double)pdf;
    }
    LodBounds lb{};
    for (uint32_t l = 0; l < p.n_lods; ++l) {
        const double c = cdf[l] / cdf[p.n_lods - 1];
        float f = (float)c;
        if ((double)f < c) f = std::nextafter(f, INFINITY);
        lb.b[l] = f;
    }
    return lb;
}

struct Voxel {
    float center[3];
    float extent;
};

// compute_lod_voxel (neural_lod_learning_grid.cuh:50-74)
__device__ inline Voxel lod_voxel(const nlod_sampler_params& p, uint32_t x, uint32_t y, uint32_t z, uint32_t lod) {
    const float step = ldexpf(p.voxel_size, (int)lod);
    const uint32_t v[3] = {x, y, z};
    Voxel vx;
    for (int k = 0; k < 3; ++k) {
        const float vmin = p.aabb_min[k] + (float)v[k] * step;
        vx.center[k] = vmin + step * 0.5f;
    }
    vx.extent = step;
    return vx;
}

// sample_voxel (kernels.cuh:72-98)
__device__ inline Voxel pick_voxel(Lcg& rng, const nlod_sampler_params& p, const LodBounds& lb, const uint32_t* morton, uint32_t n_voxels,
                                   uint32_t& lod) {
    const uint32_t sparse_idx = (uint32_t)(rng.next() * (float)n_voxels) % n_voxels;
    const uint32_t code = morton[sparse_idx];
    lod = sample_lod(rng.next(), lb, p.n_lods);
    return lod_voxel(p, compact1by2(code) >> lod, compact1by2(code >> 1) >> lod, compact1by2(code >> 2) >> lod, lod);
}

// The dilation of the cube the chord is drawn on (kernels.cuh:164-176, 457-474).
__device__ inline float sample_dilation(Lcg& rng, const nlod_sampler_params& p) {
    if (rng.next() < p.dilation_outward / (p.dilation_inward + p.dilation_outward))
        return rng.next() * (p.dilation_outward - p.min_dilation) + p.min_dilation;
    return -(rng.next() * (p.dilation_inward - p.min_dilation) + p.min_dilation);
}

// The plane basis perpendicular to w (kernels.cuh:146-163): u from the smallest |component| of -w.
__device__ inline void perp_basis(const float (&w)[3], float (&u)[3], float (&v)[3]) {
    const float m = min3(fabsf(-w[0]), fabsf(-w[1]), fabsf(-w[2]));
    u[0] = u[1] = u[2] = 0.f;
    if (fabsf(-w[0]) == m) {
        u[1] = w[2];
        u[2] = -w[1];
    } else if (fabsf(-w[1]) == m) {
        u[0] = -w[2];
        u[2] = w[0];
    } else {
        u[0] = -w[1];
        u[1] = w[0];
    }
    // glm::cross(w, u)
    v[0] = w[1] * u[2] - u[1] * w[2];
    v[1] = w[2] * u[0] - u[2] * w[0];
    v[2] = w[0] * u[1] - u[0] * w[1];
}

// One rejection-sampled ray of the orthographic camera at w * dist towards the cube of edge
// 1 + dil centred at 0; its entry / exit points (kernels.cuh:185-205, 478-496).
__device__ inline bool chord(Lcg& rng, const float (&w)[3], const float (&u)[3], const float (&v)[3], float dist, float dil,
                             uint32_t max_attempts, float (&a)[3], float (&b)[3]) {
    const float dir[3] = {-w[0], -w[1], -w[2]};
    for (uint32_t t = 0; t < max_attempts; ++t) {
        const float r0 = rng.next();
        const float r1 = rng.next();
        const float ox = (r0 - 0.5f) * dist, oy = (r1 - 0.5f) * dist;
        float o[3];
        for (int k = 0; k < 3; ++k) o[k] = w[k] * dist + u[k] * ox + v[k] * oy;
        float tn, tf;
        if (intersect_box0(o, dir, 1.0f + dil, tn, tf)) {
            for (int k = 0; k < 3; ++k) {
                a[k] = o[k] + dir[k] * tn;
                b[k] = o[k] + dir[k] * tf;
            }
            return true;
        }
    }
    return false;
}

// Cube face of a point on the cube (largest |component|, first wins; + side 2i, - side 2i+1).
__device__ inline int cube_face(const float (&q)[3]) {
    float largest = -2e20f;
    int face = 0;
    for (int i = 0; i < 3; ++i) {
        const float dd = fabsf(q[i]);
        if (dd > largest) {
            face = (double)q[i] > 0.0 ? 2 * i : 2 * i + 1;
            largest = dd;
        }
    }
    return face;
}

// get_deterministic_local_pi_po: pi is the point on the lower-numbered face (the reference's
// table of the 15 face pairs in increasing order).  Equal faces (a tangent chord) keep the order.
__device__ inline bool pi_first(const float (&a)[3], const float (&b)[3]) {
    const int fa = cube_face(a), fb = cube_face(b);
    return !(fb < fa);
}

__device__ inline void mark_invalid(float* in, uint32_t n_in, nlod_ray_query& q) {
    for (uint32_t k = 0; k < n_in; ++k) in[k] = -1.f;
    q.t_max = -1.f;
}

__device__ inline void normalise_input(const nlod_sampler_params& p, const float (&w)[3], float* out) {
    for (int k = 0; k < 3; ++k) out[k] = (w[k] - p.aabb_min[k]) / (p.aabb_max[k] - p.aabb_min[k]);
}

// Body of fill_ray_queries_visibility after the voxel is chosen.
__device__ void visibility_sample(Lcg& rng, const nlod_sampler_params& p, const Voxel& vx, float* in, nlod_ray_query& q) {
    const float dist = 2.f * (1.f + p.dilation_outward);
    float wi[3];
    {
        const float u1 = rng.next();
        const float u2 = rng.next();
        uniform_sphere(u1, u2, wi);
    }
    float pu[3], pv[3];
    perp_basis(wi, pu, pv);
    float a[3], b[3], dil = 0.f;
    bool done = false;
    for (uint32_t attempt = 0; attempt < p.max_attempts && !done; ++attempt) {
        dil = sample_dilation(rng, p);
        if (!chord(rng, wi, pu, pv, dist, dil, p.max_attempts, a, b)) break;
        if (p.increase_boundary_density) {
            float md[3];
            for (int k = 0; k < 3; ++k) md[k] = 0.5f * (a[k] + b[k]) / (1.0f + dil);
            const float umd = min3(fabsf(md[0]), fabsf(md[1]), fabsf(md[2])) * 2.0f;
            if (rng.next() < umd * 1.5f + 0.1f) done = true;
        } else {
            done = true;
        }
    }
    if (!done) {
        mark_invalid(in, 6, q);
        return;
    }
    const bool keep = pi_first(a, b);
    float lpi[3], lpo[3], pi[3], po[3];
    for (int k = 0; k < 3; ++k) {
        lpi[k] = keep ? a[k] : b[k];
        lpo[k] = keep ? b[k] : a[k];
        pi[k] = vx.center[k] + lpi[k] * vx.extent;
        po[k] = vx.center[k] + lpo[k] * vx.extent;
    }
    float d[3];
    for (int k = 0; k < 3; ++k) d[k] = lpo[k] - lpi[k];
    const float isq = 1.0f / sqrtf(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);   // glm::normalize
    for (int k = 0; k < 3; ++k) {
        q.origin[k] = vx.center[k] + lpi[k] * vx.extent;
        q.dir[k] = d[k] * isq;
        q.voxel_center[k] = vx.center[k];
    }
    q.voxel_extent = vx.extent * (1.f + (dil < p.bound_bias ? p.bound_bias : dil));
    q.t_max = 1e20f;
    q.mode_or_data = 0;
    normalise_input(p, pi, in);
    normalise_input(p, po, in + 3);
}

__global__ void __launch_bounds__(kBlock) k_sample_visibility(nlod_sampler_params p, LodBounds lb, const uint32_t* __restrict__ morton,
                                                               const uint32_t* __restrict__ n_voxels_dev, uint32_t batch_index,
                                                               uint32_t n, float* __restrict__ input, nlod_ray_query* __restrict__ queries,
                                                               uint32_t* __restrict__ lod_out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t n_voxels = *n_voxels_dev;
    float* in = input + (size_t)i * 6;
    nlod_ray_query q{};
    Lcg rng = lcg_rng(batch_index * n, 0u, i);
    uint32_t lod = 0;
    if (n_voxels == 0) {
        mark_invalid(in, 6, q);
    } else {
        const Voxel vx = pick_voxel(rng, p, lb, morton, n_voxels, lod);
        visibility_sample(rng, p, vx, in, q);
    }
    if (queries) queries[i] = q;
    if (lod_out) lod_out[i] = lod;
}

// Threshold-optimisation mode (kernels.cuh:392-413): sample s of voxel first + v of a LoD's own
// sorted mapping, i = s + v * n_samples, RNG stream (first + v, 0, s).
__global__ void __launch_bounds__(kBlock) k_sample_visibility_voxels(nlod_sampler_params p, const uint32_t* __restrict__ lod_morton,
                                                                      uint32_t first, uint32_t n_voxels, uint32_t n_samples, uint32_t lod,
                                                                      float* __restrict__ input, nlod_ray_query* __restrict__ queries) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_samples * n_voxels) return;
    const uint32_t s = i % n_samples, v = (i / n_samples) % n_voxels;
    Lcg rng = lcg_rng(first + v, 0u, s);
    const uint32_t code = lod_morton[first + v];
    const Voxel vx = lod_voxel(p, compact1by2(code), compact1by2(code >> 1), compact1by2(code >> 2), lod);
    nlod_ray_query q{};
    visibility_sample(rng, p, vx, input + (size_t)i * 6, q);
    if (queries) queries[i] = q;
}

__global__ void __launch_bounds__(kBlock) k_sample_throughput(nlod_sampler_params p, LodBounds lb, const uint32_t* __restrict__ morton,
                                                               const uint32_t* __restrict__ n_voxels_dev, uint32_t batch_index,
                                                               uint32_t n, int32_t max_orders, float* __restrict__ input,
                                                               nlod_ray_query* __restrict__ queries, uint32_t* __restrict__ lod_out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t n_voxels = *n_voxels_dev;
    float* in = input + (size_t)i * 9;
    nlod_ray_query q{};
    uint32_t lod = 0;
    Lcg rng = lcg_rng(batch_index * n, 0u, i);
    bool ok = n_voxels > 0;
    Voxel vx{};
    float wo[3] = {0.f, 0.f, 0.f}, a[3], b[3], dil = 0.f;
    if (ok) {
        vx = pick_voxel(rng, p, lb, morton, n_voxels, lod);
        const float dist = 2.f * (1.f + p.dilation_outward);
        const float u1 = rng.next();
        const float u2 = rng.next();
        uniform_sphere(u1, u2, wo);
        float pu[3], pv[3];
        perp_basis(wo, pu, pv);
        dil = sample_dilation(rng, p);
        ok = chord(rng, wo, pu, pv, dist, dil, p.max_attempts, a, b);
    }
    if (!ok) {
        mark_invalid(in, 9, q);
    } else {
        for (int k = 0; k < 3; ++k) {
            q.origin[k] = vx.center[k] + a[k] * vx.extent;
            q.dir[k] = -wo[k];
            q.voxel_center[k] = vx.center[k];
        }
        q.voxel_extent = vx.extent * (1.f + (dil < p.bound_bias ? p.bound_bias : dil));
        q.t_max = 1e20f;
        q.mode_or_data = max_orders;
        normalise_input(p, vx.center, in);
        for (int k = 0; k < 3; ++k) in[3 + k] = (wo[k] + 1.0f) * 0.5f;
        for (int k = 6; k < 9; ++k) in[k] = 0.f;   // wi: written by the trace
    }
    if (queries) queries[i] = q;
    if (lod_out) lod_out[i] = lod;
}

// ---- exact-DDA stand-ins for the ray queries -------------------------------------------------

struct Frame {
    float E[3], D[3];     // index-space ray
    float c[3], h;        // index-space box centre and half edge
};

__device__ inline Frame to_index(const nlod_sampler_params& p, const nlod_ray_query& q) {
    Frame f;
    for (int k = 0; k < 3; ++k) {
        f.E[k] = (q.origin[k] - p.aabb_min[k]) / p.voxel_size;
        f.D[k] = q.dir[k];
        f.c[k] = (q.voxel_center[k] - p.aabb_min[k]) / p.voxel_size;
    }
    f.h = q.voxel_extent * 0.5f / p.voxel_size;
    return f;
}

// Exit parameter of the ray (E, D) from the box c +- h (the ray starts inside or on it).
__device__ inline float box_exit(const float (&E)[3], const float (&D)[3], const float (&c)[3], float h) {
    float t = FLT_MAX;
    for (int k = 0; k < 3; ++k) {
        if (D[k] == 0.f) continue;
        const float bound = D[k] > 0.f ? c[k] + h : c[k] - h;
        const float tk = (bound - E[k]) / D[k];
        t = tk < t ? tk : t;
    }
    return t < 0.f ? 0.f : t;
}

__device__ inline bool inside_box(const float (&P)[3], const float (&c)[3], float h) {
    return !(fabsf(P[0] - c[0]) > h || fabsf(P[1] - c[1]) > h || fabsf(P[2] - c[2]) > h);
}

// The first occupied level-0 voxel along the ray within the box; its entry point (clamped to the
// ray origin) must lie inside the box.  Returns 1 (hit), 0 (none), -1 (step budget exhausted).
__device__ inline int first_hit_in_box(const LodLevelDev& L, const float (&E)[3], const float (&D)[3], const float (&c)[3], float h,
                                       const int32_t (&prev)[3], int32_t (&v)[3], float (&P)[3]) {
    const float t_exit = box_exit(E, D, c, h);
    float tn, tf;
    const int r = dda::first_active_voxel(L, E, D, 0.f, prev, v, tn, tf, kDdaBudget, t_exit);
    if (r != 1) return r;
    const float t = tn < 0.f ? 0.f : tn;
    for (int k = 0; k < 3; ++k) P[k] = E[k] + t * D[k];
    return inside_box(P, c, h) ? 1 : 0;
}

__global__ void __launch_bounds__(128) k_trace_visibility(LodLevelDev L, nlod_sampler_params p, const nlod_ray_query* __restrict__ queries,
                                                          uint32_t n, float* __restrict__ target, uint32_t* __restrict__ status) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const nlod_ray_query q = queries[i];
    if (q.t_max < 0.f) {
        target[i] = -1.f;
        return;
    }
    const Frame f = to_index(p, q);
    const int32_t none[3] = {-1, -1, -1};
    int32_t v[3];
    float P[3];
    const int r = first_hit_in_box(L, f.E, f.D, f.c, f.h, none, v, P);
    if (r < 0) atomicOr(status, 1u);
    target[i] = r == 1 ? 1.f : 0.f;
}

// Per-voxel albedo in [0.1, 0.9]^3 (the synthetic scene's material).
__device__ inline float voxel_albedo(const int32_t (&v)[3], uint32_t ch) {
    uint32_t h = murmur_mix(0x9e3779b9u, (uint32_t)v[0]);
    h = murmur_mix(h, (uint32_t)v[1]);
    h = murmur_mix(h, (uint32_t)v[2]);
    h = murmur_fin(h + ch);
    return 0.1f + 0.8f * ((float)(h >> 8) * 5.9604644775390625e-08f);
}

__global__ void __launch_bounds__(128) k_trace_throughput(LodLevelDev L, nlod_sampler_params p, const nlod_ray_query* __restrict__ queries,
                                                          uint32_t n, uint32_t batch_index, int log_learning, float* __restrict__ input,
                                                          float* __restrict__ target, uint32_t* __restrict__ n_invalid,
                                                          uint32_t* __restrict__ status) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const nlod_ray_query q = queries[i];
    float* in = input + (size_t)i * 9;
    float* tg = target + (size_t)i * 3;
    bool valid = q.t_max >= 0.f;
    int32_t v[3];
    float P[3];
    Frame f{};
    if (valid) {
        f = to_index(p, q);
        const int32_t none[3] = {-1, -1, -1};
        const int r = first_hit_in_box(L, f.E, f.D, f.c, f.h, none, v, P);
        if (r < 0) atomicOr(status, 1u);
        valid = r == 1;
    }
    if (!valid) {
        for (int k = 0; k < 9; ++k) in[k] = -1.f;
        for (int k = 0; k < 3; ++k) tg[k] = -1.f;
        if (n_invalid) atomicAdd(n_invalid, 1u);
        return;
    }
    Lcg rng = lcg_rng(batch_index * n, 1u, i);
    float wi[3];
    {
        const float u1 = rng.next();
        const float u2 = rng.next();
        uniform_sphere(u1, u2, wi);
    }
    int32_t v2[3];
    float P2[3];
    const int r2 = first_hit_in_box(L, P, wi, f.c, f.h, v, v2, P2);
    if (r2 < 0) atomicOr(status, 1u);
    const float vis = r2 == 1 ? 0.f : 1.f;
    for (int k = 0; k < 3; ++k) {
        float t = voxel_albedo(v, (uint32_t)k) * vis;
        if (log_learning) t = logf(1.f + t);
        tg[k] = t;
        in[6 + k] = (wi[k] + 1.0f) * 0.5f;
    }
}

// ---- order-preserving selection: per-block counts, one scan, per-block writes -----------------

struct MortonSel {
    const uint32_t* bits;
    uint32_t res;
    __device__ bool keep(uint64_t code) const {
        const uint32_t c = (uint32_t)code;
        return bit_set(bits, res, compact1by2(c), compact1by2(c >> 1), compact1by2(c >> 2));
    }
};
struct ValidSel {
    const float* target;
    uint32_t n_out;
    __device__ bool keep(uint64_t i) const { return target[i * n_out] != -1.f; }
};

template <typename Sel>
__global__ void __launch_bounds__(kBlock) k_count(Sel sel, uint64_t n, uint32_t* __restrict__ block_counts) {
    __shared__ uint32_t warp_sum[kBlock / 32];
    const uint64_t base = (uint64_t)blockIdx.x * kItemsPerBlock;
    uint32_t c = 0;
    for (uint32_t j = 0; j < kItemsPerThread; ++j) {
        const uint64_t i = base + (uint64_t)j * kBlock + threadIdx.x;
        if (i < n && sel.keep(i)) ++c;
    }
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0) warp_sum[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t t = 0;
        for (uint32_t w = 0; w < kBlock / 32; ++w) t += warp_sum[w];
        block_counts[blockIdx.x] = t;
    }
}

// Exclusive scan of the block counts in place (one CTA), total into *total.
__global__ void __launch_bounds__(1024) k_scan(uint32_t* __restrict__ counts, uint32_t nb, uint32_t* __restrict__ total) {
    __shared__ uint32_t s[1024];
    __shared__ uint32_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (uint32_t base = 0; base < nb; base += 1024) {
        const uint32_t i = base + threadIdx.x;
        const uint32_t v = i < nb ? counts[i] : 0u;
        s[threadIdx.x] = v;
        __syncthreads();
        for (uint32_t o = 1; o < 1024; o <<= 1) {
            const uint32_t add = threadIdx.x >= o ? s[threadIdx.x - o] : 0u;
            __syncthreads();
            s[threadIdx.x] += add;
            __syncthreads();
        }
        if (i < nb) counts[i] = carry + s[threadIdx.x] - v;
        __syncthreads();
        if (threadIdx.x == 1023) carry += s[1023];
        __syncthreads();
    }
    if (threadIdx.x == 0) *total = carry;
}

// Writes the kept items of each block in order: out_index(rank, item).  Items whose global rank
// is >= limit (read from device memory when limit_dev is set) are dropped.
template <typename Sel, typename Out>
__global__ void __launch_bounds__(kBlock) k_write(Sel sel, uint64_t n, const uint32_t* __restrict__ offsets,
                                                  const uint32_t* __restrict__ limit_dev, uint32_t limit, Out out) {
    __shared__ uint32_t warp_base[kBlock / 32 + 1];
    const uint64_t base = (uint64_t)blockIdx.x * kItemsPerBlock;
    const uint32_t lim = limit_dev ? *limit_dev : limit;
    uint32_t run = offsets[blockIdx.x];
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (uint32_t j = 0; j < kItemsPerThread; ++j) {
        const uint64_t i = base + (uint64_t)j * kBlock + threadIdx.x;
        const bool k = i < n && sel.keep(i);
        const uint32_t m = __ballot_sync(0xffffffffu, k);
        if (lane == 0) warp_base[warp] = __popc(m);
        __syncthreads();
        if (threadIdx.x == 0) {
            uint32_t t = 0;
            for (uint32_t w = 0; w < kBlock / 32; ++w) {
                const uint32_t c = warp_base[w];
                warp_base[w] = t;
                t += c;
            }
            warp_base[kBlock / 32] = t;
        }
        __syncthreads();
        const uint32_t rank = run + warp_base[warp] + __popc(m & ((1u << lane) - 1u));
        if (k && rank < lim) out(rank, i);
        run += warp_base[kBlock / 32];
        __syncthreads();
    }
}

struct MortonOut {
    uint32_t* codes;
    __device__ void operator()(uint32_t rank, uint64_t code) const { codes[rank] = (uint32_t)code; }
};
struct SampleOut {
    const float* in;
    const float* tg;
    float* vin;
    float* vtg;
    uint32_t n_in, n_out;
    __device__ void operator()(uint32_t rank, uint64_t i) const {
        for (uint32_t k = 0; k < n_in; ++k) vin[(size_t)rank * n_in + k] = in[i * n_in + k];
        for (uint32_t k = 0; k < n_out; ++k) vtg[(size_t)rank * n_out + k] = tg[i * n_out + k];
    }
};

// count -> the reference's training-batch size: next_multiple(count, 128) - 128 (0 if none).
__global__ void k_batch_rule(const uint32_t* __restrict__ total, uint32_t* __restrict__ n_valid) {
    const uint32_t c = *total;
    const uint32_t up = (c + 127u) / 128u * 128u;
    *n_valid = up >= 128u ? up - 128u : 0u;
}

void check_params(const nlod_sampler_params* p) {
    if (!p) throw Error(NLOD_ERR_INVALID, "sampler parameters must not be NULL");
    if (p->n_lods == 0 || p->n_lods > kMaxLods) throw Error(NLOD_ERR_INVALID, "n_lods must be in [1, 16]");
    if (!(p->voxel_size > 0.f)) throw Error(NLOD_ERR_INVALID, "voxel_size must be positive");
    if (p->max_attempts == 0) throw Error(NLOD_ERR_INVALID, "max_attempts must be positive");
    for (int k = 0; k < 3; ++k)
        if (!(p->aabb_max[k] > p->aabb_min[k])) throw Error(NLOD_ERR_INVALID, "empty AABB");
}

uint32_t* scratch(size_t n, cudaStream_t s) {
    void* ptr = nullptr;
    cuda_check(cudaMallocAsync(&ptr, n * sizeof(uint32_t), s), "workspace");
    return static_cast<uint32_t*>(ptr);
}

template <typename Sel, typename Out>
void select_ordered(Sel sel, uint64_t n, Out out, uint32_t* total_dev, uint32_t* limited_dev, uint32_t limit, bool batch_rule,
                    cudaStream_t s) {
    const uint64_t nb64 = (n + kItemsPerBlock - 1) / kItemsPerBlock;
    if (nb64 == 0 || nb64 > 0x7FFFFFFFull) throw Error(NLOD_ERR_INVALID, "selection size out of range");
    const uint32_t nb = (uint32_t)nb64;
    uint32_t* counts = scratch(nb, s);
    k_count<Sel><<<nb, kBlock, 0, s>>>(sel, n, counts);
    k_scan<<<1, 1024, 0, s>>>(counts, nb, total_dev);
    if (batch_rule) k_batch_rule<<<1, 1, 0, s>>>(total_dev, limited_dev);
    k_write<Sel, Out><<<nb, kBlock, 0, s>>>(sel, n, counts, batch_rule ? limited_dev : nullptr, limit, out);
    cuda_check(cudaGetLastError(), "selection");
    cuda_check(cudaFreeAsync(counts, s), "workspace");
}

}  // namespace
}  // namespace nlod

using namespace nlod;

extern "C" int nlod_morton_voxels(const uint32_t* bits, uint32_t res, uint32_t* codes, uint32_t capacity, uint32_t* count,
                                  void* stream) {
    return guarded([&] {
        if (!bits || !count) throw Error(NLOD_ERR_INVALID, "bits and count must not be NULL");
        if (res == 0 || res > 1024 || (res & (res - 1)) != 0) throw Error(NLOD_ERR_INVALID, "res must be a power of two <= 1024");
        cudaStream_t s = (cudaStream_t)stream;
        const uint64_t n = (uint64_t)res * res * res;
        uint32_t* sink = codes;
        if (!sink) capacity = 0;
        MortonSel sel{bits, res};
        select_ordered(sel, n, MortonOut{sink}, count, nullptr, capacity, false, s);
    });
}

extern "C" int nlod_sample_visibility(const nlod_sampler_params* p, const uint32_t* morton, const uint32_t* n_voxels,
                                      uint32_t batch_index, uint32_t n, float* input, nlod_ray_query* queries, uint32_t* lod,
                                      void* stream) {
    return guarded([&] {
        check_params(p);
        if (n == 0) return;
        if (!morton || !n_voxels || !input) throw Error(NLOD_ERR_INVALID, "morton, n_voxels and input must not be NULL");
        k_sample_visibility<<<(n + kBlock - 1) / kBlock, kBlock, 0, (cudaStream_t)stream>>>(*p, lod_bounds(*p), morton, n_voxels, batch_index,
                                                                                             n, input, queries, lod);
        cuda_check(cudaGetLastError(), "visibility samples");
    });
}

extern "C" int nlod_sample_visibility_voxels(const nlod_sampler_params* p, const uint32_t* lod_morton, uint32_t first_voxel,
                                             uint32_t n_voxels, uint32_t n_samples, uint32_t lod, float* input, nlod_ray_query* queries,
                                             void* stream) {
    return guarded([&] {
        check_params(p);
        if (n_voxels == 0 || n_samples == 0) return;
        if (!lod_morton || !input) throw Error(NLOD_ERR_INVALID, "lod_morton and input must not be NULL");
        if (lod >= p->n_lods) throw Error(NLOD_ERR_INVALID, "lod out of range");
        const uint64_t total = (uint64_t)n_voxels * n_samples;
        if (total > 0xFFFFFFFFull) throw Error(NLOD_ERR_INVALID, "too many samples");
        k_sample_visibility_voxels<<<(uint32_t)((total + kBlock - 1) / kBlock), kBlock, 0, (cudaStream_t)stream>>>(
            *p, lod_morton, first_voxel, n_voxels, n_samples, lod, input, queries);
        cuda_check(cudaGetLastError(), "visibility samples");
    });
}

extern "C" int nlod_sample_throughput(const nlod_sampler_params* p, const uint32_t* morton, const uint32_t* n_voxels,
                                      uint32_t batch_index, uint32_t n, int32_t max_orders, float* input, nlod_ray_query* queries,
                                      uint32_t* lod, void* stream) {
    return guarded([&] {
        check_params(p);
        if (n == 0) return;
        if (!morton || !n_voxels || !input) throw Error(NLOD_ERR_INVALID, "morton, n_voxels and input must not be NULL");
        k_sample_throughput<<<(n + kBlock - 1) / kBlock, kBlock, 0, (cudaStream_t)stream>>>(*p, lod_bounds(*p), morton, n_voxels,
                                                                                             batch_index, n, max_orders, input, queries, lod);
        cuda_check(cudaGetLastError(), "throughput samples");
    });
}

static const LodLevelDev& level0(const nlod_lod_grid* g, const nlod_sampler_params* p) {
    if (!g || g->n_levels == 0) throw Error(NLOD_ERR_INVALID, "grid must not be NULL");
    if ((uint32_t)g->res0 != p->grid_res) throw Error(NLOD_ERR_INVALID, "grid resolution differs from the sampler's grid_res");
    return g->levels[0];
}

extern "C" int nlod_trace_visibility(const nlod_lod_grid* g, const nlod_sampler_params* p, const nlod_ray_query* queries, uint32_t n,
                                     float* target, void* stream) {
    return guarded([&] {
        check_params(p);
        const LodLevelDev& L = level0(g, p);
        if (n == 0) return;
        if (!queries || !target) throw Error(NLOD_ERR_INVALID, "queries and target must not be NULL");
        k_trace_visibility<<<(n + 127) / 128, 128, 0, (cudaStream_t)stream>>>(L, *p, queries, n, target, g->status);
        cuda_check(cudaGetLastError(), "visibility trace");
    });
}

extern "C" int nlod_trace_throughput(const nlod_lod_grid* g, const nlod_sampler_params* p, const nlod_ray_query* queries, uint32_t n,
                                     uint32_t batch_index, int log_learning, float* input, float* target, uint32_t* n_invalid,
                                     void* stream) {
    return guarded([&] {
        check_params(p);
        const LodLevelDev& L = level0(g, p);
        if (n == 0) return;
        if (!queries || !input || !target) throw Error(NLOD_ERR_INVALID, "queries, input and target must not be NULL");
        k_trace_throughput<<<(n + 127) / 128, 128, 0, (cudaStream_t)stream>>>(L, *p, queries, n, batch_index, log_learning, input, target,
                                                                              n_invalid, g->status);
        cuda_check(cudaGetLastError(), "throughput trace");
    });
}

extern "C" int nlod_compact_samples(const float* input, const float* target, uint32_t n, uint32_t n_in, uint32_t n_out, float* valid_input,
                                    float* valid_target, uint32_t* n_valid, void* stream) {
    return guarded([&] {
        if (!n_valid) throw Error(NLOD_ERR_INVALID, "n_valid must not be NULL");
        if (n_in == 0 || n_out == 0) throw Error(NLOD_ERR_INVALID, "n_in and n_out must be positive");
        cudaStream_t s = (cudaStream_t)stream;
        if (n == 0) {
            cuda_check(cudaMemsetAsync(n_valid, 0, sizeof(uint32_t), s), "memset");
            return;
        }
        if (!input || !target || !valid_input || !valid_target) throw Error(NLOD_ERR_INVALID, "buffers must not be NULL");
        uint32_t* total = scratch(1, s);
        select_ordered(ValidSel{target, n_out}, n, SampleOut{input, target, valid_input, valid_target, n_in, n_out}, total, n_valid, 0u,
                       true, s);
        cuda_check(cudaFreeAsync(total, s), "workspace");
    });
}
