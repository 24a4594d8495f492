/* CPU oracle (test infrastructure only) for the training-sample generator: the reference's
 * sampler restated in plain C, against which the GPU kernels are checked bit for bit.
 *
 *   orc_morton_voxels             morton_sparse_voxel_idx_mapping
 *                                 (rptr/cuda/neural-lod/neural_lod_learning_init.cu:201-294)
 *   orc_sample_visibility(_voxels) fill_ray_queries_visibility
 *                                 (rptr/cuda/neural-lod/neural_lod_learning_kernels.cuh:364-569)
 *   orc_sample_throughput         fill_ray_queries_throughput (kernels.cuh:100-238)
 *   orc_trace_visibility          exact-DDA stand-in for main_visibility_optimisation
 *                                 (rptr/vulkan/raygen.rgen:695-730)
 *   orc_trace_throughput          exact-DDA stand-in for the throughput ray query
 *                                 (raygen.rgen:505-687) + record_ray_query_results_throughput_optim
 *                                 (kernels.cuh:240-278)
 *   orc_compact_samples           copy_valid_results_throughput_optim (kernels.cuh:280-318), stable
 *
 * Helpers restated: sample_voxel / sample_discrete_lods / shifted_square_pdf (kernels.cuh:29-98),
 * compute_lod_voxel (neural_lod_learning_grid.cuh:50-74), square_to_uniform_sphere,
 * intersect_aabb(_min_max), min_component, get_deterministic_local_pi_po
 * (neural_lod_learning_common.cuh:48-54, 68-76, 255-308, 567-619), encode/decode_morton3
 * (neural_lod_learning.h:519-580), the LCG and its MurmurHash3 seeding
 * (rptr/rendering/pointsets/lcg_rng.glsl, hashing.glsl).  The sine and cosine of the sphere
 * sampling are a Taylor evaluation in double (the GPU kernels use the same), so both sides draw
 * identical directions.  Built with -ffp-contract=off: one rounding per operation.
 *
 * Parity unpinned against the reference's own binaries: its sampler needs glm and its targets
 * need the Vulkan renderer, neither of which builds here. */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include "nlod_oracle.h"

static uint32_t m3_compact(uint32_t x) {
    x &= 0x09249249u;
    x = (x ^ (x >> 2)) & 0x030c30c3u;
    x = (x ^ (x >> 4)) & 0x0300f00fu;
    x = (x ^ (x >> 8)) & 0xff0000ffu;
    x = (x ^ (x >> 16)) & 0x000003ffu;
    return x;
}

static int grid_bit(const uint32_t* bits, uint32_t res, uint32_t x, uint32_t y, uint32_t z) {
    const uint64_t idx = (uint64_t)x + (uint64_t)res * ((uint64_t)y + (uint64_t)res * z);
    return (int)((bits[idx >> 5] >> (31u - (uint32_t)(idx & 31u))) & 1u);
}

uint32_t orc_morton_voxels(const uint32_t* bits, uint32_t res, uint32_t* codes, uint32_t capacity) {
    const uint64_t n = (uint64_t)res * res * res;
    uint32_t count = 0;
    for (uint64_t c = 0; c < n; ++c) {
        const uint32_t code = (uint32_t)c;
        if (!grid_bit(bits, res, m3_compact(code), m3_compact(code >> 1), m3_compact(code >> 2))) continue;
        if (codes && count < capacity) codes[count] = code;
        ++count;
    }
    return count;
}

/* ---- RNG ---- */
static uint32_t mm_mix(uint32_t h, uint32_t k) {
    k *= 0xcc9e2d51u;
    k = (k << 15) | (k >> 17);
    k *= 0x1b873593u;
    h ^= k;
    h = ((h << 13) | (h >> 19)) * 5u + 0xe6546b64u;
    return h;
}
static uint32_t mm_final(uint32_t h) {
    h ^= h >> 16;
    h *= 0x85ebca6bu;
    h ^= h >> 13;
    h *= 0xc2b2ae35u;
    h ^= h >> 16;
    return h;
}
static uint32_t rng_seed(uint32_t index, uint32_t frame, uint32_t linear) {
    return mm_final(mm_mix(mm_mix(frame, linear), index));
}
static float rng_f(uint32_t* s) {
    *s = *s * 1664525u + 1013904223u;
    return ldexpf((float)*s, -32);
}

/* cos / sin of phi in [0, 2pi]: nearest multiple of pi/2 removed, Taylor series in double. */
static void cos_sin_f(float phi, float* c_out, float* s_out) {
    const double d = (double)phi;
    const double q = floor(d * 0.63661977236758134 + 0.5);
    const double r = d - q * 1.5707963267948966;
    const double r2 = r * r;
    /* sin r = r (1 - r^2/(2*3) (1 - r^2/(4*5) (... (1 - r^2/(16*17))))), each 1/(k(k+1)) a double
     * constant (correctly rounded reciprocal) multiplied in */
    static const double ks[8] = {1.0 / 272.0, 1.0 / 210.0, 1.0 / 156.0, 1.0 / 110.0, 1.0 / 72.0, 1.0 / 42.0, 1.0 / 20.0, 1.0 / 6.0};
    double t = 1.0 - r2 * ks[0];
    for (int i = 1; i < 7; ++i) t = 1.0 - r2 * ks[i] * t;
    const double sr = r * (1.0 - r2 * ks[7] * t);
    /* cos r = 1 - r^2/(1*2) (1 - r^2/(3*4) (... (1 - r^2/(15*16)))) */
    static const double kc[8] = {1.0 / 240.0, 1.0 / 182.0, 1.0 / 132.0, 1.0 / 90.0, 1.0 / 56.0, 1.0 / 30.0, 1.0 / 12.0, 0.5};
    double u = 1.0 - r2 * kc[0];
    for (int i = 1; i < 7; ++i) u = 1.0 - r2 * kc[i] * u;
    const double cr = 1.0 - r2 * kc[7] * u;
    switch (((int)q) & 3) {
        case 0: *c_out = (float)cr; *s_out = (float)sr; break;
        case 1: *c_out = (float)(-sr); *s_out = (float)cr; break;
        case 2: *c_out = (float)(-cr); *s_out = (float)(-sr); break;
        default: *c_out = (float)sr; *s_out = (float)(-cr); break;
    }
}

void orc_cos_sin(float phi, float* c, float* s) { cos_sin_f(phi, c, s); }

static void sphere_dir(float u1, float u2, float w[3]) {
    const double two_pi = 2.0 * 3.14159265358979323846;
    const float phi = (float)(two_pi * (double)u1);
    const float ct = u2 * 2.0f - 1.0f;
    const float st = sqrtf(1.0f - ct * ct);
    float c, s;
    cos_sin_f(phi, &c, &s);
    w[0] = st * c;
    w[1] = st * s;
    w[2] = ct;
}

static float min_comp(float a, float b, float c) {
    const float m = (b < a) ? b : a;
    return (c < m) ? c : m;
}

static int box0_hit(const float o[3], const float d[3], float edge, float* tn, float* tf) {
    const float h = 0.5f * edge, lo = 0.0f - h, hi = 0.0f + h;
    float near_t = -1e20f, far_t = 1e20f;
    for (int i = 0; i < 3; ++i) {
        const float inv = 1.f / d[i];
        if (d[i] == 0.f) {
            if (o[i] < lo || o[i] > hi) return 0;
            continue;
        }
        float t1 = (lo - o[i]) * inv, t2 = (hi - o[i]) * inv;
        if (t1 > t2) { const float t = t1; t1 = t2; t2 = t; }
        if (!(t1 < near_t)) near_t = t1;
        if (!(far_t < t2)) far_t = t2;
        if (!(near_t < far_t) || (double)far_t < 0.0) return 0;
    }
    *tn = near_t;
    *tf = far_t;
    return 1;
}

static float lod_weight(uint32_t l, float strength, float shift, uint32_t n_lods) {
    const float x = (float)l / (float)n_lods + shift - 0.5f + 0.0625f;
    const float sxx = strength * x * x;
    return (float)(1.0 + (double)sxx);
}

static uint32_t pick_lod(float sample, const OrcSamplerParams* p) {
    double cdf[16];
    for (uint32_t l = 0; l < p->n_lods; ++l) {
        const double w = (double)lod_weight(l, p->pdf_strength, p->pdf_shift, p->n_lods);
        cdf[l] = l == 0 ? w : cdf[l - 1] + w;
    }
    for (uint32_t l = 0; l < p->n_lods; ++l)
        if ((double)sample < cdf[l] / cdf[p->n_lods - 1]) return l;
    return p->n_lods - 1;
}

typedef struct {
    float c[3];
    float e;
} Vox;

static Vox make_vox(const OrcSamplerParams* p, const uint32_t xyz[3], uint32_t lod) {
    Vox v;
    const float step = ldexpf(p->voxel_size, (int)lod);
    for (int k = 0; k < 3; ++k) {
        const float lo = p->aabb_min[k] + (float)xyz[k] * step;
        v.c[k] = lo + step * 0.5f;
    }
    v.e = step;
    return v;
}

static Vox draw_voxel(uint32_t* rng, const OrcSamplerParams* p, const uint32_t* morton, uint32_t n_voxels, uint32_t* lod) {
    const float u = rng_f(rng);
    const uint32_t idx = (uint32_t)(u * (float)n_voxels) % n_voxels;
    const uint32_t code = morton[idx];
    *lod = pick_lod(rng_f(rng), p);
    const uint32_t xyz[3] = {m3_compact(code) >> *lod, m3_compact(code >> 1) >> *lod, m3_compact(code >> 2) >> *lod};
    return make_vox(p, xyz, *lod);
}

static float draw_dilation(uint32_t* rng, const OrcSamplerParams* p) {
    const float ratio = p->dilation_outward / (p->dilation_inward + p->dilation_outward);
    if (rng_f(rng) < ratio) return rng_f(rng) * (p->dilation_outward - p->min_dilation) + p->min_dilation;
    return -(rng_f(rng) * (p->dilation_inward - p->min_dilation) + p->min_dilation);
}

static void plane_basis(const float w[3], float u[3], float v[3]) {
    const float ax = fabsf(-w[0]), ay = fabsf(-w[1]), az = fabsf(-w[2]);
    const float m = min_comp(ax, ay, az);
    u[0] = u[1] = u[2] = 0.f;
    if (ax == m) { u[1] = w[2]; u[2] = -w[1]; }
    else if (ay == m) { u[0] = -w[2]; u[2] = w[0]; }
    else { u[0] = -w[1]; u[1] = w[0]; }
    v[0] = w[1] * u[2] - u[1] * w[2];
    v[1] = w[2] * u[0] - u[2] * w[0];
    v[2] = w[0] * u[1] - u[0] * w[1];
}

static int draw_chord(uint32_t* rng, const float w[3], const float u[3], const float v[3], float dist, float dil, uint32_t attempts,
                      float a[3], float b[3]) {
    const float dir[3] = {-w[0], -w[1], -w[2]};
    for (uint32_t t = 0; t < attempts; ++t) {
        const float r0 = rng_f(rng);
        const float r1 = rng_f(rng);
        const float ox = (r0 - 0.5f) * dist, oy = (r1 - 0.5f) * dist;
        float o[3], tn, tf;
        for (int k = 0; k < 3; ++k) {
            const float cam = w[k] * dist;
            o[k] = cam + u[k] * ox + v[k] * oy;
        }
        if (box0_hit(o, dir, 1.0f + dil, &tn, &tf)) {
            for (int k = 0; k < 3; ++k) {
                a[k] = o[k] + dir[k] * tn;
                b[k] = o[k] + dir[k] * tf;
            }
            return 1;
        }
    }
    return 0;
}

static int face_of(const float q[3]) {
    float best = -2e20f;
    int f = 0;
    for (int i = 0; i < 3; ++i) {
        const float a = fabsf(q[i]);
        if (a > best) {
            f = (double)q[i] > 0.0 ? 2 * i : 2 * i + 1;
            best = a;
        }
    }
    return f;
}

static void invalidate(float* in, int n_in, OrcRayQuery* q) {
    for (int k = 0; k < n_in; ++k) in[k] = -1.f;
    q->t_max = -1.f;
}

static void to_unit(const OrcSamplerParams* p, const float w[3], float* out) {
    for (int k = 0; k < 3; ++k) out[k] = (w[k] - p->aabb_min[k]) / (p->aabb_max[k] - p->aabb_min[k]);
}

static void vis_after_voxel(uint32_t* rng, const OrcSamplerParams* p, const Vox* vx, float* in, OrcRayQuery* q) {
    const float dist = 2.f * (1.f + p->dilation_outward);
    float wi[3], pu[3], pv[3], a[3], b[3], dil = 0.f;
    {
        const float u1 = rng_f(rng);
        const float u2 = rng_f(rng);
        sphere_dir(u1, u2, wi);
    }
    plane_basis(wi, pu, pv);
    int done = 0;
    for (uint32_t attempt = 0; attempt < p->max_attempts && !done; ++attempt) {
        dil = draw_dilation(rng, p);
        if (!draw_chord(rng, wi, pu, pv, dist, dil, p->max_attempts, a, b)) break;
        if (p->increase_boundary_density) {
            float md[3];
            for (int k = 0; k < 3; ++k) {
                const float mid = 0.5f * (a[k] + b[k]);
                md[k] = mid / (1.0f + dil);
            }
            const float umd = min_comp(fabsf(md[0]), fabsf(md[1]), fabsf(md[2])) * 2.0f;
            const float thr = umd * 1.5f + 0.1f;
            if (rng_f(rng) < thr) done = 1;
        } else {
            done = 1;
        }
    }
    if (!done) {
        invalidate(in, 6, q);
        return;
    }
    /* the point on the lower-numbered face is pi (a tangent chord keeps its order) */
    const int fa = face_of(a), fb = face_of(b);
    const float* lpi = (fb < fa) ? b : a;
    const float* lpo = (fb < fa) ? a : b;
    float pi[3], po[3], d[3];
    for (int k = 0; k < 3; ++k) {
        pi[k] = vx->c[k] + lpi[k] * vx->e;
        po[k] = vx->c[k] + lpo[k] * vx->e;
        d[k] = lpo[k] - lpi[k];
    }
    const float dd = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
    const float inv_len = 1.0f / sqrtf(dd);
    for (int k = 0; k < 3; ++k) {
        q->origin[k] = pi[k];
        q->dir[k] = d[k] * inv_len;
        q->voxel_center[k] = vx->c[k];
    }
    q->voxel_extent = vx->e * (1.f + (dil < p->bound_bias ? p->bound_bias : dil));
    q->t_max = 1e20f;
    q->mode_or_data = 0;
    to_unit(p, pi, in);
    to_unit(p, po, in + 3);
}

void orc_sample_visibility(const OrcSamplerParams* p, const uint32_t* morton, uint32_t n_voxels, uint32_t batch_index, uint32_t n,
                           float* input, OrcRayQuery* queries, uint32_t* lod) {
    for (uint32_t i = 0; i < n; ++i) {
        OrcRayQuery q;
        memset(&q, 0, sizeof q);
        uint32_t rng = rng_seed(batch_index * n, 0u, i), l = 0;
        if (n_voxels == 0) {
            invalidate(input + (size_t)i * 6, 6, &q);
        } else {
            const Vox vx = draw_voxel(&rng, p, morton, n_voxels, &l);
            vis_after_voxel(&rng, p, &vx, input + (size_t)i * 6, &q);
        }
        if (queries) queries[i] = q;
        if (lod) lod[i] = l;
    }
}

void orc_sample_visibility_voxels(const OrcSamplerParams* p, const uint32_t* lod_morton, uint32_t first, uint32_t n_voxels,
                                  uint32_t n_samples, uint32_t lod, float* input, OrcRayQuery* queries) {
    for (uint32_t v = 0; v < n_voxels; ++v)
        for (uint32_t s = 0; s < n_samples; ++s) {
            const uint32_t i = s + v * n_samples;
            uint32_t rng = rng_seed(first + v, 0u, s);
            const uint32_t code = lod_morton[first + v];
            const uint32_t xyz[3] = {m3_compact(code), m3_compact(code >> 1), m3_compact(code >> 2)};
            const Vox vx = make_vox(p, xyz, lod);
            OrcRayQuery q;
            memset(&q, 0, sizeof q);
            vis_after_voxel(&rng, p, &vx, input + (size_t)i * 6, &q);
            if (queries) queries[i] = q;
        }
}

void orc_sample_throughput(const OrcSamplerParams* p, const uint32_t* morton, uint32_t n_voxels, uint32_t batch_index, uint32_t n,
                           int32_t max_orders, float* input, OrcRayQuery* queries, uint32_t* lod) {
    for (uint32_t i = 0; i < n; ++i) {
        OrcRayQuery q;
        memset(&q, 0, sizeof q);
        float* in = input + (size_t)i * 9;
        uint32_t rng = rng_seed(batch_index * n, 0u, i), l = 0;
        int ok = n_voxels > 0;
        Vox vx;
        memset(&vx, 0, sizeof vx);
        float wo[3] = {0.f, 0.f, 0.f}, a[3], b[3], dil = 0.f;
        if (ok) {
            vx = draw_voxel(&rng, p, morton, n_voxels, &l);
            const float dist = 2.f * (1.f + p->dilation_outward);
            const float u1 = rng_f(&rng);
            const float u2 = rng_f(&rng);
            sphere_dir(u1, u2, wo);
            float pu[3], pv[3];
            plane_basis(wo, pu, pv);
            dil = draw_dilation(&rng, p);
            ok = draw_chord(&rng, wo, pu, pv, dist, dil, p->max_attempts, a, b);
        }
        if (!ok) {
            invalidate(in, 9, &q);
        } else {
            for (int k = 0; k < 3; ++k) {
                q.origin[k] = vx.c[k] + a[k] * vx.e;
                q.dir[k] = -wo[k];
                q.voxel_center[k] = vx.c[k];
            }
            q.voxel_extent = vx.e * (1.f + (dil < p->bound_bias ? p->bound_bias : dil));
            q.t_max = 1e20f;
            q.mode_or_data = max_orders;
            to_unit(p, vx.c, in);
            for (int k = 0; k < 3; ++k) in[3 + k] = (wo[k] + 1.0f) * 0.5f;
            for (int k = 6; k < 9; ++k) in[k] = 0.f;
        }
        if (queries) queries[i] = q;
        if (lod) lod[i] = l;
    }
}

/* ---- exact-DDA targets ---- */
static float exit_t(const float E[3], const float D[3], const float c[3], float h) {
    float t = FLT_MAX;
    for (int k = 0; k < 3; ++k) {
        if (D[k] == 0.f) continue;
        const float bound = D[k] > 0.f ? c[k] + h : c[k] - h;
        const float tk = (bound - E[k]) / D[k];
        if (tk < t) t = tk;
    }
    return t < 0.f ? 0.f : t;
}

static int hit_in_box(const OrcLodLevel* L, const float E[3], const float D[3], const float c[3], float h, const int32_t prev[3],
                      int32_t v[3], float P[3]) {
    float tn, tf;
    if (!orc_first_active_voxel_clip(L, E, D, 0.f, exit_t(E, D, c, h), prev, v, &tn, &tf)) return 0;
    const float t = tn < 0.f ? 0.f : tn;
    for (int k = 0; k < 3; ++k) P[k] = E[k] + t * D[k];
    return !(fabsf(P[0] - c[0]) > h || fabsf(P[1] - c[1]) > h || fabsf(P[2] - c[2]) > h);
}

static void index_frame(const OrcSamplerParams* p, const OrcRayQuery* q, float E[3], float D[3], float c[3], float* h) {
    for (int k = 0; k < 3; ++k) {
        E[k] = (q->origin[k] - p->aabb_min[k]) / p->voxel_size;
        D[k] = q->dir[k];
        c[k] = (q->voxel_center[k] - p->aabb_min[k]) / p->voxel_size;
    }
    *h = q->voxel_extent * 0.5f / p->voxel_size;
}

void orc_trace_visibility(const OrcLodLevel* L0, const OrcSamplerParams* p, const OrcRayQuery* queries, uint32_t n, float* target) {
    const int32_t none[3] = {-1, -1, -1};
    for (uint32_t i = 0; i < n; ++i) {
        if (queries[i].t_max < 0.f) {
            target[i] = -1.f;
            continue;
        }
        float E[3], D[3], c[3], h, P[3];
        int32_t v[3];
        index_frame(p, &queries[i], E, D, c, &h);
        target[i] = hit_in_box(L0, E, D, c, h, none, v, P) ? 1.f : 0.f;
    }
}

static float albedo_ch(const int32_t v[3], uint32_t ch) {
    uint32_t h = mm_mix(mm_mix(mm_mix(0x9e3779b9u, (uint32_t)v[0]), (uint32_t)v[1]), (uint32_t)v[2]);
    h = mm_final(h + ch);
    return 0.1f + 0.8f * ((float)(h >> 8) * 5.9604644775390625e-08f);
}

uint32_t orc_trace_throughput(const OrcLodLevel* L0, const OrcSamplerParams* p, const OrcRayQuery* queries, uint32_t n,
                              uint32_t batch_index, int log_learning, float* input, float* target) {
    const int32_t none[3] = {-1, -1, -1};
    uint32_t invalid = 0;
    for (uint32_t i = 0; i < n; ++i) {
        float* in = input + (size_t)i * 9;
        float* tg = target + (size_t)i * 3;
        float E[3], D[3], c[3], h, P[3];
        int32_t v[3];
        int ok = queries[i].t_max >= 0.f;
        if (ok) {
            index_frame(p, &queries[i], E, D, c, &h);
            ok = hit_in_box(L0, E, D, c, h, none, v, P);
        }
        if (!ok) {
            for (int k = 0; k < 9; ++k) in[k] = -1.f;
            for (int k = 0; k < 3; ++k) tg[k] = -1.f;
            ++invalid;
            continue;
        }
        uint32_t rng = rng_seed(batch_index * n, 1u, i);
        float wi[3];
        {
            const float u1 = rng_f(&rng);
            const float u2 = rng_f(&rng);
            sphere_dir(u1, u2, wi);
        }
        int32_t v2[3];
        float P2[3];
        const float vis = hit_in_box(L0, P, wi, c, h, v, v2, P2) ? 0.f : 1.f;
        for (int k = 0; k < 3; ++k) {
            float t = albedo_ch(v, (uint32_t)k) * vis;
            if (log_learning) t = logf(1.f + t);
            tg[k] = t;
            in[6 + k] = (wi[k] + 1.0f) * 0.5f;
        }
    }
    return invalid;
}

uint32_t orc_compact_samples(const float* input, const float* target, uint32_t n, uint32_t n_in, uint32_t n_out, float* valid_input,
                             float* valid_target) {
    uint32_t count = 0;
    for (uint32_t i = 0; i < n; ++i)
        if (target[(size_t)i * n_out] != -1.f) ++count;
    const uint32_t up = (count + 127u) / 128u * 128u;
    const uint32_t keep = up >= 128u ? up - 128u : 0u;
    uint32_t r = 0;
    for (uint32_t i = 0; i < n && r < keep; ++i) {
        if (target[(size_t)i * n_out] == -1.f) continue;
        memcpy(valid_input + (size_t)r * n_in, input + (size_t)i * n_in, n_in * sizeof(float));
        memcpy(valid_target + (size_t)r * n_out, target + (size_t)i * n_out, n_out * sizeof(float));
        ++r;
    }
    return keep;
}
