// Per-ray state and per-ray steps of the neural-LoD render query, shared by the wavefront form
// (render.cu: rounds in a conditional graph loop, a chain of queries per ray and round) and the persistent
// form (render_pk.cu: tile pipelines that refill their ray slots from a global queue).  Both forms
// call these functions, so a ray takes the same steps with the same roundings in either.
//
// The steps are the reference's wavefront loop (rptr/cuda/neural-lod/
// wavefront_neural_throughput_visibility_lod.cu:470-720; per-ray work in
// rptr/cuda/wavefront_neural_pt.cuh: raymarch_impl, generate_*_inference_data_impl,
// process_ray_bounce) with the network inputs of this library's workloads:
//   visibility input  = voxel-local entry point in [0,1]^3, (dir + 1) / 2;
//   throughput input  = voxel centre / res, (wi + 1) / 2, (wo + 1) / 2, LoD column.
// Every floating-point operation is written with an explicit rounding (__f*_rn) so that the host
// restatement reproduces rays, traversal and sampling bit for bit.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "lod.h"
#include "lod_dda.cuh"

namespace nlod {
namespace render {

constexpr uint32_t kFull = 0xFFFFFFFFu;
constexpr float kFourPi = 12.566370614359172f;

// One ray's state between queries (80 bytes).
struct alignas(16) RayState {
    float o[3];
    float tmin;
    float d[3];
    float tnear;
    float tp[3];
    float tfar;
    int32_t ijk[3];
    uint32_t meta;     // bits 0-7 bounce, 8-23 visibility queries in this bounce
    float wi[3];
    uint32_t pad;
};

struct RenderConsts {
    LodLevelDev L;
    uint32_t width, height, n_rays;
    float cam_o[3], cam_u[3], cam_v[3], cam_w[3];
    uint32_t max_depth, max_vis;
    float threshold;
    float background[3], env[3];
    float res;
    float lod_input;
    uint32_t seed_lo, seed_hi;
    uint32_t budget;
    uint32_t max_rounds;
    uint32_t max_chain;   // wavefront form: longest chain of visibility queries a ray marches ahead
};

// Control words: [0..3] list counters [parity * 2 + kind] (the persistent form uses [0] as its
// ray queue), [4] visibility rows, [5] throughput list length of the current round, [6] round,
// [7] rays dropped at the per-bounce query cap; then 64-bit totals: visibility queries,
// throughput queries, rounds (the persistent form: the most tile iterations of any pipeline);
// then the wavefront form's throughput rows evaluated this round (0 while a short list is
// carried over) and the rounds the list has been carried over in a row; its visibility row
// counters [parity], the rows of the current round, the chain length of the next round, the
// visibility results consumed and accepted in the last round, and the total rows evaluated.
struct Control {
    uint32_t cnt[4];
    uint32_t n_vis, n_thr, round, dropped;
    unsigned long long tot_vis, tot_thr, tot_rounds;
    uint32_t thr_rows, thr_deferred;
    uint32_t rows[2], n_rows, chain, consumed, accepted;
    unsigned long long tot_rows;
};

__device__ __forceinline__ uint32_t mix32(uint32_t h) {
    h ^= h >> 16;
    h *= 0x7feb352du;
    h ^= h >> 15;
    h *= 0x846ca68bu;
    h ^= h >> 16;
    return h;
}

__device__ __forceinline__ float u01(uint32_t h) { return (float)(h >> 8) * (1.0f / 16777216.0f); }

// Uniform direction on the sphere by rejection from the cube (correctly rounded operations only,
// so that the host restatement draws the identical direction).
__device__ __forceinline__ void sample_sphere(uint32_t key, float (&w)[3]) {
    for (uint32_t t = 0; t < 16; ++t) {
        const uint32_t h = mix32(key + t * 0x632BE5ABu);
        const float x = __fsub_rn(__fmul_rn(2.f, u01(h)), 1.f);
        const float y = __fsub_rn(__fmul_rn(2.f, u01(mix32(h ^ 0x68E31DA4u))), 1.f);
        const float z = __fsub_rn(__fmul_rn(2.f, u01(mix32(h ^ 0xB5297A4Du))), 1.f);
        const float r2 = __fadd_rn(__fadd_rn(__fmul_rn(x, x), __fmul_rn(y, y)), __fmul_rn(z, z));
        if (r2 <= 1.f && r2 >= 1e-4f) {
            const float r = __fsqrt_rn(r2);
            w[0] = __fdiv_rn(x, r);
            w[1] = __fdiv_rn(y, r);
            w[2] = __fdiv_rn(z, r);
            return;
        }
    }
    w[0] = 0.f;
    w[1] = 0.f;
    w[2] = 1.f;
}

// Camera ray of pixel j; its image pixel and query counters start at zero.
__device__ __forceinline__ void ray_generate(const RenderConsts& C, uint32_t j, RayState& st) {
    const uint32_t px = j % C.width, py = j / C.width;
    const float W = (float)C.width, H = (float)C.height;
    const float a = __fdiv_rn(__fsub_rn(__fmul_rn(2.f, __fadd_rn((float)px, 0.5f)), W), W);
    const float b = __fdiv_rn(__fsub_rn(H, __fmul_rn(2.f, __fadd_rn((float)py, 0.5f))), H);
    float dd[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) dd[k] = __fadd_rn(__fadd_rn(__fmul_rn(a, C.cam_u[k]), __fmul_rn(b, C.cam_v[k])), C.cam_w[k]);
    const float len = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(dd[0], dd[0]), __fmul_rn(dd[1], dd[1])), __fmul_rn(dd[2], dd[2])));
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        st.o[k] = C.cam_o[k];
        st.d[k] = __fdiv_rn(dd[k], len);
        st.tp[k] = 1.f;
        st.ijk[k] = -1;
        st.wi[k] = 0.f;
    }
    st.tmin = 0.f;
    st.tnear = st.tfar = 0.f;
    st.meta = 0u;
    st.pad = 0u;
}

enum : int { MARCH_DONE = 0, MARCH_VIS = 1, MARCH_FAIL = 2, MARCH_DROPPED = 3 };

// The pixel of a ray that escaped: the background before the first bounce, the environment
// times the path throughput after.
__device__ __forceinline__ void write_escape(const RenderConsts& C, const RayState& st, float* __restrict__ pixel) {
    const uint32_t bounce = st.meta & 0xFFu;
#pragma unroll
    for (int k = 0; k < 3; ++k) pixel[k] = bounce == 0 ? C.background[k] : __fmul_rn(st.tp[k], C.env[k]);
}

// Marches to the next occupied voxel.  MARCH_VIS: the ray's next visibility query is set up
// (voxel, t_near / t_far, query count).  MARCH_DONE: the ray escaped (the caller writes its
// pixel).  MARCH_DROPPED: the per-bounce query cap was reached.  MARCH_FAIL: the DDA ran out of
// its step budget.
__device__ __forceinline__ int march_query(const RenderConsts& C, RayState& st) {
    const uint32_t nvis = (st.meta >> 8) & 0xFFFFu;
    if (nvis >= C.max_vis) return MARCH_DROPPED;
    int32_t v3[3] = {0, 0, 0};
    float tn = 0.f, tf = 0.f;
    const int r = dda::first_active_voxel(C.L, st.o, st.d, st.tmin, st.ijk, v3, tn, tf, C.budget);
    if (r < 0) return MARCH_FAIL;
    if (r == 0) return MARCH_DONE;
#pragma unroll
    for (int k = 0; k < 3; ++k) st.ijk[k] = v3[k];
    st.tnear = tn;
    st.tfar = tf;
    st.meta += 1u << 8;
    return MARCH_VIS;
}

// march_query, with the pixel of an escaped ray written.
__device__ __forceinline__ int ray_march(const RenderConsts& C, RayState& st, float* __restrict__ pixel) {
    const int r = march_query(C, st);
    if (r == MARCH_DONE) write_escape(C, st, pixel);
    return r;
}

enum : int { VIS_REJECT = 0, VIS_ACCEPT_THR = 1, VIS_ACCEPT_END = 2 };

// The ray parameter a rejected voxel's march restarts from: the voxel's middle.
__device__ __forceinline__ float past_voxel(const RayState& st) { return __fmul_rn(__fadd_rn(st.tnear, st.tfar), 0.5f); }

// Applies a visibility value: rejected -> the ray continues past the voxel (tmin moved to the
// voxel's middle; the caller marches); accepted -> a throughput query with a sampled incoming
// direction, or the end of the path (dark) on its last vertex.
__device__ __forceinline__ int vis_resolve(const RenderConsts& C, RayState& st, uint32_t ray, float v) {
    if (v >= C.threshold) {
        const uint32_t bounce = st.meta & 0xFFu;
        if (bounce + 1 < C.max_depth) {
            sample_sphere(mix32(mix32(ray ^ mix32(C.seed_lo ^ mix32(C.seed_hi))) ^ (bounce * 0x9E3779B9u)), st.wi);
            return VIS_ACCEPT_THR;
        }
        return VIS_ACCEPT_END;
    }
    st.tmin = past_voxel(st);
    return VIS_REJECT;
}

// Applies a throughput value: the path throughput is scaled, the ray restarts just past the
// voxel's entry along the sampled direction with a new bounce.  Returns whether the path still
// carries throughput (the caller marches it).
__device__ __forceinline__ bool thr_resolve(RayState& st, const float (&t)[3]) {
    const float t_eps = __fadd_rn(st.tnear, __fmul_rn(1e-4f, __fsub_rn(st.tfar, st.tnear)));
    bool alive = false;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float tv = fmaxf(t[k], 0.f);
        st.tp[k] = __fmul_rn(st.tp[k], __fmul_rn(tv, kFourPi));
        alive |= st.tp[k] != 0.f;
        st.o[k] = __fadd_rn(st.o[k], __fmul_rn(st.d[k], t_eps));
        st.d[k] = st.wi[k];
    }
    st.tmin = 0.f;
    st.meta = (st.meta & 0xFFu) + 1u;   // next bounce, no visibility query yet
    return alive;
}

// Network input rows of a ray's pending query.
// (the query in voxel ijk entered at t_near)
__device__ __forceinline__ void vis_row_at(const RayState& st, const int32_t (&ijk)[3], float t_near, float* __restrict__ row) {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float pk = __fadd_rn(st.o[k], __fmul_rn(st.d[k], t_near));
        row[k] = fminf(fmaxf(__fsub_rn(pk, (float)ijk[k]), 0.f), 1.f);
        row[3 + k] = __fmul_rn(__fadd_rn(st.d[k], 1.f), 0.5f);
    }
}

__device__ __forceinline__ void vis_row(const RayState& st, float* __restrict__ row) { vis_row_at(st, st.ijk, st.tnear, row); }

__device__ __forceinline__ void thr_row(const RenderConsts& C, const RayState& st, float* __restrict__ row) {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        row[k] = __fdiv_rn(__fadd_rn((float)st.ijk[k], 0.5f), C.res);
        row[3 + k] = __fmul_rn(__fadd_rn(st.wi[k], 1.f), 0.5f);
        row[6 + k] = __fmul_rn(__fadd_rn(-st.d[k], 1.f), 0.5f);
    }
    row[9] = C.lod_input;
}

}  // namespace render
}  // namespace nlod
