// Wavefront neural-LoD render query: pinhole rays through one level of the LoD pyramid, a
// visibility query per occupied voxel a ray enters, a throughput query and a bounce at every
// voxel the visibility network accepts.  The algorithm is the reference's wavefront loop
// (rptr/cuda/neural-lod/wavefront_neural_throughput_visibility_lod.cu:470-720: raymarch,
// compact_for_visibility_and_accumulate, check_visibility, generate_throughput_inference_data,
// process_ray_bounce, compact_for_next_bounce_and_accumulate; the per-ray steps in
// rptr/cuda/wavefront_neural_pt.cuh: raymarch_impl, generate_*_inference_data_impl), with the
// network inputs of this library's visibility / throughput workloads:
//   visibility input  = voxel-local entry point in [0,1]^3, (dir + 1) / 2; LoD as the grid's
//                       per-element max level;
//   throughput input  = voxel centre / res, (wi + 1) / 2, (wo + 1) / 2, LoD column.
//
// GB300 organisation.  The reference synchronises with the host after every wavefront to size
// the next launch.  Here every ray advances independently by one query per round, and one round
// is four launches: visibility inference and throughput inference over the current lists (the
// tensor-core kernels read their row count from device memory), k_step (resolve every queued
// ray: accept / reject the voxel, apply a throughput result and bounce, march to the next
// occupied voxel with the bit-exact DDA, append the ray's next query to the compacted lists with
// warp-aggregated atomics) and k_round (publish the list sizes, set the loop condition).  The
// rounds run inside a CUDA graph as the body of a conditional while node, so a frame is one
// graph launch with no host round trip; the loop ends when both lists are empty (bounded by
// construction: each round moves every live ray one query forward).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "abi_util.h"
#include "kernels.h"
#include "lod.h"
#include "lod_dda.cuh"
#include "nlod.h"

struct nlod_module;

namespace nlod {

cudaError_t module_inference_device_count(nlod_module* m, uint32_t n_max, const float* in, float* out, const uint32_t* n_dev,
                                          float max_level, cudaStream_t s);

namespace {

constexpr uint32_t kFull = 0xFFFFFFFFu;
constexpr float kFourPi = 12.566370614359172f;

// One ray's state between rounds (80 bytes).
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
};

// Control words: [0..3] list counters [parity * 2 + kind], [4] visibility rows, [5] throughput
// rows of the current round, [6] round, [7] rays dropped at the per-bounce query cap;
// then 64-bit totals: visibility queries, throughput queries, rounds.
struct Control {
    uint32_t cnt[4];
    uint32_t n_vis, n_thr, round, dropped;
    unsigned long long tot_vis, tot_thr, tot_rounds, pad;
};

struct RenderBufs {
    RayState* rays;
    uint32_t* lists;      // [2 parity][2 kind][n_rays]
    Control* ctl;
    float* vis_in;        // [n_pad][6]
    float* vis_out;       // [n_pad][1]
    float* thr_in;        // [n_pad][10]
    float* thr_out;       // [n_pad][3]
    float* image;         // [n_rays][3]
    uint32_t* ray_stats;  // [n_rays][2]
    uint32_t* status;
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

// Appends the lanes with `want` to a list; returns each wanting lane's slot.  All lanes call.
__device__ __forceinline__ uint32_t push(uint32_t* counter, bool want) {
    const unsigned m = __ballot_sync(kFull, want);
    if (!m) return 0;
    const int lane = threadIdx.x & 31, leader = __ffs(m) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(counter, (uint32_t)__popc(m));
    base = __shfl_sync(kFull, base, leader);
    return base + (uint32_t)__popc(m & ((1u << lane) - 1u));
}

enum : int { ACT_NONE_ = 0, ACT_VIS = 1, ACT_THR = 2 };

// One round for every queued ray (first = true: ray generation, every pixel's ray).
__global__ void __launch_bounds__(256) k_step(const __grid_constant__ RenderConsts C, RenderBufs B, int first) {
    const uint32_t round = first ? 0u : B.ctl->round;
    const uint32_t p = (round + 1u) & 1u, q = round & 1u;   // lists read / written
    const uint32_t nv = first ? C.n_rays : B.ctl->n_vis;
    const uint32_t total = first ? C.n_rays : nv + B.ctl->n_thr;
    for (uint32_t base = blockIdx.x * blockDim.x; base < total; base += gridDim.x * blockDim.x) {
        const uint32_t j = base + threadIdx.x;
        const bool valid = j < total;
        int act = ACT_NONE_;
        uint32_t ray = 0;
        RayState st;
        if (valid) {
            bool march = false;
            if (first) {
                ray = j;
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
                    B.image[3 * ray + k] = 0.f;
                }
                st.tmin = 0.f;
                st.tnear = st.tfar = 0.f;
                st.meta = 0u;
                st.pad = 0u;
                B.ray_stats[2 * ray] = 0u;
                B.ray_stats[2 * ray + 1] = 0u;
                march = true;
            } else if (j < nv) {
                ray = B.lists[(p * 2 + 0) * C.n_rays + j];
                st = B.rays[ray];
                const float v = B.vis_out[j];
                if (v >= C.threshold) {
                    const uint32_t bounce = st.meta & 0xFFu;
                    if (bounce + 1 < C.max_depth) {
                        sample_sphere(mix32(mix32(ray ^ mix32(C.seed_lo ^ mix32(C.seed_hi))) ^ (bounce * 0x9E3779B9u)), st.wi);
                        act = ACT_THR;
                    }
                    // a hit on the last bounce ends the path without radiance
                } else {
                    st.tmin = __fmul_rn(__fadd_rn(st.tnear, st.tfar), 0.5f);
                    march = true;
                }
            } else {
                const uint32_t jj = j - nv;
                ray = B.lists[(p * 2 + 1) * C.n_rays + jj];
                st = B.rays[ray];
                const float t_eps = __fadd_rn(st.tnear, __fmul_rn(1e-4f, __fsub_rn(st.tfar, st.tnear)));
                bool alive = false;
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    const float tv = fmaxf(B.thr_out[3 * jj + k], 0.f);
                    st.tp[k] = __fmul_rn(st.tp[k], __fmul_rn(tv, kFourPi));
                    alive |= st.tp[k] != 0.f;
                    st.o[k] = __fadd_rn(st.o[k], __fmul_rn(st.d[k], t_eps));
                    st.d[k] = st.wi[k];
                }
                st.tmin = 0.f;
                st.meta = (st.meta & 0xFFu) + 1u;   // next bounce, no visibility query yet
                march = alive;
            }
            if (march) {
                const uint32_t nvis = (st.meta >> 8) & 0xFFFFu;
                if (nvis >= C.max_vis) {
                    atomicAdd(&B.ctl->dropped, 1u);
                } else {
                    int32_t v3[3] = {0, 0, 0};
                    float tn = 0.f, tf = 0.f;
                    const int r = dda::first_active_voxel(C.L, st.o, st.d, st.tmin, st.ijk, v3, tn, tf, C.budget);
                    if (r < 0) {
                        atomicOr(B.status, 2u);
                    } else if (r == 0) {
                        // escaped: background before the first bounce, environment after
                        const uint32_t bounce = st.meta & 0xFFu;
#pragma unroll
                        for (int k = 0; k < 3; ++k) B.image[3 * ray + k] = bounce == 0 ? C.background[k] : __fmul_rn(st.tp[k], C.env[k]);
                    } else {
#pragma unroll
                        for (int k = 0; k < 3; ++k) st.ijk[k] = v3[k];
                        st.tnear = tn;
                        st.tfar = tf;
                        st.meta += 1u << 8;
                        act = ACT_VIS;
                    }
                }
            }
        }
        const uint32_t slot_v = push(&B.ctl->cnt[q * 2 + 0], act == ACT_VIS);
        const uint32_t slot_t = push(&B.ctl->cnt[q * 2 + 1], act == ACT_THR);
        if (act == ACT_VIS) {
            B.lists[(q * 2 + 0) * C.n_rays + slot_v] = ray;
            float* row = B.vis_in + 6 * (size_t)slot_v;
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const float pk = __fadd_rn(st.o[k], __fmul_rn(st.d[k], st.tnear));
                row[k] = fminf(fmaxf(__fsub_rn(pk, (float)st.ijk[k]), 0.f), 1.f);
                row[3 + k] = __fmul_rn(__fadd_rn(st.d[k], 1.f), 0.5f);
            }
            B.ray_stats[2 * ray] += 1u;
        } else if (act == ACT_THR) {
            B.lists[(q * 2 + 1) * C.n_rays + slot_t] = ray;
            float* row = B.thr_in + 10 * (size_t)slot_t;
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                row[k] = __fdiv_rn(__fadd_rn((float)st.ijk[k], 0.5f), C.res);
                row[3 + k] = __fmul_rn(__fadd_rn(st.wi[k], 1.f), 0.5f);
                row[6 + k] = __fmul_rn(__fadd_rn(-st.d[k], 1.f), 0.5f);
            }
            row[9] = C.lod_input;
            B.ray_stats[2 * ray + 1] += 1u;
        }
        if (valid) B.rays[ray] = st;
    }
}

// Publishes the lists built this round, resets the other parity, sets the loop condition.
__global__ void k_round(Control* ctl, uint32_t max_rounds, uint32_t* status, cudaGraphConditionalHandle cond, int use_cond) {
    const uint32_t q = ctl->round & 1u;
    const uint32_t nv = ctl->cnt[q * 2 + 0], nt = ctl->cnt[q * 2 + 1];
    ctl->n_vis = nv;
    ctl->n_thr = nt;
    ctl->tot_vis += nv;
    ctl->tot_thr += nt;
    ctl->tot_rounds += 1;
    ctl->cnt[(q ^ 1u) * 2 + 0] = 0u;
    ctl->cnt[(q ^ 1u) * 2 + 1] = 0u;
    ctl->round += 1u;
    bool more = nv + nt > 0;
    if (more && ctl->round > max_rounds) {
        atomicOr(status, 4u);
        more = false;
    }
    if (use_cond) cudaGraphSetConditional(cond, more ? 1u : 0u);
}

__global__ void k_reset(Control* ctl) {
    Control c{};
    *ctl = c;
}

}  // namespace
}  // namespace nlod

using namespace nlod;

struct nlod_renderer {
    nlod_module* vis = nullptr;
    nlod_module* thr = nullptr;
    RenderConsts C{};
    RenderBufs B{};
    uint32_t n_pad = 0;
    float vis_max_level = 1000.f;
    cudaStream_t cap_stream = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    std::vector<void*> owned;
};

namespace {

void camera_basis(const nlod_render_params& p, float res, float out[12]) {
    double e[3], t[3], up[3];
    for (int k = 0; k < 3; ++k) {
        e[k] = p.eye[k];
        t[k] = p.target[k];
        up[k] = p.up[k];
    }
    double w[3] = {t[0] - e[0], t[1] - e[1], t[2] - e[2]};
    double wl = std::sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
    if (!(wl > 0)) throw Error(NLOD_ERR_INVALID, "camera eye and target coincide");
    for (double& v : w) v /= wl;
    double u[3] = {w[1] * up[2] - w[2] * up[1], w[2] * up[0] - w[0] * up[2], w[0] * up[1] - w[1] * up[0]};
    double ul = std::sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
    if (!(ul > 0)) throw Error(NLOD_ERR_INVALID, "camera up vector is parallel to the view direction");
    for (double& v : u) v /= ul;
    const double v[3] = {u[1] * w[2] - u[2] * w[1], u[2] * w[0] - u[0] * w[2], u[0] * w[1] - u[1] * w[0]};
    const double th = std::tan(0.5 * (double)p.fov_y_deg * 3.14159265358979323846 / 180.0);
    const double aspect = (double)p.width / (double)p.height;
    for (int k = 0; k < 3; ++k) {
        out[k] = (float)(e[k] * res);
        out[3 + k] = (float)(u[k] * th * aspect);
        out[6 + k] = (float)(v[k] * th);
        out[9 + k] = (float)w[k];
    }
}

void validate(const nlod_render_params& p) {
    if (p.width == 0 || p.height == 0 || (uint64_t)p.width * p.height > (1ull << 26))
        throw Error(NLOD_ERR_INVALID, "image must have between 1 and 2^26 pixels");
    if (p.max_depth == 0 || p.max_depth > 255) throw Error(NLOD_ERR_INVALID, "max_depth must be in [1, 255]");
    if (p.max_vis_queries == 0 || p.max_vis_queries > 65535) throw Error(NLOD_ERR_INVALID, "max_vis_queries must be in [1, 65535]");
    if (!(p.fov_y_deg > 0.f && p.fov_y_deg < 180.f)) throw Error(NLOD_ERR_INVALID, "fov_y_deg must be in (0, 180)");
}

}  // namespace

extern "C" {

int nlod_render_camera(const nlod_render_params* p, uint32_t level_res, float* out12) {
    return guarded([&] {
        if (!p || !out12) throw Error(NLOD_ERR_INVALID, "pointers must not be NULL");
        validate(*p);
        camera_basis(*p, (float)level_res, out12);
    });
}

void nlod_renderer_destroy(nlod_renderer* r) {
    if (!r) return;
    cudaDeviceSynchronize();
    if (r->exec) cudaGraphExecDestroy(r->exec);
    if (r->graph) cudaGraphDestroy(r->graph);
    if (r->cap_stream) cudaStreamDestroy(r->cap_stream);
    for (void* p : r->owned) dev_free(p);
    delete r;
}

int nlod_renderer_create(nlod_module* visibility, nlod_module* throughput, const nlod_lod_grid* grid, const nlod_render_params* p,
                         nlod_renderer** out) {
    return guarded([&] {
        if (!out) throw Error(NLOD_ERR_INVALID, "out must not be NULL");
        *out = nullptr;
        if (!visibility || !throughput || !grid || !p) throw Error(NLOD_ERR_INVALID, "modules, grid and params must not be NULL");
        validate(*p);
        if (nlod_n_input_dims(visibility) != 6 || nlod_n_output_dims(visibility) != 1)
            throw Error(NLOD_ERR_INVALID, "the visibility module must map 6 inputs to 1 output");
        if (nlod_n_input_dims(throughput) != 10 || nlod_n_output_dims(throughput) != 3)
            throw Error(NLOD_ERR_INVALID, "the throughput module must map 10 inputs to 3 outputs");
        if (p->level >= grid->n_levels) throw Error(NLOD_ERR_INVALID, "level out of range");
        std::unique_ptr<nlod_renderer> r(new nlod_renderer());
        try {
            r->vis = visibility;
            r->thr = throughput;
            RenderConsts& C = r->C;
            C.L = grid->levels[p->level];
            C.width = p->width;
            C.height = p->height;
            C.n_rays = p->width * p->height;
            float cam[12];
            camera_basis(*p, (float)C.L.res, cam);
            for (int k = 0; k < 3; ++k) {
                C.cam_o[k] = cam[k];
                C.cam_u[k] = cam[3 + k];
                C.cam_v[k] = cam[6 + k];
                C.cam_w[k] = cam[9 + k];
                C.background[k] = p->background[k];
                C.env[k] = p->env_color[k];
            }
            C.max_depth = p->max_depth;
            C.max_vis = p->max_vis_queries;
            C.threshold = p->threshold;
            C.res = (float)C.L.res;
            C.lod_input = p->lod_input;
            C.seed_lo = (uint32_t)p->seed;
            C.seed_hi = (uint32_t)(p->seed >> 32);
            C.budget = 64u * (uint32_t)C.L.res + 4096u;
            C.max_rounds = p->max_depth * (p->max_vis_queries + 2u) + 4u;
            r->vis_max_level = p->lod_max_level;
            const uint32_t n = C.n_rays;
            r->n_pad = (n + 127u) / 128u * 128u;
            auto alloc = [&](size_t bytes) {
                void* q = dev_alloc<uint8_t>(bytes);
                r->owned.push_back(q);
                cuda_check(cudaMemset(q, 0, bytes), "memset");
                return q;
            };
            RenderBufs& B = r->B;
            B.rays = static_cast<RayState*>(alloc(sizeof(RayState) * n));
            B.lists = static_cast<uint32_t*>(alloc(sizeof(uint32_t) * 4 * (size_t)n));
            B.ctl = static_cast<Control*>(alloc(sizeof(Control)));
            B.vis_in = static_cast<float*>(alloc(sizeof(float) * 6 * (size_t)r->n_pad));
            B.vis_out = static_cast<float*>(alloc(sizeof(float) * (size_t)r->n_pad));
            B.thr_in = static_cast<float*>(alloc(sizeof(float) * 10 * (size_t)r->n_pad));
            B.thr_out = static_cast<float*>(alloc(sizeof(float) * 3 * (size_t)r->n_pad));
            B.image = static_cast<float*>(alloc(sizeof(float) * 3 * (size_t)n));
            B.ray_stats = static_cast<uint32_t*>(alloc(sizeof(uint32_t) * 2 * (size_t)n));
            B.status = static_cast<uint32_t*>(alloc(sizeof(uint32_t)));
            cuda_check(cudaStreamCreateWithFlags(&r->cap_stream, cudaStreamNonBlocking), "stream");
            cudaStream_t s = r->cap_stream;
            // One launch of each inference with zero rows (outside any capture): sets the kernels'
            // shared-memory attributes before the graph is recorded.
            cuda_check(module_inference_device_count(r->vis, r->n_pad, B.vis_in, B.vis_out, &B.ctl->n_vis, r->vis_max_level, s), "inference");
            cuda_check(module_inference_device_count(r->thr, r->n_pad, B.thr_in, B.thr_out, &B.ctl->n_thr, 1000.f, s), "inference");
            cuda_check(cudaStreamSynchronize(s), "synchronize");

            // ---- the frame graph: reset, ray generation, then rounds in a conditional while node ----
            const unsigned blocks = (unsigned)std::min<uint64_t>((n + 255) / 256, 152ull * 8);
            cuda_check(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal), "capture");
            k_reset<<<1, 1, 0, s>>>(B.ctl);
            k_step<<<blocks, 256, 0, s>>>(C, B, 1);
            k_round<<<1, 1, 0, s>>>(B.ctl, C.max_rounds, B.status, 0, 0);
            cudaStreamCaptureStatus cst;
            cudaGraph_t cap_graph = nullptr;
            const cudaGraphNode_t* deps = nullptr;
            size_t n_deps = 0;
            cuda_check(cudaStreamGetCaptureInfo(s, &cst, nullptr, &cap_graph, &deps, nullptr, &n_deps), "capture info");
            cudaGraphConditionalHandle cond;
            cuda_check(cudaGraphConditionalHandleCreate(&cond, cap_graph, 1, cudaGraphCondAssignDefault), "conditional handle");
            cudaGraphNodeParams cp{};
            cp.type = cudaGraphNodeTypeConditional;
            cp.conditional.handle = cond;
            cp.conditional.type = cudaGraphCondTypeWhile;
            cp.conditional.size = 1;
            cudaGraphNode_t loop_node;
            cuda_check(cudaGraphAddNode(&loop_node, cap_graph, deps, nullptr, n_deps, &cp), "conditional node");
            cuda_check(cudaStreamUpdateCaptureDependencies(s, &loop_node, nullptr, 1, cudaStreamSetCaptureDependencies), "capture deps");
            cudaGraph_t body = cp.conditional.phGraph_out[0];
            cudaStream_t bs;
            cuda_check(cudaStreamCreateWithFlags(&bs, cudaStreamNonBlocking), "stream");
            cudaError_t e = cudaStreamBeginCaptureToGraph(bs, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
            if (e == cudaSuccess) {
                e = module_inference_device_count(r->vis, r->n_pad, B.vis_in, B.vis_out, &B.ctl->n_vis, r->vis_max_level, bs);
                if (e == cudaSuccess) e = module_inference_device_count(r->thr, r->n_pad, B.thr_in, B.thr_out, &B.ctl->n_thr, 1000.f, bs);
                if (e == cudaSuccess) {
                    k_step<<<blocks, 256, 0, bs>>>(C, B, 0);
                    k_round<<<1, 1, 0, bs>>>(B.ctl, C.max_rounds, B.status, cond, 1);
                    e = cudaGetLastError();
                }
                cudaGraph_t body_out = body;
                const cudaError_t e2 = cudaStreamEndCapture(bs, &body_out);
                if (e == cudaSuccess) e = e2;
            }
            cudaStreamDestroy(bs);
            cudaGraph_t g = nullptr;
            const cudaError_t e3 = cudaStreamEndCapture(s, &g);
            r->graph = g;
            cuda_check(e, "frame graph body");
            cuda_check(e3, "frame graph");
            cuda_check(cudaGraphInstantiate(&r->exec, r->graph, 0), "graph instantiate");
        } catch (...) {
            nlod_renderer_destroy(r.release());
            throw;
        }
        *out = r.release();
    });
}

int nlod_render_frame(nlod_renderer* r, void* stream, float* image, uint32_t* ray_stats) {
    return guarded([&] {
        if (!r) throw Error(NLOD_ERR_INVALID, "renderer is NULL");
        cudaStream_t s = (cudaStream_t)stream;
        cuda_check(cudaGraphLaunch(r->exec, s), "graph launch");
        if (image)
            cuda_check(cudaMemcpyAsync(image, r->B.image, sizeof(float) * 3 * (size_t)r->C.n_rays, cudaMemcpyDeviceToDevice, s), "copy image");
        if (ray_stats)
            cuda_check(cudaMemcpyAsync(ray_stats, r->B.ray_stats, sizeof(uint32_t) * 2 * (size_t)r->C.n_rays, cudaMemcpyDeviceToDevice, s),
                       "copy stats");
    });
}

int nlod_render_stats(nlod_renderer* r, void* stream, uint64_t* out4) {
    return guarded([&] {
        if (!r || !out4) throw Error(NLOD_ERR_INVALID, "renderer and output must not be NULL");
        Control c;
        uint32_t st = 0;
        cuda_check(cudaStreamSynchronize((cudaStream_t)stream), "synchronize");
        cuda_check(cudaMemcpy(&c, r->B.ctl, sizeof c, cudaMemcpyDeviceToHost), "copy");
        cuda_check(cudaMemcpy(&st, r->B.status, sizeof st, cudaMemcpyDeviceToHost), "copy");
        out4[0] = c.tot_vis;
        out4[1] = c.tot_thr;
        out4[2] = c.tot_rounds;
        out4[3] = c.dropped;
        if (st) {
            cuda_check(cudaMemset(r->B.status, 0, sizeof st), "status");
            throw Error(NLOD_ERR_TIMEOUT, (st & 4u) ? "the frame exceeded its round bound" : "a ray exceeded its traversal step budget");
        }
    });
}

}  // extern "C"
