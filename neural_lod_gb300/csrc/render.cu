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
// the next launch.  Here every ray advances independently, and one round is four launches:
// visibility inference and throughput inference over the current lists (the tensor-core kernels
// read their row count from device memory), k_step (resolve every queued ray: apply its chain of
// visibility values up to the first accepted one, apply a throughput result and bounce, march the
// next chain of occupied voxels with the bit-exact DDA, append the ray and its query rows to the
// compacted lists with warp-aggregated atomics) and k_round (publish the list sizes, set the next
// chain length and the loop condition).  The rounds run inside a CUDA graph as the body of a
// conditional while node, so a frame is one graph launch with no host round trip; the loop ends
// when both lists are empty (bounded by construction: each round moves every live ray at least
// one query forward).  A chain of visibility queries marched ahead (k_step) takes a ray through
// several rejected voxels per round, so a frame whose voxels are mostly rejected needs a few
// rounds instead of one per voxel.
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
#include "render_common.cuh"
#include "render_pk.h"

struct nlod_module;

namespace nlod {

cudaError_t module_inference_device_count(nlod_module* m, uint32_t n_max, const float* in, float* out, const uint32_t* n_dev,
                                          float max_level, cudaStream_t s, int variant = -1);
int module_variant(nlod_module* m);
bool module_variant_ok(nlod_module* m, int variant);
bool module_tc_operands(nlod_module* m, const ModelDesc** d, const void** weights, const void** table, int* kind);
cudaError_t module_prepare_inference(nlod_module* m, cudaStream_t s);

namespace {

using namespace render;

struct RenderBufs {
    RayState* rays;
    uint32_t* lists;      // [2 parity][2 kind][n_rays]
    Control* ctl;
    float* vis_in;        // [max_chain * n_pad][6]
    float* vis_out;       // [max_chain * n_pad][1]
    float* thr_in;        // [n_pad][10]
    float* thr_out;       // [n_pad][3]
    float* image;         // [n_rays][3]
    uint32_t* ray_stats;  // [n_rays][2]
    uint32_t* status;
    int4* chain_q;        // [max_chain][n_rays] a chain's queries: voxel, t_near bits
    float* chain_t;       // [max_chain][n_rays] their t_far
    uint32_t* vis_row0;   // [2 parity][n_rays] first visibility row of each visibility-list entry
};

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

// Reserves n consecutive slots for each lane; returns the lane's first.  All lanes call.
__device__ __forceinline__ uint32_t push_n(uint32_t* counter, uint32_t n) {
    const uint32_t lane = threadIdx.x & 31u;
    uint32_t incl = n;
#pragma unroll
    for (uint32_t o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(kFull, incl, o);
        if (lane >= o) incl += t;
    }
    const uint32_t total = __shfl_sync(kFull, incl, 31);
    uint32_t base = 0;
    if (lane == 31u && total) base = atomicAdd(counter, total);
    return __shfl_sync(kFull, base, 31) + incl - n;
}

__device__ __forceinline__ uint32_t warp_sum(uint32_t v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
    return v;
}

enum : int { ACT_NONE_ = 0, ACT_VIS = 1, ACT_THR = 2 };

// How a ray's chain of visibility queries ended (RayState::pad bits 8-15): open (the chain
// reached its length; the ray marches on if every query is rejected) or the outcome of the
// march after its last query, applied when every query of the chain is rejected.
enum : uint32_t { CHAIN_OPEN = 0, CHAIN_DONE = 1, CHAIN_DROPPED = 2, CHAIN_FAIL = 3 };

// Throughput lists shorter than this are carried over (k_round), at most this many rounds in a
// row (divided by the round's chain length).
constexpr uint32_t kThrDeferBelow = 32768u;
constexpr uint32_t kThrDeferRounds = 8u;

// The pixel that ray generation's thread j takes: strips of four rows, each walked column by
// column, so that a warp's 32 rays cover 8 x 4 pixels (their directions, and with them the
// distances they march, are closer than along 32 pixels of one row).  The ray's index stays its
// pixel's, which keys its image entry, counts and sampled directions, so the order changes
// nothing but the lists' initial order.  Frame (1024^2): 6.33 ms with one row, 6.23 ms with
// strips of 4 rows, 6.41 / 6.58 / 6.66 ms with 8 / 16 / 32.
constexpr uint32_t kStripRows = 4u;
__device__ __forceinline__ uint32_t tiled_pixel(const RenderConsts& C, uint32_t j) {
    const uint32_t strip = j / (kStripRows * C.width);
    const uint32_t rows = min(kStripRows, C.height - kStripRows * strip);
    const uint32_t idx = j - strip * kStripRows * C.width;
    return (kStripRows * strip + idx % rows) * C.width + idx / rows;
}

// The end of a march that produced no query: the escaped ray's pixel, a dropped ray or a failed
// traversal.
__device__ __forceinline__ void march_end(const RenderConsts& C, const RenderBufs& B, const RayState& st, uint32_t ray, uint32_t end) {
    if (end == CHAIN_DONE) write_escape(C, st, B.image + 3 * (size_t)ray);
    else if (end == CHAIN_DROPPED) atomicAdd(&B.ctl->dropped, 1u);
    else atomicOr(B.status, 2u);
}

// One round for every queued ray (first = true: ray generation, every pixel's ray).
//
// Query chains.  A ray that marches marches up to `chain` visibility queries ahead: query i+1 is
// the march that follows query i's rejection (from t_min = query i's middle, query i's voxel
// excluded), exactly the march the ray would make in the next round after that rejection.  The
// next round applies the chain's values in order and stops at the first accepted one; the later
// queries of the chain are dropped, with their query counts.  So every ray takes the same steps as
// with one query per round, in fewer rounds; a chain costs the queries past an acceptance, and
// k_round sets the chain length from the fraction of accepted values.
// Four 256-thread blocks per SM at 64 registers (ptxas spills about 30 words; three blocks at
// 85 registers without spills render the 1024^2 frame no faster).
__global__ void __launch_bounds__(256, 4) k_step(const __grid_constant__ RenderConsts C, RenderBufs B, int first) {
    const uint32_t round = first ? 0u : B.ctl->round;
    const uint32_t p = (round + 1u) & 1u, q = round & 1u;   // lists read / written
    const uint32_t nv = first ? C.n_rays : B.ctl->n_vis;
    const uint32_t total = first ? C.n_rays : nv + B.ctl->n_thr;
    // the throughput list was not evaluated this round: its rays go unchanged into the next list
    const bool thr_carried = !first && B.ctl->thr_rows == 0u;
    const uint32_t chain = first ? 1u : max(B.ctl->chain, 1u);
    const size_t n = C.n_rays;
    __shared__ uint32_t s_used, s_accepted;   // visibility values applied / accepted by the block
    if (threadIdx.x == 0) s_used = s_accepted = 0u;
    __syncthreads();
    for (uint32_t base = blockIdx.x * blockDim.x; base < total; base += gridDim.x * blockDim.x) {
        const uint32_t j = base + threadIdx.x;
        const bool valid = j < total;
        int act = ACT_NONE_;
        bool carried = false;
        uint32_t ray = 0, kr = 0, n_used = 0, n_accepted = 0;
        RayState st;
        if (valid) {
            bool march = false;
            if (first) {
                ray = tiled_pixel(C, j);
                ray_generate(C, ray, st);
#pragma unroll
                for (int k = 0; k < 3; ++k) B.image[3 * ray + k] = 0.f;
                B.ray_stats[2 * ray] = 0u;
                B.ray_stats[2 * ray + 1] = 0u;
                march = true;
            } else if (j < nv) {
                ray = B.lists[(p * 2 + 0) * n + j];
                st = B.rays[ray];
                const uint32_t row0 = B.vis_row0[p * n + j];
                const uint32_t pending = st.pad & 0xFFu, end = (st.pad >> 8) & 0xFFu;
                // the chain's last query is the state's own; the earlier ones are in chain_q / chain_t
                const int32_t li = st.ijk[0], lj = st.ijk[1], lk = st.ijk[2];
                const float ln = st.tnear, lf = st.tfar;
                int vr = VIS_REJECT;
                uint32_t used = 0;
                while (used < pending && vr == VIS_REJECT) {
                    if (used + 1u < pending) {
                        const int4 a = B.chain_q[used * n + ray];
                        st.ijk[0] = a.x;
                        st.ijk[1] = a.y;
                        st.ijk[2] = a.z;
                        st.tnear = __int_as_float(a.w);
                        st.tfar = B.chain_t[used * n + ray];
                    } else {
                        st.ijk[0] = li;
                        st.ijk[1] = lj;
                        st.ijk[2] = lk;
                        st.tnear = ln;
                        st.tfar = lf;
                    }
                    vr = vis_resolve(C, st, ray, B.vis_out[row0 + used]);
                    ++used;
                }
                n_used = used;
                n_accepted = vr != VIS_REJECT;
                st.meta -= (pending - used) << 8;   // the queries past the accepted one are not taken
                st.pad = 0u;
                B.ray_stats[2 * ray] += used;
                if (vr == VIS_ACCEPT_THR) act = ACT_THR;
                else if (vr == VIS_REJECT) {
                    if (end == CHAIN_OPEN) march = true;
                    else march_end(C, B, st, ray, end);
                }
            } else {
                const uint32_t jj = j - nv;
                ray = B.lists[(p * 2 + 1) * n + jj];
                st = B.rays[ray];
                if (thr_carried) {
                    act = ACT_THR;
                    carried = true;
                } else {
                    const float t[3] = {B.thr_out[3 * jj], B.thr_out[3 * jj + 1], B.thr_out[3 * jj + 2]};
                    march = thr_resolve(st, t);
                }
            }
            if (march) {
                st.pad = 0u;
                for (; kr < chain; ++kr) {
                    if (kr) st.tmin = past_voxel(st);   // the march after the previous query's rejection
                    const int mr = march_query(C, st);
                    if (mr == MARCH_VIS) {
                        // a query that another one may follow is also kept in chain_q / chain_t
                        if (kr + 1u < chain) {
                            B.chain_q[(size_t)kr * C.n_rays + ray] = make_int4(st.ijk[0], st.ijk[1], st.ijk[2], __float_as_int(st.tnear));
                            B.chain_t[(size_t)kr * C.n_rays + ray] = st.tfar;
                        }
                        continue;
                    }
                    const uint32_t end = mr == MARCH_DONE ? CHAIN_DONE : mr == MARCH_DROPPED ? CHAIN_DROPPED : CHAIN_FAIL;
                    if (kr == 0) march_end(C, B, st, ray, end);   // no query pending: the ray ends now
                    else st.pad = end << 8;
                    break;
                }
                if (kr) {
                    act = ACT_VIS;
                    st.pad |= kr;
                }
            }
        }
        const uint32_t slot_v = push(&B.ctl->cnt[q * 2 + 0], act == ACT_VIS);
        const uint32_t row_v = push_n(&B.ctl->rows[q], act == ACT_VIS ? kr : 0u);
        const uint32_t slot_t = push(&B.ctl->cnt[q * 2 + 1], act == ACT_THR);
        if (act == ACT_VIS) {
            B.lists[(q * 2 + 0) * n + slot_v] = ray;
            B.vis_row0[q * n + slot_v] = row_v;
            // the chain's input rows: the earlier queries from chain_q, the last from the state
            for (uint32_t i = 0; i + 1u < kr; ++i) {
                const int4 a = B.chain_q[i * n + ray];
                const int32_t v[3] = {a.x, a.y, a.z};
                vis_row_at(st, v, __int_as_float(a.w), B.vis_in + 6 * (size_t)(row_v + i));
            }
            vis_row(st, B.vis_in + 6 * (size_t)(row_v + kr - 1u));
        } else if (act == ACT_THR) {
            B.lists[(q * 2 + 1) * n + slot_t] = ray;
            thr_row(C, st, B.thr_in + 10 * (size_t)slot_t);
            if (!carried) B.ray_stats[2 * ray + 1] += 1u;
        }
        if (valid) B.rays[ray] = st;
        n_used = warp_sum(n_used);
        n_accepted = warp_sum(n_accepted);
        if ((threadIdx.x & 31u) == 0u && n_used) {
            atomicAdd(&s_used, n_used);
            atomicAdd(&s_accepted, n_accepted);
        }
    }
    __syncthreads();
    if (threadIdx.x == 0 && s_used) {
        atomicAdd(&B.ctl->consumed, s_used);
        atomicAdd(&B.ctl->accepted, s_accepted);
    }
}

// Publishes the lists built this round, resets the other parity, sets the next round's chain
// length and the loop condition.
// use_cond: the launch is the loop body's (graph form): it sets the loop condition and the
// condition of the next round's throughput inference (skipped in rounds that carry the list over
// or have none).
__global__ void k_round(Control* ctl, uint32_t max_rounds, uint32_t max_chain, uint32_t* status, cudaGraphConditionalHandle cond,
                        cudaGraphConditionalHandle thr_cond, int use_cond) {
    const uint32_t q = ctl->round & 1u;
    const uint32_t nv = ctl->cnt[q * 2 + 0], nt = ctl->cnt[q * 2 + 1];
    // Chain length: the queries past an accepted one are evaluated for nothing.  With a fraction a
    // of accepted values, a chain of c queries evaluates about (c - 1) a / 2 of them in vain; the
    // chain is the longest power of two up to max_chain that keeps this at 1/32, from the last
    // round's values (kept when that round resolved too few to tell).
    const uint32_t used = ctl->consumed, acc = ctl->accepted;
    uint32_t chain = ctl->chain ? ctl->chain : 1u;
    if (used >= 1024u) {
        chain = 1u;
        while (chain * 2u <= max_chain && (uint64_t)(chain * 2u - 1u) * acc * 16u <= used) chain *= 2u;
    }
    ctl->chain = min(chain, max_chain);
    ctl->tot_vis += used;
    ctl->consumed = 0u;
    ctl->accepted = 0u;
    // A short throughput list waits for more rows instead of paying a whole inference launch for a
    // few of them (a launch costs about as much for one tile as for a few hundred): it is carried
    // into the next round, at most kThrDeferRounds / chain rounds in a row and only while
    // visibility queries keep the rounds going.  A carried ray's state and queries are unchanged,
    // so every ray takes the same steps; only the round it takes them in moves.
    const uint32_t defer_rounds = kThrDeferRounds / ctl->chain;
    const bool defer = nt > 0u && nt < kThrDeferBelow && nv > 0u && ctl->thr_deferred < defer_rounds;
    ctl->n_vis = nv;
    ctl->n_thr = nt;
    ctl->n_rows = ctl->rows[q];
    ctl->tot_rows += ctl->rows[q];
    ctl->thr_rows = defer ? 0u : nt;
    ctl->thr_deferred = defer ? ctl->thr_deferred + 1u : 0u;
    ctl->tot_thr += defer ? 0u : nt;
    ctl->tot_rounds += 1;
    ctl->cnt[(q ^ 1u) * 2 + 0] = 0u;
    ctl->cnt[(q ^ 1u) * 2 + 1] = 0u;
    ctl->rows[q ^ 1u] = 0u;
    ctl->round += 1u;
    bool more = nv + nt > 0;
    if (more && ctl->round > max_rounds) {
        atomicOr(status, 4u);
        more = false;
    }
    if (use_cond) {
        cudaGraphSetConditional(cond, more ? 1u : 0u);
        cudaGraphSetConditional(thr_cond, ctl->thr_rows > 0u ? 1u : 0u);
    }
}

__global__ void k_reset(Control* ctl) {
    Control c{};
    *ctl = c;
}

// Appends to the graph being captured on `s` a conditional node of `type` (its condition set by
// kernels of that graph; no value is assigned at launch) whose body is what `body(stream)`
// records, and makes it the capture's next dependency.
template <typename Body>
cudaError_t add_conditional_body(cudaStream_t s, cudaGraphConditionalNodeType type, cudaGraphConditionalHandle* handle, Body&& body) {
    cudaStreamCaptureStatus cst;
    cudaGraph_t g = nullptr;
    const cudaGraphNode_t* deps = nullptr;
    size_t n_deps = 0;
    cudaError_t e = cudaStreamGetCaptureInfo(s, &cst, nullptr, &g, &deps, nullptr, &n_deps);
    if (e != cudaSuccess) return e;
    e = cudaGraphConditionalHandleCreate(handle, g, 0, 0);
    if (e != cudaSuccess) return e;
    cudaGraphNodeParams cp{};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = *handle;
    cp.conditional.type = type;
    cp.conditional.size = 1;
    cudaGraphNode_t node;
    e = cudaGraphAddNode(&node, g, deps, nullptr, n_deps, &cp);
    if (e != cudaSuccess) return e;
    e = cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1, cudaStreamSetCaptureDependencies);
    if (e != cudaSuccess) return e;
    cudaGraph_t inner = cp.conditional.phGraph_out[0];
    cudaStream_t bs;
    e = cudaStreamCreateWithFlags(&bs, cudaStreamNonBlocking);
    if (e != cudaSuccess) return e;
    e = cudaStreamBeginCaptureToGraph(bs, inner, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        e = body(bs);
        cudaGraph_t out = inner;
        const cudaError_t e2 = cudaStreamEndCapture(bs, &out);
        if (e == cudaSuccess) e = e2;
    }
    cudaStreamDestroy(bs);
    return e;
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
    uint32_t vis_rows_max = 0;      // visibility rows of the wavefront forms' buffers
    float vis_max_level = 1000.f;
    int mode = NLOD_RENDER_WAVEFRONT;
    int pk_groups = 0;              // tile pipelines per CTA of the persistent form (autotuned)
    int vis_variant = -1, thr_variant = -1;   // the wavefront forms' inference organisations (-1: the module's)
    unsigned step_blocks = 0;       // k_step grid of the wavefront forms
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
    if (p.max_chain > 64) throw Error(NLOD_ERR_INVALID, "max_chain must be in [0, 64]");
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
            C.max_rounds = p->max_depth * (p->max_vis_queries + 2u + kThrDeferRounds) + 4u;
            r->vis_max_level = p->lod_max_level;
            const uint32_t n = C.n_rays;
            r->n_pad = (n + 127u) / 128u * 128u;
            // ---- the persistent form, when both modules are tensor-core modules of one type ----
            const ModelDesc *dv = nullptr, *dt = nullptr;
            PkArgs pk{};
            int kv = 0, kt = 0, groups = 0;
            const bool tc_v = module_tc_operands(visibility, &dv, &pk.vis.weights_op, &pk.vis.table, &kv);
            const bool tc_t = module_tc_operands(throughput, &dt, &pk.thr.weights_op, &pk.thr.table, &kt);
            int candidates[4] = {0, 0, 0, 0}, n_candidates = 0;
            if (tc_v && tc_t && kv == kt) {
                for (int g : {kWsForm16, kWsForm8, 4, 6})
                    if (render_pk_supported(*dv, *dt, g)) candidates[n_candidates++] = g;
            }
            if ((p->mode & 0x100u) != 0) {
                // one organisation forced
                const int f = (int)(p->mode & 0xFFu);
                bool ok = false;
                for (int i = 0; i < n_candidates; ++i) ok |= candidates[i] == f;
                if (!ok) throw Error(NLOD_ERR_UNSUPPORTED, "persistent organisation " + std::to_string(f) + " is not available for these modules");
                candidates[0] = f;
                n_candidates = 1;
            } else if (p->mode != NLOD_RENDER_AUTO && p->mode != NLOD_RENDER_WAVEFRONT && p->mode != NLOD_RENDER_PERSISTENT &&
                       p->mode != NLOD_RENDER_HOST_ROUNDS) {
                throw Error(NLOD_ERR_INVALID, "unknown render mode");
            }
            const bool wavefront = p->mode == NLOD_RENDER_WAVEFRONT || p->mode == NLOD_RENDER_HOST_ROUNDS;
            if (n_candidates && !wavefront) groups = candidates[0];
            if (p->mode != NLOD_RENDER_AUTO && !wavefront && !groups)
                throw Error(NLOD_ERR_UNSUPPORTED, "the persistent form needs two tensor-core modules of one operand type with "
                                                  "64-wide networks of 6 and 10 inputs");
            if (!wavefront && groups) {
                auto alloc = [&](size_t bytes) {
                    void* q = dev_alloc<uint8_t>(bytes);
                    r->owned.push_back(q);
                    cuda_check(cudaMemset(q, 0, bytes), "memset");
                    return q;
                };
                RenderBufs& B = r->B;
                B.ctl = static_cast<Control*>(alloc(sizeof(Control)));
                B.image = static_cast<float*>(alloc(sizeof(float) * 3 * (size_t)n));
                B.ray_stats = static_cast<uint32_t*>(alloc(sizeof(uint32_t) * 2 * (size_t)n));
                B.status = static_cast<uint32_t*>(alloc(sizeof(uint32_t)));
                pk.C = C;
                pk.vis.max_level = p->lod_max_level;
                pk.thr.max_level = 1000.f;
                pk.image = B.image;
                pk.ray_stats = B.ray_stats;
                pk.ctl = B.ctl;
                pk.status = B.status;
                cuda_check(cudaStreamCreateWithFlags(&r->cap_stream, cudaStreamNonBlocking), "stream");
                cudaStream_t s = r->cap_stream;
                // Autotune: one frame per supported pipeline count, outside any capture (which also
                // sets the kernels' shared-memory attributes); the fastest is captured.
                float best = 0.f;
                cudaEvent_t e0, e1;
                cuda_check(cudaEventCreate(&e0), "event");
                cuda_check(cudaEventCreate(&e1), "event");
                for (int i = 0; i < n_candidates; ++i) {
                    cuda_check(launch_render_pk(*dv, *dt, pk, kv, candidates[i], s), "persistent frame");   // warm-up
                    cuda_check(cudaEventRecord(e0, s), "event");
                    cuda_check(launch_render_pk(*dv, *dt, pk, kv, candidates[i], s), "persistent frame");
                    cuda_check(cudaEventRecord(e1, s), "event");
                    cuda_check(cudaEventSynchronize(e1), "synchronize");
                    float ms = 0.f;
                    cuda_check(cudaEventElapsedTime(&ms, e0, e1), "event");
                    if (i == 0 || ms < best) {
                        best = ms;
                        groups = candidates[i];
                    }
                }
                cudaEventDestroy(e0);
                cudaEventDestroy(e1);
                r->pk_groups = groups;
                r->mode = NLOD_RENDER_PERSISTENT_FORM(groups);
                cuda_check(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal), "capture");
                const cudaError_t e = launch_render_pk(*dv, *dt, pk, kv, groups, s);
                cudaGraph_t g = nullptr;
                const cudaError_t e2 = cudaStreamEndCapture(s, &g);
                r->graph = g;
                cuda_check(e, "persistent frame graph");
                cuda_check(e2, "persistent frame graph");
                cuda_check(cudaGraphInstantiate(&r->exec, r->graph, 0), "graph instantiate");
                if (p->mode == NLOD_RENDER_AUTO) {
                    // The automatic choice also times the wavefront form on this scene and keeps
                    // whichever frame is faster (one timed frame of each graph after a warm-up).
                    nlod_render_params pw = *p;
                    pw.mode = NLOD_RENDER_WAVEFRONT;
                    nlod_renderer* wf = nullptr;
                    if (nlod_renderer_create(visibility, throughput, grid, &pw, &wf) == NLOD_OK) {
                        auto frame_ms = [&](cudaGraphExec_t x) {
                            cudaEvent_t a0, a1;
                            float ms = 3.0e38f;
                            if (cudaEventCreate(&a0) != cudaSuccess) return ms;
                            if (cudaEventCreate(&a1) == cudaSuccess) {
                                if (cudaGraphLaunch(x, s) == cudaSuccess && cudaEventRecord(a0, s) == cudaSuccess &&
                                    cudaGraphLaunch(x, s) == cudaSuccess && cudaEventRecord(a1, s) == cudaSuccess &&
                                    cudaEventSynchronize(a1) == cudaSuccess)
                                    cudaEventElapsedTime(&ms, a0, a1);
                                cudaEventDestroy(a1);
                            }
                            cudaEventDestroy(a0);
                            return ms;
                        };
                        const float ms_pk = frame_ms(r->exec), ms_wf = frame_ms(wf->exec);
                        cuda_check(cudaStreamSynchronize(s), "synchronize");
                        if (ms_wf < ms_pk) {
                            nlod_renderer_destroy(r.release());
                            *out = wf;
                            return;
                        }
                        nlod_renderer_destroy(wf);
                    }
                }
                *out = r.release();
                return;
            }
            auto alloc = [&](size_t bytes) {
                void* q = dev_alloc<uint8_t>(bytes);
                r->owned.push_back(q);
                cuda_check(cudaMemset(q, 0, bytes), "memset");
                return q;
            };
            RenderBufs& B = r->B;
            // query chains of up to max_chain (0: 8) visibility queries per ray, within 2^23 rows
            C.max_chain = std::max<uint32_t>(1u, std::min<uint32_t>(p->max_chain ? p->max_chain : 8u, (1u << 23) / r->n_pad));
            const size_t vis_cap = (size_t)C.max_chain * r->n_pad;
            r->vis_rows_max = (uint32_t)vis_cap;
            B.rays = static_cast<RayState*>(alloc(sizeof(RayState) * n));
            B.lists = static_cast<uint32_t*>(alloc(sizeof(uint32_t) * 4 * (size_t)n));
            B.ctl = static_cast<Control*>(alloc(sizeof(Control)));
            B.vis_in = static_cast<float*>(alloc(sizeof(float) * 6 * vis_cap));
            B.vis_out = static_cast<float*>(alloc(sizeof(float) * vis_cap));
            B.chain_q = static_cast<int4*>(alloc(sizeof(int4) * C.max_chain * (size_t)n));
            B.chain_t = static_cast<float*>(alloc(sizeof(float) * C.max_chain * (size_t)n));
            B.vis_row0 = static_cast<uint32_t*>(alloc(sizeof(uint32_t) * 2 * (size_t)n));
            B.thr_in = static_cast<float*>(alloc(sizeof(float) * 10 * (size_t)r->n_pad));
            B.thr_out = static_cast<float*>(alloc(sizeof(float) * 3 * (size_t)r->n_pad));
            B.image = static_cast<float*>(alloc(sizeof(float) * 3 * (size_t)n));
            B.ray_stats = static_cast<uint32_t*>(alloc(sizeof(uint32_t) * 2 * (size_t)n));
            B.status = static_cast<uint32_t*>(alloc(sizeof(uint32_t)));
            cuda_check(cudaStreamCreateWithFlags(&r->cap_stream, cudaStreamNonBlocking), "stream");
            cudaStream_t s = r->cap_stream;
            cuda_check(module_prepare_inference(r->vis, s), "inference tables");
            cuda_check(module_prepare_inference(r->thr, s), "inference tables");
            // One launch of each inference with zero rows (outside any capture): sets the kernels'
            // shared-memory attributes before the graph is recorded.
            cuda_check(module_inference_device_count(r->vis, r->vis_rows_max, B.vis_in, B.vis_out, &B.ctl->n_rows, r->vis_max_level, s), "inference");
            cuda_check(module_inference_device_count(r->thr, r->n_pad, B.thr_in, B.thr_out, &B.ctl->thr_rows, 1000.f, s), "inference");
            cuda_check(cudaStreamSynchronize(s), "synchronize");

            // ---- the frame graph: reset, ray generation, then rounds in a conditional while node ----
            // up to 32 blocks per SM (8 waves of 4): rays' marches differ in length, and small
            // blocks balance them (frame 6.41 ms with 8 per SM, 6.33 ms with 32)
            const unsigned blocks = (unsigned)std::min<uint64_t>((n + 255) / 256, 152ull * 32);
            r->step_blocks = blocks;
            if (p->mode == NLOD_RENDER_HOST_ROUNDS) r->mode = NLOD_RENDER_HOST_ROUNDS;
            // Records the frame graph with the given inference organisations into r->graph / r->exec.
            auto capture = [&](int vv, int tv) {
                if (r->exec) cudaGraphExecDestroy(r->exec);
                if (r->graph) cudaGraphDestroy(r->graph);
                r->exec = nullptr;
                r->graph = nullptr;
                r->vis_variant = vv;
                r->thr_variant = tv;
                cuda_check(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal), "capture");
                k_reset<<<1, 1, 0, s>>>(B.ctl);
                k_step<<<blocks, 256, 0, s>>>(C, B, 1);
                k_round<<<1, 1, 0, s>>>(B.ctl, C.max_rounds, C.max_chain, B.status, 0, 0, 0);
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
                    e = module_inference_device_count(r->vis, r->vis_rows_max, B.vis_in, B.vis_out, &B.ctl->n_rows, r->vis_max_level, bs, vv);
                    // the throughput inference inside an if node: most rounds carry its list over
                    // (or have none), and a launch that finds no rows still costs its grid's start-up
                    cudaGraphConditionalHandle thr_cond{};
                    if (e == cudaSuccess) e = add_conditional_body(bs, cudaGraphCondTypeIf, &thr_cond, [&](cudaStream_t ts) {
                        return module_inference_device_count(r->thr, r->n_pad, B.thr_in, B.thr_out, &B.ctl->thr_rows, 1000.f, ts, tv);
                    });
                    if (e == cudaSuccess) {
                        k_step<<<blocks, 256, 0, bs>>>(C, B, 0);
                        k_round<<<1, 1, 0, bs>>>(B.ctl, C.max_rounds, C.max_chain, B.status, cond, thr_cond, 1);
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
            };
            capture(-1, -1);
            if (p->mode != NLOD_RENDER_HOST_ROUNDS && module_variant(r->vis) >= 0 && module_variant(r->thr) >= 0) {
                // The inference organisations for this frame: the modules' own (tuned on batches of
                // their own) against the ones that suit the frame's rounds (four and six pipelines
                // with two and one threads per tile row), one network at a time, each timed on a
                // frame of its graph after a warm-up frame.  The modules' settings are unchanged.
                cudaEvent_t e0, e1;
                cuda_check(cudaEventCreate(&e0), "event");
                cuda_check(cudaEventCreate(&e1), "event");
                auto frame_ms = [&]() {
                    float ms = 3.0e38f;
                    if (cudaGraphLaunch(r->exec, s) == cudaSuccess && cudaEventRecord(e0, s) == cudaSuccess &&
                        cudaGraphLaunch(r->exec, s) == cudaSuccess && cudaEventRecord(e1, s) == cudaSuccess &&
                        cudaEventSynchronize(e1) == cudaSuccess)
                        cudaEventElapsedTime(&ms, e0, e1);
                    return ms;
                };
                const int own_v = module_variant(r->vis), own_t = module_variant(r->thr);
                const uint32_t* no_rows = static_cast<const uint32_t*>(alloc(sizeof(uint32_t)));   // a zero row count
                int best_v = own_v, best_t = own_t;
                float best = frame_ms();
                for (int which = 0; which < 2; ++which) {
                    nlod_module* m = which == 0 ? r->thr : r->vis;
                    const int own = which == 0 ? own_t : own_v;
                    for (int cand : {12, 6}) {
                        if (cand == own || !module_variant_ok(m, cand)) continue;
                        const int vv = which == 0 ? best_v : cand, tv = which == 0 ? cand : best_t;
                        // zero-row launch outside the capture: the kernel's shared-memory attribute
                        cuda_check(module_inference_device_count(m, which == 0 ? r->n_pad : r->vis_rows_max, which == 0 ? B.thr_in : B.vis_in,
                                                                 which == 0 ? B.thr_out : B.vis_out, no_rows, 1000.f, s, cand),
                                   "inference");
                        capture(vv, tv);
                        const float ms = frame_ms();
                        if (ms < best) {
                            best = ms;
                            best_v = vv;
                            best_t = tv;
                        }
                    }
                }
                cudaEventDestroy(e0);
                cudaEventDestroy(e1);
                cuda_check(cudaStreamSynchronize(s), "synchronize");
                if (best_v != r->vis_variant || best_t != r->thr_variant) capture(best_v == own_v ? -1 : best_v, best_t == own_t ? -1 : best_t);
            }
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
        // tables derived from the modules' parameters (rebuilt when a training step changed them)
        cuda_check(module_prepare_inference(r->vis, s), "inference tables");
        cuda_check(module_prepare_inference(r->thr, s), "inference tables");
        if (r->mode == NLOD_RENDER_HOST_ROUNDS) {
            // the graph's rounds, issued from the host: it reads the list sizes after each round
            RenderBufs& B = r->B;
            const RenderConsts& C = r->C;
            k_reset<<<1, 1, 0, s>>>(B.ctl);
            k_step<<<r->step_blocks, 256, 0, s>>>(C, B, 1);
            k_round<<<1, 1, 0, s>>>(B.ctl, C.max_rounds, C.max_chain, B.status, 0, 0, 0);
            cuda_check(cudaGetLastError(), "launch");
            for (;;) {
                Control c;
                cuda_check(cudaMemcpyAsync(&c, B.ctl, sizeof c, cudaMemcpyDeviceToHost, s), "copy");
                cuda_check(cudaStreamSynchronize(s), "synchronize");
                if (c.n_vis + c.n_thr == 0 || c.round > C.max_rounds) break;
                cuda_check(module_inference_device_count(r->vis, r->vis_rows_max, B.vis_in, B.vis_out, &B.ctl->n_rows, r->vis_max_level, s,
                                                         r->vis_variant), "inference");
                cuda_check(module_inference_device_count(r->thr, r->n_pad, B.thr_in, B.thr_out, &B.ctl->thr_rows, 1000.f, s, r->thr_variant),
                           "inference");
                k_step<<<r->step_blocks, 256, 0, s>>>(C, B, 0);
                k_round<<<1, 1, 0, s>>>(B.ctl, C.max_rounds, C.max_chain, B.status, 0, 0, 0);
                cuda_check(cudaGetLastError(), "launch");
            }
        } else {
            cuda_check(cudaGraphLaunch(r->exec, s), "graph launch");
        }
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
            throw Error(NLOD_ERR_TIMEOUT, (st & 8u)   ? "a tensor-core wait of the persistent frame timed out"
                                          : (st & 4u) ? "the frame exceeded its round or time bound"
                                                      : "a ray exceeded its traversal step budget");
        }
    });
}

int nlod_renderer_mode(const nlod_renderer* r) { return r ? r->mode : -1; }

}  // extern "C"
