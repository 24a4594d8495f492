// Persistent form of the neural-LoD render query: one launch renders the whole frame.
//
// Every CTA (one per SM) keeps both networks' weights in shared memory and runs G independent
// four-warp tile pipelines.  A pipeline owns 128 ray slots, one per thread (the thread keeps its
// ray's state in registers), and loops:
//   1. refill: each empty slot takes the next ray id from the frame's queue (warp-aggregated
//      atomics), generates the camera ray and marches it to its first occupied voxel; rays that
//      escape are finished on the spot and the slot takes another;
//   2. visibility pass: the slots with a pending visibility query encode their input rows into
//      the pipeline's A-operand tile and the tile runs through the visibility MLP (tcgen05.mma,
//      M = 128, FP32 accumulate in TMEM; one thread issues, the group drains TMEM); each slot
//      resolves its value: rejected rays march on, accepted rays get a throughput query (or end);
//   3. throughput pass, when any slot has one: the same with the throughput MLP; the ray bounces
//      and marches to its next voxel.
// The pipelines never wait for each other or for other CTAs, and the tiles stay full until the
// queue runs dry (compaction by refilling), so the frame has no per-wavefront launches, no host
// round trips and no global barrier; it is captured in a CUDA graph with its control reset.
// The per-ray steps are those of the wavefront form (render_common.cuh) and the network math is
// that of the tensor-core query kernel (tc.cu), so a ray's queries, values and pixel are the same
// bits in both forms.  Every wait is bounded (mbarrier waits by clock cycles, the frame by the
// global timer) and reports through the status word.
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <type_traits>

#include "desc.h"
#include "encoding.cuh"
#include "kernels.h"
#include "render_common.cuh"
#include "render_pk.h"
#include "tc_common.cuh"
#include "tc_tile.cuh"

namespace nlod {

namespace {

using namespace render;

constexpr int kTile = 128;
constexpr int kGroupThreads = 128;
constexpr int kWidth = 64;
constexpr int kNL = 2;                             // grid levels per gather batch
constexpr uint32_t kInLd = 11;                     // staged input row stride (floats): 10 inputs + 1
constexpr long long kWaitCycles = 4000000000ll;    // ~2 s at 2 GHz per MMA wait
constexpr unsigned long long kFrameNs = 30000000000ull;   // 30 s per frame at most

struct PkLayout {
    uint32_t wv, wt;          // byte offsets of the two networks' weights
    uint32_t lv, lt;          // level tables
    uint32_t groups, group_stride, a_bytes, in_rel;
    uint32_t bar;             // G mbarriers, then the TMEM base address
    uint32_t total;
    uint32_t tmem_cols;
};

__host__ __device__ inline uint32_t up128(uint32_t v) { return (v + 127u) / 128u * 128u; }

__host__ __device__ inline PkLayout pk_layout(const ModelDesc& dv, const ModelDesc& dt, int G) {
    PkLayout L{};
    uint32_t off = 0;
    L.wv = off;
    off += up128(dv.n_params_network * 2u);
    L.wt = off;
    off += up128(dt.n_params_network * 2u);
    L.lv = off;
    off += kMaxGrids * kMaxLevels * (uint32_t)sizeof(GridLevel);
    L.lt = off;
    off += kMaxGrids * kMaxLevels * (uint32_t)sizeof(GridLevel);
    uint32_t ka = dv.enc_width > dt.enc_width ? dv.enc_width : dt.enc_width;
    if (ka < (uint32_t)kWidth) ka = kWidth;
    L.a_bytes = kTile * ka * 2u;
    L.in_rel = up128(L.a_bytes);
    L.group_stride = L.in_rel + up128(kTile * kInLd * 4u);
    L.groups = off;
    off += (uint32_t)G * L.group_stride;
    L.bar = off;
    off += 8u * (uint32_t)G + 8u;
    L.total = up128(off);
    uint32_t cols = 32;
    while (cols < (uint32_t)G * kWidth) cols <<= 1;
    L.tmem_cols = cols;
    return L;
}

// Stores the encoded features of one row (the calling thread's slot) into the A tile.
template <typename T>
struct RowStore {
    TcStore<T> inner;
    uint32_t row;
    template <int M>
    __device__ __forceinline__ void run(uint32_t, uint32_t col, const float (&f)[M], uint32_t n) { inner.run(row, col, f, n); }
    __device__ __forceinline__ void one(uint32_t, uint32_t col, float v) { inner.one(row, col, v); }
};

// Stages one network's weights (row-major [out][in], operand type) into the K-major layout and
// its grid level tables, as the query kernel does.
__device__ __forceinline__ void stage_network(const ModelDesc& d, const void* weights, uint8_t* wdst, GridLevel* ldst, uint32_t tid,
                                              uint32_t nthreads) {
    const uint16_t* wsrc = static_cast<const uint16_t*>(weights);
    for (uint32_t l = 0; l < d.n_layers; ++l) {
        const uint32_t K = d.layer_in[l], N = d.layer_out[l];
        const uint32_t sbo = K * 16u;
        const uint32_t chunks = N * (K / 8u);
        const uint4* src = reinterpret_cast<const uint4*>(wsrc + d.layer_offset[l]);
        for (uint32_t c = tid; c < chunks; c += nthreads) {
            const uint32_t n = c / (K / 8u), k0 = (c - n * (K / 8u)) * 8u;
            *reinterpret_cast<uint4*>(wdst + 2u * d.layer_offset[l] + tc::kmajor_offset(n, k0, sbo)) = src[c];
        }
    }
    for (uint32_t i = tid; i < d.n_grids * (uint32_t)kMaxLevels; i += nthreads) {
        const uint32_t g = i / kMaxLevels, l = i % kMaxLevels;
        if (l < d.grids[g].n_levels) ldst[i] = d.grids[g].levels[l];
    }
}

// Runs the encoded A tile through one network: per layer one thread issues the MMAs and commits
// them to the group's mbarrier, the group drains its TMEM lanes, applies the activation and writes
// the next A operand; the output layer's activated values of the calling thread's row land in out.
// Returns false when an MMA wait timed out (the caller aborts).  Group-uniform.
template <typename T>
__device__ __forceinline__ bool run_mlp(const ModelDesc& d, const uint8_t* w, uint8_t* a_tile, uint32_t a_addr, uint32_t tmem_base,
                                        uint32_t taddr_row, uint64_t* bar, uint32_t& phase, uint32_t bar_id, uint32_t gtid, uint32_t row,
                                        float (&out)[3]) {
    using Op = tc::OpType<T>;
    for (uint32_t l = 0; l < d.n_layers; ++l) {
        const bool last = l + 1 == d.n_layers;
        const uint32_t K = d.layer_in[l];
        const uint32_t N = d.layer_out[l];
        const uint32_t sbo = K * 16u;
        if (gtid == 0) {
            tc::fence_after_sync();
            const uint32_t idesc = tc::make_idesc_f16(Op::kFmt, kTile, N);
            const uint32_t b_addr = tc::smem_addr(w + 2u * d.layer_offset[l]);
            for (uint32_t k = 0; k < K; k += 16) {
                const uint64_t adesc = tc::make_smem_desc(a_addr + (k / 8u) * 128u, 128u, sbo);
                const uint64_t bdesc = tc::make_smem_desc(b_addr + (k / 8u) * 128u, 128u, sbo);
                tc::mma_f16_ss(tmem_base, adesc, bdesc, idesc, k > 0 ? 1u : 0u);
            }
            tc::mma_commit(bar);
        }
        const bool ok = gtid != 0 || tc::mbar_wait_bounded(bar, phase, kWaitCycles);
        phase ^= 1u;
        if (group_sync_or(bar_id, !ok)) return false;
        tc::fence_after_sync();
        if (!last) {
            const uint32_t out_sbo = (uint32_t)kWidth * 16u;
            const ReluOrNone act{d.act == ACT_RELU};
#pragma unroll
            for (uint32_t col = 0; col < (uint32_t)kWidth; col += 32) {
                uint32_t r[32];
                tc::tmem_ld32(taddr_row + col, r);
                tc::tmem_wait_ld();
#pragma unroll
                for (uint32_t j = 0; j < 4; ++j) {
                    uint4 pk;
                    pk.x = Op::pack2(act(__uint_as_float(r[8 * j + 0])), act(__uint_as_float(r[8 * j + 1])));
                    pk.y = Op::pack2(act(__uint_as_float(r[8 * j + 2])), act(__uint_as_float(r[8 * j + 3])));
                    pk.z = Op::pack2(act(__uint_as_float(r[8 * j + 4])), act(__uint_as_float(r[8 * j + 5])));
                    pk.w = Op::pack2(act(__uint_as_float(r[8 * j + 6])), act(__uint_as_float(r[8 * j + 7])));
                    *reinterpret_cast<uint4*>(a_tile + tc::kmajor_offset(row, col + 8u * j, out_sbo)) = pk;
                }
            }
            tc::fence_proxy_async_smem();
        } else {
            uint32_t r[16];
            tc::tmem_ld16(taddr_row, r);
            tc::tmem_wait_ld();
#pragma unroll
            for (uint32_t c = 0; c < 3; ++c) out[c] = c < d.n_output ? act_fwd(d.out_act, __uint_as_float(r[c])) : 0.f;
        }
        tc::fence_before_sync();
        group_sync(bar_id);
    }
    return true;
}

enum : int { SLOT_EMPTY = 0, SLOT_VIS = 1, SLOT_THR = 2 };

__device__ __forceinline__ unsigned long long globaltimer_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

template <typename T, int G>
__global__ void __launch_bounds__(G * kGroupThreads, 1)
    k_render_pk(const __grid_constant__ ModelDesc dv, const __grid_constant__ ModelDesc dt, const __grid_constant__ PkArgs A) {
    using TT = typename std::conditional<std::is_same<T, __half>::value, __half, float>::type;   // grid table type
    constexpr int kThreads = G * kGroupThreads;
    extern __shared__ __align__(1024) uint8_t smem[];
    const PkLayout L = pk_layout(dv, dt, G);
    const RenderConsts& C = A.C;
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + L.bar);
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem + L.bar + 8 * G);

    const uint32_t tid = threadIdx.x;
    const uint32_t warp = tid >> 5, lane = tid & 31;
    const uint32_t grp = warp >> 2;
    const uint32_t gtid = tid & (kGroupThreads - 1);
    const uint32_t quarter = warp & 3u;
    const uint32_t bar_id = 1u + grp;
    const uint32_t row = gtid;                         // the slot, and the tile row, of this thread
    const unsigned long long t_start = globaltimer_ns();

    // ---- set-up: barriers, TMEM, both networks ----
    if (tid == 0) {
        for (int g = 0; g < G; ++g) tc::mbar_init(&bars[g], 1);
        tc::fence_barrier_init();
    }
    if (warp == 0) {
        tc::tmem_alloc(tmem_slot, L.tmem_cols);
        tc::tmem_relinquish();
    }
    GridLevel* lvl_v = reinterpret_cast<GridLevel*>(smem + L.lv);
    GridLevel* lvl_t = reinterpret_cast<GridLevel*>(smem + L.lt);
    stage_network(dv, A.vis.weights_op, smem + L.wv, lvl_v, tid, kThreads);
    stage_network(dt, A.thr.weights_op, smem + L.wt, lvl_t, tid, kThreads);
    tc::fence_proxy_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();

    const uint32_t tmem_base = *tmem_slot + grp * (uint32_t)kWidth;
    const uint32_t taddr_row = tmem_base + ((quarter * 32u) << 16);
    uint8_t* a_tile = smem + L.groups + grp * L.group_stride;
    float* in_row = reinterpret_cast<float*>(a_tile + L.in_rel) + row * kInLd;
    const uint32_t a_addr = tc::smem_addr(a_tile);
    uint64_t* bar = &bars[grp];
    const TT* vtab = static_cast<const TT*>(A.vis.table);
    const TT* ttab = static_cast<const TT*>(A.thr.table);

    uint32_t phase = 0;
    bool aborted = false;
    int state = SLOT_EMPTY;
    bool queue_done = false;
    uint32_t ray = 0, nv_ray = 0, nt_ray = 0;
    RayState st{};
    unsigned long long tot_v = 0, tot_t = 0;
    uint32_t iters = 0;

    // the ray of this slot is finished: its query counts go out
    auto finish = [&]() {
        A.ray_stats[2 * ray] = nv_ray;
        A.ray_stats[2 * ray + 1] = nt_ray;
        state = SLOT_EMPTY;
    };
    // marches the slot's ray; sets up its next visibility query or finishes it
    auto march = [&]() {
        const int mr = ray_march(C, st, A.image + 3 * (size_t)ray);
        if (mr == MARCH_VIS) {
            state = SLOT_VIS;
            ++nv_ray;
            return;
        }
        if (mr == MARCH_DROPPED) atomicAdd(&A.ctl->dropped, 1u);
        else if (mr == MARCH_FAIL) atomicOr(A.status, 2u);
        finish();
    };

    for (;;) {
        // ---- 1. refill empty slots from the frame's ray queue (warp-uniform loop) ----
        for (;;) {
            const bool want = state == SLOT_EMPTY && !queue_done;
            const unsigned m = __ballot_sync(kFull, want);
            if (!m) break;
            const int leader = __ffs(m) - 1;
            uint32_t base = 0;
            if ((int)lane == leader) base = atomicAdd(&A.ctl->cnt[0], (uint32_t)__popc(m));
            base = __shfl_sync(kFull, base, leader);
            if (want) {
                const uint32_t id = base + (uint32_t)__popc(m & ((1u << lane) - 1u));
                if (id >= C.n_rays) {
                    queue_done = true;
                } else {
                    ray = id;
                    nv_ray = nt_ray = 0;
                    ray_generate(C, id, st);
#pragma unroll
                    for (int k = 0; k < 3; ++k) A.image[3 * (size_t)ray + k] = 0.f;
                    march();
                }
            }
        }
        // every slot now has a visibility query, or is empty with the queue exhausted
        const bool timed_out = globaltimer_ns() - t_start > kFrameNs;
        if (group_sync_or(bar_id, timed_out)) {
            if (gtid == 0) atomicOr(A.status, 4u);
            break;
        }
        if (!group_sync_or(bar_id, state == SLOT_VIS)) break;
        ++iters;

        // ---- 2. visibility pass ----
        if (state == SLOT_VIS) {
            vis_row(st, in_row);
            RowStore<T> rs{TcStore<T>{a_tile, dv.enc_width * 16u}, row};
            encode_tile_rows<kNL>(dv, lvl_v, vtab, in_row, kInLd, nullptr, A.vis.max_level, 0, 1, 0, 1, rs);
            ++tot_v;
        }
        tc::fence_proxy_async_smem();
        tc::fence_before_sync();
        group_sync(bar_id);
        float out[3];
        if (!run_mlp<T>(dv, smem + L.wv, a_tile, a_addr, tmem_base, taddr_row, bar, phase, bar_id, gtid, row, out)) {
            aborted = true;
            break;
        }
        if (state == SLOT_VIS) {
            const int vr = vis_resolve(C, st, ray, out[0]);
            if (vr == VIS_ACCEPT_THR) {
                state = SLOT_THR;
                ++nt_ray;
            } else if (vr == VIS_ACCEPT_END) {
                finish();
            } else {
                march();
            }
        }

        // ---- 3. throughput pass, when a slot has a throughput query ----
        if (group_sync_or(bar_id, state == SLOT_THR)) {
            if (state == SLOT_THR) {
                thr_row(C, st, in_row);
                RowStore<T> rs{TcStore<T>{a_tile, dt.enc_width * 16u}, row};
                encode_tile_rows<kNL>(dt, lvl_t, ttab, in_row, kInLd, nullptr, A.thr.max_level, 0, 1, 0, 1, rs);
                ++tot_t;
            }
            tc::fence_proxy_async_smem();
            tc::fence_before_sync();
            group_sync(bar_id);
            if (!run_mlp<T>(dt, smem + L.wt, a_tile, a_addr, tmem_base, taddr_row, bar, phase, bar_id, gtid, row, out)) {
                aborted = true;
                break;
            }
            if (state == SLOT_THR) {
                const float t3[3] = {out[0], out[1], out[2]};
                if (thr_resolve(st, t3)) march();
                else finish();
            }
        }
    }

    // ---- totals, teardown ----
    for (int o = 16; o > 0; o >>= 1) {
        tot_v += __shfl_xor_sync(kFull, tot_v, o);
        tot_t += __shfl_xor_sync(kFull, tot_t, o);
    }
    if (lane == 0) {
        atomicAdd(&A.ctl->tot_vis, tot_v);
        atomicAdd(&A.ctl->tot_thr, tot_t);
        if (gtid == 0) atomicMax(&A.ctl->tot_rounds, (unsigned long long)iters);
    }
    if (aborted) {
        (void)tc::mbar_wait_bounded(bar, phase ^ 1u, kWaitCycles);
        if (gtid == 0) atomicOr(A.status, 8u);
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) {
        tc::fence_after_sync();
        tc::tmem_dealloc(*tmem_slot, L.tmem_cols);
    }
}

// ---- warp-specialized form --------------------------------------------------------------------
// The tile pipelines above march their own rays between network passes, so the DDA's dependent
// loads run with only G x 4 warps per SM to hide them, and each pipeline's barriers wait for its
// slowest ray.  Here the two jobs are split: MW "marcher" warps own a pool of ray slots in shared
// memory (K per lane) and do all ray generation and DDA marching; two four-warp tensor-core groups
// own half of the slots each and run the networks on the slots whose queries are ready.  A slot's
// state word says who holds it: EMPTY / MARCH belong to its marcher lane, VIS / THR to its network
// group; a side hands a slot over by writing the ray data, a block fence, then the state (and
// reads the state, a fence, then the data).  A group runs a full tile of 128 ready visibility
// queries, or after a short wait whatever is ready, and a throughput pass whenever throughput
// queries are ready.  The frame ends when the ray queue is exhausted and every slot is empty.

enum : uint32_t { WS_EMPTY = 0, WS_MARCH = 1, WS_VIS = 2, WS_THR = 3 };

template <int MW, int K>
struct WsLayout {
    static constexpr int kSlots = MW * 32 * K;
    PkLayout base;            // weights, level tables, the two groups' A tiles (base.groups)
    uint32_t rays, ray_id, counts, state, rows, ctl;
    uint32_t total;
};

template <int MW, int K>
__host__ __device__ inline WsLayout<MW, K> ws_layout(const ModelDesc& dv, const ModelDesc& dt) {
    WsLayout<MW, K> L{};
    L.base = pk_layout(dv, dt, 2);
    uint32_t off = L.base.total;
    constexpr uint32_t S = (uint32_t)WsLayout<MW, K>::kSlots;
    L.rays = off;
    off += S * (uint32_t)sizeof(RayState);
    L.ray_id = off;
    off += S * 4u;
    L.counts = off;
    off += S * 4u;
    L.state = off;
    off += S * 4u;
    L.rows = off;             // per group: [2][128] slot of each visibility / throughput row, 2 counters
    off += 2u * (2u * 128u + 4u) * 4u;
    L.ctl = off;              // active marcher warps
    off += 16u;
    L.total = up128(off);
    return L;
}

__device__ __forceinline__ uint32_t ld_state(const uint32_t* p) { return *reinterpret_cast<const volatile uint32_t*>(p); }
__device__ __forceinline__ void st_state(uint32_t* p, uint32_t v) { *reinterpret_cast<volatile uint32_t*>(p) = v; }

template <typename T, int MW, int K>
__global__ void __launch_bounds__(2 * kGroupThreads + MW * 32, 1)
    k_render_ws(const __grid_constant__ ModelDesc dv, const __grid_constant__ ModelDesc dt, const __grid_constant__ PkArgs A) {
    using TT = typename std::conditional<std::is_same<T, __half>::value, __half, float>::type;
    constexpr int kThreads = 2 * kGroupThreads + MW * 32;
    constexpr uint32_t S = (uint32_t)WsLayout<MW, K>::kSlots;
    constexpr uint32_t kHalf = S / 2u;
    extern __shared__ __align__(1024) uint8_t smem[];
    const WsLayout<MW, K> L = ws_layout<MW, K>(dv, dt);
    const RenderConsts& C = A.C;
    RayState* rays = reinterpret_cast<RayState*>(smem + L.rays);
    uint32_t* ray_id = reinterpret_cast<uint32_t*>(smem + L.ray_id);
    uint32_t* counts = reinterpret_cast<uint32_t*>(smem + L.counts);     // vis | thr << 16 of the slot's ray
    uint32_t* state = reinterpret_cast<uint32_t*>(smem + L.state);
    uint32_t* active_marchers = reinterpret_cast<uint32_t*>(smem + L.ctl);
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + L.base.bar);
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem + L.base.bar + 16);

    const uint32_t tid = threadIdx.x;
    const uint32_t warp = tid >> 5, lane = tid & 31;
    const unsigned long long t_start = globaltimer_ns();

    // ---- set-up ----
    if (tid == 0) {
        tc::mbar_init(&bars[0], 1);
        tc::mbar_init(&bars[1], 1);
        tc::fence_barrier_init();
        *active_marchers = MW;
    }
    if (warp == 0) {
        tc::tmem_alloc(tmem_slot, L.base.tmem_cols);
        tc::tmem_relinquish();
    }
    for (uint32_t i = tid; i < S; i += kThreads) st_state(&state[i], WS_EMPTY);
    GridLevel* lvl_v = reinterpret_cast<GridLevel*>(smem + L.base.lv);
    GridLevel* lvl_t = reinterpret_cast<GridLevel*>(smem + L.base.lt);
    stage_network(dv, A.vis.weights_op, smem + L.base.wv, lvl_v, tid, kThreads);
    stage_network(dt, A.thr.weights_op, smem + L.base.wt, lvl_t, tid, kThreads);
    tc::fence_proxy_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();

    if (warp >= 8) {
        // ================= marcher warps =================
        const uint32_t mlane = (warp - 8) * 32 + lane;      // 0 .. MW*32-1
        bool queue_done = false;
        for (uint32_t it = 0;; ++it) {
            bool progress = false;
            // march every slot handed back for marching
#pragma unroll
            for (int k = 0; k < K; ++k) {
                const uint32_t s = mlane + (uint32_t)k * (MW * 32);
                if (ld_state(&state[s]) == WS_MARCH) {
                    __threadfence_block();
                    RayState st = rays[s];
                    const uint32_t ray = ray_id[s];
                    const int mr = ray_march(C, st, A.image + 3 * (size_t)ray);
                    if (mr == MARCH_VIS) {
                        rays[s] = st;
                        counts[s] += 1u;
                        __threadfence_block();
                        st_state(&state[s], WS_VIS);
                    } else {
                        if (mr == MARCH_DROPPED) atomicAdd(&A.ctl->dropped, 1u);
                        else if (mr == MARCH_FAIL) atomicOr(A.status, 2u);
                        const uint32_t c = counts[s];
                        A.ray_stats[2 * ray] = c & 0xFFFFu;
                        A.ray_stats[2 * ray + 1] = c >> 16;
                        st_state(&state[s], WS_EMPTY);
                    }
                    progress = true;
                }
            }
            // refill one empty slot per lane from the ray queue (warp-aggregated)
            int empty_k = -1;
#pragma unroll
            for (int k = K - 1; k >= 0; --k)
                if (ld_state(&state[mlane + (uint32_t)k * (MW * 32)]) == WS_EMPTY) empty_k = k;
            const bool want = !queue_done && empty_k >= 0;
            const unsigned m = __ballot_sync(kFull, want);
            if (m) {
                const int leader = __ffs(m) - 1;
                uint32_t base = 0;
                if ((int)lane == leader) base = atomicAdd(&A.ctl->cnt[0], (uint32_t)__popc(m));
                base = __shfl_sync(kFull, base, leader);
                if (want) {
                    const uint32_t id = base + (uint32_t)__popc(m & ((1u << lane) - 1u));
                    if (id >= C.n_rays) {
                        queue_done = true;
                    } else {
                        const uint32_t s = mlane + (uint32_t)empty_k * (MW * 32);
                        RayState st;
                        ray_generate(C, id, st);
#pragma unroll
                        for (int c = 0; c < 3; ++c) A.image[3 * (size_t)id + c] = 0.f;
                        const int mr = ray_march(C, st, A.image + 3 * (size_t)id);
                        if (mr == MARCH_VIS) {
                            rays[s] = st;
                            ray_id[s] = id;
                            counts[s] = 1u;
                            __threadfence_block();
                            st_state(&state[s], WS_VIS);
                        } else {
                            if (mr == MARCH_DROPPED) atomicAdd(&A.ctl->dropped, 1u);
                            else if (mr == MARCH_FAIL) atomicOr(A.status, 2u);
                            A.ray_stats[2 * id] = 0u;
                            A.ray_stats[2 * id + 1] = 0u;
                        }
                    }
                }
                progress = true;
            }
            // the lane is done when the queue is exhausted and all its slots are empty
            bool mine_empty = true;
#pragma unroll
            for (int k = 0; k < K; ++k) mine_empty &= ld_state(&state[mlane + (uint32_t)k * (MW * 32)]) == WS_EMPTY;
            if (__all_sync(kFull, queue_done && mine_empty)) break;
            if (!__any_sync(kFull, progress)) {
                // the time bound is decided for the whole warp, so that no lane leaves alone
                if ((it & 63u) == 0 && __any_sync(kFull, globaltimer_ns() - t_start > kFrameNs)) {
                    if (lane == 0) atomicOr(A.status, 4u);
                    break;
                }
                __nanosleep(256);
            }
        }
        __threadfence_block();
        if (lane == 0) atomicSub(active_marchers, 1u);
    } else {
        // ================= tensor-core groups =================
        const uint32_t grp = warp >> 2;                     // 0 or 1
        const uint32_t gtid = tid & (kGroupThreads - 1);
        const uint32_t quarter = warp & 3u;
        const uint32_t bar_id = 1u + grp;
        const uint32_t row = gtid;
        const uint32_t tmem_base = *tmem_slot + grp * (uint32_t)kWidth;
        const uint32_t taddr_row = tmem_base + ((quarter * 32u) << 16);
        uint8_t* a_tile = smem + L.base.groups + grp * L.base.group_stride;
        float* in_row = reinterpret_cast<float*>(a_tile + L.base.in_rel) + row * kInLd;
        const uint32_t a_addr = tc::smem_addr(a_tile);
        uint64_t* bar = &bars[grp];
        uint32_t* vis_rows = reinterpret_cast<uint32_t*>(smem + L.rows) + grp * (2u * 128u + 4u);
        uint32_t* thr_rows = vis_rows + 128;
        uint32_t* cnt = vis_rows + 256;                     // [0] visibility, [1] throughput ready, [2] active marchers
        const TT* vtab = static_cast<const TT*>(A.vis.table);
        const TT* ttab = static_cast<const TT*>(A.thr.table);
        const uint32_t first = grp * kHalf;
        uint32_t phase = 0;
        bool aborted = false;
        unsigned long long tot_v = 0, tot_t = 0;
        uint32_t waited = 0, passes = 0;
        for (uint32_t it = 0;; ++it) {
            // ---- collect the ready slots of this group's half ----
            // Every decision below is taken on values the whole group reads after a group
            // barrier (one thread samples the marcher count), so no thread of the group leaves the
            // loop or skips a pass alone: the group barriers have 128 arrivals on every path.
            if (gtid == 0) {
                cnt[0] = 0u;
                cnt[1] = 0u;
                cnt[2] = ld_state(active_marchers);
            }
            group_sync(bar_id);
            const bool marchers_gone = cnt[2] == 0u;
            for (uint32_t j = gtid; j < kHalf; j += kGroupThreads) {
                const uint32_t s = first + j;
                const uint32_t v = ld_state(&state[s]);
                if (v == WS_VIS) {
                    const uint32_t pos = atomicAdd(&cnt[0], 1u);
                    if (pos < 128u) vis_rows[pos] = s;
                } else if (v == WS_THR) {
                    const uint32_t pos = atomicAdd(&cnt[1], 1u);
                    if (pos < 128u) thr_rows[pos] = s;
                }
            }
            group_sync(bar_id);
            const uint32_t n_vis = min(cnt[0], 128u), n_thr = min(cnt[1], 128u);
            const bool timed_out = (it & 63u) == 0 && globaltimer_ns() - t_start > kFrameNs;
            if (group_sync_or(bar_id, timed_out)) {
                if (gtid == 0) atomicOr(A.status, 4u);
                break;
            }
            // a full visibility tile, or after a short wait (or at the end) whatever is ready
            const bool run_vis = n_vis == 128u || (n_vis > 0u && (waited >= 4u || marchers_gone));
            const bool run_thr = n_thr > 0u && (n_thr == 128u || !run_vis);
            if (!run_vis && !run_thr) {
                if (marchers_gone && n_vis == 0u && n_thr == 0u) break;
                ++waited;
                __nanosleep(128);
                continue;
            }
            waited = 0;
            ++passes;
            float out[3];
            if (run_vis) {
                __threadfence_block();
                const bool mine = row < n_vis;
                const uint32_t s = mine ? vis_rows[row] : 0u;
                RayState st;
                if (mine) {
                    st = rays[s];
                    vis_row(st, in_row);
                    RowStore<T> rs{TcStore<T>{a_tile, dv.enc_width * 16u}, row};
                    encode_tile_rows<kNL>(dv, lvl_v, vtab, in_row, kInLd, nullptr, A.vis.max_level, 0, 1, 0, 1, rs);
                    ++tot_v;
                }
                tc::fence_proxy_async_smem();
                tc::fence_before_sync();
                group_sync(bar_id);
                if (!run_mlp<T>(dv, smem + L.base.wv, a_tile, a_addr, tmem_base, taddr_row, bar, phase, bar_id, gtid, row, out)) {
                    aborted = true;
                    break;
                }
                if (mine) {
                    const uint32_t ray = ray_id[s];
                    const int vr = vis_resolve(C, st, ray, out[0]);
                    rays[s] = st;
                    if (vr == VIS_ACCEPT_THR) {
                        counts[s] += 1u << 16;
                        __threadfence_block();
                        st_state(&state[s], WS_THR);
                    } else if (vr == VIS_ACCEPT_END) {
                        const uint32_t c = counts[s];
                        A.ray_stats[2 * ray] = c & 0xFFFFu;
                        A.ray_stats[2 * ray + 1] = c >> 16;
                        __threadfence_block();
                        st_state(&state[s], WS_EMPTY);
                    } else {
                        __threadfence_block();
                        st_state(&state[s], WS_MARCH);
                    }
                }
            }
            if (run_thr) {
                __threadfence_block();
                const bool mine = row < n_thr;
                const uint32_t s = mine ? thr_rows[row] : 0u;
                RayState st;
                if (mine) {
                    st = rays[s];
                    thr_row(C, st, in_row);
                    RowStore<T> rs{TcStore<T>{a_tile, dt.enc_width * 16u}, row};
                    encode_tile_rows<kNL>(dt, lvl_t, ttab, in_row, kInLd, nullptr, A.thr.max_level, 0, 1, 0, 1, rs);
                    ++tot_t;
                }
                tc::fence_proxy_async_smem();
                tc::fence_before_sync();
                group_sync(bar_id);
                if (!run_mlp<T>(dt, smem + L.base.wt, a_tile, a_addr, tmem_base, taddr_row, bar, phase, bar_id, gtid, row, out)) {
                    aborted = true;
                    break;
                }
                if (mine) {
                    const float t3[3] = {out[0], out[1], out[2]};
                    const bool alive = thr_resolve(st, t3);
                    rays[s] = st;
                    if (alive) {
                        __threadfence_block();
                        st_state(&state[s], WS_MARCH);
                    } else {
                        const uint32_t ray = ray_id[s], c = counts[s];
                        A.ray_stats[2 * ray] = c & 0xFFFFu;
                        A.ray_stats[2 * ray + 1] = c >> 16;
                        __threadfence_block();
                        st_state(&state[s], WS_EMPTY);
                    }
                }
            }
        }
        for (int o = 16; o > 0; o >>= 1) {
            tot_v += __shfl_xor_sync(kFull, tot_v, o);
            tot_t += __shfl_xor_sync(kFull, tot_t, o);
        }
        if (lane == 0) {
            atomicAdd(&A.ctl->tot_vis, tot_v);
            atomicAdd(&A.ctl->tot_thr, tot_t);
            if (gtid == 0) atomicMax(&A.ctl->tot_rounds, (unsigned long long)passes);
        }
        if (aborted) {
            (void)tc::mbar_wait_bounded(bar, phase ^ 1u, kWaitCycles);
            if (gtid == 0) atomicOr(A.status, 8u);
        }
    }

    // ---- teardown ----
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) {
        tc::fence_after_sync();
        tc::tmem_dealloc(*tmem_slot, L.base.tmem_cols);
    }
}

template <typename T, int MW, int K>
cudaError_t launch_ws(const ModelDesc& dv, const ModelDesc& dt, const PkArgs& a, int n_sms, cudaStream_t s) {
    const WsLayout<MW, K> L = ws_layout<MW, K>(dv, dt);
    if (L.total > 227u * 1024u) return cudaErrorInvalidConfiguration;
    const uint32_t bytes = L.total > 120u * 1024u ? L.total : 120u * 1024u;
    cudaError_t e = ensure_dynamic_smem((const void*)k_render_ws<T, MW, K>, bytes);
    if (e != cudaSuccess) return e;
    k_render_ws<T, MW, K><<<(uint32_t)n_sms, 2 * kGroupThreads + MW * 32, bytes, s>>>(dv, dt, a);
    return cudaGetLastError();
}

__global__ void k_reset_pk(Control* ctl) {
    Control c{};
    *ctl = c;
}

template <typename T, int G>
cudaError_t launch_pk(const ModelDesc& dv, const ModelDesc& dt, const PkArgs& a, int n_sms, cudaStream_t s) {
    const PkLayout L = pk_layout(dv, dt, G);
    if (L.total > 227u * 1024u) return cudaErrorInvalidConfiguration;
    // at least 120 KB per CTA, so that one CTA runs per SM and its TMEM columns are always free
    const uint32_t bytes = L.total > 120u * 1024u ? L.total : 120u * 1024u;
    cudaError_t e = ensure_dynamic_smem((const void*)k_render_pk<T, G>, bytes);
    if (e != cudaSuccess) return e;
    uint32_t blocks = (uint32_t)n_sms;
    const uint32_t need = (a.C.n_rays + G * kTile - 1) / (G * kTile);
    if (blocks > need) blocks = need;
    if (blocks == 0) blocks = 1;
    k_render_pk<T, G><<<blocks, G * kGroupThreads, bytes, s>>>(dv, dt, a);
    return cudaGetLastError();
}

}  // namespace

bool render_pk_supported(const ModelDesc& dv, const ModelDesc& dt, int groups) {
    for (const ModelDesc* d : {&dv, &dt}) {
        if (d->width != (uint32_t)kWidth || d->n_output > 3 || d->n_output_padded != 16) return false;
        if (d->act != ACT_RELU && d->act != ACT_NONE) return false;
        if (d->enc_width % 16 != 0 || d->enc_width > 256) return false;
        if (d->n_input + 1 > kInLd) return false;
    }
    if (dv.n_input != 6 || dt.n_input != 10) return false;
    if (groups == kWsForm16) return ws_layout<16, 2>(dv, dt).total <= 227u * 1024u;
    if (groups == kWsForm8) return ws_layout<8, 4>(dv, dt).total <= 227u * 1024u;
    if (groups != 4 && groups != 6) return false;
    return pk_layout(dv, dt, groups).total <= 227u * 1024u;
}

cudaError_t launch_render_pk(const ModelDesc& dv, const ModelDesc& dt, const PkArgs& a, int kind, int groups, cudaStream_t s) {
    int dev = 0, n_sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&n_sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    k_reset_pk<<<1, 1, 0, s>>>(a.ctl);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if (kind == 1 && groups == kWsForm16) return launch_ws<__half, 16, 2>(dv, dt, a, n_sms, s);
    if (kind == 1 && groups == kWsForm8) return launch_ws<__half, 8, 4>(dv, dt, a, n_sms, s);
    if (kind == 2 && groups == kWsForm16) return launch_ws<__nv_bfloat16, 16, 2>(dv, dt, a, n_sms, s);
    if (kind == 2 && groups == kWsForm8) return launch_ws<__nv_bfloat16, 8, 4>(dv, dt, a, n_sms, s);
    if (kind == 1 && groups == 6) return launch_pk<__half, 6>(dv, dt, a, n_sms, s);
    if (kind == 1 && groups == 4) return launch_pk<__half, 4>(dv, dt, a, n_sms, s);
    if (kind == 2 && groups == 6) return launch_pk<__nv_bfloat16, 6>(dv, dt, a, n_sms, s);
    if (kind == 2 && groups == 4) return launch_pk<__nv_bfloat16, 4>(dv, dt, a, n_sms, s);
    return cudaErrorInvalidValue;
}

}  // namespace nlod
