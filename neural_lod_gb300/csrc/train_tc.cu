// Tensor-core form of the training step: encoding, forward, loss, backward through the MLP,
// weight gradients and the grid-gradient scatter of a batch in one persistent kernel.
//
// A CTA (one per SM) holds the network's weights in shared memory (FP16/BF16, K-major core
// matrices) and runs G four-warp tile pipelines ("groups") plus one MMA warp:
//   * a group stages a 128-element tile, encodes it into X0 (shared memory), and for each of the
//     2L MMA jobs of the tile (L forward layers, then L backward layers) signals READY, waits for
//     DONE and runs the job's epilogue from TMEM:
//       forward l < L-1 : ReLU, hidden activations H[l+1] kept in shared memory;
//       forward L-1     : output activation, loss value, dL/dy (per element, unscaled) -> DZ;
//       backward b >= 1 : dL/dH[b] * act'(H[b]) = delta of layer b-1, written over H[b];
//       backward 0      : dL/dX0 -> grid-table gradients (FP32 reductions, one per corner or one
//                         16-byte reduction per aligned x-adjacent entry pair; most levels are
//                         handed to a scatter team, see ST below).
//   * the MMA warp's elected thread serves the groups' READY signals in turn: per job it issues
//     tcgen05.mma (M = 128 rows of the tile, FP32 accumulate in the group's TMEM columns) and, for
//     a backward job, the weight-gradient MMA dW_b += delta_b^T A_b (M = 64, contraction over the
//     tile's 128 rows, both operands read MN-major straight from the activation buffers) into
//     TMEM columns that persist over all tiles of the CTA, then commits to the group's DONE.
//     One issuing thread keeps every accumulation into the shared dW columns ordered.
// At the end the CTA adds its dW (scaled) to the FP32 gradient vector and its loss partial sum.
//
// The operand precision is FP16 or BF16 with FP32 accumulation.  The deltas are kept per element
// (without the 1/N of the mean and the static loss scale, which are applied in FP32 when the
// gradients leave the kernel), so they stay well inside the FP16 range.
//
// Semantics: tiny-cuda-nn's FullyFusedMLP forward/backward (src/fully_fused_mlp.cu:499-633,
// 153-372), the losses (losses/binary_cross_entropy.h, relative_l2.h, l2.h) and the grid
// encoding backward (encodings/grid.h:394-517), paths relative to rptr/ext/tiny-cuda-nn.
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <type_traits>

#include "desc.h"
#include "encoding.cuh"
#include "kernels.h"
#include "tc_common.cuh"
#include "tc_tile.cuh"

namespace nlod {

namespace {

constexpr int kTile = 128;
constexpr int kGT = 128;                         // threads of a group
constexpr long long kWaitCycles = 4000000000ll;  // ~2 s at 2 GHz
constexpr uint32_t kHBytes = kTile * 64u * 2u;   // one hidden activation buffer (128 x 64, 16-bit)
// Merging the lanes of a warp that hit the same entry before the reduction (grid_level_scatter8's
// AGG form) costs eight warp matches per level and pays only for spatially coherent batches; the
// training batches here are random, so every corner goes straight to the L2.
constexpr bool kScatterAggregate = false;

__host__ __device__ inline uint32_t al(uint32_t v, uint32_t a) { return (v + a - 1) / a * a; }

constexpr uint32_t kMmaSeqBytes = 40;   // sizeof(MmaSeq)

struct TrainLayout {
    uint32_t grp_base;       // first group region (after the weights)
    uint32_t h_rel;          // H[1] within a group region (X0 at 0)
    uint32_t dz_rel;
    uint32_t group_stride;
    uint32_t lvl_off;
    uint32_t bar_off;        // ready[G], done[G], fin, xbar[G], full[G], empty[G], then the TMEM
                             // slot, the abort flag, the scatter team's pick and the hand-off tiles [G]
    uint32_t red_off;        // per-warp loss sums
    uint32_t seq_off;        // MMA runs: [G][2L jobs][2]
    uint32_t total;
    uint32_t work_col, work_stride, tmem_cols;   // TMEM: dW columns of every layer, then G work regions
};

// First TMEM column of layer b's weight-gradient accumulator (layers in order, each rounded up to
// 32 columns; the output layer's is stored transposed, 64 rows x 16 columns).
__host__ __device__ inline uint32_t dw_col(const ModelDesc& d, uint32_t b) {
    uint32_t col = 0;
    for (uint32_t l = 0; l < b; ++l) col += (l + 1 < d.n_layers) ? al(d.layer_in[l], 32) : 32u;
    return col;
}

__host__ __device__ inline TrainLayout train_layout(const ModelDesc& d, int G) {
    TrainLayout L{};
    uint32_t off = al(d.n_params_network * 2u, 128);
    L.grp_base = off;
    const uint32_t nh = d.n_layers - 1;
    L.h_rel = al(kTile * d.enc_width * 2u, 128);
    L.dz_rel = L.h_rel + nh * kHBytes;
    L.group_stride = al(L.dz_rel + kTile * 16u * 2u, 128);
    off += (uint32_t)G * L.group_stride;
    L.lvl_off = off;
    off += kMaxGrids * kMaxLevels * (uint32_t)sizeof(GridLevel);
    L.bar_off = off;
    off += 8u * (5u * G + 1u) + 12u + 4u * G;
    L.red_off = al(off, 16);
    off = L.red_off + 4u * (4u * G + 5u);
    L.seq_off = al(off, 16);
    off = L.seq_off + (uint32_t)G * 2u * d.n_layers * 2u * kMmaSeqBytes;
    L.total = al(off, 128);
    uint32_t col = dw_col(d, d.n_layers);
    L.work_col = col;
    L.work_stride = al(d.enc_width > 64u ? d.enc_width : 64u, 32);
    col += (uint32_t)G * L.work_stride;
    L.tmem_cols = 32;
    while (L.tmem_cols < col) L.tmem_cols <<= 1;
    return L;
}

// Loss value and dL/dprediction of one output, without the 1/N of the mean (the callers scale).
__device__ __forceinline__ float loss_unit(int32_t kind, float pred, float target, float& grad) {
    switch (kind) {
        case LOSS_BCE: {
            const float eps = 1e-5f;
            const float p = fminf(fmaxf(pred, eps), 1.f - eps);
            grad = -(target - p) / (p - p * p);
            return -(target * logf(p) + (1.f - target) * logf(1.f - p));
        }
        case LOSS_RELATIVE_L2: {
            const float den = pred * pred + 0.01f;
            const float diff = pred - target;
            grad = 2.f * diff / den;
            return diff * diff / den;
        }
        case LOSS_L2: {
            const float diff = pred - target;
            grad = 2.f * diff;
            return diff * diff;
        }
        default: grad = 0.f; return 0.f;
    }
}

// Saturating conversion for the 16-bit delta buffers.
__device__ __forceinline__ float sat16(float v) { return fminf(fmaxf(v, -65504.f), 65504.f); }

template <typename T>
__device__ __forceinline__ float lo16(uint32_t w);
template <>
__device__ __forceinline__ float lo16<__half>(uint32_t w) { return __half2float(__ushort_as_half((unsigned short)(w & 0xFFFFu))); }
template <>
__device__ __forceinline__ float lo16<__nv_bfloat16>(uint32_t w) { return __uint_as_float(w << 16); }
template <typename T>
__device__ __forceinline__ float hi16(uint32_t w) { return lo16<T>(w >> 16); }

__device__ __forceinline__ uint64_t desc(uint32_t addr, uint32_t lbo, uint32_t sbo) { return tc::make_smem_desc(addr, lbo, sbo); }

// One run of dependent MMAs: count instructions whose operand descriptors advance by a_step /
// b_step (16-byte units) per instruction.  Built once per CTA so that issuing a job is a short
// loop of descriptor additions.
struct MmaSeq {
    uint64_t a, b;        // operand descriptors of the first MMA
    uint32_t d, idesc;    // accumulator (TMEM address) and instruction descriptor
    uint32_t a_step, b_step;
    uint32_t count;
    int32_t dw_layer;     // >= 0: weight-gradient run of that layer (accumulates across tiles)
};

// The MMA runs of job j of group g (forward layers 0..L-1, then backward layers L-1..0).
template <typename T>
__device__ void build_job(const ModelDesc& d, const TrainLayout& L, uint8_t* smem, uint32_t tmem, uint32_t g, uint32_t j, MmaSeq (&q)[2]) {
    using Op = tc::OpType<T>;
    const uint32_t nl = d.n_layers;
    const uint32_t grp = tc::smem_addr(smem + L.grp_base + g * L.group_stride);
    const uint32_t x0 = grp, dz = grp + L.dz_rel;
    auto hbuf = [&](uint32_t i) { return grp + L.h_rel + (i - 1u) * kHBytes; };   // H[i], i >= 1
    const uint32_t work = tmem + L.work_col + g * L.work_stride;
    const uint32_t K0 = d.enc_width;
    q[0].count = q[1].count = 0;
    q[0].dw_layer = q[1].dw_layer = -1;
    if (j < nl) {
        const uint32_t f = j, K = d.layer_in[f], N = d.layer_out[f];
        const uint32_t a = f == 0 ? x0 : hbuf(f);
        const uint32_t b = tc::smem_addr(smem + 2u * d.layer_offset[f]);
        // K-major operands: 16 more K columns = two core matrices = 256 bytes
        q[0] = MmaSeq{desc(a, 128u, K * 16u), desc(b, 128u, K * 16u), work, tc::make_idesc_f16(Op::kFmt, 128, N), 16u, 16u, K / 16u, -1};
        return;
    }
    const uint32_t b = 2u * nl - 1u - j;
    const uint32_t in_b = d.layer_in[b], out_b = d.layer_out[b];
    const bool last = b + 1 == nl;
    const uint32_t delta = last ? dz : hbuf(b + 1);           // delta of layer b (rows x out_b)
    const uint32_t delta_ld = out_b * 16u;                    // its 8-row stride
    // delta propagation: dL/d(input of layer b) = delta_b W_b  (B = W_b read MN-major)
    if (b > 0 || d.n_grids > 0) {
        const uint32_t w = tc::smem_addr(smem + 2u * d.layer_offset[b]);
        q[0] = MmaSeq{desc(delta, 128u, delta_ld), desc(w, in_b * 16u, 128u), work,
                      tc::make_idesc_f16(Op::kFmt, 128, in_b) | tc::kIdescBMajorMN, 16u, (2u * in_b * 16u) >> 4, out_b / 16u, -1};
    }
    // weight gradient over the tile's rows (both operands MN-major, K = rows)
    const uint32_t dw = tmem + dw_col(d, b);
    if (last) {
        // dW_out^T[in][out] += H[L-1]^T dz
        const uint32_t hin = nl >= 2 ? hbuf(nl - 1) : x0;
        const uint32_t hin_ld = nl >= 2 ? 64u * 16u : K0 * 16u;
        q[1] = MmaSeq{desc(hin, hin_ld, 128u), desc(dz, 256u, 128u), dw,
                      tc::make_idesc_f16(Op::kFmt, 64, 16) | tc::kIdescAMajorMN | tc::kIdescBMajorMN, (2u * hin_ld) >> 4, (2u * 256u) >> 4,
                      kTile / 16u, (int32_t)b};
    } else {
        // dW_b[out][in] += delta_b^T A_b
        const uint32_t ain = b == 0 ? x0 : hbuf(b);
        const uint32_t ain_ld = in_b * 16u;
        q[1] = MmaSeq{desc(delta, delta_ld, 128u), desc(ain, ain_ld, 128u), dw,
                      tc::make_idesc_f16(Op::kFmt, 64, in_b) | tc::kIdescAMajorMN | tc::kIdescBMajorMN, (2u * delta_ld) >> 4,
                      (2u * ain_ld) >> 4, kTile / 16u, (int32_t)b};
    }
}

static_assert(sizeof(MmaSeq) == kMmaSeqBytes, "MmaSeq layout");

__device__ __forceinline__ void issue_seq(const MmaSeq& q, uint32_t& dw_started) {
    uint32_t acc = 0;
    if (q.dw_layer >= 0) {
        acc = (dw_started >> q.dw_layer) & 1u;
        dw_started |= 1u << q.dw_layer;
    }
    uint64_t a = q.a, b = q.b;
    for (uint32_t k = 0; k < q.count; ++k) {
        tc::mma_f16_ss(q.d, a, b, q.idesc, (k > 0 || acc) ? 1u : 0u);
        a += q.a_step;
        b += q.b_step;
    }
}

// Waits for phase `parity` of `bar`; gives up (false) when the CTA's abort flag is raised or after
// kWaitCycles.
__device__ __forceinline__ bool wait_unless_aborted(uint64_t* bar, uint32_t parity, volatile uint32_t* abort_flag) {
    const long long t0 = clock64();
    while (!tc::mbar_test_wait(bar, parity)) {
        if (*abort_flag || clock64() - t0 > kWaitCycles) return false;
    }
    return true;
}

// Grid-gradient scatter of one tile row, levels [l_begin, l_end) of every grid: dL/d(grid
// features) of the row are read from `dx` (column c of the grid features at dx[c * col_stride])
// and reduced into the FP32 gradient tables.
__device__ __forceinline__ void scatter_row(const ModelDesc& d, const TrainTcArgs& a, const GridLevel* lvl_s, size_t grow,
                                            const float* dx, uint32_t col_stride, uint32_t l_begin, uint32_t l_end) {
    uint32_t hc = 0;
    for (uint32_t si = 0; si < d.n_slots; ++si) {
        const Slot& s = d.slots[si];
        if (s.type != SLOT_GRID) continue;
        const GridDesc& gd = d.grids[s.grid];
        const GridLevel* lv = lvl_s + s.grid * kMaxLevels;
        const float* prow = a.in + grow * d.n_input + s.in_begin;
        const float px = __ldg(prow), py = __ldg(prow + 1), pz = __ldg(prow + 2);
        const float ml = a.max_level_gpu ? __ldg(a.max_level_gpu + grow) : a.max_level;
        float* gtab = a.grads + gd.param_offset;
        uint32_t p0, p1, p2;
        hash_primes(gd.hash, p0, p1, p2);
        const uint32_t le = min(l_end, gd.n_levels);
#pragma unroll 1
        for (uint32_t level = l_begin; level < le; ++level) {
            const bool act = !grid_level_skipped_backward(level, ml, gd.n_levels);
            const float2 dy = make_float2(dx[(hc + 2u * level) * col_stride] * a.grad_scale, dx[(hc + 2u * level + 1u) * col_stride] * a.grad_scale);
            if (gd.interp == INTERP_NEAREST) grid_level_backward(gd, level, gtab, px, py, pz, dy, act);
            else grid_level_scatter8<kScatterAggregate>(gd, lv[level], gtab, p0, p1, p2, px, py, pz, dy, act);
        }
        hc += 2u * gd.n_levels;
    }
}

// ST (scatter team): most of the grid-gradient scatter runs in four extra warps.  A group that
// finishes a tile's last backward job copies dL/d(grid features) (FP32, column-major 128 rows x
// <= 32 columns) from TMEM into its last hidden-activation buffer, which no MMA reads until the
// next tile's forward reaches it, hands it over (full[g]), scatters the first a.group_levels
// levels itself and goes on with its next tile; the team scatters the other levels of the
// hand-offs in arrival order and releases each buffer (empty[g]).  A group's last tile is not
// handed over: the group scatters all of it, which keeps the team's queue short at the end.  The reductions, bound by the
// L2's reduction rate, then run continuously instead of stalling every group for the whole
// scatter of its own tile.
template <typename T, int G, bool ST>
__global__ void __launch_bounds__(G * kGT + 32 + (ST ? kGT : 0), 1)
    k_train_tc(const __grid_constant__ ModelDesc d, const __grid_constant__ TrainTcArgs a, uint32_t* __restrict__ status) {
    using Op = tc::OpType<T>;
    constexpr uint32_t kThreads = G * kGT + 32 + (ST ? kGT : 0);
    extern __shared__ __align__(1024) uint8_t smem[];
    const TrainLayout L = train_layout(d, G);
    uint64_t* ready = reinterpret_cast<uint64_t*>(smem + L.bar_off);
    uint64_t* done = ready + G;
    uint64_t* fin = done + G;
    uint64_t* xbar = fin + 1;                    // X0 tile arrival (pre-encoded tiles)
    uint64_t* full = xbar + G;                   // hand-off of a tile's grid gradients to the team
    uint64_t* empty = full + G;                  // the team has finished reading a hand-off
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(empty + G);
    volatile uint32_t* abort_flag = tmem_slot + 1;
    volatile uint32_t* team_pick = tmem_slot + 2;
    volatile uint32_t* hand_tile = tmem_slot + 3;
    float* red = reinterpret_cast<float*>(smem + L.red_off);

    const uint32_t tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t nl = d.n_layers;
    const uint32_t n_tiles = a.n / kTile;

    if (tid == 0) {
        for (int g = 0; g < G; ++g) {
            tc::mbar_init(&ready[g], 1);
            tc::mbar_init(&done[g], 1);
            tc::mbar_init(&xbar[g], 1);
            tc::mbar_init(&full[g], 1);
            tc::mbar_init(&empty[g], 1);
        }
        tc::mbar_init(fin, 1);
        *abort_flag = 0u;
        tc::fence_barrier_init();
    }
    if (warp == 0) {
        tc::tmem_alloc(tmem_slot, L.tmem_cols);
        tc::tmem_relinquish();
    }
    {
        const uint16_t* wsrc = reinterpret_cast<const uint16_t*>(a.weights_op);
        for (uint32_t l = 0; l < nl; ++l) {
            const uint32_t K = d.layer_in[l], N = d.layer_out[l];
            const uint32_t chunks = N * (K / 8u);
            const uint4* src = reinterpret_cast<const uint4*>(wsrc + d.layer_offset[l]);
            for (uint32_t c = tid; c < chunks; c += kThreads) {
                const uint32_t n = c / (K / 8u), k0 = (c - n * (K / 8u)) * 8u;
                *reinterpret_cast<uint4*>(smem + 2u * d.layer_offset[l] + tc::kmajor_offset(n, k0, K * 16u)) = src[c];
            }
        }
    }
    GridLevel* lvl_s = reinterpret_cast<GridLevel*>(smem + L.lvl_off);
    for (uint32_t i = tid; i < d.n_grids * (uint32_t)kMaxLevels; i += kThreads) {
        const uint32_t g = i / kMaxLevels, l = i % kMaxLevels;
        if (l < d.grids[g].n_levels) lvl_s[i] = d.grids[g].levels[l];
    }
    tc::fence_proxy_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    // Everything above reads only parameters; the X0 tiles, zeroed gradients and the batch come
    // from the encoding kernel, which may still be finishing (programmatic dependent launch).
    asm volatile("griddepcontrol.wait;" ::: "memory");
    const uint32_t tmem = *tmem_slot;
    // The CTA's tiles are one contiguous range (13 or 14 of 2048 tiles over 152 CTAs, where a
    // round-robin over all groups would give 16 to some CTAs and 12 to the rest); its groups take
    // every G-th tile of it.
    const uint32_t first_tile = (uint32_t)(((uint64_t)blockIdx.x * n_tiles) / gridDim.x);
    const uint32_t end_tile = (uint32_t)(((uint64_t)(blockIdx.x + 1u) * n_tiles) / gridDim.x);
    constexpr uint32_t stride = G;
    bool aborted = false;
    float loss_acc = 0.f;

    if (warp == (uint32_t)G * 4u) {
        // ---- MMA warp ----
        if (lane == 0) {
            uint32_t left[G], job[G];
            uint32_t rpar = 0, active = 0, dw_started = 0;
#pragma unroll
            for (int g = 0; g < G; ++g) {
                const uint32_t t0 = first_tile + g;
                left[g] = t0 < end_tile ? (end_tile - t0 + stride - 1) / stride : 0u;
                job[g] = 0;
                if (left[g]) active |= 1u << g;
            }
            MmaSeq* seqs = reinterpret_cast<MmaSeq*>(smem + L.seq_off);
            for (uint32_t g = 0; g < (uint32_t)G; ++g)
                for (uint32_t j = 0; j < 2u * nl; ++j) {
                    MmaSeq q[2];
                    build_job<T>(d, L, smem, tmem, g, j, q);
                    seqs[(g * 2u * nl + j) * 2u] = q[0];
                    seqs[(g * 2u * nl + j) * 2u + 1u] = q[1];
                }
            long long last = clock64();
            while (active) {
                if (*abort_flag) break;
                bool prog = false;
#pragma unroll
                for (int g = 0; g < G; ++g) {
                    if (!((active >> g) & 1u)) continue;
                    if (!tc::mbar_test_wait(&ready[g], (rpar >> g) & 1u)) continue;
                    rpar ^= 1u << g;
                    tc::fence_after_sync();
                    const MmaSeq* js = seqs + ((uint32_t)g * 2u * nl + job[g]) * 2u;
                    issue_seq(js[0], dw_started);
                    issue_seq(js[1], dw_started);
                    tc::mma_commit(&done[g]);
                    if (++job[g] == 2u * nl) {
                        job[g] = 0;
                        if (--left[g] == 0) active &= ~(1u << g);
                    }
                    prog = true;
                }
                if (prog) {
                    last = clock64();
                } else if (clock64() - last > kWaitCycles) {
                    *abort_flag = 1u;
                    atomicOr(status, 1u);
                    break;
                }
            }
            tc::mma_commit(fin);
            if (!tc::mbar_wait_bounded(fin, 0, kWaitCycles)) atomicOr(status, 1u);
        }
        __syncwarp();
    } else if (warp < (uint32_t)G * 4u) {
        // ---- tile pipeline (group) ----
        const uint32_t grp_i = warp >> 2;
        const uint32_t gtid = tid & (kGT - 1);
        const uint32_t quarter = warp & 3u;
        const uint32_t bar_id = 1u + grp_i;
        uint8_t* grp = smem + L.grp_base + grp_i * L.group_stride;
        uint8_t* x0 = grp;
        uint8_t* dzb = grp + L.dz_rel;
        auto hbuf = [&](uint32_t i) { return grp + L.h_rel + (i - 1u) * kHBytes; };
        const uint32_t row = quarter * 32u + lane;
        const uint32_t taddr = tmem + L.work_col + grp_i * L.work_stride + ((quarter * 32u) << 16);
        uint32_t dpar = 0, xpar = 0, epar = 0;
        bool x_pending = false;   // a bulk copy of X0 is in flight (thread gtid 0)
        bool hand_pending = false;   // the scatter team still reads this group's last hidden buffer
        const uint32_t x0_bytes = kTile * d.enc_width * 2u;
        const uint8_t* enc_tiles = reinterpret_cast<const uint8_t*>(a.enc_tiles);
        if (gtid == 0 && first_tile + grp_i < end_tile) {
            tc::mbar_arrive_expect_tx(&xbar[grp_i], x0_bytes);
            tc::bulk_copy_g2s(x0, enc_tiles + (size_t)(first_tile + grp_i) * x0_bytes, x0_bytes, &xbar[grp_i]);
            x_pending = true;
        }

        for (uint32_t tile = first_tile + grp_i; tile < end_tile; tile += stride) {
            const uint32_t row0 = tile * kTile;
            {
                // X0 was encoded by k_encode_tiles; its copy was issued when the previous tile's
                // last MMA job had finished reading X0.
                const bool ok = gtid != 0 || tc::mbar_wait_bounded(&xbar[grp_i], xpar, kWaitCycles);
                x_pending = x_pending && !ok;
                xpar ^= 1u;
                if (group_sync_or(bar_id, !ok)) {
                    aborted = true;
                    break;
                }
            }
            if (gtid == 0) tc::mbar_arrive(&ready[grp_i]);

            for (uint32_t j = 0; j < 2u * nl; ++j) {
                const bool ok = gtid != 0 || tc::mbar_wait_bounded(&done[grp_i], dpar, kWaitCycles);
                dpar ^= 1u;
                if (group_sync_or(bar_id, !ok)) {
                    aborted = true;
                    break;
                }
                tc::fence_after_sync();
                const size_t grow = (size_t)row0 + row;
                if (j + 1 < nl) {
                    if (ST && j + 2u == nl && hand_pending) {
                        // H[L-1] still holds the previous tile's hand-off until the team releases it
                        const bool ok = gtid != 0 || wait_unless_aborted(&empty[grp_i], epar, abort_flag);
                        epar ^= 1u;
                        hand_pending = false;
                        if (group_sync_or(bar_id, !ok)) {
                            aborted = true;
                            break;
                        }
                    }
                    // hidden layer j: activation -> H[j+1]
                    uint8_t* h = hbuf(j + 1);
                    const ReluOrNone act{d.act == ACT_RELU};
#pragma unroll
                    for (uint32_t col = 0; col < 64u; col += 32) {
                        uint32_t r[32];
                        tc::tmem_ld32(taddr + col, r);
                        tc::tmem_wait_ld();
#pragma unroll
                        for (uint32_t q = 0; q < 4; ++q) {
                            uint4 pk;
                            pk.x = Op::pack2(act(__uint_as_float(r[8 * q + 0])), act(__uint_as_float(r[8 * q + 1])));
                            pk.y = Op::pack2(act(__uint_as_float(r[8 * q + 2])), act(__uint_as_float(r[8 * q + 3])));
                            pk.z = Op::pack2(act(__uint_as_float(r[8 * q + 4])), act(__uint_as_float(r[8 * q + 5])));
                            pk.w = Op::pack2(act(__uint_as_float(r[8 * q + 6])), act(__uint_as_float(r[8 * q + 7])));
                            *reinterpret_cast<uint4*>(h + tc::kmajor_offset(row, col + 8u * q, 1024u)) = pk;
                        }
                    }
                } else if (j + 1 == nl) {
                    // output layer: activation, loss, dL/dz per element -> DZ
                    uint32_t r[16];
                    tc::tmem_ld16(taddr, r);
                    tc::tmem_wait_ld();
                    float dzv[16];
#pragma unroll
                    for (uint32_t c = 0; c < 16; ++c) {
                        float gv = 0.f;
                        if (c < d.n_output) {
                            const float y = act_fwd(d.out_act, __uint_as_float(r[c]));
                            loss_acc += loss_unit(a.loss_kind, y, __ldg(a.target + grow * d.n_output + c), gv) * a.inv_n_total;
                            gv *= act_grad_from_output(d.out_act, y);
                        }
                        dzv[c] = sat16(gv);
                    }
#pragma unroll
                    for (uint32_t q = 0; q < 2; ++q) {
                        uint4 pk;
                        pk.x = Op::pack2(dzv[8 * q + 0], dzv[8 * q + 1]);
                        pk.y = Op::pack2(dzv[8 * q + 2], dzv[8 * q + 3]);
                        pk.z = Op::pack2(dzv[8 * q + 4], dzv[8 * q + 5]);
                        pk.w = Op::pack2(dzv[8 * q + 6], dzv[8 * q + 7]);
                        *reinterpret_cast<uint4*>(dzb + tc::kmajor_offset(row, 8u * q, 256u)) = pk;
                    }
                } else {
                    const uint32_t b = 2u * nl - 1u - j;
                    if (b == 0 && gtid == 0 && tile + stride < end_tile) {
                        // every MMA reading X0 has completed: fetch the next tile during this epilogue
                        tc::mbar_arrive_expect_tx(&xbar[grp_i], x0_bytes);
                        tc::bulk_copy_g2s(x0, enc_tiles + (size_t)(tile + stride) * x0_bytes, x0_bytes, &xbar[grp_i]);
                        x_pending = true;
                    }
                    if (b > 0) {
                        // delta of layer b-1 = dL/dH[b] * act'(H[b]), in place over H[b]
                        uint8_t* h = hbuf(b);
#pragma unroll
                        for (uint32_t col = 0; col < 64u; col += 32) {
                            uint32_t r[32];
                            tc::tmem_ld32(taddr + col, r);
                            tc::tmem_wait_ld();
#pragma unroll
                            for (uint32_t q = 0; q < 4; ++q) {
                                uint4* p = reinterpret_cast<uint4*>(h + tc::kmajor_offset(row, col + 8u * q, 1024u));
                                const uint4 hv = *p;
                                const uint32_t hw[4] = {hv.x, hv.y, hv.z, hv.w};
                                uint32_t ow[4];
#pragma unroll
                                for (uint32_t e = 0; e < 4; ++e) {
                                    float g0 = __uint_as_float(r[8 * q + 2 * e]), g1 = __uint_as_float(r[8 * q + 2 * e + 1]);
                                    if (d.act == ACT_RELU) {
                                        g0 = lo16<T>(hw[e]) > 0.f ? g0 : 0.f;
                                        g1 = hi16<T>(hw[e]) > 0.f ? g1 : 0.f;
                                    }
                                    ow[e] = Op::pack2(sat16(g0), sat16(g1));
                                }
                                *p = make_uint4(ow[0], ow[1], ow[2], ow[3]);
                            }
                        }
                    } else if (ST) {
                        // dL/d(grid features) -> H[L-1] (column-major FP32) for the scatter team
                        float* hand = reinterpret_cast<float*>(hbuf(nl - 1u));
                        // (all grid levels; the group reads its own share back from here)
                        uint32_t hc = 0;
                        for (uint32_t si = 0; si < d.n_slots; ++si) {
                            const Slot& s = d.slots[si];
                            if (s.type != SLOT_GRID) continue;
                            const uint32_t nlv = d.grids[s.grid].n_levels;
#pragma unroll 1
                            for (uint32_t level = 0; level < nlv; ++level) {
                                uint32_t r0, r1;
                                tc::tmem_ld2(taddr + s.out_begin + 2u * level, r0, r1);
                                tc::tmem_wait_ld();
                                hand[(hc + 2u * level) * kTile + row] = __uint_as_float(r0);
                                hand[(hc + 2u * level + 1u) * kTile + row] = __uint_as_float(r1);
                            }
                            hc += 2u * nlv;
                        }
                        group_sync(bar_id);
                        if (tile + stride < end_tile) {
                            if (gtid == 0) {
                                hand_tile[grp_i] = tile;
                                tc::mbar_arrive(&full[grp_i]);
                            }
                            hand_pending = true;
                            // the group's own share of the levels (the team takes the rest)
                            scatter_row(d, a, lvl_s, grow, hand + row, kTile, 0u, a.group_levels);
                        } else {
                            // the group's last tile: nothing left to overlap, so no hand-off
                            scatter_row(d, a, lvl_s, grow, hand + row, kTile, 0u, kMaxLevels);
                        }
                    } else if (d.n_grids > 0) {
                        // dL/dX0 -> grid-table gradients
                        for (uint32_t si = 0; si < d.n_slots; ++si) {
                            const Slot& s = d.slots[si];
                            if (s.type != SLOT_GRID) continue;
                            const GridDesc& gd = d.grids[s.grid];
                            const GridLevel* lv = lvl_s + s.grid * kMaxLevels;
                            const float* prow = a.in + grow * d.n_input + s.in_begin;
                            const float px = __ldg(prow), py = __ldg(prow + 1), pz = __ldg(prow + 2);
                            const float ml = a.max_level_gpu ? __ldg(a.max_level_gpu + grow) : a.max_level;
                            float* gtab = a.grads + gd.param_offset;
                            uint32_t p0, p1, p2;
                            hash_primes(gd.hash, p0, p1, p2);
#pragma unroll 1
                            for (uint32_t level = 0; level < gd.n_levels; ++level) {
                                uint32_t r0, r1;
                                tc::tmem_ld2(taddr + s.out_begin + 2u * level, r0, r1);
                                tc::tmem_wait_ld();
                                const bool act = !grid_level_skipped_backward(level, ml, gd.n_levels);
                                const float2 dy = make_float2(__uint_as_float(r0) * a.grad_scale, __uint_as_float(r1) * a.grad_scale);
                                if (gd.interp == INTERP_NEAREST) grid_level_backward(gd, level, gtab, px, py, pz, dy, act);
                                else grid_level_scatter8<kScatterAggregate>(gd, lv[level], gtab, p0, p1, p2, px, py, pz, dy, act);
                            }
                        }
                    }
                }
                tc::fence_proxy_async_smem();
                tc::fence_before_sync();
                group_sync(bar_id);
                if (j + 1 < 2u * nl && gtid == 0) tc::mbar_arrive(&ready[grp_i]);
            }
            if (aborted) break;
        }
        if (aborted) {
            *abort_flag = 1u;
            if (gtid == 0) atomicOr(status, 1u);
        }
        // a copy still in flight (only after an abort) must land before the CTA's shared memory goes
        if (x_pending) (void)tc::mbar_wait_bounded(&xbar[grp_i], xpar, kWaitCycles);
    } else {
        if constexpr (ST) {
            // ---- scatter team: one thread per tile row ----
            const uint32_t st = tid - (uint32_t)G * kGT - 32u;
            const uint32_t team_bar = 1u + G;
            // every tile but each group's last one is handed over
            const uint32_t n_cta = end_tile > first_tile ? end_tile - first_tile : 0u;
            const uint32_t total = n_cta > (uint32_t)G ? n_cta - (uint32_t)G : 0u;
            constexpr uint32_t kNone = 0xFFFFFFFFu;
            uint32_t fpar = 0, next = 0;
            for (uint32_t k = 0; k < total; ++k) {
                if (st == 0) {
                    // the next hand-off in arrival order, groups polled round-robin
                    uint32_t pick = kNone;
                    const long long t0 = clock64();
                    for (;;) {
                        for (uint32_t i = 0; i < (uint32_t)G; ++i) {
                            const uint32_t g = (next + i) % (uint32_t)G;
                            if (tc::mbar_test_wait(&full[g], (fpar >> g) & 1u)) {
                                pick = g;
                                break;
                            }
                        }
                        if (pick != kNone || *abort_flag || clock64() - t0 > kWaitCycles) break;
                    }
                    if (pick != kNone) {
                        fpar ^= 1u << pick;
                        next = (pick + 1u) % (uint32_t)G;
                    } else {
                        *abort_flag = 1u;
                        atomicOr(status, 1u);
                    }
                    *team_pick = pick;
                }
                group_sync(team_bar);
                const uint32_t pick = *team_pick;
                if (pick == kNone) break;
                const float* hand = reinterpret_cast<const float*>(smem + L.grp_base + pick * L.group_stride + L.h_rel + (nl - 2u) * kHBytes);
                scatter_row(d, a, lvl_s, (size_t)hand_tile[pick] * kTile + st, hand + st, kTile, a.group_levels, kMaxLevels);
                group_sync(team_bar);
                if (st == 0) tc::mbar_arrive(&empty[pick]);
            }
        }
    }

    // ---- drain the weight gradients, loss partial sum ----
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const bool any_tile = first_tile < end_tile;
    if (!*abort_flag && any_tile && warp < (uint32_t)G * 4u) {
        const uint32_t grp_i = warp >> 2, quarter = warp & 3u;
        const uint32_t m = quarter * 16u + lane;   // accumulator row (M = 64 layout)
        for (uint32_t b = grp_i; b < nl; b += G) {
            const bool last = b + 1 == nl;
            const uint32_t ncols = last ? 16u : d.layer_in[b];
            float* gw = a.grads + d.layer_offset[b];
            for (uint32_t c0 = 0; c0 < ncols; c0 += 16) {
                uint32_t r[16];
                tc::tmem_ld16(tmem + dw_col(d, b) + c0 + ((quarter * 32u) << 16), r);
                tc::tmem_wait_ld();
                if (lane < 16) {
#pragma unroll
                    for (uint32_t c = 0; c < 16; ++c) {
                        if (c0 + c >= ncols) break;
                        const float v = __uint_as_float(r[c]) * a.grad_scale;
                        if (last) atomicAdd(gw + (c0 + c) * d.layer_in[b] + m, v);
                        else atomicAdd(gw + m * d.layer_in[b] + c0 + c, v);
                    }
                }
            }
        }
    }
    if (a.loss_partial) {
        float v = loss_acc;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) red[warp] = v;
    }
    tc::fence_before_sync();
    __syncthreads();
    if (a.loss_partial && tid == 0) {
        float s = 0.f;
        for (uint32_t w = 0; w < (uint32_t)G * 4u; ++w) s += red[w];
        a.loss_partial[blockIdx.x] = s;
    }
    if (warp == 0) {
        tc::fence_after_sync();
        tc::tmem_dealloc(tmem, L.tmem_cols);
    }
}

// Encoding of the batch into X0 tiles in HBM, each tile laid out exactly as the fused kernel's
// shared-memory A operand (128 rows x enc_width, K-major core matrices), so that one bulk copy
// brings it in.  Full occupancy (128-thread CTAs) for the gather-bound grid levels.
// TT: element type of the grid tables gathered (float: the FP32 parameters; __half / __nv_bfloat16:
// their 16-bit copy of the training values, a.grid_h).  One table type per instantiation keeps the gather code at its register count.
template <typename T, int NL, typename TT>
__global__ void __launch_bounds__(kTile) k_encode_tiles(const __grid_constant__ ModelDesc d, const __grid_constant__ TrainTcArgs a) {
    extern __shared__ __align__(1024) uint8_t smem[];
    GridLevel* lvl_s = reinterpret_cast<GridLevel*>(smem);
    float* in_s = reinterpret_cast<float*>(smem + kMaxGrids * kMaxLevels * sizeof(GridLevel));
    const uint32_t tid = threadIdx.x;
    const uint32_t in_ld = d.n_input + 1;
    for (uint32_t i = tid; i < d.n_grids * (uint32_t)kMaxLevels; i += kTile) {
        const uint32_t g = i / kMaxLevels, l = i % kMaxLevels;
        if (l < d.grids[g].n_levels) lvl_s[i] = d.grids[g].levels[l];
    }
    // the fused training kernel may start its set-up now (programmatic dependent launch); it waits
    // for this grid's completion before touching what it writes
    asm volatile("griddepcontrol.launch_dependents;");
    // the fused kernel accumulates into the gradient vector: zero it here, the stores overlapping
    // the gathers' latency (no separate memset pass)
    for (uint32_t i = blockIdx.x * kTile + tid; i < a.zero_grads_n / 4u; i += gridDim.x * kTile)
        reinterpret_cast<float4*>(a.grads)[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    const uint32_t n_tiles = a.n / kTile;
    const size_t x0_bytes = (size_t)kTile * d.enc_width * 2u;
    for (uint32_t tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
        const uint32_t row0 = tile * kTile;
        __syncthreads();
        const float* in_tile = a.in + (size_t)row0 * d.n_input;
        for (uint32_t idx = tid; idx < kTile * d.n_input; idx += kTile) {
            const uint32_t r = idx / d.n_input, c = idx - r * d.n_input;
            in_s[r * in_ld + c] = __ldg(in_tile + idx);
        }
        __syncthreads();
        TcStore<T> st{reinterpret_cast<uint8_t*>(a.enc_tiles) + tile * x0_bytes, d.enc_width * 16u};
        const TT* table = std::is_same<TT, float>::value ? reinterpret_cast<const TT*>(a.params) : static_cast<const TT*>(a.grid_h);
        encode_tile_rows<NL>(d, lvl_s, table, in_s, in_ld, a.max_level_gpu, a.max_level, row0, kTile, tid, kTile, st);
    }
}

int g_sms = 0;
int sm_count() {
    if (!g_sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&g_sms, cudaDevAttrMultiProcessorCount, dev);
        if (g_sms <= 0) g_sms = 1;
    }
    return g_sms;
}

constexpr size_t kMaxSmem = 227u * 1024u;

bool layout_ok(const ModelDesc& d, int G) {
    const TrainLayout L = train_layout(d, G);
    return L.total <= kMaxSmem && L.tmem_cols <= 512u;
}

// Grid-feature columns of the encoding (the width of a scatter-team hand-off).
uint32_t grid_columns(const ModelDesc& d) {
    uint32_t c = 0;
    for (uint32_t si = 0; si < d.n_slots; ++si)
        if (d.slots[si].type == SLOT_GRID) c += 2u * d.grids[d.slots[si].grid].n_levels;
    return c;
}

// A hand-off (128 rows x grid columns, FP32) fits one hidden-activation buffer.
bool use_scatter_team(const ModelDesc& d) {
    const uint32_t c = grid_columns(d);
    return d.n_grids > 0 && c > 0 && c * kTile * 4u <= kHBytes;
}

// Levels of every grid that a group scatters itself, the scatter team taking the rest: 2 of 16
// (measured on the visibility and throughput networks; anything from 0 to 6 is within a few
// percent, the step being bound by the L2 reduction rate).
uint32_t group_scatter_levels(const ModelDesc& d, int) {
    uint32_t nlev = 0;
    for (uint32_t g = 0; g < d.n_grids; ++g) nlev = d.grids[g].n_levels > nlev ? d.grids[g].n_levels : nlev;
    return nlev / 8u;
}

}  // namespace

uint32_t train_tc_blocks(uint32_t n, int groups) {
    const uint32_t n_tiles = n / kTile;
    uint32_t blocks = (uint32_t)sm_count();
    const uint32_t need = (n_tiles + groups - 1) / groups;
    return blocks > need ? need : blocks;
}

namespace {

template <typename T, int G, bool ST>
cudaError_t launch_gs(const ModelDesc& d, const TrainTcArgs& a_in, uint32_t* status, cudaStream_t s) {
    TrainTcArgs a = a_in;
    a.group_levels = ST ? group_scatter_levels(d, G) : 0u;
    const TrainLayout L = train_layout(d, G);
    const uint32_t blocks = train_tc_blocks(a.n, G);
    if (blocks == 0) return cudaSuccess;
    cudaError_t e = ensure_dynamic_smem((const void*)k_train_tc<T, G, ST>, L.total);
    if (e != cudaSuccess) return e;
    // programmatic dependent launch: the set-up overlaps the encoding kernel's last wave
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(blocks);
    cfg.blockDim = dim3(G * kGT + 32 + (ST ? kGT : 0));
    cfg.dynamicSmemBytes = L.total;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k_train_tc<T, G, ST>, d, a, status);
}

template <typename T, int G>
cudaError_t launch_g(const ModelDesc& d, const TrainTcArgs& a, uint32_t* status, cudaStream_t s) {
    return use_scatter_team(d) ? launch_gs<T, G, true>(d, a, status, s) : launch_gs<T, G, false>(d, a, status, s);
}

template <typename T>
cudaError_t launch_t(const ModelDesc& d, const TrainTcArgs& a, int G, uint32_t* status, cudaStream_t s) {
    switch (G) {
        case 2: return launch_g<T, 2>(d, a, status, s);
        case 3: return launch_g<T, 3>(d, a, status, s);
        case 4: return launch_g<T, 4>(d, a, status, s);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace

int train_tc_groups(const ModelDesc& d) {
    if (d.width != 64 || d.n_layers < 2 || d.n_layers > 8) return 0;
    if (d.act != ACT_RELU && d.act != ACT_NONE) return 0;
    if (d.enc_width % 16 != 0 || d.enc_width > 128 || d.n_output_padded != 16) return 0;
    if (d.n_input + 1 > 32) return 0;
    for (uint32_t l = 1; l + 1 < d.n_layers; ++l)
        if (d.layer_in[l] != 64 || d.layer_out[l] != 64) return 0;
    if (d.layer_out[0] != 64 || d.layer_in[d.n_layers - 1] != 64 || d.layer_out[d.n_layers - 1] != 16) return 0;
    for (int G = 4; G >= 2; --G)
        if (layout_ok(d, G)) return G;
    return 0;
}

cudaError_t launch_encode_tiles(const ModelDesc& d, const TrainTcArgs& a, int kind, cudaStream_t s) {
    const uint32_t n_tiles = a.n / kTile;
    if (n_tiles == 0) return cudaSuccess;
    uint32_t blocks = (uint32_t)sm_count() * 16u;
    if (blocks > n_tiles) blocks = n_tiles;
    const size_t smem = kMaxGrids * kMaxLevels * sizeof(GridLevel) + (size_t)kTile * (d.n_input + 1) * 4u;
    // the FP16 form gathers from the FP16 grid copy when the caller passes one (training values
    // equal to the inference values: no EMA)
    if (kind == 1 && a.grid_h) k_encode_tiles<__half, 2, __half><<<blocks, kTile, smem, s>>>(d, a);
    else if (kind == 1) k_encode_tiles<__half, 2, float><<<blocks, kTile, smem, s>>>(d, a);
    else if (kind == 2 && a.grid_h) k_encode_tiles<__nv_bfloat16, 2, __nv_bfloat16><<<blocks, kTile, smem, s>>>(d, a);
    else if (kind == 2) k_encode_tiles<__nv_bfloat16, 2, float><<<blocks, kTile, smem, s>>>(d, a);
    else return cudaErrorInvalidValue;
    return cudaGetLastError();
}

cudaError_t launch_train_tc(const ModelDesc& d, const TrainTcArgs& a, int kind, int G, uint32_t* status, cudaStream_t s) {
    if (G < 2 || G > 4 || !layout_ok(d, G) || !a.enc_tiles) return cudaErrorInvalidValue;
    if (kind == 1) return launch_t<__half>(d, a, G, status, s);
    if (kind == 2) return launch_t<__nv_bfloat16>(d, a, G, status, s);
    return cudaErrorInvalidValue;
}

}  // namespace nlod
