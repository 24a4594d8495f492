// The tensor-core query kernel (k_forward_tc), its organisations (the autotuner's variant table)
// and their launcher, instantiated per operand type and width in tc_f16_w64.cu, tc_bf16_w64.cu,
// tc_f16_w128.cu and tc_bf16_w128.cu (separate units, so that the library builds in parallel) and
// dispatched by tc.cu.  Internal to those files.
//
// A CTA holds every weight matrix of the network in shared memory (loaded once, FP16/BF16,
// K-major core-matrix layout) and runs G independent tile pipelines ("groups") of 4 warps, or 8
// with two threads per tile row (TPR).  Each group owns a 128-element tile at a time (persistent
// grid-stride loop), its own A-operand buffer, staged inputs, mbarrier and W columns of the CTA's
// TMEM:
//   1. the tile's input rows are staged in shared memory (one coalesced copy);
//   2. the group's threads evaluate the encoding (a row per thread, grid levels NL at a time; with
//      TPR = 2 two threads share a row's levels) straight into the A operand;
//   3. per layer, one thread issues K/16 tcgen05.mma (M=128, N=width or 16, FP32 accumulate in
//      TMEM) and commits them to the group's mbarrier; after the wait each of the 4 warps reads
//      its 32-lane TMEM quarter (tcgen05.ld), applies the activation, converts and writes the
//      next A operand back into the same buffer (the MMAs have finished reading it);
//   4. the 16-wide output layer (accumulated into the same TMEM columns, which the previous
//      epilogue has drained) applies the output activation and writes FP32 rows.
// While one group runs its serial MMA/epilogue chain the other groups' gather-bound encodings keep
// the SM busy.  (G, NL) variants are instantiated and chosen by a measured autotune.
//
// The math is tiny-cuda-nn's FullyFusedMLP forward (rptr/ext/tiny-cuda-nn/src/fully_fused_mlp.cu:499-633)
// with FP32 instead of FP16 accumulation, fed by the composite encoding of encoding.cuh.
#pragma once

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


constexpr int kTcTile = 128;
constexpr int kGroupThreads = 128;
constexpr long long kWaitCycles = 4000000000ll;  // ~2 s at 2 GHz

// Shared-memory plan.  Layer l's B operand starts at byte 2 * layer_offset[l]: the network's
// matrices are contiguous and each is a multiple of 16 x 16 elements (512 bytes).
struct TcLayout {
    uint32_t w_bytes;             // resident weights; group g's region starts at w_bytes + g * group_stride
    uint32_t a_bytes;             // A operand tile (first in a group's region)
    uint32_t in_rel;              // staged input rows (FP32), relative to the region
    uint32_t in_ld;
    uint32_t group_stride;
    uint32_t lvl_off;             // grid level tables (kMaxGrids x kMaxLevels GridLevel)
    uint32_t bar_off;             // G + 1 mbarriers (the last for the staged levels), then the TMEM base address
    uint32_t total;
    uint32_t tmem_cols;           // G * width rounded up to a power of two
    uint32_t tab_off, tab_bytes;  // leading levels of the first grid staged in shared memory (FP16)
    uint32_t tab_levels;
};

__host__ __device__ inline uint32_t align_up(uint32_t v, uint32_t a) { return (v + a - 1) / a * a; }

__host__ __device__ inline TcLayout tc_layout(const ModelDesc& d, int G, bool stage_levels = false) {
    TcLayout L{};
    uint32_t off = align_up(d.n_params_network * 2u, 128);
    L.w_bytes = off;
    const uint32_t ka = d.enc_width > d.width ? d.enc_width : d.width;
    L.a_bytes = kTcTile * ka * 2u;
    L.in_ld = d.n_input + 1;
    L.in_rel = align_up(L.a_bytes, 128);
    L.group_stride = L.in_rel + align_up(kTcTile * L.in_ld * 4u, 128);
    off += (uint32_t)G * L.group_stride;
    L.lvl_off = off;
    off += kMaxGrids * kMaxLevels * (uint32_t)sizeof(GridLevel);
    if (stage_levels && d.n_grids > 0 && d.grids[0].interp != INTERP_NEAREST && d.grids[0].n_features == 2) {
        // as many leading levels of the first grid (4 bytes per FP16 entry pair) as fit in what is
        // left of the 227 KB a CTA may use
        const uint32_t tab_off = align_up(off, 128);
        const uint32_t tail = 8u * (uint32_t)G + 16u + 256u;
        const uint32_t room = 227u * 1024u > tab_off + tail ? 227u * 1024u - tab_off - tail : 0u;
        const GridDesc& g = d.grids[0];
        for (uint32_t l = 0; l < g.n_levels; ++l) {
            const uint32_t end = (g.levels[l].offset + g.levels[l].size) * 4u;
            if (end > room) break;
            L.tab_levels = l + 1;
            L.tab_bytes = end;
        }
        if (L.tab_levels) {
            L.tab_off = tab_off;
            off = tab_off + L.tab_bytes;
        }
    }
    L.bar_off = off;
    off += 8 * G + 16;
    L.total = align_up(off, 128);
    uint32_t cols = 32;
    while (cols < (uint32_t)G * d.width) cols <<= 1;   // TMEM allocations are powers of two
    L.tmem_cols = cols;
    return L;
}

template <int W, typename T, int G, int NL, bool ST, int TPR>
__global__ void __launch_bounds__(G * kGroupThreads * TPR, (G * TPR == 2 ? 2 : 1))
    k_forward_tc(const __grid_constant__ ModelDesc d, const __grid_constant__ ForwardArgs a, uint32_t* __restrict__ status) {
    using Op = tc::OpType<T>;
    // TPR threads per tile row: a pipeline has 4 * TPR warps; the encoding of a row is split in
    // TPR parts (encode_row_part) and each hidden epilogue in TPR column ranges, which halves
    // the latency chain of a tile when there are few tiles per pipeline (small batches)
    constexpr int kGT = kGroupThreads * TPR;     // threads of one tile pipeline
    constexpr int kThreads = G * kGT;
    extern __shared__ __align__(1024) uint8_t smem[];
    // ST: the first grid's leading levels are staged in shared memory (FP16 form), so their
    // gathers are shared-memory loads instead of L1/L2 requests
    const TcLayout L = tc_layout(d, G, ST && std::is_same<T, __half>::value);
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + L.bar_off);
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem + L.bar_off + 8 * G + 8);

    const uint32_t tid = threadIdx.x;
    const uint32_t warp = tid >> 5, lane = tid & 31;
    const uint32_t grp = warp / (4u * TPR);      // tile pipeline of this thread
    const uint32_t gtid = tid % (uint32_t)kGT;
    const uint32_t quarter = warp & 3u;          // TMEM lane quarter this warp may access
    const uint32_t part = gtid >> 7;             // row part (encoding) and column range (epilogue)
    const uint32_t bar_id = 1u + grp;
    // A CTA without a tile (device row counts below the launch size: the renderer's late rounds)
    // leaves before staging weights and allocating TMEM.  The test is uniform over the CTA.
    if (blockIdx.x * G >= forward_rows(a) / kTcTile) return;

    // Grid tables into L2 ahead of the gathers, when the batch's corner lookups number at least
    // a sixteenth of the entries (rows x levels x 8 corners x 16 >= entries): each CTA prefetches
    // its slice in 4 KB pieces.  A batch that starts with a cold L2 then meets L2 latency instead
    // of DRAM latency on its gathers.  Tables start on 512-byte boundaries and span multiples of
    // 32 bytes.
    if (d.n_grids > 0 && d.n_params_encoding > 0) {
        const uint32_t esz = std::is_same<T, __half>::value ? 2u : 4u;
        const uint8_t* base = std::is_same<T, __half>::value ? static_cast<const uint8_t*>(a.grid_h) + 2u * d.n_params_network
                                                             : reinterpret_cast<const uint8_t*>(a.params + d.n_params_network);
        const uint64_t total = (uint64_t)d.n_params_encoding * esz;
        const uint64_t touched = (uint64_t)forward_rows(a) * d.grids[0].n_levels * 8u * d.grids[0].n_features;
        if (16u * touched >= d.n_params_encoding) {
            const uint64_t per = ((total + gridDim.x - 1) / gridDim.x + 15u) & ~uint64_t(15);
            const uint64_t lo = (uint64_t)blockIdx.x * per, hi = lo + per < total ? lo + per : total;
            for (uint64_t off = lo + (uint64_t)threadIdx.x * 4096u; off < hi; off += (uint64_t)blockDim.x * 4096u)
                tc::prefetch_l2_bulk(base + off, (uint32_t)(hi - off < 4096u ? hi - off : 4096u));
        }
    }

    // ---- set-up: barriers, TMEM, resident weights ----
    if (tid == 0) {
        for (int g = 0; g <= G; ++g) tc::mbar_init(&bars[g], 1);
        tc::fence_barrier_init();
        if (L.tab_levels) {
            // one bulk copy of the staged levels (16-byte aligned: the grid starts on a 512-byte
            // boundary of the FP16 copy, levels on multiples of 8 entries)
            const uint8_t* src = static_cast<const uint8_t*>(a.grid_h) + 2u * d.grids[0].param_offset;
            tc::mbar_arrive_expect_tx(&bars[G], L.tab_bytes);
            tc::bulk_copy_g2s(smem + L.tab_off, src, L.tab_bytes, &bars[G]);
        }
    }
    if (warp == 0) {
        tc::tmem_alloc(tmem_slot, L.tmem_cols);
        tc::tmem_relinquish();
    }
    {
        // weights_op holds every layer as row-major [out][in] operand-typed values.
        const uint16_t* wsrc = reinterpret_cast<const uint16_t*>(a.weights_op);
        for (uint32_t l = 0; l < d.n_layers; ++l) {
            const uint32_t K = d.layer_in[l], N = d.layer_out[l];
            const uint32_t sbo = K * 16u;
            const uint32_t chunks = N * (K / 8u);
            const uint4* src = reinterpret_cast<const uint4*>(wsrc + d.layer_offset[l]);
            for (uint32_t c = tid; c < chunks; c += kThreads) {
                const uint32_t n = c / (K / 8u), k0 = (c - n * (K / 8u)) * 8u;
                *reinterpret_cast<uint4*>(smem + 2u * d.layer_offset[l] + tc::kmajor_offset(n, k0, sbo)) = src[c];
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
    bool aborted = false;
    if (L.tab_levels && !tc::mbar_wait_bounded(&bars[G], 0, kWaitCycles)) aborted = true;
    aborted = __syncthreads_or(aborted);
    const uint32_t* tab_s = reinterpret_cast<const uint32_t*>(smem + L.tab_off);
    const uint32_t tmem_base = *tmem_slot + grp * (uint32_t)W;
    uint8_t* a_tile = smem + L.w_bytes + grp * L.group_stride;
    float* in_s = reinterpret_cast<float*>(a_tile + L.in_rel);
    uint64_t* bar = &bars[grp];
    const uint32_t a_addr = tc::smem_addr(a_tile);

    uint32_t phase = 0;
    const uint32_t n_tiles = aborted ? 0u : forward_rows(a) / kTcTile;
    // the cell table of the FP16 tables, unless an optimizer step has changed them since it was
    // built (the corners are then gathered)
    const CellTable cells{a.cells && __ldg(a.cells_stale) == 0u ? static_cast<const uint4*>(a.cells) : nullptr, a.cell_base, a.cells_levels};
    const uint32_t row = quarter * 32u + lane;   // TMEM lane == tile row owned in the epilogue
    const uint32_t taddr_row = tmem_base + ((quarter * 32u) << 16);

    for (uint32_t tile = blockIdx.x * G + grp; tile < n_tiles; tile += gridDim.x * G) {
        const uint32_t row0 = tile * kTcTile;
        // 1. stage inputs (read once: streaming loads, so that they do not evict the grid tables
        //    from L2)
        const float* in_tile = a.in + (size_t)row0 * d.n_input;
        for (uint32_t idx = gtid; idx < kTcTile * d.n_input; idx += kGT) {
            const uint32_t r = idx / d.n_input, c = idx - r * d.n_input;
            in_s[r * L.in_ld + c] = __ldcs(in_tile + idx);
        }
        group_sync<kGT>(bar_id);
        // 2. encoding into the A operand (K = enc_width)
        {
            TcStore<T> st{a_tile, d.enc_width * 16u};
            // the FP16 form gathers from the FP16 copy of the grid tables (half the bytes per
            // entry, tiny-cuda-nn's half-precision parameters), the BF16 form from the FP32 tables
            if constexpr (TPR > 1) {
                if constexpr (std::is_same<T, __half>::value)
                    encode_row_part<NL, TPR>(d, lvl_s, static_cast<const __half*>(a.grid_h), in_s, L.in_ld, a.max_level_gpu, a.max_level, row0,
                                             gtid & 127u, part, st, tab_s, L.tab_levels, cells);
                else
                    encode_row_part<NL, TPR>(d, lvl_s, a.params, in_s, L.in_ld, a.max_level_gpu, a.max_level, row0, gtid & 127u, part, st);
            } else if constexpr (std::is_same<T, __half>::value) {
                encode_tile_rows<NL>(d, lvl_s, static_cast<const __half*>(a.grid_h), in_s, L.in_ld, a.max_level_gpu, a.max_level, row0, kTcTile,
                                     gtid, kGroupThreads, st, tab_s, L.tab_levels, cells);
            } else {
                encode_tile_rows<NL>(d, lvl_s, a.params, in_s, L.in_ld, a.max_level_gpu, a.max_level, row0, kTcTile, gtid, kGroupThreads, st);
            }
        }
        tc::fence_proxy_async_smem();
        tc::fence_before_sync();
        group_sync<kGT>(bar_id);

        // 3. layer chain
        for (uint32_t l = 0; l < d.n_layers; ++l) {
            const bool last = l + 1 == d.n_layers;
            const uint32_t K = d.layer_in[l];
            const uint32_t N = d.layer_out[l];
            const uint32_t sbo = K * 16u;
            if (gtid == 0) {
                tc::fence_after_sync();
                const uint32_t idesc = tc::make_idesc_f16(Op::kFmt, kTcTile, N);
                const uint32_t b_addr = tc::smem_addr(smem + 2u * d.layer_offset[l]);
                for (uint32_t k = 0; k < K; k += 16) {
                    const uint64_t adesc = tc::make_smem_desc(a_addr + (k / 8u) * 128u, 128u, sbo);
                    const uint64_t bdesc = tc::make_smem_desc(b_addr + (k / 8u) * 128u, 128u, sbo);
                    tc::mma_f16_ss(tmem_base, adesc, bdesc, idesc, k > 0 ? 1u : 0u);
                }
                tc::mma_commit(bar);
            }
            // Only the issuing thread polls the mbarrier; the rest of the group sleeps in the
            // named barrier instead of burning issue slots the other groups need.
            const bool ok = gtid != 0 || tc::mbar_wait_bounded(bar, phase, kWaitCycles);
            phase ^= 1u;
            if (group_sync_or<kGT>(bar_id, !ok)) { aborted = true; break; }
            tc::fence_after_sync();

            if (!last) {
                // hidden epilogue: each warp converts W / TPR columns of its 32 rows
                const uint32_t out_sbo = (uint32_t)W * 16u;
                const ReluOrNone act{d.act == ACT_RELU};
#pragma unroll
                for (uint32_t col = part * (uint32_t)(W / TPR); col < (part + 1u) * (uint32_t)(W / TPR); col += 32) {
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
            } else if (part == 0) {
                uint32_t r[16];
                tc::tmem_ld16(taddr_row, r);
                tc::tmem_wait_ld();
                const size_t grow = (size_t)row0 + row;
                if (a.out) {
                    // written once: streaming stores (evict-first in L2)
#pragma unroll
                    for (uint32_t c = 0; c < 16u; ++c)
                        if (c < d.n_output) __stcs(a.out + grow * d.n_output + c, act_fwd(d.out_act, __uint_as_float(r[c])));
                }
                if (a.y) {
                    float4* yv = reinterpret_cast<float4*>(a.y + grow * 16);
#pragma unroll
                    for (uint32_t j = 0; j < 4; ++j)
                        __stcs(yv + j, make_float4(act_fwd(d.out_act, __uint_as_float(r[4 * j])), act_fwd(d.out_act, __uint_as_float(r[4 * j + 1])),
                                                   act_fwd(d.out_act, __uint_as_float(r[4 * j + 2])), act_fwd(d.out_act, __uint_as_float(r[4 * j + 3]))));
                }
            }
            tc::fence_before_sync();
            group_sync<kGT>(bar_id);
        }
        if (aborted) break;
    }

    // ---- teardown ----
    if (aborted) {
        // Give the group's outstanding MMAs (and the staging copy) one more bounded chance to
        // finish before TMEM and shared memory are released.
        (void)tc::mbar_wait_bounded(bar, phase ^ 1u, kWaitCycles);
        if (L.tab_levels) (void)tc::mbar_wait_bounded(&bars[G], 0, kWaitCycles);
        if (gtid == 0) atomicOr(status, 1u);
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) {
        tc::fence_after_sync();
        tc::tmem_dealloc(*tmem_slot, L.tmem_cols);
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

// Dynamic shared memory request: what the tiles need, raised so that TMEM (512 columns per SM)
// can never be over-subscribed by co-resident CTAs.
size_t tc_smem_bytes(const ModelDesc& d, int G, bool stage_levels, int* per_sm_out) {
    const TcLayout L = tc_layout(d, G, stage_levels);
    const uint32_t cap = 512u / L.tmem_cols;               // CTAs whose TMEM fits on one SM
    const size_t sm_bytes = 233472;                        // 228 KB per SM
    size_t bytes = L.total;
    // With 1 KB reserved per CTA, at most floor(sm_bytes / (bytes + 1024)) CTAs fit.
    const size_t min_bytes = sm_bytes / (cap + 1) - 1024 + 16;
    if (bytes < min_bytes) bytes = min_bytes;
    bytes = (bytes + 127) / 128 * 128;
    int per_sm = (int)(sm_bytes / (bytes + 1024));
    if (per_sm > (int)cap) per_sm = (int)cap;
    if (per_sm_out) *per_sm_out = per_sm;
    return bytes;
}

struct Variant {
    int G, NL;
    bool stage_levels;
    int tpr;   // threads per tile row
};
constexpr Variant kVariants[] = {{2, 2, false, 1}, {2, 4, false, 1}, {4, 2, false, 1}, {4, 4, false, 1}, {6, 2, false, 1},
                                 {5, 2, false, 1}, {6, 1, false, 1}, {4, 2, true, 1},  {4, 1, true, 1},  {6, 1, true, 1},
                                 {2, 4, false, 2}, {4, 2, false, 2}, {4, 1, false, 2}, {3, 2, false, 2}};
constexpr int kNumVariants = sizeof(kVariants) / sizeof(kVariants[0]);

template <int W, typename T, int G, int NL, bool ST = false, int TPR = 1>
cudaError_t launch_variant(const ModelDesc& d, const ForwardArgs& a, uint32_t* status, cudaStream_t s) {
    int per_sm = 1;
    const size_t bytes = tc_smem_bytes(d, G, ST && std::is_same<T, __half>::value, &per_sm);
    if (bytes > 227u * 1024u || per_sm < 1) return cudaErrorInvalidConfiguration;
    const uint32_t n_tiles = a.n / kTcTile;
    const void* kern = (const void*)k_forward_tc<W, T, G, NL, ST, TPR>;
    cudaError_t e = ensure_dynamic_smem(kern, bytes);
    if (e != cudaSuccess) return e;
    if (TPR > 1) {
        // eight warps per pipeline: registers, not shared memory or TMEM, bound the CTAs that are
        // resident at once, and a grid larger than that would run in two waves
        const int fit = resident_blocks(kern, G * kGroupThreads * TPR, bytes);
        if (fit < 1) return cudaErrorInvalidConfiguration;
        if (per_sm > fit) per_sm = fit;
    }
    uint32_t blocks = (uint32_t)(per_sm * sm_count());
    const uint32_t need = (n_tiles + G - 1) / G;
    if (blocks > need) blocks = need;
    if (blocks == 0) return cudaSuccess;
    k_forward_tc<W, T, G, NL, ST, TPR><<<blocks, G * kGroupThreads * TPR, bytes, s>>>(d, a, status);
    return cudaGetLastError();
}

template <int W, typename T>
cudaError_t launch_typed(const ModelDesc& d, const ForwardArgs& a, int variant, uint32_t* status, cudaStream_t s) {
    switch (variant) {
        case 0: return launch_variant<W, T, 2, 2>(d, a, status, s);
        case 1: return launch_variant<W, T, 2, 4>(d, a, status, s);
        case 2: return launch_variant<W, T, 4, 2>(d, a, status, s);
        case 3: return launch_variant<W, T, 4, 4>(d, a, status, s);
        case 4: return launch_variant<W, T, 6, 2>(d, a, status, s);
        case 5: return launch_variant<W, T, 5, 2>(d, a, status, s);
        case 6: return launch_variant<W, T, 6, 1>(d, a, status, s);
        // the staging variants exist for the FP16 form (its grid tables have an FP16 copy)
        case 7: return std::is_same<T, __half>::value ? launch_variant<W, T, 4, 2, true>(d, a, status, s) : cudaErrorInvalidValue;
        case 8: return std::is_same<T, __half>::value ? launch_variant<W, T, 4, 1, true>(d, a, status, s) : cudaErrorInvalidValue;
        case 9: return std::is_same<T, __half>::value ? launch_variant<W, T, 6, 1, true>(d, a, status, s) : cudaErrorInvalidValue;
        // two threads per tile row (small batches: about one tile per pipeline)
        case 10: return launch_variant<W, T, 2, 4, false, 2>(d, a, status, s);
        case 11: return launch_variant<W, T, 4, 2, false, 2>(d, a, status, s);
        case 12: return launch_variant<W, T, 4, 1, false, 2>(d, a, status, s);
        case 13: return launch_variant<W, T, 3, 2, false, 2>(d, a, status, s);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace
}  // namespace nlod
