// Host-side launchers of the device kernels.  All launchers are asynchronous on `stream`,
// validate nothing (the C ABI validates first) and return the cudaError_t of the launch.
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <map>
#include <mutex>
#include <utility>

#include "desc.h"

namespace nlod {

// Raises a kernel's dynamic shared-memory limit to at least `bytes` on the current device.  The
// attribute is set only when the limit recorded for (kernel, device) is lower, so that repeated
// launches of small batches do not pay for a cudaFuncSetAttribute call each.
inline cudaError_t ensure_dynamic_smem(const void* kernel, size_t bytes) {
    static std::mutex mu;
    static std::map<std::pair<const void*, int>, size_t> limits;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lock(mu);
    size_t& cur = limits[{kernel, dev}];
    if (cur >= bytes) return cudaSuccess;
    e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e == cudaSuccess) cur = bytes;
    return e;
}

// CTAs of `kernel` with `threads` threads and `bytes` of dynamic shared memory that fit on one SM
// at once (registers, threads and shared memory; cudaOccupancyMaxActiveBlocksPerMultiprocessor),
// computed once per (kernel, device, bytes).  0 on an error.
inline int resident_blocks(const void* kernel, int threads, size_t bytes) {
    static std::mutex mu;
    static std::map<std::pair<std::pair<const void*, int>, size_t>, int> cache;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    std::lock_guard<std::mutex> lock(mu);
    auto it = cache.find({{kernel, dev}, bytes});
    if (it != cache.end()) return it->second;
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel, threads, bytes) != cudaSuccess) n = 0;
    cache[{{kernel, dev}, bytes}] = n;
    return n;
}

// Inputs shared by every forward-style launch.
struct ForwardArgs {
    uint32_t n;                       // elements (multiple of 128)
    const float* in;                  // [n][n_input]
    const float* params;              // FP32 parameters (network then encoding)
    const void* weights_op;           // network weights in the operand type (FP16/BF16 forms)
    const void* grid_h;               // FP16 copy of the parameters' grid tables (FP16 tensor-core inference)
    const void* cells;                // nullable: cell table of grid_h's leading levels (cells.cu)
    uint32_t cells_levels;            // levels of the first grid that the cell table covers
    const uint32_t* cells_stale;      // device word: nonzero while the table lags grid_h (then unused)
    uint32_t cell_base[kMaxLevels];   // first record of each covered level
    const float* max_level_gpu;       // nullable, [n]
    float max_level;                  // scalar fallback (1000 = off)
    float* out;                       // nullable, [n][n_output]
    // training extras (all nullable)
    float* enc;                       // [n][enc_width] encoded input
    float* hidden;                    // [n_hidden_layers][n][width] post-activation hidden values
    float* y;                         // [n][16] post-activation outputs (padded)
    // fused loss (loss_kind != LOSS_NONE)
    int32_t loss_kind;
    const float* target;              // [n][n_output]
    float loss_scale;
    float* dz;                        // [n][16] dL/d(pre-activation output) * loss_scale
    float* loss_partial;              // [gridDim.x] per-block loss sums (mean-normalised)
    // inference only: when set, the rows to process are min(n, *n_dev rounded up to 128); rows
    // past *n_dev inside the last tile are computed from whatever the input holds and ignored
    const uint32_t* n_dev;
};

// Rows an inference launch processes (n, or the device-side count when given).
__device__ __forceinline__ uint32_t forward_rows(const ForwardArgs& a) {
    if (!a.n_dev) return a.n;
    const uint32_t c = (*a.n_dev + 127u) & ~127u;
    return c < a.n ? c : a.n;
}

// Plain FP32 form.
cudaError_t launch_forward_simt(const ModelDesc& d, const ForwardArgs& a, int n_blocks_hint, cudaStream_t s);
int forward_simt_blocks(const ModelDesc& d);

// dz -> per-layer deltas + dL/d(encoding) (plain FP32).
struct BackwardArgs {
    uint32_t n;
    const float* params;              // FP32 weights
    const float* hidden;              // [n_hidden][n][width]
    const float* dz;                  // [n][16]
    float* delta;                     // [n_hidden][n][width]: delta of hidden layer l (pre-activation)
    float* d_enc;                     // [n][enc_width]
};
cudaError_t launch_backward_delta_simt(const ModelDesc& d, const BackwardArgs& a, cudaStream_t s);

// dW_l += delta_l^T a_{l-1} for every layer (split over rows, FP32 atomics into grads).
struct WeightGradArgs {
    uint32_t n;
    const float* enc;                 // [n][enc_width]
    const float* hidden;              // [n_hidden][n][width]
    const float* delta;               // [n_hidden][n][width]
    const float* dz;                  // [n][16]
    float* grads;                     // FP32 gradient vector (network part accumulated)
};
cudaError_t launch_weight_grad_simt(const ModelDesc& d, const WeightGradArgs& a, cudaStream_t s);

// Grid-table gradient scatter from dL/d(encoding).
struct GridBackwardArgs {
    uint32_t n;
    const float* in;
    const float* d_enc;               // [n][enc_width]
    const float* max_level_gpu;
    float max_level;
    float* grads;
};
cudaError_t launch_grid_backward(const ModelDesc& d, const GridBackwardArgs& a, cudaStream_t s);

// dz[r][c] = dL_dout[r][c] * act'(y[r][c]) for c < n_output, 0 for the padding columns.
cudaError_t launch_dz_from_dout(const ModelDesc& d, uint32_t n, const float* dL_dout, const float* y, float* dz, cudaStream_t s);

// Sum of per-block partials into *out (single block).
cudaError_t launch_reduce_sum(const float* partial, uint32_t n, float* out, float scale, cudaStream_t s);

// FP32 -> operand type copy of the network weights (kind 1 = FP16, 2 = BF16).
cudaError_t launch_convert_weights(const float* src, void* dst, uint32_t n, int kind, cudaStream_t s);

// Parameter initialisation: uniform(lo, hi) from a counter-based PCG stream.
cudaError_t launch_init_uniform(float* p, uint32_t n, uint64_t seed, uint64_t stream_id, float lo, float hi, cudaStream_t s);

// Optimizer step over all parameters (Adam + optional EMA), see optim.cu.
struct AdamStepArgs {
    uint32_t n_params;
    uint32_t n_matrix;                // leading matrix (network) parameters
    AdamParams hp;
    float learning_rate;              // after exponential decay
    float loss_scale;
    float lower_lr_bound, upper_lr_bound;
    float log2_beta1, log2_beta2;     // log2 of the moment decay rates (bias correction)
    float* params;                    // FP32 master
    const float* grads;               // FP32, scaled by loss_scale
    float* m1;
    float* m2;
    uint32_t* steps;
    // EMA (nullable ema)
    float* ema;
    float ema_decay, ema_debias_old, ema_debias_new;
    // nullable: FP16 copy of the inference values (the EMA when present) of the non-matrix
    // parameters, refreshed in the same pass
    __half* grid_h;
    // nullable: FP16 copy of the training values of the non-matrix parameters, kept apart from
    // grid_h when an EMA makes the inference values differ (the FP16 training step gathers from it)
    __half* grid_h_train;
    // nullable: BF16 copy of the training values of the non-matrix parameters (the BF16 training
    // step gathers from it)
    __nv_bfloat16* grid_b_train;
    // nullable: operand-type copies of the matrix parameters (training values, inference values),
    // refreshed in the same pass; op_kind 1 = FP16, 2 = BF16
    void* w_op;
    void* w_op_inf;
    int32_t op_kind;
    // nullable: set to 1 by the step (grid_h changes, the cell table of grid_h is out of date)
    uint32_t* cells_stale;
};
cudaError_t launch_adam_step(const AdamStepArgs& a, cudaStream_t s);

// Fixed scratch of the training step that allocates nothing (noalloc.cu): 16 MiB.
constexpr size_t kNoAllocScratchBytes = size_t(16) << 20;
cudaError_t noalloc_scratch(void** ptr, size_t* bytes);

// Tensor-core (tcgen05) forms.  kind 1 = FP16, 2 = BF16.  `variant` selects the CTA
// organisation (tile pipelines per CTA, grid levels per gather unit); see tc.cu.
bool tc_supported(const ModelDesc& d);
int tc_num_variants();
// kind: operand type of the module (1 = FP16, 2 = BF16); the variants that stage grid levels in
// shared memory read the FP16 copy of the tables and exist for the FP16 form only.
bool tc_variant_ok(const ModelDesc& d, int variant, int kind = 1);
int tc_default_variant(const ModelDesc& d);
cudaError_t launch_forward_tc(const ModelDesc& d, const ForwardArgs& a, int kind, int variant, uint32_t* status, cudaStream_t s);

// cells.cu: the cell table of the first grid's leading levels (FP16 tables), its (re)build from
// the FP16 copy grid_h.
// Levels it covers (0: none) and their record bases (base[l], base[levels] = all records).
uint32_t cells_levels_of(const ModelDesc& d, uint32_t (&base)[kMaxLevels + 1]);
cudaError_t launch_build_cells(const ModelDesc& d, const void* grid_h, uint32_t levels, const uint32_t (&base)[kMaxLevels + 1], void* cells,
                               cudaStream_t s);

// calib.cu
cudaError_t launch_calib_gathers(const ModelDesc& d, const void* params, bool half_tables, uint32_t n, float* sink, cudaStream_t s,
                                 const void* cells = nullptr, uint32_t cells_levels = 0, const uint32_t* cell_base = nullptr);
cudaError_t launch_calib_scatter(const ModelDesc& d, float* grads, uint32_t n, cudaStream_t s);

// Fused tensor-core training step (train_tc.cu): encoding, forward, loss, backward, weight
// gradients and grid-gradient scatter.  grads must be zeroed by the caller; gradients are
// accumulated as dL/dparam * grad_scale.
struct TrainTcArgs {
    uint32_t n;
    const float* in;                  // [n][n_input]
    const float* params;              // FP32 parameters (grid tables read by the encoding)
    const void* weights_op;           // network weights in the operand type
    const float* max_level_gpu;
    float max_level;
    int32_t loss_kind;
    const float* target;              // [n][n_output]
    float inv_n_total;                // 1 / (n * n_output): the loss is a mean
    float grad_scale;                 // loss_scale * inv_n_total
    float* grads;                     // FP32 gradient vector
    float* loss_partial;              // [gridDim.x] per-CTA loss sums (nullable)
    void* enc_tiles;                  // [n/128][128 x enc_width] operand-type X0 tiles written by
                                      // launch_encode_tiles and bulk-copied by the fused kernel
    const void* grid_h;               // nullable: 16-bit copy of the training values' grid tables in
                                      // the operand type (FP16 or BF16), read by launch_encode_tiles
    uint32_t zero_grads_n;            // launch_encode_tiles zeroes grads[0, zero_grads_n) (multiple of 4)
    uint32_t group_levels;            // grid levels a tile pipeline scatters itself when a
                                      // scatter team takes the rest (set by launch_train_tc)
};
// Tile pipelines per CTA that fit the network (0 = network not supported by the fused kernel).
int train_tc_groups(const ModelDesc& d);
cudaError_t launch_train_tc(const ModelDesc& d, const TrainTcArgs& a, int kind, int groups, uint32_t* status, cudaStream_t s);
// CTAs launch_train_tc uses for a batch of n (each writes its loss_partial entry).
uint32_t train_tc_blocks(uint32_t n, int groups);
// Encodes the batch into a.enc_tiles (kind 1 = FP16, 2 = BF16).
cudaError_t launch_encode_tiles(const ModelDesc& d, const TrainTcArgs& a, int kind, cudaStream_t s);

}  // namespace nlod
