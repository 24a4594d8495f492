// Plain FP32 form of the neural-LoD query and its training (CUDA cores only).
//
// Forward: one CTA handles 64 elements at a time (grid-stride over tiles): the tile's input
// rows are staged in shared memory, every (element, encoding part) pair is evaluated by one
// thread into the encoded tile, then each layer is a shared-memory tiled GEMM
// (act[64][K] x W^T[K][N]) with a 4-column x N/16-row register block per thread.
// The output activation and the loss (value + scaled gradient) are fused into the epilogue.
//
// Semantics follow tiny-cuda-nn's FullyFusedMLP / losses (paths relative to
// rptr/ext/tiny-cuda-nn/): src/fully_fused_mlp.cu:499-633 (layer chain, output padded to 16),
// include/tiny-cuda-nn/common_device.h:68-230 (activations),
// include/tiny-cuda-nn/losses/binary_cross_entropy.h:7-43, losses/relative_l2.h:39-76.
#include <cuda_runtime.h>

#include <cstdint>

#include "activation.cuh"
#include "desc.h"
#include "encoding.cuh"
#include "kernels.h"

namespace nlod {

namespace {

constexpr int kTile = 64;
constexpr int kThreads = 256;

// Per-element loss value (already divided by n_total) and d loss / d prediction (scaled).
__device__ __forceinline__ float loss_eval(int32_t kind, float pred, float target, float inv_n_total, float loss_scale, float& grad) {
    switch (kind) {
        case LOSS_BCE: {
            const float eps = 1e-5f;
            const float p = fminf(fmaxf(pred, eps), 1.f - eps);
            const float value = -(target * logf(p) + (1.f - target) * logf(1.f - p)) * inv_n_total;
            grad = loss_scale * (-(target - p) / (p - p * p)) * inv_n_total;
            return value;
        }
        case LOSS_RELATIVE_L2: {
            const float den = pred * pred + 0.01f;
            const float diff = pred - target;
            grad = loss_scale * (2.f * diff / den) * inv_n_total;
            return diff * diff / den * inv_n_total;
        }
        case LOSS_L2: {
            const float diff = pred - target;
            grad = loss_scale * (2.f * diff) * inv_n_total;
            return diff * diff * inv_n_total;
        }
        default: grad = 0.f; return 0.f;
    }
}

// acc[r][j] = sum_k A[row(r)][k] * WT[k][c0 + 4 cg + j] for NC output columns starting at c0.
// Thread layout: NC/4 column groups x (kThreads / (NC/4)) row groups of RPT rows.
template <int NC>
struct LayerBlock {
    static constexpr int CG = NC / 4;
    static constexpr int RG = kThreads / CG;
    static constexpr int RPT = kTile / RG;
    static_assert(RPT >= 1 && RPT * RG == kTile, "bad tiling");
    float acc[RPT][4];

    __device__ __forceinline__ int cg() const { return threadIdx.x % CG; }
    __device__ __forceinline__ int row(int r) const { return (threadIdx.x / CG) * RPT + r; }

    __device__ __forceinline__ void compute(const float* __restrict__ A, int lda, int K, const float* __restrict__ WT, int ldw, int c0) {
#pragma unroll
        for (int r = 0; r < RPT; ++r)
#pragma unroll
            for (int j = 0; j < 4; ++j) acc[r][j] = 0.f;
        const int col = c0 + 4 * cg();
        for (int k = 0; k < K; k += 4) {
            float4 a[RPT];
#pragma unroll
            for (int r = 0; r < RPT; ++r) a[r] = *reinterpret_cast<const float4*>(A + row(r) * lda + k);
#pragma unroll
            for (int kk = 0; kk < 4; ++kk) {
                const float4 w = *reinterpret_cast<const float4*>(WT + (k + kk) * ldw + col);
#pragma unroll
                for (int r = 0; r < RPT; ++r) {
                    const float av = kk == 0 ? a[r].x : kk == 1 ? a[r].y : kk == 2 ? a[r].z : a[r].w;
                    acc[r][0] = fmaf(av, w.x, acc[r][0]);
                    acc[r][1] = fmaf(av, w.y, acc[r][1]);
                    acc[r][2] = fmaf(av, w.z, acc[r][2]);
                    acc[r][3] = fmaf(av, w.w, acc[r][3]);
                }
            }
        }
    }
};

// Encoded features as FP32 into a row-major shared tile.
struct SimtStore {
    float* act;
    uint32_t lda;
    template <int M>
    __device__ __forceinline__ void run(uint32_t r, uint32_t col, const float (&f)[M], uint32_t n) {
        float* dst = act + r * lda + col;
        if (n == (uint32_t)M && (col & 3u) == 0) {
#pragma unroll
            for (int i = 0; i < M; i += 4) *reinterpret_cast<float4*>(dst + i) = make_float4(f[i], f[i + 1], f[i + 2], f[i + 3]);
        } else {
#pragma unroll
            for (uint32_t i = 0; i < (uint32_t)M; ++i)
                if (i < n) dst[i] = f[i];
        }
    }
    __device__ __forceinline__ void one(uint32_t r, uint32_t col, float v) { act[r * lda + col] = v; }
};

// Loads W [out][in] (row-major, global) transposed into WT[in][out] in shared memory.
__device__ __forceinline__ void load_weights_transposed(const float* __restrict__ W, int n_out, int n_in, float* WT) {
    for (int idx = threadIdx.x; idx < n_out * n_in; idx += kThreads) {
        const int o = idx / n_in, i = idx - o * n_in;
        WT[i * n_out + o] = W[idx];
    }
}

// Loads W [rows][cols] as is (row-major) into shared memory.
__device__ __forceinline__ void load_weights(const float* __restrict__ W, int count, float* Ws) {
    for (int idx = threadIdx.x; idx < count; idx += kThreads) Ws[idx] = W[idx];
}

struct SimtSmem {
    int lda_in, lda_a, lda_b;
    size_t off_in, off_a, off_b, off_w, off_red, total_floats;
};

__host__ __device__ inline SimtSmem simt_smem_layout(const ModelDesc& d) {
    SimtSmem s;
    s.lda_in = (int)d.n_input + 1;
    const int ka = (int)(d.enc_width > d.width ? d.enc_width : d.width);
    s.lda_a = ka + 4;
    s.lda_b = (int)d.width + 4;
    uint32_t wmax = 0;
    for (uint32_t l = 0; l < d.n_layers; ++l) {
        const uint32_t c = d.layer_in[l] * d.layer_out[l];
        wmax = c > wmax ? c : wmax;
    }
    s.off_in = 0;
    s.off_a = s.off_in + (size_t)kTile * s.lda_in;
    s.off_a = (s.off_a + 3) & ~size_t(3);
    s.off_b = s.off_a + (size_t)kTile * s.lda_a;
    s.off_w = s.off_b + (size_t)kTile * s.lda_b;
    s.off_red = s.off_w + wmax;
    s.total_floats = s.off_red + kThreads / 32;
    return s;
}

template <int W>
__global__ void __launch_bounds__(kThreads) k_forward_simt(const __grid_constant__ ModelDesc d, const __grid_constant__ ForwardArgs a) {
    extern __shared__ float4 smem4[];
    float* smem = reinterpret_cast<float*>(smem4);
    const SimtSmem L = simt_smem_layout(d);
    float* in_s = smem + L.off_in;
    float* act_a = smem + L.off_a;
    float* act_b = smem + L.off_b;
    float* w_s = smem + L.off_w;
    float* red_s = smem + L.off_red;

    const uint32_t n_tiles = forward_rows(a) / kTile;
    const float inv_n_total = 1.0f / ((float)a.n * (float)d.n_output);
    float loss_acc = 0.f;

    for (uint32_t tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
        const uint32_t row0 = tile * kTile;
        // 1. stage the input rows (contiguous in global memory)
        const float* in_tile = a.in + (size_t)row0 * d.n_input;
        for (uint32_t idx = threadIdx.x; idx < kTile * d.n_input; idx += kThreads) {
            const uint32_t r = idx / d.n_input, c = idx - r * d.n_input;
            in_s[r * L.lda_in + c] = in_tile[idx];
        }
        __syncthreads();
        // 2. encoding into act_a
        {
            SimtStore st{act_a, (uint32_t)L.lda_a};
            encode_tile<2>(d, a.params, in_s, (uint32_t)L.lda_in, a.max_level_gpu, a.max_level, row0, kTile, threadIdx.x, kThreads, st);
        }
        __syncthreads();
        if (a.enc) {
            for (uint32_t idx = threadIdx.x; idx < kTile * d.enc_width; idx += kThreads) {
                const uint32_t r = idx / d.enc_width, c = idx - r * d.enc_width;
                a.enc[(size_t)(row0 + r) * d.enc_width + c] = act_a[r * L.lda_a + c];
            }
        }
        // 3. hidden layers (ping-pong between act_a and act_b)
        float* cur = act_a;
        int ld_cur = L.lda_a;
        for (uint32_t l = 0; l + 1 < d.n_layers; ++l) {
            const int K = (int)d.layer_in[l];
            load_weights_transposed(a.params + d.layer_offset[l], W, K, w_s);
            __syncthreads();
            float* nxt = (cur == act_a) ? act_b : act_a;
            const int ld_nxt = (cur == act_a) ? L.lda_b : L.lda_a;
            LayerBlock<W> lb;
            lb.compute(cur, ld_cur, K, w_s, W, 0);
            __syncthreads();  // everyone done reading cur / w_s
            const ReluOrNone act{d.act == ACT_RELU};
#pragma unroll
            for (int r = 0; r < LayerBlock<W>::RPT; ++r) {
                float4 v;
                v.x = act(lb.acc[r][0]);
                v.y = act(lb.acc[r][1]);
                v.z = act(lb.acc[r][2]);
                v.w = act(lb.acc[r][3]);
                *reinterpret_cast<float4*>(nxt + lb.row(r) * ld_nxt + 4 * lb.cg()) = v;
                if (a.hidden) {
                    *reinterpret_cast<float4*>(a.hidden + ((size_t)l * a.n + row0 + lb.row(r)) * W + 4 * lb.cg()) = v;
                }
            }
            cur = nxt;
            ld_cur = ld_nxt;
            __syncthreads();
        }
        // 4. output layer (16 padded rows) + output activation + fused loss
        {
            const uint32_t l = d.n_layers - 1;
            load_weights_transposed(a.params + d.layer_offset[l], 16, W, w_s);
            __syncthreads();
            LayerBlock<16> lb;
            lb.compute(cur, ld_cur, W, w_s, 16, 0);
            const uint32_t r = lb.row(0);
            const uint32_t grow = row0 + r;
            float yv[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) yv[j] = act_fwd(d.out_act, lb.acc[0][j]);
            if (a.y) *reinterpret_cast<float4*>(a.y + (size_t)grow * 16 + 4 * lb.cg()) = make_float4(yv[0], yv[1], yv[2], yv[3]);
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const uint32_t c = 4 * lb.cg() + j;
                if (a.out && c < d.n_output) a.out[(size_t)grow * d.n_output + c] = yv[j];
            }
            if (a.loss_kind != LOSS_NONE) {
                float dzv[4];
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const uint32_t c = 4 * lb.cg() + j;
                    float g = 0.f;
                    if (c < d.n_output) {
                        loss_acc += loss_eval(a.loss_kind, yv[j], a.target[(size_t)grow * d.n_output + c], inv_n_total, a.loss_scale, g);
                        g *= act_grad_from_output(d.out_act, yv[j]);
                    }
                    dzv[j] = g;
                }
                *reinterpret_cast<float4*>(a.dz + (size_t)grow * 16 + 4 * lb.cg()) = make_float4(dzv[0], dzv[1], dzv[2], dzv[3]);
            }
            __syncthreads();
        }
    }
    if (a.loss_kind != LOSS_NONE && a.loss_partial) {
        float v = loss_acc;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) == 0) red_s[threadIdx.x >> 5] = v;
        __syncthreads();
        if (threadIdx.x == 0) {
            float s = 0.f;
            for (int w = 0; w < kThreads / 32; ++w) s += red_s[w];
            a.loss_partial[blockIdx.x] = s;
        }
    }
}

// Backward through the layer chain: delta_{l-1} = (delta_l W_l) * act'(h_{l-1}); d_enc = delta_0 W_0.
template <int W>
__global__ void __launch_bounds__(kThreads) k_backward_delta_simt(const __grid_constant__ ModelDesc d, const __grid_constant__ BackwardArgs a) {
    extern __shared__ float4 smem4[];
    float* smem = reinterpret_cast<float*>(smem4);
    const int lda = (int)(d.enc_width > d.width ? d.enc_width : d.width) + 4;
    float* buf_a = smem;                         // [64][lda]
    float* buf_b = buf_a + kTile * lda;          // [64][lda]
    float* w_s = buf_b + kTile * lda;            // weights as stored [out][in]

    const uint32_t n_tiles = a.n / kTile;
    for (uint32_t tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
        const uint32_t row0 = tile * kTile;
        // delta of the output (pre-activation), 16 wide
        for (uint32_t idx = threadIdx.x; idx < kTile * 16; idx += kThreads) {
            const uint32_t r = idx / 16, c = idx % 16;
            buf_a[r * lda + c] = a.dz[(size_t)(row0 + r) * 16 + c];
        }
        float* cur = buf_a;
        int K = 16;
        for (int l = (int)d.n_layers - 1; l >= 0; --l) {
            // cur: delta_l [64][K=out_l]; W_l [out_l][in_l] is the [K][N] operand as stored.
            const int n_in = (int)d.layer_in[l];
            load_weights(a.params + d.layer_offset[l], K * n_in, w_s);
            __syncthreads();
            float* nxt = cur == buf_a ? buf_b : buf_a;
            if (l > 0) {
                LayerBlock<W> lb;
                lb.compute(cur, lda, K, w_s, n_in, 0);
                const float* h = a.hidden + (size_t)(l - 1) * a.n * W;
#pragma unroll
                for (int r = 0; r < LayerBlock<W>::RPT; ++r) {
                    const size_t g = (size_t)(row0 + lb.row(r)) * W + 4 * lb.cg();
                    const float4 hv = *reinterpret_cast<const float4*>(h + g);
                    float4 v;
                    v.x = d.act == ACT_RELU ? (hv.x > 0.f ? lb.acc[r][0] : 0.f) : lb.acc[r][0];
                    v.y = d.act == ACT_RELU ? (hv.y > 0.f ? lb.acc[r][1] : 0.f) : lb.acc[r][1];
                    v.z = d.act == ACT_RELU ? (hv.z > 0.f ? lb.acc[r][2] : 0.f) : lb.acc[r][2];
                    v.w = d.act == ACT_RELU ? (hv.w > 0.f ? lb.acc[r][3] : 0.f) : lb.acc[r][3];
                    *reinterpret_cast<float4*>(nxt + lb.row(r) * lda + 4 * lb.cg()) = v;
                    *reinterpret_cast<float4*>(a.delta + (size_t)(l - 1) * a.n * W + g) = v;
                }
            } else {
                // dL/d(encoding), in 16-column chunks
                for (int c0 = 0; c0 < n_in; c0 += 16) {
                    LayerBlock<16> lb;
                    lb.compute(cur, lda, K, w_s, n_in, c0);
                    const size_t g = (size_t)(row0 + lb.row(0)) * d.enc_width + c0 + 4 * lb.cg();
                    *reinterpret_cast<float4*>(a.d_enc + g) = make_float4(lb.acc[0][0], lb.acc[0][1], lb.acc[0][2], lb.acc[0][3]);
                }
            }
            __syncthreads();
            cur = nxt;
            K = W;
        }
    }
}

// dW_l[o][i] += sum_r D_l[r][o] * A_l[r][i] over a chunk of rows.  blockIdx.z = layer,
// blockIdx.y = 64x64 output block, blockIdx.x = row chunk.
__global__ void __launch_bounds__(kThreads) k_weight_grad_simt(const __grid_constant__ ModelDesc d, const __grid_constant__ WeightGradArgs a, uint32_t rows_per_chunk) {
    __shared__ float Ds[32][64 + 4];
    __shared__ float As[32][64 + 4];
    const uint32_t l = blockIdx.z;
    if (l >= d.n_layers) return;
    const uint32_t n_out = d.layer_out[l], n_in = d.layer_in[l];
    const uint32_t ob_count = (n_out + 63) / 64, ib_count = (n_in + 63) / 64;
    if (blockIdx.y >= ob_count * ib_count) return;
    const uint32_t o0 = (blockIdx.y / ib_count) * 64, i0 = (blockIdx.y % ib_count) * 64;
    const float* D;
    uint32_t ldd;
    if (l + 1 == d.n_layers) { D = a.dz; ldd = 16; }
    else { D = a.delta + (size_t)l * a.n * d.width; ldd = d.width; }
    const float* A;
    uint32_t lda;
    if (l == 0) { A = a.enc; lda = d.enc_width; }
    else { A = a.hidden + (size_t)(l - 1) * a.n * d.width; lda = d.width; }

    const uint32_t r_begin = blockIdx.x * rows_per_chunk;
    const uint32_t r_end = min(a.n, r_begin + rows_per_chunk);
    const int ti = threadIdx.x % 16, to = threadIdx.x / 16;  // 16 x 16 threads, 4x4 outputs each
    float acc[4][4] = {};
    for (uint32_t r0 = r_begin; r0 < r_end; r0 += 32) {
        for (uint32_t idx = threadIdx.x; idx < 32 * 64; idx += kThreads) {
            const uint32_t rr = idx / 64, c = idx % 64;
            const uint32_t row = r0 + rr;
            Ds[rr][c] = (row < r_end && o0 + c < n_out) ? D[(size_t)row * ldd + o0 + c] : 0.f;
            As[rr][c] = (row < r_end && i0 + c < n_in) ? A[(size_t)row * lda + i0 + c] : 0.f;
        }
        __syncthreads();
#pragma unroll 8
        for (int rr = 0; rr < 32; ++rr) {
            float dv[4], av[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) { dv[j] = Ds[rr][to * 4 + j]; av[j] = As[rr][ti * 4 + j]; }
#pragma unroll
            for (int x = 0; x < 4; ++x)
#pragma unroll
                for (int y = 0; y < 4; ++y) acc[x][y] = fmaf(dv[x], av[y], acc[x][y]);
        }
        __syncthreads();
    }
    float* G = a.grads + d.layer_offset[l];
#pragma unroll
    for (int x = 0; x < 4; ++x) {
        const uint32_t o = o0 + to * 4 + x;
        if (o >= n_out) continue;
#pragma unroll
        for (int y = 0; y < 4; ++y) {
            const uint32_t i = i0 + ti * 4 + y;
            if (i < n_in) atomicAdd(G + (size_t)o * n_in + i, acc[x][y]);
        }
    }
}

// One thread per (element, grid level); lanes of a warp share the level.
__global__ void __launch_bounds__(kThreads) k_grid_backward(const __grid_constant__ ModelDesc d, const __grid_constant__ GridBackwardArgs a, uint32_t slot_idx) {
    const Slot& s = d.slots[slot_idx];
    const GridDesc& g = d.grids[s.grid];
    const uint32_t level = blockIdx.y;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool in_range = i < a.n;
    const uint32_t ii = in_range ? i : 0;
    const float ml = a.max_level_gpu ? a.max_level_gpu[ii] : a.max_level;
    const bool active = in_range && !grid_level_skipped_backward(level, ml, g.n_levels);
    const float* row = a.in + (size_t)ii * d.n_input + s.in_begin;
    const float2 dy = *reinterpret_cast<const float2*>(a.d_enc + (size_t)ii * d.enc_width + s.out_begin + 2 * level);
    grid_level_backward(g, level, a.grads + g.param_offset, row[0], row[1], row[2], dy, active);
}

__global__ void k_dz_from_dout(const __grid_constant__ ModelDesc d, uint32_t n, const float* __restrict__ dL_dout,
                               const float* __restrict__ y, float* __restrict__ dz) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n * 16u) return;
    const uint32_t r = i / 16u, c = i % 16u;
    dz[i] = c < d.n_output ? dL_dout[(size_t)r * d.n_output + c] * act_grad_from_output(d.out_act, y[i]) : 0.f;
}

__global__ void k_reduce_sum(const float* __restrict__ partial, uint32_t n, float* __restrict__ out, float scale) {
    __shared__ float red[32];
    float v = 0.f;
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) v += partial[i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        float s = 0.f;
        for (uint32_t w = 0; w < (blockDim.x + 31) / 32; ++w) s += red[w];
        *out = s * scale;
    }
}

int g_num_sms = 0;
int num_sms() {
    if (g_num_sms == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev);
        if (g_num_sms <= 0) g_num_sms = 1;
    }
    return g_num_sms;
}

template <typename K>
cudaError_t set_smem(K kernel, size_t bytes) {
    return ensure_dynamic_smem((const void*)kernel, bytes);
}

}  // namespace

int forward_simt_blocks(const ModelDesc& d) {
    const SimtSmem L = simt_smem_layout(d);
    const size_t bytes = L.total_floats * sizeof(float);
    int per_sm = (int)((220 * 1024) / (bytes + 1024));
    if (per_sm < 1) per_sm = 1;
    if (per_sm > 8) per_sm = 8;
    return per_sm * num_sms();
}

cudaError_t launch_forward_simt(const ModelDesc& d, const ForwardArgs& a, int n_blocks_hint, cudaStream_t s) {
    const SimtSmem L = simt_smem_layout(d);
    const size_t bytes = L.total_floats * sizeof(float);
    const uint32_t n_tiles = a.n / kTile;
    uint32_t blocks = n_blocks_hint > 0 ? (uint32_t)n_blocks_hint : (uint32_t)forward_simt_blocks(d);
    if (blocks > n_tiles) blocks = n_tiles;
    if (blocks == 0) return cudaSuccess;
    cudaError_t e = cudaSuccess;
    switch (d.width) {
#define NLOD_CASE(WD)                                                                 \
        case WD:                                                                      \
            e = set_smem(k_forward_simt<WD>, bytes);                                  \
            if (e != cudaSuccess) return e;                                           \
            k_forward_simt<WD><<<blocks, kThreads, bytes, s>>>(d, a);                 \
            break;
        NLOD_CASE(16) NLOD_CASE(32) NLOD_CASE(64) NLOD_CASE(128)
#undef NLOD_CASE
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launch_backward_delta_simt(const ModelDesc& d, const BackwardArgs& a, cudaStream_t s) {
    const int lda = (int)(d.enc_width > d.width ? d.enc_width : d.width) + 4;
    uint32_t wmax = 0;
    for (uint32_t l = 0; l < d.n_layers; ++l) wmax = max(wmax, d.layer_in[l] * d.layer_out[l]);
    const size_t bytes = ((size_t)2 * kTile * lda + wmax) * sizeof(float);
    const uint32_t n_tiles = a.n / kTile;
    int per_sm = (int)((220 * 1024) / (bytes + 1024));
    per_sm = per_sm < 1 ? 1 : (per_sm > 8 ? 8 : per_sm);
    uint32_t blocks = min((uint32_t)(per_sm * num_sms()), n_tiles);
    if (blocks == 0) return cudaSuccess;
    cudaError_t e;
    switch (d.width) {
#define NLOD_CASE(WD)                                                                 \
        case WD:                                                                      \
            e = set_smem(k_backward_delta_simt<WD>, bytes);                           \
            if (e != cudaSuccess) return e;                                           \
            k_backward_delta_simt<WD><<<blocks, kThreads, bytes, s>>>(d, a);          \
            break;
        NLOD_CASE(16) NLOD_CASE(32) NLOD_CASE(64) NLOD_CASE(128)
#undef NLOD_CASE
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launch_weight_grad_simt(const ModelDesc& d, const WeightGradArgs& a, cudaStream_t s) {
    uint32_t max_blocks = 1;
    for (uint32_t l = 0; l < d.n_layers; ++l) {
        const uint32_t b = ((d.layer_out[l] + 63) / 64) * ((d.layer_in[l] + 63) / 64);
        max_blocks = max(max_blocks, b);
    }
    // Split the rows so that the whole launch has a few waves of CTAs.
    const uint32_t target_chunks = max(1u, (uint32_t)(2 * num_sms()) / (max_blocks * d.n_layers) + 1);
    uint32_t rows_per_chunk = (a.n + target_chunks - 1) / target_chunks;
    rows_per_chunk = (rows_per_chunk + 31) / 32 * 32;
    if (rows_per_chunk < 512) rows_per_chunk = 512;
    const uint32_t chunks = (a.n + rows_per_chunk - 1) / rows_per_chunk;
    dim3 grid(chunks, max_blocks, d.n_layers);
    k_weight_grad_simt<<<grid, kThreads, 0, s>>>(d, a, rows_per_chunk);
    return cudaGetLastError();
}

cudaError_t launch_grid_backward(const ModelDesc& d, const GridBackwardArgs& a, cudaStream_t s) {
    for (uint32_t i = 0; i < d.n_slots; ++i) {
        if (d.slots[i].type != SLOT_GRID) continue;
        dim3 grid((a.n + kThreads - 1) / kThreads, d.grids[d.slots[i].grid].n_levels);
        k_grid_backward<<<grid, kThreads, 0, s>>>(d, a, i);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

cudaError_t launch_dz_from_dout(const ModelDesc& d, uint32_t n, const float* dL_dout, const float* y, float* dz, cudaStream_t s) {
    const uint32_t total = n * 16u;
    if (total == 0) return cudaSuccess;
    k_dz_from_dout<<<(total + 255) / 256, 256, 0, s>>>(d, n, dL_dout, y, dz);
    return cudaGetLastError();
}

cudaError_t launch_reduce_sum(const float* partial, uint32_t n, float* out, float scale, cudaStream_t s) {
    k_reduce_sum<<<1, 1024, 0, s>>>(partial, n, out, scale);
    return cudaGetLastError();
}

}  // namespace nlod
