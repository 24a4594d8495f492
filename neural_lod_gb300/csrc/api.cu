// C ABI of libnlod (include/nlod.h): module life cycle, inference, training, parameters and
// checkpoints.  Every entry point validates its arguments before any launch, never throws
// across the boundary and reports failures through a status code + nlod_last_error().
#include <cuda_runtime.h>

#include <cmath>
#include <functional>
#include <cstdint>
#include <cstdio>
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <new>
#include <stdexcept>
#include <string>
#include <vector>

#include "nlod.h"
#include "abi_util.h"
#include "desc.h"
#include "json.h"
#include "kernels.h"
#include "model.h"

using namespace nlod;

namespace {
thread_local std::string g_last_error;
}  // namespace

std::string& nlod::last_error() { return g_last_error; }

namespace {

// Growable device workspace for training-mode forward/backward intermediates.
struct Workspace {
    uint32_t cap = 0;
    float* enc = nullptr;
    float* hidden = nullptr;
    float* y = nullptr;
    float* dz = nullptr;
    float* delta = nullptr;
    float* d_enc = nullptr;
    float* loss_partial = nullptr;
    uint32_t n_partial = 0;

    void release() {
        dev_free(enc); dev_free(hidden); dev_free(y); dev_free(dz); dev_free(delta); dev_free(d_enc); dev_free(loss_partial);
        *this = Workspace{};
    }
};

}  // namespace

struct nlod_module {
    ModelDesc d{};
    LossDesc loss{};
    OptimizerDesc opt{};
    bool has_loss = false;
    bool has_opt = false;
    int precision = NLOD_PRECISION_FP32;
    uint32_t n_params = 0;

    float* params = nullptr;        // FP32 master weights
    float* grads = nullptr;         // FP32 gradients (scaled by grad_scale)
    float* m1 = nullptr;
    float* m2 = nullptr;
    uint32_t* steps = nullptr;
    float* ema = nullptr;           // EMA of the parameters = inference parameters when present
    void* w_op = nullptr;           // operand copy (FP16/BF16) of the network part of `params`
    void* w_op_inf = nullptr;       // operand copy of the inference network weights
    uint16_t* grid_h = nullptr;     // FP16 copy of the inference parameters (grid part used), FP16 modules with grids
    uint16_t* grid_b_train = nullptr;   // BF16 copy of the training values (grid part), BF16 modules with grids
    // Cell table of grid_h's leading levels (cells.cu).  An optimizer step marks it out of
    // date on the device (cells_stale, which the kernels read before using it) and on the host
    // (cells_dirty); the next inference call rebuilds it, so training steps do not pay for it and
    // captured inference stays correct (it gathers while the table is out of date).
    void* cells = nullptr;
    uint32_t cells_levels = 0;
    uint32_t cell_base[kMaxLevels + 1] = {};
    uint32_t* cells_stale = nullptr;
    bool cells_dirty = false;
    uint16_t* grid_h_train = nullptr;  // FP16 copy of the training values (grid part), FP16 modules with grids and an EMA
    uint32_t* status = nullptr;     // device status word (bounded-wait timeouts)

    const float* max_level_gpu = nullptr;
    float max_level = 1000.0f;

    // optimizer host state (Adam::m_current_step, ExponentialDecay factor)
    uint32_t step = 0;
    float base_lr = 1e-3f;
    float lr_factor = 1.0f;
    float grad_scale = 1.0f;

    Workspace ws;
    int tc_variant = -1;            // tensor-core kernel organisation (autotuned or default)
    int train_groups = 0;           // tile pipelines of the fused tensor-core training kernel (0 = SIMT kernels)
    float* loss_partial = nullptr;  // per-CTA loss sums of the fused training kernel
    void* enc_tiles = nullptr;      // encoded X0 tiles of the fused training step (operand type)
    size_t enc_tiles_bytes = 0;
    uint8_t* host_io = nullptr;     // device outputs (and staged pageable inputs) of nlod_inference_host
    size_t host_io_bytes = 0;
    // executable graphs of the fused training step, per kind (optimizer step yes/no x loss output yes/no)
    cudaGraphExec_t step_graph[4] = {};
    bool step_graph_warm = false;

    const float* inference_params() const { return ema ? ema : params; }
    int op_kind() const { return precision == NLOD_PRECISION_FP16 ? 1 : 2; }
};

struct nlod_ctx {
    nlod_module* m = nullptr;
    uint32_t n = 0;
    float* enc = nullptr;
    float* hidden = nullptr;
    float* y = nullptr;
};

namespace {

void ensure_workspace(nlod_module* m, uint32_t n) {
    if (m->ws.cap >= n) return;
    m->ws.release();
    const ModelDesc& d = m->d;
    Workspace w;
    w.cap = n;
    w.enc = dev_alloc<float>((size_t)n * d.enc_width);
    w.hidden = dev_alloc<float>((size_t)n * d.width * d.n_hidden_layers);
    w.y = dev_alloc<float>((size_t)n * 16);
    w.dz = dev_alloc<float>((size_t)n * 16);
    w.delta = dev_alloc<float>((size_t)n * d.width * d.n_hidden_layers);
    w.d_enc = dev_alloc<float>((size_t)n * d.enc_width);
    w.n_partial = 4096;
    w.loss_partial = dev_alloc<float>(w.n_partial);
    m->ws = w;
}

constexpr uint32_t kTrainPartials = 1024;   // >= CTAs of the fused training kernel (one per SM)

void check_batch(uint32_t n) {
    if (n % NLOD_BATCH_GRANULARITY != 0)
        throw Error(NLOD_ERR_INVALID, "batch size must be a multiple of 128 (got " + std::to_string(n) + ")");
}

// Rebuilds the cell table when an optimizer step has changed the FP16 tables since the last build.
void ensure_cells(nlod_module* m, cudaStream_t s) {
    if (!m->cells || !m->cells_dirty) return;
    cuda_check(launch_build_cells(m->d, m->grid_h, m->cells_levels, m->cell_base, m->cells, s), "cell table");
    cuda_check(cudaMemsetAsync(m->cells_stale, 0, sizeof(uint32_t), s), "cell table");
    m->cells_dirty = false;
}

// Derived copies of the parameters after they were set from outside (an optimizer step refreshes
// them in its own pass).
void refresh_operand_copies(nlod_module* m, cudaStream_t s) {
    if (m->precision == NLOD_PRECISION_FP32) return;
    if (m->grid_b_train) {
        const uint32_t off = m->d.n_params_network, n = (uint32_t)(m->d.n_params - m->d.n_params_network);
        cuda_check(launch_convert_weights(m->params + off, m->grid_b_train + off, n, 2, s), "convert grid tables");
    }
    cuda_check(launch_convert_weights(m->params, m->w_op, m->d.n_params_network, m->op_kind(), s), "convert weights");
    if (m->w_op_inf != m->w_op)
        cuda_check(launch_convert_weights(m->ema, m->w_op_inf, m->d.n_params_network, m->op_kind(), s), "convert inference weights");
    if (m->grid_h) {
        // after every parameter change, so that captured inference (the renderer's graph) reads
        // the current values
        const uint32_t off = m->d.n_params_network, n = (uint32_t)(m->d.n_params - m->d.n_params_network);
        cuda_check(launch_convert_weights(m->inference_params() + off, m->grid_h + off, n, 1, s), "convert grid tables");
        if (m->grid_h_train)
            cuda_check(launch_convert_weights(m->params + off, m->grid_h_train + off, n, 1, s), "convert grid tables");
        m->cells_dirty = m->cells != nullptr;
        ensure_cells(m, s);
    }
}

ForwardArgs base_forward_args(nlod_module* m, uint32_t n, const float* in, bool inference) {
    ForwardArgs a{};
    a.n = n;
    a.in = in;
    a.params = inference ? m->inference_params() : m->params;
    a.weights_op = inference ? m->w_op_inf : m->w_op;
    a.grid_h = inference ? m->grid_h : nullptr;
    a.cells = inference ? m->cells : nullptr;
    a.cells_levels = inference ? m->cells_levels : 0u;
    a.cells_stale = m->cells_stale;
    for (uint32_t l = 0; l < (uint32_t)kMaxLevels; ++l) a.cell_base[l] = m->cell_base[l];
    a.max_level_gpu = m->max_level_gpu;
    a.max_level = m->max_level;
    return a;
}

// Forward (training parameters) filling the workspace; optional fused loss.
void run_training_forward(nlod_module* m, cudaStream_t s, uint32_t n, const float* in, float* out, const float* target,
                          float loss_scale, float* enc, float* hidden, float* y) {
    ForwardArgs a = base_forward_args(m, n, in, false);
    a.out = out;
    a.enc = enc;
    a.hidden = hidden;
    a.y = y;
    if (target) {
        a.loss_kind = m->loss.kind;
        a.target = target;
        a.loss_scale = loss_scale;
        a.dz = m->ws.dz;
        a.loss_partial = m->ws.loss_partial;
    }
    int blocks = forward_simt_blocks(m->d);
    if ((uint32_t)blocks > m->ws.n_partial) blocks = (int)m->ws.n_partial;
    cuda_check(launch_forward_simt(m->d, a, blocks, s), "forward");
}

void run_backward(nlod_module* m, cudaStream_t s, uint32_t n, const float* in, const float* enc, const float* hidden) {
    const ModelDesc& d = m->d;
    cuda_check(cudaMemsetAsync(m->grads, 0, sizeof(float) * (size_t)m->n_params, s), "memset grads");
    BackwardArgs b{};
    b.n = n;
    b.params = m->params;
    b.hidden = hidden;
    b.dz = m->ws.dz;
    b.delta = m->ws.delta;
    b.d_enc = m->ws.d_enc;
    cuda_check(launch_backward_delta_simt(d, b, s), "backward delta");
    WeightGradArgs w{};
    w.n = n;
    w.enc = enc;
    w.hidden = hidden;
    w.delta = m->ws.delta;
    w.dz = m->ws.dz;
    w.grads = m->grads;
    cuda_check(launch_weight_grad_simt(d, w, s), "weight gradients");
    if (d.n_grids) {
        GridBackwardArgs g{};
        g.n = n;
        g.in = in;
        g.d_enc = m->ws.d_enc;
        g.max_level_gpu = m->max_level_gpu;
        g.max_level = m->max_level;
        g.grads = m->grads;
        cuda_check(launch_grid_backward(d, g, s), "grid backward");
    }
}

void run_optimizer(nlod_module* m, cudaStream_t s) {
    if (!m->has_opt) throw Error(NLOD_ERR_STATE, "module was created without an optimizer");
    const OptimizerDesc& o = m->opt;
    // ExponentialDecay::step (optimizers/exponential_decay.h:60-71), evaluated on the nested
    // optimizer's step count before it increments.
    if (o.has_decay) {
        if (m->step == 0) m->lr_factor = 1.0f;
        if (m->step >= o.decay_start && (m->step - o.decay_start) % o.decay_interval == 0 && m->step <= o.decay_end)
            m->lr_factor *= o.decay_base;
    }
    const float lr = m->base_lr * (o.has_decay ? m->lr_factor : 1.0f);
    ++m->step;
    AdamStepArgs a{};
    a.n_params = m->n_params;
    a.n_matrix = m->d.n_params_network;
    a.hp = o.adam;
    a.learning_rate = lr;
    a.loss_scale = m->grad_scale;
    a.lower_lr_bound = 0.0f;
    a.upper_lr_bound = 3.402823466e38f;
    a.log2_beta1 = (float)std::log2((double)o.adam.beta1);
    a.log2_beta2 = (float)std::log2((double)o.adam.beta2);
    if (o.adam.adabound) {
        a.lower_lr_bound = 0.1f - 0.1f / ((1.f - o.adam.beta2) * (float)m->step + 1.f);
        a.upper_lr_bound = 0.1f + 0.1f / ((1.f - o.adam.beta2) * (float)m->step);
    }
    a.params = m->params;
    a.grads = m->grads;
    a.m1 = m->m1;
    a.m2 = m->m2;
    a.steps = m->steps;
    if (m->ema) {
        a.ema = m->ema;
        a.ema_decay = o.ema_decay;
        a.ema_debias_old = 1.f - (float)std::pow(o.ema_decay, (float)(m->step - 1));
        a.ema_debias_new = 1.0f / (1.f - (float)std::pow(o.ema_decay, (float)m->step));
    }
    // the same pass refreshes every derived copy: operand-type weights and the FP16 grid tables
    a.grid_h = reinterpret_cast<__half*>(m->grid_h);
    a.grid_h_train = reinterpret_cast<__half*>(m->grid_h_train);
    a.grid_b_train = reinterpret_cast<__nv_bfloat16*>(m->grid_b_train);
    a.w_op = m->precision == NLOD_PRECISION_FP32 ? nullptr : m->w_op;
    a.w_op_inf = m->precision == NLOD_PRECISION_FP32 ? nullptr : m->w_op_inf;
    a.op_kind = m->op_kind();
    a.cells_stale = m->cells_stale;
    cuda_check(launch_adam_step(a, s), "adam step");
    m->cells_dirty = m->cells != nullptr;
}

void init_params(nlod_module* m, uint64_t seed) {
    const ModelDesc& d = m->d;
    for (uint32_t l = 0; l < d.n_layers; ++l) {
        // Xavier-uniform (gpu_matrix.h:291-306): +-sqrt(6 / (fan_in + fan_out)).
        const float sc = std::sqrt(6.0f / (float)(d.layer_in[l] + d.layer_out[l]));
        cuda_check(launch_init_uniform(m->params + d.layer_offset[l], d.layer_in[l] * d.layer_out[l], seed, 1 + l, -sc, sc, 0), "init");
    }
    for (uint32_t g = 0; g < d.n_grids; ++g) {
        // grid.h:1353-1356: U[-1e-4, 1e-4]
        cuda_check(launch_init_uniform(m->params + d.grids[g].param_offset, d.grids[g].n_params, seed, 100 + g, -1e-4f, 1e-4f, 0), "init");
    }
}

}  // namespace

namespace nlod {

// Inference launch used by the wavefront renderer: inference parameters, a scalar max level, and
// the row count read from device memory at launch time (n_max rows of input/output storage).
// variant: the tensor-core kernel organisation (< 0: the module's own).
cudaError_t module_inference_device_count(nlod_module* m, uint32_t n_max, const float* in, float* out, const uint32_t* n_dev,
                                          float max_level, cudaStream_t s, int variant) {
    ForwardArgs a = base_forward_args(m, n_max, in, true);
    a.out = out;
    a.n_dev = n_dev;
    a.max_level_gpu = nullptr;
    a.max_level = max_level;
    if (m->precision == NLOD_PRECISION_FP32) return launch_forward_simt(m->d, a, 0, s);
    return launch_forward_tc(m->d, a, m->op_kind(), variant < 0 ? m->tc_variant : variant, m->status, s);
}

// The module's own tensor-core kernel organisation (-1 for the FP32 form), and whether another
// one fits it.
int module_variant(nlod_module* m) { return m->precision == NLOD_PRECISION_FP32 ? -1 : m->tc_variant; }
bool module_variant_ok(nlod_module* m, int variant) {
    return m->precision != NLOD_PRECISION_FP32 && variant >= 0 && tc_variant_ok(m->d, variant, m->op_kind());
}

uint32_t* module_status_word(nlod_module* m) { return m->status; }

// Before inference that a graph captured earlier runs (the renderer's frame): derived tables that
// lag the parameters are rebuilt on the stream.
cudaError_t module_prepare_inference(nlod_module* m, cudaStream_t s) {
    try {
        ensure_cells(m, s);
    } catch (const Error&) {
        return cudaErrorUnknown;
    }
    return cudaSuccess;
}

// Inference operands of a tensor-core module for the persistent renderer: its description, the
// inference weights in the operand type and the parameter vector its encoding gathers (FP16 copy
// for the FP16 form, FP32 inference values for the BF16 form).  False for the plain FP32 form.
bool module_tc_operands(nlod_module* m, const ModelDesc** d, const void** weights, const void** table, int* kind) {
    if (!m || m->precision == NLOD_PRECISION_FP32) return false;
    if (m->precision == NLOD_PRECISION_FP16 && m->d.n_grids > 0 && !m->grid_h) return false;
    *d = &m->d;
    *weights = m->w_op_inf;
    *table = m->precision == NLOD_PRECISION_FP16 && m->grid_h ? static_cast<const void*>(m->grid_h)
                                                             : static_cast<const void*>(m->inference_params());
    *kind = m->op_kind();
    return true;
}

}  // namespace nlod

namespace {

// Times `launch` on stream s with CUDA events (synchronous); ms = its duration.
template <typename Launch>
void time_on_stream(cudaStream_t s, float* ms, Launch&& launch) {
    cudaEvent_t e0, e1;
    cuda_check(cudaEventCreate(&e0), "event");
    cudaError_t e = cudaEventCreate(&e1);
    if (e != cudaSuccess) {
        cudaEventDestroy(e0);
        cuda_check(e, "event");
    }
    e = cudaEventRecord(e0, s);
    if (e == cudaSuccess) e = launch();
    if (e == cudaSuccess) e = cudaEventRecord(e1, s);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    if (e == cudaSuccess) e = cudaEventElapsedTime(ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cuda_check(e, "calibration");
}

}  // namespace

extern "C" {

const char* nlod_last_error(void) { return g_last_error.c_str(); }

const char* nlod_version(void) { return "nlod-gb300 0.1 (sm_103a)"; }

int nlod_module_create(const char* encoding_json, const char* network_json, const char* loss_json, const char* optimizer_json,
                       uint32_t n_input_dims, uint32_t n_output_dims, int precision, uint64_t seed, nlod_module** out) {
    return guarded([&] {
        if (!out) throw Error(NLOD_ERR_INVALID, "out must not be NULL");
        *out = nullptr;
        if (!encoding_json || !network_json) throw Error(NLOD_ERR_INVALID, "encoding and network configs are required");
        if (precision < NLOD_PRECISION_FP32 || precision > NLOD_PRECISION_BF16) throw Error(NLOD_ERR_INVALID, "invalid precision");
        std::unique_ptr<nlod_module> m(new nlod_module());
        Json enc = Json::parse(encoding_json);
        Json net = Json::parse(network_json);
        build_model_desc(enc, net, n_input_dims, n_output_dims, m->d);
        if (loss_json) {
            build_loss_desc(Json::parse(loss_json), m->loss);
            m->has_loss = true;
        }
        if (optimizer_json) {
            build_optimizer_desc(Json::parse(optimizer_json), m->opt);
            m->has_opt = true;
            m->base_lr = m->opt.adam.learning_rate;
        }
        m->precision = precision;
        if (precision != NLOD_PRECISION_FP32) {
            if (!tc_supported(m->d))
                throw Error(NLOD_ERR_UNSUPPORTED, "tensor-core form needs n_neurons 64 or 128 and an encoded width <= 256");
            m->tc_variant = tc_default_variant(m->d);
            m->train_groups = train_tc_groups(m->d);
        }
        const size_t np = m->d.n_params;
        m->n_params = (uint32_t)np;
        try {
            m->params = dev_alloc<float>(np);
            m->grads = dev_alloc<float>(np);
            m->status = dev_alloc<uint32_t>(1);
            cuda_check(cudaMemset(m->status, 0, sizeof(uint32_t)), "memset");
            cuda_check(cudaMemset(m->grads, 0, sizeof(float) * np), "memset");
            if (m->has_opt) {
                m->m1 = dev_alloc<float>(np);
                m->m2 = dev_alloc<float>(np);
                m->steps = dev_alloc<uint32_t>(np);
                cuda_check(cudaMemset(m->m1, 0, sizeof(float) * np), "memset");
                cuda_check(cudaMemset(m->m2, 0, sizeof(float) * np), "memset");
                cuda_check(cudaMemset(m->steps, 0, sizeof(uint32_t) * np), "memset");
                if (m->opt.has_ema) {
                    // tiny-cuda-nn zero-initialises the EMA weights (ema.h:101-110) and uses them
                    // as inference parameters (trainer.h:322-327).
                    m->ema = dev_alloc<float>(np);
                    cuda_check(cudaMemset(m->ema, 0, sizeof(float) * np), "memset");
                }
            }
            if (precision != NLOD_PRECISION_FP32) {
                m->w_op = dev_alloc<uint16_t>(m->d.n_params_network);
                m->w_op_inf = m->ema ? dev_alloc<uint16_t>(m->d.n_params_network) : m->w_op;
            }
            if (precision == NLOD_PRECISION_BF16 && m->d.n_grids > 0 && m->has_loss) m->grid_b_train = dev_alloc<uint16_t>(np);
            if (precision == NLOD_PRECISION_FP16 && m->d.n_grids > 0) {
                m->grid_h = dev_alloc<uint16_t>(np);
                if (m->ema) m->grid_h_train = dev_alloc<uint16_t>(np);
                m->cells_levels = cells_levels_of(m->d, m->cell_base);
                if (m->cells_levels) {
                    m->cells = dev_alloc<uint8_t>(32u * (size_t)m->cell_base[m->cells_levels]);
                    m->cells_stale = dev_alloc<uint32_t>(1);
                    cuda_check(cudaMemset(m->cells_stale, 0xFF, sizeof(uint32_t)), "memset");
                }
            }
            init_params(m.get(), seed);
            refresh_operand_copies(m.get(), 0);
            cuda_check(cudaDeviceSynchronize(), "init");
        } catch (...) {
            nlod_module_destroy(m.release());
            throw;
        }
        *out = m.release();
    });
}

int nlod_layout_json(const char* encoding_json, const char* network_json, uint32_t n_input_dims, uint32_t n_output_dims,
                     char** json_out) {
    return guarded([&] {
        if (!json_out) throw Error(NLOD_ERR_INVALID, "json_out must not be NULL");
        *json_out = nullptr;
        if (!encoding_json || !network_json) throw Error(NLOD_ERR_INVALID, "encoding and network configs are required");
        ModelDesc d;
        build_model_desc(Json::parse(encoding_json), Json::parse(network_json), n_input_dims, n_output_dims, d);
        Json j = Json::object();
        j.set("n_input", Json::number(d.n_input));
        j.set("n_output", Json::number(d.n_output));
        j.set("enc_width", Json::number(d.enc_width));
        j.set("width", Json::number(d.width));
        j.set("n_layers", Json::number(d.n_layers));
        j.set("act", Json::number(d.act));
        j.set("out_act", Json::number(d.out_act));
        j.set("n_params_network", Json::number(d.n_params_network));
        j.set("n_params", Json::number(d.n_params));
        Json layers = Json::array();
        for (uint32_t l = 0; l < d.n_layers; ++l) {
            Json e = Json::object();
            e.set("in", Json::number(d.layer_in[l]));
            e.set("out", Json::number(d.layer_out[l]));
            e.set("offset", Json::number(d.layer_offset[l]));
            layers.push(e);
        }
        j.set("layers", layers);
        Json slots = Json::array();
        for (uint32_t i = 0; i < d.n_slots; ++i) {
            const Slot& s = d.slots[i];
            Json e = Json::object();
            e.set("type", Json::number(s.type));
            e.set("in_begin", Json::number(s.in_begin));
            e.set("n_in", Json::number(s.n_in));
            e.set("out_begin", Json::number(s.out_begin));
            e.set("out_width", Json::number(s.out_width));
            e.set("n_pad", Json::number(s.n_pad));
            e.set("grid", Json::number(s.grid));
            e.set("degree", Json::number(s.degree));
            e.set("n_bins", Json::number(s.n_bins));
            slots.push(e);
        }
        j.set("slots", slots);
        Json grids = Json::array();
        for (uint32_t g = 0; g < d.n_grids; ++g) {
            const GridDesc& gd = d.grids[g];
            Json e = Json::object();
            e.set("n_levels", Json::number(gd.n_levels));
            e.set("hash", Json::number(gd.hash));
            e.set("kind", Json::number(gd.kind));
            e.set("interp", Json::number(gd.interp));
            e.set("param_offset", Json::number(gd.param_offset));
            e.set("n_params", Json::number(gd.n_params));
            Json off = Json::array(), res = Json::array(), sc = Json::array();
            for (uint32_t l = 0; l < gd.n_levels; ++l) {
                off.push(Json::number(gd.levels[l].offset));
                res.push(Json::number(gd.levels[l].res_flags & kLevelResMask));
                sc.push(Json::number(gd.levels[l].scale));
            }
            off.push(Json::number(gd.levels[gd.n_levels - 1].offset + gd.levels[gd.n_levels - 1].size));
            e.set("offset", off);
            e.set("res", res);
            e.set("scale", sc);
            grids.push(e);
        }
        j.set("grids", grids);
        const std::string s = j.dump();
        char* outp = (char*)std::malloc(s.size() + 1);
        if (!outp) throw std::bad_alloc();
        std::memcpy(outp, s.c_str(), s.size() + 1);
        *json_out = outp;
    });
}

void nlod_module_destroy(nlod_module* m) {
    if (!m) return;
    cudaDeviceSynchronize();
    m->ws.release();
    dev_free(m->params);
    dev_free(m->grads);
    dev_free(m->m1);
    dev_free(m->m2);
    dev_free(m->steps);
    dev_free(m->ema);
    if (m->w_op_inf != m->w_op) dev_free(m->w_op_inf);
    dev_free(m->grid_h);
    dev_free(m->grid_h_train);
    dev_free(m->grid_b_train);
    dev_free(m->cells);
    dev_free(m->cells_stale);
    dev_free(m->w_op);
    dev_free(m->status);
    dev_free(m->loss_partial);
    dev_free(m->enc_tiles);
    dev_free(m->host_io);
    for (cudaGraphExec_t& g : m->step_graph)
        if (g) cudaGraphExecDestroy(g);
    delete m;
}

size_t nlod_n_params(const nlod_module* m) { return m ? m->d.n_params : 0; }
size_t nlod_n_network_params(const nlod_module* m) { return m ? m->d.n_params_network : 0; }
uint32_t nlod_n_input_dims(const nlod_module* m) { return m ? m->d.n_input : 0; }
uint32_t nlod_n_output_dims(const nlod_module* m) { return m ? m->d.n_output : 0; }
uint32_t nlod_encoded_width(const nlod_module* m) { return m ? m->d.enc_width : 0; }
uint32_t nlod_padded_output_width(const nlod_module* m) { return m ? m->d.n_output_padded : 0; }
int nlod_precision(const nlod_module* m) { return m ? m->precision : -1; }

int nlod_set_max_level_gpu(nlod_module* m, const float* max_level_gpu) {
    return guarded([&] {
        if (!m) throw Error(NLOD_ERR_INVALID, "module is NULL");
        m->max_level_gpu = max_level_gpu;
    });
}

int nlod_set_max_level(nlod_module* m, float max_level) {
    return guarded([&] {
        if (!m) throw Error(NLOD_ERR_INVALID, "module is NULL");
        if (!(max_level >= 0.0f)) throw Error(NLOD_ERR_INVALID, "max_level must be >= 0");
        m->max_level = max_level;
    });
}

int nlod_inference(nlod_module* m, void* stream, uint32_t n, const float* in, float* out) {
    return guarded([&] {
        if (!m) throw Error(NLOD_ERR_INVALID, "module is NULL");
        check_batch(n);
        if (n == 0) return;
        if (!in || !out) throw Error(NLOD_ERR_INVALID, "input and output must not be NULL");
        cudaStream_t s = (cudaStream_t)stream;
        ensure_cells(m, s);
        ForwardArgs a = base_forward_args(m, n, in, true);
        a.out = out;
        if (m->precision == NLOD_PRECISION_FP32) cuda_check(launch_forward_simt(m->d, a, 0, s), "inference");
        else cuda_check(launch_forward_tc(m->d, a, m->op_kind(), m->tc_variant, m->status, s), "inference");
    });
}

// Device address of memory the GPU can read in place: device / managed memory, or page-locked host
// memory (mapped under unified addressing; on Grace the kernel reads it over NVLink-C2C).  NULL for
// pageable host memory.
static const float* device_readable(const float* p) {
    cudaPointerAttributes attr{};
    if (cudaPointerGetAttributes(&attr, p) != cudaSuccess) {
        (void)cudaGetLastError();
        return nullptr;
    }
    if (attr.type == cudaMemoryTypeDevice || attr.type == cudaMemoryTypeManaged) return p;
    if (attr.type == cudaMemoryTypeHost && attr.devicePointer) return static_cast<const float*>(attr.devicePointer);
    return nullptr;
}

int nlod_inference_host(nlod_module* m, void* stream, uint32_t n, const float* host_in, float* host_out) {
    return guarded([&] {
        if (!m) throw Error(NLOD_ERR_INVALID, "module is NULL");
        check_batch(n);
        if (n == 0) return;
        if (!host_in || !host_out) throw Error(NLOD_ERR_INVALID, "input and output must not be NULL");
        cudaStream_t s = (cudaStream_t)stream;
        const size_t in_bytes = (size_t)n * m->d.n_input * sizeof(float);
        const size_t out_bytes = (size_t)n * m->d.n_output * sizeof(float);
        const size_t out_span = (out_bytes + 255) / 256 * 256;
        const float* in_dev = device_readable(host_in);
        const size_t need = out_span + (in_dev ? 0 : in_bytes);
        if (m->host_io_bytes < need) {
            dev_free(m->host_io);
            m->host_io = nullptr;
            m->host_io_bytes = 0;
            m->host_io = dev_alloc<uint8_t>(need);
            m->host_io_bytes = need;
        }
        float* out_dev = reinterpret_cast<float*>(m->host_io);
        if (!in_dev) {
            float* stage = reinterpret_cast<float*>(m->host_io + out_span);
            cuda_check(cudaMemcpyAsync(stage, host_in, in_bytes, cudaMemcpyHostToDevice, s), "input copy");
            in_dev = stage;
        }
        ensure_cells(m, s);
        ForwardArgs a = base_forward_args(m, n, in_dev, true);
        a.out = out_dev;
        if (m->precision == NLOD_PRECISION_FP32) cuda_check(launch_forward_simt(m->d, a, 0, s), "inference");
        else cuda_check(launch_forward_tc(m->d, a, m->op_kind(), m->tc_variant, m->status, s), "inference");
        cuda_check(cudaMemcpyAsync(host_out, out_dev, out_bytes, cudaMemcpyDeviceToHost, s), "output copy");
    });
}

int nlod_forward(nlod_module* m, void* stream, uint32_t n, const float* in, float* out, nlod_ctx** ctx) {
    return guarded([&] {
        if (!m || !ctx) throw Error(NLOD_ERR_INVALID, "module and ctx must not be NULL");
        *ctx = nullptr;
        check_batch(n);
        if (n == 0) throw Error(NLOD_ERR_INVALID, "empty batch");
        if (!in) throw Error(NLOD_ERR_INVALID, "input must not be NULL");
        std::unique_ptr<nlod_ctx> c(new nlod_ctx());
        c->m = m;
        c->n = n;
        try {
            c->enc = dev_alloc<float>((size_t)n * m->d.enc_width);
            c->hidden = dev_alloc<float>((size_t)n * m->d.width * m->d.n_hidden_layers);
            c->y = dev_alloc<float>((size_t)n * 16);
            ensure_workspace(m, n);
            run_training_forward(m, (cudaStream_t)stream, n, in, out, nullptr, 1.0f, c->enc, c->hidden, c->y);
        } catch (...) {
            nlod_ctx_destroy(c.release());
            throw;
        }
        *ctx = c.release();
    });
}

int nlod_backward(nlod_module* m, void* stream, nlod_ctx* ctx, const float* in, const float* dL_dout) {
    return guarded([&] {
        if (!m || !ctx || ctx->m != m) throw Error(NLOD_ERR_INVALID, "context does not belong to this module");
        if (!in || !dL_dout) throw Error(NLOD_ERR_INVALID, "input and dL_dout must not be NULL");
        cudaStream_t s = (cudaStream_t)stream;
        ensure_workspace(m, ctx->n);
        cuda_check(launch_dz_from_dout(m->d, ctx->n, dL_dout, ctx->y, m->ws.dz, s), "dz");
        run_backward(m, s, ctx->n, in, ctx->enc, ctx->hidden);
        m->grad_scale = 1.0f;
    });
}

void nlod_ctx_destroy(nlod_ctx* ctx) {
    if (!ctx) return;
    cudaDeviceSynchronize();
    dev_free(ctx->enc);
    dev_free(ctx->hidden);
    dev_free(ctx->y);
    delete ctx;
}

// Runs the launches `issue` makes on s as one CUDA graph, as tiny-cuda-nn's Trainer does for its
// step (trainer.h:175-180), here including the optimizer: the launches are captured on s, the
// module's executable graph for this kind of step is updated in place with the new arguments
// (cudaGraphExecUpdate; instantiated again only when the update is refused), and launched.  The
// programmatic (PDL) edge between the encoding and the fused kernel is kept by the capture.
// The module's first step, a step on the legacy default stream (which cannot be captured) and a
// step on a stream the caller is capturing issue the launches directly.
static void launch_step_graph(nlod_module* m, cudaStream_t s, int kind, const std::function<void(cudaStream_t)>& issue) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    const bool capturable = m->step_graph_warm && s != nullptr && s != cudaStreamLegacy &&
                            cudaStreamIsCapturing(s, &cs) == cudaSuccess && cs == cudaStreamCaptureStatusNone;
    if (!capturable) {
        issue(s);
        m->step_graph_warm = true;   // kernel attributes and buffers are set up by the direct launches
        return;
    }
    cuda_check(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal), "begin step capture");
    cudaGraph_t g = nullptr;
    try {
        issue(s);
    } catch (...) {
        cudaStreamEndCapture(s, &g);
        if (g) cudaGraphDestroy(g);
        throw;
    }
    cuda_check(cudaStreamEndCapture(s, &g), "end step capture");
    cudaGraphExec_t& exec = m->step_graph[kind & 3];
    if (exec) {
        cudaGraphExecUpdateResultInfo info{};
        if (cudaGraphExecUpdate(exec, g, &info) != cudaSuccess) {
            (void)cudaGetLastError();
            cudaGraphExecDestroy(exec);
            exec = nullptr;
        }
    }
    cudaError_t e = cudaSuccess;
    if (!exec) e = cudaGraphInstantiate(&exec, g, 0);
    cudaGraphDestroy(g);
    cuda_check(e, "instantiate step graph");
    cuda_check(cudaGraphLaunch(exec, s), "launch step graph");
}

static int train_impl(nlod_module* m, void* stream, uint32_t n, const float* in, const float* target, float* loss_out, bool run_opt) {
    return guarded([&] {
        if (!m) throw Error(NLOD_ERR_INVALID, "module is NULL");
        if (!m->has_loss) throw Error(NLOD_ERR_STATE, "module was created without a loss");
        if (run_opt && !m->has_opt) throw Error(NLOD_ERR_STATE, "module was created without an optimizer");
        check_batch(n);
        if (n == 0) throw Error(NLOD_ERR_INVALID, "empty batch");
        if (!in || !target) throw Error(NLOD_ERR_INVALID, "input and target must not be NULL");
        cudaStream_t s = (cudaStream_t)stream;
        const float loss_scale = 128.0f;  // Trainer::training_step's static loss scale (trainer.h:171)
        if (m->train_groups > 0) {
            // fused tensor-core step: one kernel for encoding, forward, loss and all gradients
            if (!m->loss_partial) m->loss_partial = dev_alloc<float>(kTrainPartials);
            TrainTcArgs t{};
            t.n = n;
            t.in = in;
            t.params = m->params;
            t.weights_op = m->w_op;
            t.max_level_gpu = m->max_level_gpu;
            t.max_level = m->max_level;
            t.loss_kind = m->loss.kind;
            t.target = target;
            t.inv_n_total = 1.0f / ((float)n * (float)m->d.n_output);
            t.grad_scale = loss_scale * t.inv_n_total;
            t.grads = m->grads;
            t.loss_partial = m->loss_partial;
            // FP16 training values: the inference copy without an EMA, the separate training copy with one
            t.grid_h = m->grid_b_train ? static_cast<const void*>(m->grid_b_train)
                                       : m->ema ? static_cast<const void*>(m->grid_h_train) : static_cast<const void*>(m->grid_h);
            // the encoding kernel zeroes the gradients (4-float tail, if any, by a memset)
            t.zero_grads_n = (uint32_t)(m->n_params & ~size_t(3));
            const size_t enc_bytes = (size_t)n * m->d.enc_width * 2u;
            if (m->enc_tiles_bytes < enc_bytes) {
                dev_free(m->enc_tiles);
                m->enc_tiles = nullptr;
                m->enc_tiles_bytes = 0;
                m->enc_tiles = dev_alloc<uint8_t>(enc_bytes);
                m->enc_tiles_bytes = enc_bytes;
            }
            t.enc_tiles = m->enc_tiles;
            const auto issue = [&](cudaStream_t st) {
                if (t.zero_grads_n != m->n_params)
                    cuda_check(cudaMemsetAsync(m->grads + t.zero_grads_n, 0, sizeof(float) * (m->n_params - t.zero_grads_n), st),
                               "memset grads");
                cuda_check(launch_encode_tiles(m->d, t, m->op_kind(), st), "encoding");
                cuda_check(launch_train_tc(m->d, t, m->op_kind(), m->train_groups, m->status, st), "training step");
                // every CTA of the fused kernel wrote its partial: no memset, sum exactly those
                if (loss_out)
                    cuda_check(launch_reduce_sum(m->loss_partial, train_tc_blocks(n, m->train_groups), loss_out, 1.0f, st), "loss");
                m->grad_scale = loss_scale;
                if (run_opt) run_optimizer(m, st);
            };
            launch_step_graph(m, s, (run_opt ? 2 : 0) | (loss_out ? 1 : 0), issue);
            return;
        }
        ensure_workspace(m, n);
        cuda_check(cudaMemsetAsync(m->ws.loss_partial, 0, sizeof(float) * m->ws.n_partial, s), "memset");
        run_training_forward(m, s, n, in, nullptr, target, loss_scale, m->ws.enc, m->ws.hidden, m->ws.y);
        if (loss_out) cuda_check(launch_reduce_sum(m->ws.loss_partial, m->ws.n_partial, loss_out, 1.0f, s), "loss");
        run_backward(m, s, n, in, m->ws.enc, m->ws.hidden);
        m->grad_scale = loss_scale;
        if (run_opt) run_optimizer(m, s);
    });
}

int nlod_training_step(nlod_module* m, void* stream, uint32_t n, const float* in, const float* target, float* loss_out) {
    return train_impl(m, stream, n, in, target, loss_out, true);
}

int nlod_forward_backward_loss(nlod_module* m, void* stream, uint32_t n, const float* in, const float* target, float* loss_out) {
    return train_impl(m, stream, n, in, target, loss_out, false);
}

// Scratch plan of nlod_training_step_noalloc: the workspace buffers of one step, each 256-byte
// aligned, followed by the per-block loss partial sums.
struct NoAllocPlan {
    size_t enc, hidden, y, dz, delta, d_enc, partial, total;
};

static NoAllocPlan noalloc_plan(const ModelDesc& d, uint32_t n) {
    auto al = [](size_t b) { return (b + 255) / 256 * 256; };
    NoAllocPlan p{};
    size_t off = 0;
    p.enc = off;     off += al(sizeof(float) * (size_t)n * d.enc_width);
    p.hidden = off;  off += al(sizeof(float) * (size_t)n * d.width * d.n_hidden_layers);
    p.y = off;       off += al(sizeof(float) * (size_t)n * 16);
    p.dz = off;      off += al(sizeof(float) * (size_t)n * 16);
    p.delta = off;   off += al(sizeof(float) * (size_t)n * d.width * d.n_hidden_layers);
    p.d_enc = off;   off += al(sizeof(float) * (size_t)n * d.enc_width);
    p.partial = off; off += al(sizeof(float) * 4096);
    p.total = off;
    return p;
}

int nlod_training_step_noalloc(nlod_module* m, void* stream, uint32_t n, const float* in, const float* target, float* loss_out) {
    return guarded([&] {
        if (!m) throw Error(NLOD_ERR_INVALID, "module is NULL");
        if (!m->has_loss) throw Error(NLOD_ERR_STATE, "module was created without a loss");
        if (!m->has_opt) throw Error(NLOD_ERR_STATE, "module was created without an optimizer");
        check_batch(n);
        if (n == 0) throw Error(NLOD_ERR_INVALID, "empty batch");
        if (!in || !target) throw Error(NLOD_ERR_INVALID, "input and target must not be NULL");
        const ModelDesc& d = m->d;
        const NoAllocPlan plan = noalloc_plan(d, n);
        if (plan.total > kNoAllocScratchBytes) {
            uint32_t max_n = 0;
            for (uint32_t k = 128; noalloc_plan(d, k).total <= kNoAllocScratchBytes; k += 128) max_n = k;
            throw Error(NLOD_ERR_INVALID, "batch of " + std::to_string(n) + " needs " + std::to_string(plan.total) +
                                              " bytes of scratch; the no-allocation training step has a fixed 16 MiB scratch, "
                                              "which holds at most " + std::to_string(max_n) + " elements for this network");
        }
        void* base = nullptr;
        size_t cap = 0;
        cuda_check(noalloc_scratch(&base, &cap), "no-allocation scratch address");
        unsigned char* b = static_cast<unsigned char*>(base);
        float* enc = reinterpret_cast<float*>(b + plan.enc);
        float* hidden = reinterpret_cast<float*>(b + plan.hidden);
        float* y = reinterpret_cast<float*>(b + plan.y);
        float* dz = reinterpret_cast<float*>(b + plan.dz);
        float* delta = reinterpret_cast<float*>(b + plan.delta);
        float* d_enc = reinterpret_cast<float*>(b + plan.d_enc);
        float* partial = reinterpret_cast<float*>(b + plan.partial);
        cudaStream_t s = (cudaStream_t)stream;
        const float loss_scale = 128.0f;
        // The partial sums are reduced over all 4096 slots: they must start at zero.
        cuda_check(cudaMemsetAsync(partial, 0, sizeof(float) * 4096, s), "memset");
        ForwardArgs a = base_forward_args(m, n, in, false);
        a.enc = enc;
        a.hidden = hidden;
        a.y = y;
        a.loss_kind = m->loss.kind;
        a.target = target;
        a.loss_scale = loss_scale;
        a.dz = dz;
        a.loss_partial = partial;
        int blocks = forward_simt_blocks(d);
        if (blocks > 4096) blocks = 4096;
        cuda_check(launch_forward_simt(d, a, blocks, s), "forward");
        if (loss_out) cuda_check(launch_reduce_sum(partial, 4096, loss_out, 1.0f, s), "loss");
        cuda_check(cudaMemsetAsync(m->grads, 0, sizeof(float) * (size_t)m->n_params, s), "memset grads");
        BackwardArgs bw{};
        bw.n = n;
        bw.params = m->params;
        bw.hidden = hidden;
        bw.dz = dz;
        bw.delta = delta;
        bw.d_enc = d_enc;
        cuda_check(launch_backward_delta_simt(d, bw, s), "backward delta");
        WeightGradArgs wg{};
        wg.n = n;
        wg.enc = enc;
        wg.hidden = hidden;
        wg.delta = delta;
        wg.dz = dz;
        wg.grads = m->grads;
        cuda_check(launch_weight_grad_simt(d, wg, s), "weight gradients");
        if (d.n_grids) {
            GridBackwardArgs g{};
            g.n = n;
            g.in = in;
            g.d_enc = d_enc;
            g.max_level_gpu = m->max_level_gpu;
            g.max_level = m->max_level;
            g.grads = m->grads;
            cuda_check(launch_grid_backward(d, g, s), "grid backward");
        }
        m->grad_scale = loss_scale;
        run_optimizer(m, s);
    });
}

int nlod_optimizer_step(nlod_module* m, void* stream) {
    return guarded([&] {
        if (!m) throw Error(NLOD_ERR_INVALID, "module is NULL");
        run_optimizer(m, (cudaStream_t)stream);
    });
}

uint32_t nlod_optimizer_step_count(const nlod_module* m) { return m ? m->step : 0; }

float nlod_learning_rate(const nlod_module* m) {
    if (!m) return 0.f;
    return m->base_lr * (m->opt.has_decay ? m->lr_factor : 1.0f);
}

int nlod_set_learning_rate(nlod_module* m, float lr) {
    return guarded([&] {
        if (!m) throw Error(NLOD_ERR_INVALID, "module is NULL");
        if (!(lr >= 0.f)) throw Error(NLOD_ERR_INVALID, "learning rate must be >= 0");
        // ExponentialDecay::set_learning_rate keeps the decay factor (exponential_decay.h:78-81).
        m->base_lr = (m->opt.has_decay && m->lr_factor != 0.f) ? lr / m->lr_factor : lr;
    });
}

int nlod_set_params(nlod_module* m, const float* params, size_t n_params, int device_ptr) {
    return guarded([&] {
        if (!m || !params) throw Error(NLOD_ERR_INVALID, "module and params must not be NULL");
        if (n_params != m->d.n_params) throw Error(NLOD_ERR_INVALID, "Can't set fp params because buffer has the wrong size.");
        cuda_check(cudaMemcpy(m->params, params, sizeof(float) * n_params, device_ptr ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice), "set params");
        // set_params_full_precision also overwrites the inference (EMA) weights (trainer.h:234-246).
        if (m->ema) cuda_check(cudaMemcpy(m->ema, m->params, sizeof(float) * n_params, cudaMemcpyDeviceToDevice), "set params");
        refresh_operand_copies(m, 0);
        cuda_check(cudaDeviceSynchronize(), "set params");
    });
}

int nlod_get_params(nlod_module* m, float* params, size_t n_params, int which, int device_ptr) {
    return guarded([&] {
        if (!m || !params) throw Error(NLOD_ERR_INVALID, "module and params must not be NULL");
        if (n_params != m->d.n_params) throw Error(NLOD_ERR_INVALID, "buffer has the wrong size");
        cuda_check(cudaDeviceSynchronize(), "get params");
        const float* src = which == 0 ? m->params : which == 1 ? m->inference_params() : which == 2 ? m->grads : nullptr;
        if (!src) throw Error(NLOD_ERR_INVALID, "which must be 0 (params), 1 (inference params) or 2 (gradients)");
        std::vector<float> host;
        float* dst = params;
        if (!device_ptr) {
            host.resize(n_params);
            dst = host.data();
        }
        if (device_ptr) cuda_check(cudaMemcpy(dst, src, sizeof(float) * n_params, cudaMemcpyDeviceToDevice), "get params");
        else cuda_check(cudaMemcpy(dst, src, sizeof(float) * n_params, cudaMemcpyDeviceToHost), "get params");
        if (which == 2 && m->grad_scale != 1.0f) {
            if (device_ptr) {
                std::vector<float> tmp(n_params);
                cuda_check(cudaMemcpy(tmp.data(), dst, sizeof(float) * n_params, cudaMemcpyDeviceToHost), "get grads");
                for (auto& v : tmp) v /= m->grad_scale;
                cuda_check(cudaMemcpy(dst, tmp.data(), sizeof(float) * n_params, cudaMemcpyHostToDevice), "get grads");
            } else {
                for (auto& v : host) v /= m->grad_scale;
            }
        }
        if (!device_ptr) std::memcpy(params, host.data(), sizeof(float) * n_params);
    });
}

int nlod_serialize(nlod_module* m, int half_precision, char** json_out) {
    return guarded([&] {
        if (!m || !json_out) throw Error(NLOD_ERR_INVALID, "module and json_out must not be NULL");
        *json_out = nullptr;
        const size_t np = m->d.n_params;
        std::vector<float> p(np);
        cuda_check(cudaDeviceSynchronize(), "serialize");
        cuda_check(cudaMemcpy(p.data(), m->inference_params(), sizeof(float) * np, cudaMemcpyDeviceToHost), "serialize");
        std::vector<uint8_t> bytes;
        if (half_precision) {
            bytes.resize(np * 2);
            for (size_t i = 0; i < np; ++i) {
                // round-to-nearest-even FP32 -> FP16 (IEEE 754 binary16)
                uint32_t x;
                std::memcpy(&x, &p[i], 4);
                const uint32_t sign = (x >> 16) & 0x8000u;
                int32_t e = (int32_t)((x >> 23) & 0xFF) - 127 + 15;
                uint32_t mant = x & 0x7FFFFFu;
                uint16_t h;
                if (((x >> 23) & 0xFF) == 0xFF) h = (uint16_t)(sign | 0x7C00u | (mant ? 0x200u : 0u));
                else if (e >= 31) h = (uint16_t)(sign | 0x7C00u);
                else if (e <= 0) {
                    if (e < -10) h = (uint16_t)sign;
                    else {
                        mant |= 0x800000u;
                        const uint32_t shift = (uint32_t)(14 - e);
                        uint32_t hm = mant >> shift;
                        const uint32_t rem = mant & ((1u << shift) - 1u), halfway = 1u << (shift - 1);
                        if (rem > halfway || (rem == halfway && (hm & 1u))) ++hm;
                        h = (uint16_t)(sign | hm);
                    }
                } else {
                    uint32_t hm = mant >> 13;
                    const uint32_t rem = mant & 0x1FFFu;
                    uint32_t he = (uint32_t)e;
                    if (rem > 0x1000u || (rem == 0x1000u && (hm & 1u))) {
                        ++hm;
                        if (hm == 0x400u) { hm = 0; ++he; }
                    }
                    h = he >= 31 ? (uint16_t)(sign | 0x7C00u) : (uint16_t)(sign | (he << 10) | hm);
                }
                bytes[2 * i] = (uint8_t)(h & 0xFF);
                bytes[2 * i + 1] = (uint8_t)(h >> 8);
            }
        } else {
            bytes.resize(np * 4);
            std::memcpy(bytes.data(), p.data(), np * 4);
        }
        std::string s = "{\"n_params\":" + std::to_string(np) + ",\"params_type\":\"" + (half_precision ? "__half" : "float") +
                        "\",\"params_binary\":{\"bytes\":[";
        s.reserve(s.size() + bytes.size() * 4 + 64);
        char buf[8];
        for (size_t i = 0; i < bytes.size(); ++i) {
            int k = std::snprintf(buf, sizeof buf, i ? ",%u" : "%u", (unsigned)bytes[i]);
            s.append(buf, (size_t)k);
        }
        s += "],\"subtype\":null}}";
        char* outp = (char*)std::malloc(s.size() + 1);
        if (!outp) throw std::bad_alloc();
        std::memcpy(outp, s.c_str(), s.size() + 1);
        *json_out = outp;
    });
}

static float half_to_float(uint16_t h) {
    const uint32_t sign = (uint32_t)(h & 0x8000u) << 16;
    uint32_t e = (h >> 10) & 0x1F, mant = h & 0x3FFu;
    uint32_t x;
    if (e == 0) {
        if (mant == 0) x = sign;
        else {
            int shift = 0;
            while (!(mant & 0x400u)) { mant <<= 1; ++shift; }
            mant &= 0x3FFu;
            x = sign | ((uint32_t)(127 - 15 + 1 - shift) << 23) | (mant << 13);
        }
    } else if (e == 31) {
        x = sign | 0x7F800000u | (mant << 13);
    } else {
        x = sign | ((e - 15 + 127) << 23) | (mant << 13);
    }
    float f;
    std::memcpy(&f, &x, 4);
    return f;
}

int nlod_deserialize(nlod_module* m, const char* json) {
    return guarded([&] {
        if (!m || !json) throw Error(NLOD_ERR_INVALID, "module and json must not be NULL");
        Json j = Json::parse(json);
        std::string type = j.value_str("params_type", "__half");
        const Json& b = j.at("params_binary");
        const Json& arr = b.is_object() ? b.at("bytes") : b;
        const auto& items = arr.items();
        std::vector<float> p;
        if (type == "float") {
            if (items.size() % 4) throw Error(NLOD_ERR_INVALID, "params_binary size is not a multiple of 4");
            p.resize(items.size() / 4);
            std::vector<uint8_t> raw(items.size());
            for (size_t i = 0; i < items.size(); ++i) raw[i] = (uint8_t)items[i].as_number();
            std::memcpy(p.data(), raw.data(), raw.size());
        } else if (type == "__half") {
            if (items.size() % 2) throw Error(NLOD_ERR_INVALID, "params_binary size is not a multiple of 2");
            p.resize(items.size() / 2);
            for (size_t i = 0; i < p.size(); ++i) {
                const uint16_t h = (uint16_t)((uint32_t)items[2 * i].as_number() | ((uint32_t)items[2 * i + 1].as_number() << 8));
                p[i] = half_to_float(h);
            }
        } else {
            throw Error(NLOD_ERR_INVALID, "Trainer: snapshot parameters must be of type float of __half");
        }
        if (p.size() != m->d.n_params) throw Error(NLOD_ERR_INVALID, "checkpoint has " + std::to_string(p.size()) + " params, module has " + std::to_string(m->d.n_params));
        cuda_check(cudaMemcpy(m->params, p.data(), sizeof(float) * p.size(), cudaMemcpyHostToDevice), "deserialize");
        if (m->ema) cuda_check(cudaMemcpy(m->ema, m->params, sizeof(float) * p.size(), cudaMemcpyDeviceToDevice), "deserialize");
        refresh_operand_copies(m, 0);
        cuda_check(cudaDeviceSynchronize(), "deserialize");
    });
}

void nlod_free_string(char* s) { std::free(s); }

int nlod_kernel_variants(const nlod_module* m) {
    if (!m || m->precision == NLOD_PRECISION_FP32) return 1;
    return tc_num_variants();
}

int nlod_set_kernel_variant(nlod_module* m, int variant) {
    return guarded([&] {
        if (!m) throw Error(NLOD_ERR_INVALID, "module is NULL");
        if (m->precision == NLOD_PRECISION_FP32) {
            if (variant != 0) throw Error(NLOD_ERR_INVALID, "the FP32 form has a single kernel variant");
            return;
        }
        if (!tc_variant_ok(m->d, variant, m->op_kind())) throw Error(NLOD_ERR_UNSUPPORTED, "kernel variant does not fit this network");
        m->tc_variant = variant;
    });
}

int nlod_get_kernel_variant(const nlod_module* m) { return m ? (m->precision == NLOD_PRECISION_FP32 ? 0 : m->tc_variant) : -1; }

int nlod_autotune(nlod_module* m, void* stream, uint32_t n, const float* in, float* out) {
    return guarded([&] {
        if (!m) throw Error(NLOD_ERR_INVALID, "module is NULL");
        check_batch(n);
        if (n == 0 || m->precision == NLOD_PRECISION_FP32) return;
        if (!in || !out) throw Error(NLOD_ERR_INVALID, "input and output must not be NULL");
        cudaStream_t s = (cudaStream_t)stream;
        ensure_cells(m, s);
        ForwardArgs a = base_forward_args(m, n, in, true);
        a.out = out;
        // Each organisation is timed on single launches that find the L2 holding other data (a
        // scratch write of twice the L2's size before each), in three rounds over all of them; the
        // median of an organisation's three decides.  Without the scratch (allocation refused) the
        // launches run back to back.
        int dev = 0, l2 = 0;
        cuda_check(cudaGetDevice(&dev), "device");
        cuda_check(cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, dev), "device");
        void* scratch = nullptr;
        const size_t scratch_bytes = 2u * (size_t)(l2 > 0 ? l2 : 0);
        if (scratch_bytes && cudaMalloc(&scratch, scratch_bytes) != cudaSuccess) {
            (void)cudaGetLastError();
            scratch = nullptr;
        }
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        std::vector<int> cand;
        for (int v = 0; v < tc_num_variants(); ++v)
            if (tc_variant_ok(m->d, v, m->op_kind())) cand.push_back(v);
        std::vector<float> times(cand.size() * 3u, 0.f);
        cudaError_t e = cudaEventCreate(&e0);
        if (e == cudaSuccess) e = cudaEventCreate(&e1);
        for (size_t i = 0; i < cand.size() && e == cudaSuccess; ++i)   // warm-up (also sets each kernel's attributes)
            e = launch_forward_tc(m->d, a, m->op_kind(), cand[i], m->status, s);
        for (int round = 0; round < 3 && e == cudaSuccess; ++round) {
            for (size_t i = 0; i < cand.size() && e == cudaSuccess; ++i) {
                if (scratch) e = cudaMemsetAsync(scratch, round + 1, scratch_bytes, s);
                if (e == cudaSuccess) e = cudaEventRecord(e0, s);
                if (e == cudaSuccess) e = launch_forward_tc(m->d, a, m->op_kind(), cand[i], m->status, s);
                if (e == cudaSuccess) e = cudaEventRecord(e1, s);
                if (e == cudaSuccess) e = cudaEventSynchronize(e1);
                if (e == cudaSuccess) e = cudaEventElapsedTime(&times[i * 3u + round], e0, e1);
            }
        }
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        if (scratch) cudaFree(scratch);
        cuda_check(e, "autotune");
        float best = 3.0e38f;
        int best_v = m->tc_variant;
        for (size_t i = 0; i < cand.size(); ++i) {
            float t[3] = {times[i * 3u], times[i * 3u + 1u], times[i * 3u + 2u]};
            std::sort(t, t + 3);
            if (t[1] < best) {
                best = t[1];
                best_v = cand[i];
            }
        }
        m->tc_variant = best_v;
    });
}

int nlod_calib_gathers(nlod_module* m, void* stream, uint32_t n, float* ms_out) {
    return guarded([&] {
        if (!m || !ms_out) throw Error(NLOD_ERR_INVALID, "module and ms_out must not be NULL");
        if (m->d.n_grids == 0) throw Error(NLOD_ERR_UNSUPPORTED, "the module has no grid encoding");
        cudaStream_t s = (cudaStream_t)stream;
        // the gathers' results go into a sum that is stored (to the gradient buffer's first entry,
        // which the next training step clears) only if it equals a value no table sum takes
        const bool half = m->grid_h != nullptr;
        const void* tables = half ? static_cast<const void*>(m->grid_h) : static_cast<const void*>(m->inference_params());
        ensure_cells(m, s);
        time_on_stream(s, ms_out, [&] { return launch_calib_gathers(m->d, tables, half, n, m->grads, s, half ? m->cells : nullptr, m->cells_levels, m->cell_base); });
    });
}

int nlod_calib_scatter(nlod_module* m, void* stream, uint32_t n, float* ms_out) {
    return guarded([&] {
        if (!m || !ms_out) throw Error(NLOD_ERR_INVALID, "module and ms_out must not be NULL");
        if (m->d.n_grids == 0) throw Error(NLOD_ERR_UNSUPPORTED, "the module has no grid encoding");
        cudaStream_t s = (cudaStream_t)stream;
        time_on_stream(s, ms_out, [&] { return launch_calib_scatter(m->d, m->grads, n, s); });
    });
}

int nlod_sync_status(nlod_module* m, void* stream) {
    if (!m) {
        g_last_error = "module is NULL";
        return NLOD_ERR_INVALID;
    }
    uint32_t st = 0;
    cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
    if (e != cudaSuccess) {
        g_last_error = std::string("stream synchronize: ") + cudaGetErrorString(e);
        return NLOD_ERR_CUDA;
    }
    e = cudaMemcpy(&st, m->status, sizeof st, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
        g_last_error = std::string("status read: ") + cudaGetErrorString(e);
        return NLOD_ERR_CUDA;
    }
    if (st) {
        cudaMemset(m->status, 0, sizeof st);
        g_last_error = "a bounded device-side wait timed out";
        return NLOD_ERR_TIMEOUT;
    }
    g_last_error.clear();
    return NLOD_OK;
}

}  // extern "C"
