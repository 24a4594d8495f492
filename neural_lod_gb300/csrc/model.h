// Host-side construction of a ModelDesc / optimizer chain from tiny-cuda-nn JSON configs.
#pragma once

#include <string>

#include "desc.h"
#include "json.h"

namespace nlod {

// Parameters of the optimizer chain Ema(ExponentialDecay(Adam)) with either wrapper
// optional, as built by rptr/cuda/neural-lod/neural_lod_learning_init.cu:581-602, 824-848.
struct OptimizerDesc {
    AdamParams adam{};
    bool has_decay = false;
    uint32_t decay_start = 0, decay_interval = 1, decay_end = 0xFFFFFFFFu;
    float decay_base = 1.0f;
    bool has_ema = false;
    float ema_decay = 0.99f;
    bool ema_full_precision = false;
};

struct LossDesc {
    int32_t kind = LOSS_NONE;
};

// Parses `encoding` + `network` exactly as NetworkWithInputEncoding's constructor does
// (network_with_input_encoding.h:43-50 + encoding.cu create_encoding + composite.h:136-213)
// and fills every size, padding and parameter offset of `d`.  Throws std::runtime_error
// with a message on invalid or unsupported input.
void build_model_desc(const Json& encoding, const Json& network, uint32_t n_input_dims,
                      uint32_t n_output_dims, ModelDesc& d);

void build_loss_desc(const Json& loss, LossDesc& l);
void build_optimizer_desc(const Json& optimizer, OptimizerDesc& o);

// tiny-cuda-nn's per-level grid scale and resolution (grid.h:195-204), host side.
float grid_scale_host(uint32_t level, float log2_per_level_scale, uint32_t base_resolution);
uint32_t grid_resolution_host(float scale);

bool iequals(const std::string& a, const std::string& b);

}  // namespace nlod
