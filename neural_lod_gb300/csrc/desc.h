// Plain-old-data description of one network-with-input-encoding, shared by the host code
// (which builds it from the tiny-cuda-nn JSON configs) and the kernels (which receive it
// by value as a __grid_constant__ parameter).
#pragma once

#include <cstdint>

namespace nlod {

constexpr int kMaxSlots = 8;       // nested encodings after flattening Composite / RepeatedComposite
constexpr int kMaxGrids = 2;       // distinct grid encodings (each with its own parameters)
constexpr int kMaxLevels = 32;     // levels per grid (tiny-cuda-nn allows 128; neural_lod uses <= 16)
constexpr int kMaxLayers = 10;     // weight matrices of the MLP (input + hidden + output)
constexpr uint32_t kBatchGranularity = 128;

enum SlotType : int32_t { SLOT_GRID = 0, SLOT_SH = 1, SLOT_IDENTITY = 2, SLOT_ONEHOT = 3 };
enum Activation : int32_t { ACT_NONE = 0, ACT_RELU = 1, ACT_SIGMOID = 2, ACT_EXP = 3 };
enum HashKind : int32_t { HASH_COHERENT_PRIME = 0, HASH_PRIME = 1, HASH_REVERSED_PRIME = 2 };
enum GridKind : int32_t { GRID_HASH = 0, GRID_DENSE = 1, GRID_TILED = 2 };
enum Interp : int32_t { INTERP_LINEAR = 0, INTERP_NEAREST = 1, INTERP_SMOOTHSTEP = 2 };
enum LossKind : int32_t { LOSS_NONE = 0, LOSS_BCE = 1, LOSS_RELATIVE_L2 = 2, LOSS_L2 = 3 };

// One level of a grid encoding: tiny-cuda-nn's offset table entry plus the derived
// per-level scale and resolution (rptr/ext/tiny-cuda-nn/include/tiny-cuda-nn/encodings/grid.h:195-204, 982-1015).
// 16 bytes, so a kernel reads one level with a single 128-bit shared-memory load.
struct alignas(16) GridLevel {
    uint32_t offset;    // first table entry of the level (entries, not floats)
    uint32_t size;      // entries in the level ("hashmap_size")
    uint32_t res_flags; // grid_resolution(scale) in bits 0..27, per-level flags in bits 28..31
    float scale;        // grid_scale(level, log2(per_level_scale), base_resolution)
};

// Per-level flags (bits 28..31 of res_flags): the index rule of grid.h:170-187 resolved once on
// the host.
constexpr uint32_t kLevelResMask = 0x0FFFFFFFu;
constexpr uint32_t kLevelHashed = 1u << 28;     // the spatial hash replaces the dense index
constexpr uint32_t kLevelPow2 = 1u << 29;       // size is a power of two (modulo is a mask)
constexpr uint32_t kLevelDimsShift = 30u;       // dims folded into the dense index (0..3)

struct GridDesc {
    uint32_t n_levels;
    uint32_t n_features;       // per level (F)
    int32_t hash;              // HashKind
    int32_t kind;              // GridKind
    int32_t interp;            // Interp
    uint32_t param_offset;     // first float of the grid in the module's parameter vector
    uint32_t n_params;         // floats (entries * F)
    uint32_t pad_;
    GridLevel levels[kMaxLevels];
};

// One flattened nested encoding writing columns [out_begin, out_begin + out_width) of the
// encoded row.  out_width includes n_pad padding columns; SH writes its padding (1.0)
// first (spherical_harmonics.h:57-63), grid pads with 0 after its features
// (grid.h:1040-1051), identity pads with 1.0 after (identity.h:62-66).
struct Slot {
    int32_t type;              // SlotType
    uint32_t in_begin;         // first input column
    uint32_t n_in;             // input columns read
    uint32_t out_begin;
    uint32_t out_width;        // features + padding
    uint32_t n_pad;
    int32_t grid;              // index into ModelDesc::grids (SLOT_GRID)
    uint32_t degree;           // SLOT_SH
    uint32_t n_bins;           // SLOT_ONEHOT
    float scale;               // SLOT_IDENTITY
    float offset;              // SLOT_IDENTITY
    uint32_t pad_;
};

struct ModelDesc {
    uint32_t n_input;          // input columns (FP32 per element)
    uint32_t n_output;         // output columns written to the caller
    uint32_t n_output_padded;  // 16 (fully_fused_mlp.cu:646 REQUIRED_ALIGNMENT)
    uint32_t enc_width;        // padded encoded width = MLP input width (multiple of 16)
    uint32_t width;            // hidden width (n_neurons)
    uint32_t n_hidden_layers;  // tiny-cuda-nn's n_hidden_layers
    uint32_t n_layers;         // weight matrices = n_hidden_layers + 1
    int32_t act;               // hidden activation
    int32_t out_act;           // output activation
    uint32_t n_slots;
    uint32_t n_grids;
    uint32_t n_params_network;
    uint32_t n_params_encoding;
    uint32_t n_params;
    uint32_t layer_offset[kMaxLayers];   // first weight of each matrix in the parameter vector
    uint32_t layer_in[kMaxLayers];       // matrix columns
    uint32_t layer_out[kMaxLayers];      // matrix rows
    Slot slots[kMaxSlots];
    GridDesc grids[kMaxGrids];
};

// Optimizer hyper-parameters in the order of tiny-cuda-nn's adam_step arguments
// (rptr/ext/tiny-cuda-nn/include/tiny-cuda-nn/optimizers/adam.h:47-68).
struct AdamParams {
    float learning_rate;
    float beta1, beta2, epsilon;
    float l2_reg;
    float relative_decay, absolute_decay;
    float weight_clipping;
    float non_matrix_lr_factor;
    int32_t optimize_matrix;
    int32_t optimize_non_matrix;
    int32_t adabound;
};

}  // namespace nlod
