// Construction of the flattened model description from tiny-cuda-nn style JSON.
//
// The layout rules restate tiny-cuda-nn (paths relative to rptr/ext/tiny-cuda-nn/):
//  * encoding factory and per-encoding alignment: src/encoding.cu:81-164
//  * Composite concatenation + inter-encoding padding: include/tiny-cuda-nn/encodings/composite.h:136-213, 376-386
//  * RepeatedComposite (shared parameters over repetitions): encodings/repeated_composite.h:48-128, 340-361
//  * grid offset table: encodings/grid.h:982-1015; factory defaults grid.h:1417-1494
//  * SH: encodings/spherical_harmonics.h:393-412; Identity: encodings/identity.h
//  * network input alignment 16 and padded output 16: network_with_input_encoding.h:43-50,
//    src/network.cu:111-123, networks/fully_fused_mlp.h:108-110, src/fully_fused_mlp.cu:640-677
#include "model.h"

#include <algorithm>
#include <cctype>
#include <cmath>
#include <limits>
#include <stdexcept>
#include <string>
#include <vector>

namespace nlod {

bool iequals(const std::string& a, const std::string& b) {
    if (a.size() != b.size()) return false;
    for (size_t i = 0; i < a.size(); ++i)
        if (std::tolower((unsigned char)a[i]) != std::tolower((unsigned char)b[i])) return false;
    return true;
}

static uint32_t next_multiple(uint32_t v, uint32_t m) { return (v + m - 1) / m * m; }
static uint32_t gcd_u(uint32_t a, uint32_t b) { while (b) { uint32_t t = a % b; a = b; b = t; } return a; }
static uint32_t lcm_u(uint32_t a, uint32_t b) { return a / gcd_u(a, b) * b; }
static uint32_t powi_u(uint32_t b, uint32_t e) { uint32_t r = 1; for (uint32_t i = 0; i < e; ++i) r *= b; return r; }

float grid_scale_host(uint32_t level, float log2_per_level_scale, uint32_t base_resolution) {
    // exp2f(level * log2_scale) * base - 1, evaluated in FP32 like grid.h:195-200.
    return std::exp2f((float)level * log2_per_level_scale) * (float)base_resolution - 1.0f;
}

uint32_t grid_resolution_host(float scale) { return (uint32_t)std::ceil(scale) + 1; }

static uint32_t json_u32(const Json& j, const std::string& k, uint32_t def) {
    if (!j.contains(k)) return def;
    double v = j.at(k).as_number();
    if (v < 0 || v > 4294967295.0 || v != std::floor(v)) throw std::runtime_error("config: '" + k + "' must be a non-negative integer");
    return (uint32_t)v;
}

// ---------------------------------------------------------------------------------------------
// Encoding tree.  Each node mirrors one tiny-cuda-nn Encoding object: it knows its raw output
// width, its required output alignment and how to take a padded output width.
// ---------------------------------------------------------------------------------------------
namespace {

struct EncNode {
    int kind = -1;                   // SlotType, or 100 = Composite, 101 = RepeatedComposite
    uint32_t n_dims_to_encode = 0;
    uint32_t n_output = 0;           // unpadded features
    uint32_t n_pad = 0;
    // grid
    GridDesc grid{};
    uint32_t n_params = 0;
    // SH / identity / one-hot
    uint32_t degree = 0, n_bins = 0;
    float scale = 1.0f, offset = 0.0f;
    // composites
    std::vector<EncNode> nested;
    std::vector<uint32_t> dims_begin;   // per nested (Composite) or per nested*rep (Repeated)
    uint32_t n_repetitions = 1;

    bool is_composite() const { return kind >= 100; }

    uint32_t required_output_alignment() const {
        if (kind == SLOT_GRID) return grid.n_features;
        if (is_composite()) {
            uint32_t a = 1;
            for (auto& n : nested) a = lcm_u(a, n.required_output_alignment());
            return a;
        }
        return 1;
    }

    uint32_t padded_output_width() const {
        if (kind == 100) {
            uint32_t t = 0;
            for (auto& n : nested) t += n.padded_output_width();
            return t;
        }
        if (kind == 101) {
            uint32_t t = 0;
            for (auto& n : nested) t += n.padded_output_width();
            return t * n_repetitions;
        }
        return n_output + n_pad;
    }

    void set_padded_output_width(uint32_t w) {
        if (kind == 100) {
            uint32_t prev = padded_output_width() - nested.back().padded_output_width();
            if (w < prev) throw std::runtime_error("encoding: padded width too small");
            nested.back().set_padded_output_width(w - prev);
            return;
        }
        if (kind == 101) {
            if (w != padded_output_width())
                throw std::runtime_error("encoding: RepeatedComposite with padding is not supported; make its width a multiple of the network alignment");
            return;
        }
        if (w < n_output) throw std::runtime_error("encoding: padded width below output width");
        n_pad = w - n_output;
    }

    void set_alignment(uint32_t alignment) {
        set_padded_output_width(next_multiple(padded_output_width(), lcm_u(alignment, required_output_alignment())));
    }
};

EncNode make_encoding(const Json& j, uint32_t n_dims_to_encode, uint32_t alignment);

void build_grid(const Json& j, uint32_t n_dims, EncNode& n) {
    if (n_dims != 3) throw std::runtime_error("GridEncoding: only 3 input dims are supported");
    const uint32_t log2T = json_u32(j, "log2_hashmap_size", 19u);
    const std::string otype = j.value_str("otype", "Grid");
    std::string default_type = iequals(otype, "TiledGrid") ? "Tiled" : (iequals(otype, "DenseGrid") ? "Dense" : "Hash");
    const uint32_t F = json_u32(j, "n_features_per_level", 2u);
    if (F != 2) throw std::runtime_error("GridEncoding: n_features_per_level must be 2 in this build (tiny-cuda-nn also allows 1, 4, 8)");
    uint32_t n_features;
    if (j.contains("n_features") || j.contains("n_grid_features")) {
        n_features = j.contains("n_features") ? json_u32(j, "n_features", 0) : json_u32(j, "n_grid_features", 0);
        if (j.contains("n_levels")) throw std::runtime_error("GridEncoding: may not specify n_features and n_levels simultaneously (one determines the other)");
    } else {
        n_features = F * json_u32(j, "n_levels", 16u);
    }
    if (n_features % F != 0) throw std::runtime_error("GridEncoding: n_features must be a multiple of n_features_per_level");
    const uint32_t n_levels = (n_features + F - 1) / F;
    if (n_levels == 0 || n_levels > (uint32_t)kMaxLevels) throw std::runtime_error("GridEncoding: n_levels must be in [1, 32]");
    const uint32_t base_res = json_u32(j, "base_resolution", 16u);
    const float per_level_scale = (float)j.value("per_level_scale", 2.0);
    if (j.value_bool("stochastic_interpolation", false))
        throw std::runtime_error("GridEncoding: stochastic_interpolation is not supported");
    std::string interp = j.value_str("interpolation", "Linear");
    std::string type = j.value_str("type", default_type);
    std::string hash = j.value_str("hash", "CoherentPrime");
    if (log2T > 31) throw std::runtime_error("GridEncoding: log2_hashmap_size must be <= 31");

    GridDesc& g = n.grid;
    g = GridDesc{};
    g.n_levels = n_levels;
    g.n_features = F;
    if (iequals(hash, "CoherentPrime")) g.hash = HASH_COHERENT_PRIME;
    else if (iequals(hash, "Prime")) g.hash = HASH_PRIME;
    else if (iequals(hash, "ReversedPrime")) g.hash = HASH_REVERSED_PRIME;
    else if (iequals(hash, "Rng")) throw std::runtime_error("GridEncoding: hash 'Rng' is not supported");
    else throw std::runtime_error("Invalid hash type: " + hash);
    if (iequals(type, "Hash")) g.kind = GRID_HASH;
    else if (iequals(type, "Dense")) g.kind = GRID_DENSE;
    else if (iequals(type, "Tiled") || iequals(type, "Tile")) g.kind = GRID_TILED;
    else throw std::runtime_error("Invalid grid type: " + type);
    if (iequals(interp, "Linear")) g.interp = INTERP_LINEAR;
    else if (iequals(interp, "Nearest")) g.interp = INTERP_NEAREST;
    else if (iequals(interp, "Smoothstep")) g.interp = INTERP_SMOOTHSTEP;
    else throw std::runtime_error("Invalid interpolation type: " + interp);

    // Offset table, grid.h:982-1015.
    const float log2s = std::log2(per_level_scale);
    uint32_t offset = 0;
    for (uint32_t i = 0; i < n_levels; ++i) {
        const float scale = grid_scale_host(i, log2s, base_res);
        const uint32_t res = grid_resolution_host(scale);
        const uint32_t max_params = std::numeric_limits<uint32_t>::max() / 2;
        uint32_t in_level = std::pow((float)res, 3.0f) > (float)max_params ? max_params : powi_u(res, 3);
        in_level = next_multiple(in_level, 8u);
        if (g.kind == GRID_TILED) in_level = std::min(in_level, powi_u(base_res, 3));
        else if (g.kind == GRID_HASH) in_level = std::min(in_level, 1u << log2T);
        if (res > kLevelResMask) throw std::runtime_error("GridEncoding: level resolution must be below 2^28");
        g.levels[i].offset = offset;
        g.levels[i].size = in_level;
        g.levels[i].scale = scale;
        // grid_index's loop (grid.h:175-186): dims are folded while the running stride fits.
        uint32_t dims = 0;
        uint32_t stride32 = 1;
        for (uint32_t dim = 0; dim < 3 && stride32 <= in_level; ++dim) {
            ++dims;
            stride32 *= res;   // uint32 arithmetic, as on the device
        }
        uint32_t flags = dims << kLevelDimsShift;
        if (g.kind == GRID_HASH && in_level < stride32) flags |= kLevelHashed;
        if ((in_level & (in_level - 1)) == 0) flags |= kLevelPow2;
        g.levels[i].res_flags = res | flags;
        if ((uint64_t)offset + in_level > 0x7FFFFFFFull) throw std::runtime_error("GridEncoding: too many parameters");
        offset += in_level;
    }
    g.n_params = offset * F;
    n.n_params = g.n_params;
    n.n_output = n_features;
}

EncNode make_encoding(const Json& j, uint32_t n_dims_to_encode, uint32_t alignment) {
    if (!j.is_object()) throw std::runtime_error("encoding config must be a JSON object");
    EncNode n;
    n.n_dims_to_encode = n_dims_to_encode;
    const std::string otype = j.value_str("otype", "OneBlob");
    if (iequals(otype, "Composite") || iequals(otype, "RepeatedComposite")) {
        const bool repeated = iequals(otype, "RepeatedComposite");
        n.kind = repeated ? 101 : 100;
        if (!j.contains("nested") || !j.at("nested").is_array())
            throw std::runtime_error("Must provide an array of nested encodings to CompositeEncoding.");
        if (j.contains("reduction") && !iequals(j.value_str("reduction", "Concatenation"), "Concatenation"))
            throw std::runtime_error("CompositeEncoding: only Concatenation reduction is supported");
        const auto& nested = j.at("nested").items();
        n.n_repetitions = repeated ? json_u32(j, "n_repetitions", 1u) : 1u;
        if (n.n_repetitions == 0) throw std::runtime_error("RepeatedComposite: n_repetitions must be >= 1");
        uint32_t total = 0;
        for (auto& e : nested) {
            total += json_u32(e, "n_dims_to_encode", 0);
            if (e.contains("dims_to_encode_begin")) { total = 0xFFFFFFFFu; break; }
        }
        if (repeated) {
            if (total == 0xFFFFFFFFu) throw std::runtime_error("dims_to_encode_begin not supported with repeated encodings");
            total *= n.n_repetitions;
            if (total != n_dims_to_encode)
                throw std::runtime_error("RepeatedCompositeEncoding: nested encodings must encode exactly the number of dims of the composite");
        } else if (total != 0xFFFFFFFFu && total > n_dims_to_encode) {
            throw std::runtime_error("CompositeEncoding: nested encodings must not encode more dims than composite");
        }
        uint32_t unspecified = total == 0xFFFFFFFFu ? 0xFFFFFFFFu : (n_dims_to_encode - total);
        uint32_t offset = 0;
        for (uint32_t rep = 0; rep < n.n_repetitions; ++rep) {
            for (auto& e : nested) {
                uint32_t nd;
                if (e.contains("n_dims_to_encode")) {
                    if (e.contains("dims_to_encode_begin")) offset = json_u32(e, "dims_to_encode_begin", 0);
                    nd = json_u32(e, "n_dims_to_encode", 0);
                } else {
                    if (unspecified == 0xFFFFFFFFu)
                        throw std::runtime_error("CompositeEncoding: may only leave 'n_dims_to_encode' unspecified for a single nested encoding");
                    nd = unspecified;
                    unspecified = 0xFFFFFFFFu;
                }
                if (nd > 0) {
                    if (rep == 0) n.nested.push_back(make_encoding(e, nd, 1));
                    n.dims_begin.push_back(offset);
                }
                offset += nd;
            }
        }
        if (n.nested.empty()) throw std::runtime_error("CompositeEncoding: no nested encoding encodes any dimension");
        // Alignment between nested encodings (composite.h:192-200).
        uint32_t so_far = 0;
        for (size_t i = 0; i + 1 < n.nested.size(); ++i) {
            uint32_t want = n.nested[i + 1].required_output_alignment();
            uint32_t w = next_multiple(so_far + n.nested[i].padded_output_width(), want) - so_far;
            n.nested[i].set_padded_output_width(w);
            so_far += n.nested[i].padded_output_width();
        }
    } else if (iequals(otype, "Grid") || iequals(otype, "HashGrid") || iequals(otype, "TiledGrid") || iequals(otype, "DenseGrid")) {
        n.kind = SLOT_GRID;
        build_grid(j, n_dims_to_encode, n);
    } else if (iequals(otype, "SphericalHarmonics")) {
        n.kind = SLOT_SH;
        n.degree = json_u32(j, "degree", 4u);
        if (n_dims_to_encode != 3) throw std::runtime_error("Can only encode 3D directions in spherical harmonics.");
        if (n.degree == 0) throw std::runtime_error("Spherical harmonics must have positive degree.");
        if (n.degree > 8) throw std::runtime_error("Spherical harmonics are only implemented up to degree 8.");
        n.n_output = n.degree * n.degree;
    } else if (iequals(otype, "Identity")) {
        n.kind = SLOT_IDENTITY;
        n.scale = (float)j.value("scale", 1.0);
        n.offset = (float)j.value("offset", 0.0);
        n.n_output = n_dims_to_encode;
    } else if (iequals(otype, "OneHot")) {
        // Extension (no tiny-cuda-nn counterpart): x in [0,1] -> one-hot over n_bins,
        // bin = min(floor(x * n_bins), n_bins - 1).  Used for the LoD index input.
        n.kind = SLOT_ONEHOT;
        if (n_dims_to_encode != 1) throw std::runtime_error("OneHot encodes exactly 1 input dim");
        n.n_bins = json_u32(j, "n_bins", 8u);
        if (n.n_bins == 0 || n.n_bins > 64) throw std::runtime_error("OneHot: n_bins must be in [1, 64]");
        n.n_output = n.n_bins;
    } else {
        throw std::runtime_error("Unsupported encoding type in this build: " + otype);
    }
    if (alignment > 0) n.set_alignment(alignment);
    return n;
}

struct Flattener {
    ModelDesc& d;
    uint32_t param_cursor = 0;   // relative to the encoding's first parameter
    uint32_t out_cursor = 0;

    void flatten(const EncNode& n, uint32_t in_begin, int reuse_grid = -1) {
        if (n.kind == 100) {
            for (size_t i = 0; i < n.nested.size(); ++i) flatten(n.nested[i], in_begin + n.dims_begin[i]);
            return;
        }
        if (n.kind == 101) {
            const size_t k = n.nested.size();
            std::vector<int> grid_ids(k, -1);
            for (uint32_t rep = 0; rep < n.n_repetitions; ++rep) {
                for (size_t i = 0; i < k; ++i) {
                    int before = (int)d.n_grids;
                    flatten(n.nested[i], in_begin + n.dims_begin[rep * k + i], rep == 0 ? -1 : grid_ids[i]);
                    if (rep == 0 && (int)d.n_grids > before) grid_ids[i] = (int)d.n_grids - 1;
                }
            }
            return;
        }
        if (d.n_slots >= (uint32_t)kMaxSlots) throw std::runtime_error("encoding: too many nested encodings");
        Slot& s = d.slots[d.n_slots++];
        s = Slot{};
        s.type = n.kind;
        s.in_begin = in_begin;
        s.n_in = n.n_dims_to_encode;
        s.out_begin = out_cursor;
        s.out_width = n.n_output + n.n_pad;
        s.n_pad = n.n_pad;
        s.grid = -1;
        s.degree = n.degree;
        s.n_bins = n.n_bins;
        s.scale = n.scale;
        s.offset = n.offset;
        if (n.kind == SLOT_GRID) {
            if (reuse_grid >= 0) {
                s.grid = reuse_grid;
            } else {
                if (d.n_grids >= (uint32_t)kMaxGrids) throw std::runtime_error("encoding: at most 2 distinct grid encodings are supported");
                GridDesc g = n.grid;
                g.param_offset = param_cursor;   // made absolute once the network size is known
                param_cursor += g.n_params;
                d.grids[d.n_grids] = g;
                s.grid = (int)d.n_grids++;
            }
        }
        out_cursor += s.out_width;
    }
};

}  // namespace

void build_model_desc(const Json& encoding, const Json& network, uint32_t n_input_dims, uint32_t n_output_dims, ModelDesc& d) {
    d = ModelDesc{};
    if (n_input_dims == 0 || n_input_dims > 64) throw std::runtime_error("n_input_dims must be in [1, 64]");
    if (n_output_dims == 0 || n_output_dims > 16) throw std::runtime_error("n_output_dims must be in [1, 16] (fully fused output layer)");
    if (!network.is_object()) throw std::runtime_error("network config must be a JSON object");

    // Network (fully_fused_mlp.cu:640-677).
    std::string otype = network.value_str("otype", "MLP");
    if (!(iequals(otype, "FullyFusedMLP") || iequals(otype, "MegakernelMLP") || iequals(otype, "CutlassMLP") || iequals(otype, "MLP")))
        throw std::runtime_error("Unsupported network type: " + otype);
    const uint32_t width = json_u32(network, "n_neurons", 128u);
    if (width != 16 && width != 32 && width != 64 && width != 128)
        throw std::runtime_error("FullyFusedMLP only supports 16, 32, 64, and 128 neurons");
    const uint32_t n_hidden = json_u32(network, "n_hidden_layers", 5u);
    if (n_hidden == 0) throw std::runtime_error("FullyFusedMLP requires at least 1 hidden layer (3 layers in total).");
    if (n_hidden + 1 > (uint32_t)kMaxLayers) throw std::runtime_error("too many hidden layers");
    auto act_of = [](const std::string& s) -> int32_t {
        if (iequals(s, "None")) return ACT_NONE;
        if (iequals(s, "ReLU")) return ACT_RELU;
        if (iequals(s, "Sigmoid")) return ACT_SIGMOID;
        if (iequals(s, "Exponential")) return ACT_EXP;
        throw std::runtime_error("Unsupported activation in this build: " + s);
    };
    d.act = act_of(network.value_str("activation", "ReLU"));
    d.out_act = act_of(network.value_str("output_activation", "None"));
    if (d.act != ACT_RELU && d.act != ACT_NONE) throw std::runtime_error("hidden activation must be ReLU or None");

    // Encoding, aligned to the network's minimum alignment (16).
    EncNode root = make_encoding(encoding, n_input_dims, 8);
    root.set_alignment(16);

    Flattener f{d};
    f.flatten(root, 0);
    d.enc_width = root.padded_output_width();
    if (d.enc_width != f.out_cursor) throw std::runtime_error("internal: encoding width mismatch");
    if (d.enc_width % 16 != 0 || d.enc_width == 0 || d.enc_width > 256)
        throw std::runtime_error("encoded width must be a multiple of 16 in [16, 256]");
    for (uint32_t i = 0; i < d.n_slots; ++i)
        if (d.slots[i].in_begin + d.slots[i].n_in > n_input_dims)
            throw std::runtime_error("encoding reads past the input dims");

    d.n_input = n_input_dims;
    d.n_output = n_output_dims;
    d.n_output_padded = 16;
    d.width = width;
    d.n_hidden_layers = n_hidden;
    d.n_layers = n_hidden + 1;
    uint32_t off = 0;
    for (uint32_t l = 0; l < d.n_layers; ++l) {
        d.layer_in[l] = l == 0 ? d.enc_width : width;
        d.layer_out[l] = l + 1 == d.n_layers ? d.n_output_padded : width;
        d.layer_offset[l] = off;
        off += d.layer_in[l] * d.layer_out[l];
    }
    d.n_params_network = off;
    uint32_t enc_params = 0;
    for (uint32_t g = 0; g < d.n_grids; ++g) {
        d.grids[g].param_offset += d.n_params_network;
        enc_params += d.grids[g].n_params;
    }
    d.n_params_encoding = enc_params;
    if ((uint64_t)d.n_params_network + enc_params > 0x7FFFFFFFull) throw std::runtime_error("too many parameters");
    d.n_params = d.n_params_network + enc_params;
}

void build_loss_desc(const Json& loss, LossDesc& l) {
    l = LossDesc{};
    std::string t = loss.value_str("otype", "L2");
    if (iequals(t, "BinaryCrossEntropy")) l.kind = LOSS_BCE;
    else if (iequals(t, "RelativeL2")) l.kind = LOSS_RELATIVE_L2;
    else if (iequals(t, "L2")) l.kind = LOSS_L2;
    else throw std::runtime_error("Unsupported loss in this build: " + t);
}

static void parse_adam(const Json& j, AdamParams& a) {
    std::string t = j.value_str("otype", "Adam");
    if (!iequals(t, "Adam")) throw std::runtime_error("Unsupported optimizer in this build: " + t);
    a.learning_rate = (float)j.value("learning_rate", 1e-3);
    a.beta1 = (float)j.value("beta1", 0.9);
    a.beta2 = (float)j.value("beta2", 0.999);
    a.epsilon = (float)j.value("epsilon", 1e-8);
    a.l2_reg = (float)j.value("l2_reg", 1e-8);
    a.relative_decay = (float)j.value("relative_decay", 0.0);
    a.absolute_decay = (float)j.value("absolute_decay", 0.0);
    a.weight_clipping = (float)j.value("clipping_magnitude", 0.0);
    a.non_matrix_lr_factor = (float)j.value("non_matrix_learning_rate_factor", 1.0);
    a.optimize_matrix = j.value_bool("optimize_matrix_params", true) ? 1 : 0;
    a.optimize_non_matrix = j.value_bool("optimize_non_matrix_params", true) ? 1 : 0;
    a.adabound = j.value_bool("adabound", false) ? 1 : 0;
}

void build_optimizer_desc(const Json& opt, OptimizerDesc& o) {
    o = OptimizerDesc{};
    const Json* cur = &opt;
    Json empty = Json::object();
    for (int depth = 0; depth < 4; ++depth) {
        std::string t = cur->value_str("otype", "Adam");
        if (iequals(t, "Ema") || iequals(t, "EMA")) {
            if (o.has_ema || o.has_decay) throw std::runtime_error("Ema must be the outermost optimizer wrapper");
            o.has_ema = true;
            o.ema_decay = (float)cur->value("decay", 0.99);
            o.ema_full_precision = cur->value_bool("full_precision", false);
            cur = cur->contains("nested") ? &cur->at("nested") : &empty;
        } else if (iequals(t, "ExponentialDecay")) {
            if (o.has_decay) throw std::runtime_error("nested ExponentialDecay is not supported");
            o.has_decay = true;
            o.decay_base = (float)cur->value("decay_base", 0.1);
            o.decay_interval = json_u32(*cur, "decay_interval", 10000u);
            o.decay_start = json_u32(*cur, "decay_start", 10000u);
            o.decay_end = json_u32(*cur, "decay_end", 10000000u);
            if (o.decay_interval == 0) throw std::runtime_error("ExponentialDecay: decay_interval must be > 0");
            cur = cur->contains("nested") ? &cur->at("nested") : &empty;
        } else {
            parse_adam(*cur, o.adam);
            return;
        }
    }
    throw std::runtime_error("optimizer nesting too deep");
}

}  // namespace nlod
