/*
 * CPU oracle of the neural-LoD hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * Only the tests, __graft_entry__.smoke() and bench.py's CPU-baseline legs may load this
 * library; the product (libnlod.so) never calls it.  It restates, in plain C, tiny-cuda-nn's
 * algorithms for the neural_lod network path (paths relative to rptr/ext/tiny-cuda-nn/):
 *   grid offset table / resolution     include/tiny-cuda-nn/encodings/grid.h:195-204, 982-1015
 *   grid index + hashes                encodings/grid.h:111-187
 *   pos_fract                          include/tiny-cuda-nn/common_device.h:437-464
 *   grid forward / backward            encodings/grid.h:220-392 / 394-517
 *   spherical harmonics                encodings/spherical_harmonics.h:46-151
 *   composite concatenation            encodings/composite.h:215-281
 *   fully fused MLP forward/backward   src/fully_fused_mlp.cu:499-633, 733-833
 *   losses                             include/tiny-cuda-nn/losses/binary_cross_entropy.h:7-43,
 *                                      losses/relative_l2.h:39-76, losses/l2.h
 *   Adam / EMA / exponential decay     optimizers/adam.h:47-188, ema.h:45-124, exponential_decay.h:60-71
 * The continuous arithmetic is FP64 ("FP64 oracle"); the discrete choices (grid cell of a
 * position, hash index) are made in FP32 exactly as the GPU makes them, so that both pick the
 * same table entries.  Spherical harmonics are evaluated by the associated-Legendre recurrence,
 * independently of the generated polynomials the kernels use.
 *
 * Pinning: SH values against the reference's own kernel_sh polynomials (tests/golden/
 * make_sh_golden.py -> sh_golden.npz); grid sizes against the reference's offset-table sizes of the
 * three workload configurations; the DDA against NanoVDB compiled from the reference tree
 * (oracle/build_ref.py, tests/golden/make_dda_golden.py); gradients against FP64 central finite
 * differences of this oracle's own forward.
 */
#ifndef NLOD_ORACLE_H
#define NLOD_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_MAX_SLOTS 8
#define ORC_MAX_GRIDS 2
#define ORC_MAX_LEVELS 32
#define ORC_MAX_LAYERS 10

enum { ORC_GRID = 0, ORC_SH = 1, ORC_IDENTITY = 2, ORC_ONEHOT = 3 };
enum { ORC_ACT_NONE = 0, ORC_ACT_RELU = 1, ORC_ACT_SIGMOID = 2, ORC_ACT_EXP = 3 };
enum { ORC_LOSS_BCE = 1, ORC_LOSS_RELL2 = 2, ORC_LOSS_L2 = 3 };

typedef struct {
    int32_t n_levels;
    int32_t hash;      /* 0 coherent prime, 1 prime, 2 reversed prime */
    int32_t kind;      /* 0 hash, 1 dense, 2 tiled */
    int32_t interp;    /* 0 linear, 1 nearest, 2 smoothstep */
    int64_t param_offset;
    uint32_t offset[ORC_MAX_LEVELS + 1];
    uint32_t res[ORC_MAX_LEVELS];
    float scale[ORC_MAX_LEVELS];
} OrcGrid;

typedef struct {
    int32_t type;
    int32_t in_begin, n_in;
    int32_t out_begin, out_width, n_pad;
    int32_t grid;
    int32_t degree, n_bins;
    float scale, offset;
} OrcSlot;

typedef struct {
    int32_t n_input, n_output, enc_width, width, n_layers, act, out_act;
    int32_t layer_in[ORC_MAX_LAYERS], layer_out[ORC_MAX_LAYERS];
    int64_t layer_offset[ORC_MAX_LAYERS];
    int32_t n_slots, n_grids;
    OrcSlot slots[ORC_MAX_SLOTS];
    OrcGrid grids[ORC_MAX_GRIDS];
    int64_t n_params, n_params_network;
} OrcModel;

/* grid.h:195-204 + 982-1015: per-level scale/resolution and offsets (entries). Returns n entries. */
uint32_t orc_grid_offsets(int n_levels, uint32_t log2_hashmap_size, uint32_t base_resolution, float per_level_scale,
                          int kind, uint32_t* offsets /* n_levels+1 */, uint32_t* res, float* scale);

/* Real SH basis (degree^2 values) of direction (x,y,z) in [-1,1]^3 (already mapped), FP64. */
void orc_sh(int degree, double x, double y, double z, double* out);

/* Encoded rows [n][enc_width], FP64.  max_level: NULL or per-element fractions. */
void orc_encode(const OrcModel* m, int64_t n, const float* in, const double* params, const float* max_level,
                float max_level_scalar, double* enc);

/* Forward: out [n][n_output] post-activation; y16 (nullable) [n][16] padded post-activation. */
void orc_forward(const OrcModel* m, int64_t n, const float* in, const double* params, const float* max_level,
                 float max_level_scalar, double* out, double* y16);

/* Loss values (mean over n*n_output, summed into *loss) and dz16 = dL/d(pre-activation output)
 * * loss_scale (padding columns zero). */
void orc_loss(const OrcModel* m, int loss_kind, int64_t n, const double* y16, const float* target, double loss_scale,
              double* loss, double* dz16);

/* Parameter gradients from dz16, accumulated into grads[n_params]. */
void orc_backward(const OrcModel* m, int64_t n, const float* in, const double* params, const float* max_level,
                  float max_level_scalar, const double* dz16, double* grads);

/* One Adam step (adam.h:47-119) in FP32 on all parameters; m1, m2, steps updated. */
typedef struct {
    float lr, beta1, beta2, eps, l2_reg, rel_decay, abs_decay, clip, non_matrix_lr_factor;
    int32_t optimize_matrix, optimize_non_matrix;
    float lower_lr_bound, upper_lr_bound;
    float loss_scale;
} OrcAdam;
void orc_adam_step(const OrcAdam* a, int64_t n_params, int64_t n_matrix, float* params, const float* grads,
                   float* m1, float* m2, uint32_t* steps, float* ema, float ema_decay, float ema_debias_old,
                   float ema_debias_new);

/* ---- LoD occupancy pyramid and first-active-voxel search (restating
 *      rptr/cuda/neural-lod/neural_lod_learning_init.cu:194-267 (pyramid by >> lod),
 *      rptr/ext/nanovdb/nanovdb/util/HDDA.h:27-188, 190-307, 370-450 (HDDA, DDA, TreeMarcher),
 *      rptr/ext/nanovdb/nanovdb/util/Ray.h:153-158, 398-424 (ray eval, bbox clip),
 *      rptr/ext/nanovdb/nanovdb/NanoVDB.h:3358-3369, 3745-3757, 4442-4448 (getDim),
 *      rptr/cuda/neural-lod/neural_lod_learning_common.cuh:567-606, 783-832 (slab test, search)) */
typedef struct {
    int32_t res;            /* voxels per axis */
    int32_t n_active;
    int32_t bbox_min[3], bbox_max[3];   /* tight inclusive bbox of active voxels */
    const uint32_t* bits;   /* occupancy, bit x + y*res + z*res*res, MSB first in each word */
    const uint8_t* leaf;    /* [ceil(res/8)]^3 flags: 8^3 block has an active voxel */
    const uint8_t* lower;   /* [ceil(res/128)]^3 flags: 128^3 block has a leaf */
} OrcLodLevel;

/* Level `lod` of the pyramid from level-0 bits (res0 per axis): voxel (x,y,z) >> lod.
 * bits_out: ceil((res0>>lod)^3 / 32) words; leaf_out / lower_out sized as above. */
void orc_lod_level(const uint32_t* bits0, int32_t res0, int32_t lod, uint32_t* bits_out, uint8_t* leaf_out,
                   uint8_t* lower_out, OrcLodLevel* level);

/* First active voxel along an index-space ray (eye, dir, t_min; t_max = 1e38), skipping `prev`.
 * Returns 1 and ijk / t_near / t_far on a hit, 0 on a miss. */
int orc_first_active_voxel(const OrcLodLevel* level, const float eye[3], const float dir[3], float t_min,
                           const int32_t prev[3], int32_t ijk[3], float* t_near, float* t_far);

/* The same search restricted to ray parameters [t_min, t_max]. */
int orc_first_active_voxel_clip(const OrcLodLevel* level, const float eye[3], const float dir[3], float t_min, float t_max,
                                const int32_t prev[3], int32_t ijk[3], float* t_near, float* t_far);

void orc_first_active_voxel_batch(const OrcLodLevel* level, int64_t n, const float* eye, const float* dir,
                                  const float* t_min, const int32_t* prev, int32_t* hit, int32_t* ijk,
                                  float* t_near, float* t_far);

/* createMeshBBCube + voxinfo (cuda_voxelizer/src/util.h:87-112, 58-63): cube frame around the mesh
 * bbox, padded by eps * extent, and the voxel size (bmax - bmin) / grid per axis. */
void orc_mesh_frame(const float mn[3], const float mx[3], uint32_t grid, float eps, float bmin[3], float bmax[3], float unit[3]);

/* Conservative surface voxelization of n triangles (9 floats each) into grid^3 bits, OR-ed into
 * `bits` (bit x + y*grid + z*grid^2, most significant bit first per word), following
 * voxelize_triangle (cuda_voxelizer/src/voxelize.cu:58-190) in IEEE single precision. */
void orc_voxelize(const float* tris, int64_t n, const float bmin[3], const float unit[3], uint32_t grid, uint32_t* bits);

/* Wavefront render query (see orc_render in nlod_oracle.c). */
typedef struct {
    uint32_t width, height, max_depth, max_vis;
    float threshold, lod_max_level, lod_input;
    float background[3], env[3];
    uint64_t seed;
} OrcRenderParams;

/* Renders width x height rays through level L with the visibility / throughput networks;
 * cam = index-space eye, right, up, forward (12 floats).  image [n][3]; ray_stats [n][2]
 * (visibility, throughput queries) or NULL; totals[3] = visibility queries, throughput queries,
 * rays dropped at the per-bounce cap (or NULL). */
void orc_render(const OrcModel* vis, const double* vis_params, const OrcModel* thr, const double* thr_params, const OrcLodLevel* L,
                const OrcRenderParams* p, const float cam[12], float* image, uint32_t* ray_stats, uint64_t* totals);

/* Optimal per-voxel visibility thresholds (metric ids as NLOD_METRIC_* in include/nlod.h). */
void orc_optimal_thresholds(const float* truth, const float* proba, uint32_t n_samples, uint32_t n_voxels, int metric, float beta,
                            float* out);

/* ---- Training-sample generator (nlod_sampler.c) ----
 * Same layouts as nlod_ray_query / nlod_sampler_params in include/nlod.h. */
typedef struct {
    float origin[3];
    int32_t mode_or_data;
    float dir[3];
    float t_max;
    float voxel_center[3];
    float voxel_extent;
} OrcRayQuery;

typedef struct {
    float aabb_min[3];
    float aabb_max[3];
    float voxel_size;
    uint32_t grid_res;
    uint32_t n_lods;
    float dilation_outward, dilation_inward, min_dilation, bound_bias;
    float pdf_strength, pdf_shift;
    int32_t increase_boundary_density;
    uint32_t max_attempts;
} OrcSamplerParams;

/* Returns the number of set voxels; writes the first `capacity` Morton codes in increasing order. */
uint32_t orc_morton_voxels(const uint32_t* bits, uint32_t res, uint32_t* codes, uint32_t capacity);
void orc_cos_sin(float phi, float* c, float* s);
void orc_sample_visibility(const OrcSamplerParams* p, const uint32_t* morton, uint32_t n_voxels, uint32_t batch_index, uint32_t n,
                           float* input, OrcRayQuery* queries, uint32_t* lod);
void orc_sample_visibility_voxels(const OrcSamplerParams* p, const uint32_t* lod_morton, uint32_t first, uint32_t n_voxels,
                                  uint32_t n_samples, uint32_t lod, float* input, OrcRayQuery* queries);
void orc_sample_throughput(const OrcSamplerParams* p, const uint32_t* morton, uint32_t n_voxels, uint32_t batch_index, uint32_t n,
                           int32_t max_orders, float* input, OrcRayQuery* queries, uint32_t* lod);
void orc_trace_visibility(const OrcLodLevel* L0, const OrcSamplerParams* p, const OrcRayQuery* queries, uint32_t n, float* target);
/* Returns the number of invalid samples. */
uint32_t orc_trace_throughput(const OrcLodLevel* L0, const OrcSamplerParams* p, const OrcRayQuery* queries, uint32_t n,
                              uint32_t batch_index, int log_learning, float* input, float* target);
/* Returns the number of samples kept. */
uint32_t orc_compact_samples(const float* input, const float* target, uint32_t n, uint32_t n_in, uint32_t n_out, float* valid_input,
                             float* valid_target);

/* FP32 scalar forward over all host threads: the timed CPU baseline. Returns threads used. */
int orc_forward_f32(const OrcModel* m, int64_t n, const float* in, const float* params, const float* max_level,
                    float max_level_scalar, float* out, int n_threads);

#ifdef __cplusplus
}
#endif

#endif
