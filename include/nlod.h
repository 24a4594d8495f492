/*
 * nlod.h -- C ABI of the GB300-native neural level-of-detail library (libnlod.so).
 *
 * The library implements the neural-LoD query and its training: a composite input
 * encoding (multiresolution hash grid, spherical harmonics, identity, one-hot) feeding a
 * small fully fused MLP, trained with a fused forward+loss+backward and Adam
 * (+ ExponentialDecay / EMA wrappers).  The call shape mirrors tiny-cuda-nn's
 * NetworkWithInputEncoding + Trainer, the API the neural_lod learner and renderers call:
 *
 *   tcnn::NetworkWithInputEncoding<__half>
 *        rptr/ext/tiny-cuda-nn/include/tiny-cuda-nn/network_with_input_encoding.h:41-188
 *   tcnn::Trainer<float, __half, __half>
 *        rptr/ext/tiny-cuda-nn/include/tiny-cuda-nn/trainer.h:51-355
 *   tcnn::cpp::Module (type-erased form)
 *        rptr/ext/tiny-cuda-nn/include/tiny-cuda-nn/cpp_api.h:74-110
 *
 * Conventions
 *  - Every entry point that can fail returns an int status (NLOD_OK == 0) and never
 *    throws across the boundary; the message of the last failure on the calling thread
 *    is returned by nlod_last_error().
 *  - Streams are passed as void* (a cudaStream_t; NULL = legacy default stream).
 *  - Matrices are row-per-element FP32: input [n][n_input_dims], output
 *    [n][n_output_dims], target [n][n_output_dims].  This is tiny-cuda-nn's
 *    column-major GPUMatrix<float> as the neural_lod callers build it
 *    (rptr/cuda/neural-lod/neural_lod_learning_kernels.cuh:123, input_idx = i * n_in).
 *  - Unless stated otherwise every pointer argument is a device pointer and every
 *    call is asynchronous on the given stream.
 *  - The batch size n must be a multiple of NLOD_BATCH_GRANULARITY (128), as in
 *    tiny-cuda-nn (rptr/ext/tiny-cuda-nn/src/fully_fused_mlp.cu:598-602,
 *    rptr/ext/tiny-cuda-nn/include/tiny-cuda-nn/common.h:287).
 *  - Parameters are laid out network first, then encoding
 *    (network_with_input_encoding.h:113-120); the MLP's matrices are row-major
 *    [out][in], the output layer padded to 16 rows (fully_fused_mlp.cu:646-677).
 */
#ifndef NLOD_H
#define NLOD_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define NLOD_API __attribute__((visibility("default")))
#else
#define NLOD_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. */
#define NLOD_OK              0
#define NLOD_ERR_INVALID     1  /* bad argument, size or configuration (rejected before launch) */
#define NLOD_ERR_CUDA        2  /* a CUDA runtime call failed */
#define NLOD_ERR_ALLOC       3  /* device or host allocation failed */
#define NLOD_ERR_UNSUPPORTED 4  /* configuration valid for tiny-cuda-nn but not implemented here */
#define NLOD_ERR_TIMEOUT     5  /* a bounded device-side wait gave up (error flag set by a kernel) */
#define NLOD_ERR_STATE       6  /* call made in the wrong state (e.g. backward without forward) */

/* Arithmetic form of the network. */
#define NLOD_PRECISION_FP32  0  /* plain FP32 form: CUDA-core encoding + MLP, FP32 everything */
#define NLOD_PRECISION_FP16  1  /* tcgen05 tensor-core MLP, FP16 operands, FP32 accumulate   */
#define NLOD_PRECISION_BF16  2  /* tcgen05 tensor-core MLP, BF16 operands, FP32 accumulate   */

#define NLOD_BATCH_GRANULARITY 128

typedef struct nlod_module nlod_module;
typedef struct nlod_ctx nlod_ctx;

/* Thread-local message describing the last failure ("" if none). */
NLOD_API const char* nlod_last_error(void);

/* Library version string. */
NLOD_API const char* nlod_version(void);

/*
 * Build a network-with-input-encoding and its trainer from tiny-cuda-nn JSON configs.
 * Replaces `new NetworkWithInputEncoding(n_input_dims, n_output_dims, encoding, network)`
 * + create_loss + create_optimizer + `new Trainer(network, optimizer, loss, seed)`
 * (rptr/cuda/neural-lod/neural_lod_learning_init.cu:654-668, 889-903).
 * loss_json / optimizer_json may be NULL (inference-only module).  Parameters are
 * initialised from `seed` (Xavier-uniform MLP, U[-1e-4, 1e-4] grid entries).
 * Synchronous.  Allocates all device state on the current device.
 */
NLOD_API int nlod_module_create(const char* encoding_json, const char* network_json,
                       const char* loss_json, const char* optimizer_json,
                       uint32_t n_input_dims, uint32_t n_output_dims,
                       int precision, uint64_t seed, nlod_module** out);

/*
 * Host-only: the flattened layout the configs produce (encoded width, per nested encoding
 * input/output columns and padding, grid offset tables, matrix shapes, parameter counts) as a
 * malloc'ed JSON string (free with nlod_free_string).  Touches no GPU.  Mirrors the sizes
 * tiny-cuda-nn reports through n_params() / padded_output_width() / level_params_offset().
 */
NLOD_API int nlod_layout_json(const char* encoding_json, const char* network_json, uint32_t n_input_dims,
                              uint32_t n_output_dims, char** json_out);

/* Frees every resource of the module (synchronises the device first). */
NLOD_API void nlod_module_destroy(nlod_module* m);

/* Sizes: n_params() (network_with_input_encoding.h / object.h), the padded encoding width
 * fed to the MLP, and the padded output width (16 for the fully fused MLP). */
NLOD_API size_t   nlod_n_params(const nlod_module* m);
NLOD_API size_t   nlod_n_network_params(const nlod_module* m);
NLOD_API uint32_t nlod_n_input_dims(const nlod_module* m);
NLOD_API uint32_t nlod_n_output_dims(const nlod_module* m);
NLOD_API uint32_t nlod_encoded_width(const nlod_module* m);
NLOD_API uint32_t nlod_padded_output_width(const nlod_module* m);
NLOD_API int      nlod_precision(const nlod_module* m);

/* Per-element maximum grid level, as GridEncoding::set_max_level_gpu
 * (rptr/ext/tiny-cuda-nn/include/tiny-cuda-nn/encodings/grid.h:916-922, used at :242-265):
 * device pointer to n floats in [0,1] (fraction of grid levels kept), or NULL to disable.
 * The pointer is read by every later inference/forward/training call (n elements). */
NLOD_API int nlod_set_max_level_gpu(nlod_module* m, const float* max_level_gpu);
/* Scalar maximum level fraction (GridEncoding::set_max_level, grid.h:908-914); default 1000. */
NLOD_API int nlod_set_max_level(nlod_module* m, float max_level);

/*
 * Inference with the inference parameters (EMA weights when the optimizer has an EMA
 * wrapper).  Replaces DifferentiableObject::inference(stream, X, Y)
 * (rptr/ext/tiny-cuda-nn/include/tiny-cuda-nn/object.h:147-170), called at
 * rptr/cuda/neural-lod/wavefront_neural_throughput_visibility_lod.cu:595,662.
 * in: [n][n_input_dims] FP32 device; out: [n][n_output_dims] FP32 device.
 */
NLOD_API int nlod_inference(nlod_module* m, void* stream, uint32_t n, const float* in, float* out);

/*
 * The same inference on a batch in host memory (no reference counterpart: the reference's batches
 * are already on the device).  A page-locked input (cudaHostAlloc / cudaHostRegister) is read in
 * place by the kernel over the host link (NVLink-C2C on Grace), any other host input is first
 * copied to device memory; the output goes to a module-owned device buffer and comes back with one
 * copy.  in: [n][n_input_dims] FP32 host; out: [n][n_output_dims] FP32 host.  Asynchronous on
 * `stream` for page-locked buffers: out is valid after the stream synchronises.  Calls on one
 * module share that device buffer: two of them must not overlap on different streams.
 */
NLOD_API int nlod_inference_host(nlod_module* m, void* stream, uint32_t n, const float* in, float* out);

/*
 * Training-mode forward (training parameters), keeping what backward needs in a context.
 * Mirrors cpp::Module::forward (cpp_api.h:80).  out may be NULL.  The context is owned by
 * the caller and freed with nlod_ctx_destroy.
 */
NLOD_API int nlod_forward(nlod_module* m, void* stream, uint32_t n, const float* in, float* out, nlod_ctx** ctx);

/*
 * Backward from dL/d(output) ([n][n_output_dims] FP32 device) into the module's parameter
 * gradients (overwrite mode, EGradientMode::Overwrite, object.h:115).  Mirrors
 * cpp::Module::backward (cpp_api.h:81).  `in` must be the input given to nlod_forward.
 */
NLOD_API int nlod_backward(nlod_module* m, void* stream, nlod_ctx* ctx, const float* in, const float* dL_dout);
NLOD_API void nlod_ctx_destroy(nlod_ctx* ctx);

/*
 * One training step: forward + loss + backward (graph-captured in the reference) + optimizer
 * step.  Replaces Trainer::training_step(stream, X, Y) (trainer.h:161-186) followed by
 * Trainer::loss (trainer.h:197-199), called at rptr/cuda/neural-lod/neural_lod_learning.cu:590,686.
 * target: [n][n_output_dims] FP32 device.  loss_out: NULL or a device float receiving the
 * mean loss of this step (no host synchronisation).  Loss scale 128 (trainer.h:171).
 */
NLOD_API int nlod_training_step(nlod_module* m, void* stream, uint32_t n, const float* in,
                       const float* target, float* loss_out);

/*
 * nlod_training_step for callers that cannot allocate device memory while they train, for example
 * an online learner that takes one step inside a real-time frame loop with a no-allocation budget.
 * No counterpart in the reference (tiny-cuda-nn's Trainer allocates its step workspace from its
 * memory arena).  Same arguments and status codes as nlod_training_step; the step runs the plain
 * FP32 kernels whatever precision the module has (the tensor-core step needs a workspace of its
 * own), so its result is that of nlod_training_step on the module's FP32 form.  The step's
 * intermediates live in a fixed 16 MiB device scratch that the library holds on every GPU that uses
 * it until the process exits, instead of a cudaMalloc'ed workspace, and the call itself allocates
 * nothing.  A batch whose intermediates do not fit is rejected with NLOD_ERR_INVALID and a message
 * giving the largest batch this network can use (about 10k elements for a 48-wide encoding with two
 * 64-wide hidden layers).  The first call in a device's context is the set-up: it looks up the
 * scratch's device address and, under CUDA's lazy module loading (the default), that first lookup
 * and the first launches load the scratch and the step's kernels, which takes device memory once.
 * Make that first call at start-up, outside the no-allocation region and before any stream capture;
 * from the second call on nothing is allocated.  The same holds again after cudaDeviceReset, which
 * gives the device a new context.  All calls share the one scratch and it keeps the last call's
 * contents, so calls that overlap on the GPU (other streams or threads) race on it.
 */
NLOD_API int nlod_training_step_noalloc(nlod_module* m, void* stream, uint32_t n, const float* in,
                                        const float* target, float* loss_out);

/* Same as nlod_training_step without the optimizer step (run_optimizer = false). */
NLOD_API int nlod_forward_backward_loss(nlod_module* m, void* stream, uint32_t n, const float* in,
                               const float* target, float* loss_out);

/* Optimizer step over the current gradients (Trainer::optimizer_step, trainer.h:151-153). */
NLOD_API int nlod_optimizer_step(nlod_module* m, void* stream);

/* Optimizer step counter and learning rate (Optimizer::step / learning_rate). */
NLOD_API uint32_t nlod_optimizer_step_count(const nlod_module* m);
NLOD_API float    nlod_learning_rate(const nlod_module* m);
NLOD_API int      nlod_set_learning_rate(nlod_module* m, float lr);

/*
 * FP32 parameter access.  set replaces Trainer::set_params_full_precision
 * (trainer.h:234-246): writes the FP32 master weights and refreshes the operand copies
 * and inference weights.  get copies the FP32 master weights (which = 0), the inference
 * parameters (which = 1, EMA when enabled) or the last gradients (which = 2, unscaled:
 * dL/dparam of the mean loss).  device_ptr selects device (1) or host (0) buffers.
 * Both synchronise the device.
 */
NLOD_API int nlod_set_params(nlod_module* m, const float* params, size_t n_params, int device_ptr);
NLOD_API int nlod_get_params(nlod_module* m, float* params, size_t n_params, int which, int device_ptr);

/*
 * Checkpoints in tiny-cuda-nn's Trainer::serialize JSON form (trainer.h:267-306):
 * {"n_params": N, "params_type": "__half"|"float", "params_binary": {"bytes": [...]}}.
 * nlod_serialize allocates *json_out with malloc; free it with nlod_free_string.
 * half_precision = 1 writes __half inference params (the reference's format).
 */
NLOD_API int  nlod_serialize(nlod_module* m, int half_precision, char** json_out);
NLOD_API int  nlod_deserialize(nlod_module* m, const char* json);
NLOD_API void nlod_free_string(char* s);

/*
 * Kernel organisation of the tensor-core query (tile pipelines per CTA x grid levels per gather
 * unit).  No tiny-cuda-nn counterpart (its launch shapes are fixed).  nlod_autotune times every
 * variant that fits the network on the given batch and keeps the fastest (synchronous; per variant
 * one warm-up and three timed launches in rounds over all variants, each timed launch after a
 * write of twice the L2's size to a scratch buffer allocated for the call, the median deciding);
 * nlod_set_kernel_variant forces one.  The FP32 form has one.
 */
NLOD_API int nlod_kernel_variants(const nlod_module* m);
NLOD_API int nlod_get_kernel_variant(const nlod_module* m);
NLOD_API int nlod_set_kernel_variant(nlod_module* m, int variant);
NLOD_API int nlod_autotune(nlod_module* m, void* stream, uint32_t n, const float* in, float* out);

/*
 * Calibration (diagnostics; no tiny-cuda-nn counterpart): the memory-side floors of the hot path
 * on this module's grid, each kernel alone at full occupancy, timed with CUDA events on `stream`
 * (synchronous).  nlod_calib_gathers: the encoding's grid gathers of n queries (from the FP16
 * table copy when the module keeps one) -- the floor of the query kernel and of the training
 * encoding.  nlod_calib_scatter: the grid-gradient scatter of n samples (one reduction per corner,
 * x-adjacent aligned pairs merged) -- the floor of the fused training kernel; it overwrites the
 * module's gradient buffer (the next training step clears it).  Positions are seeded U[0,1)^3.
 * ms_out receives the kernel's duration.
 */
NLOD_API int nlod_calib_gathers(nlod_module* m, void* stream, uint32_t n, float* ms_out);
NLOD_API int nlod_calib_scatter(nlod_module* m, void* stream, uint32_t n, float* ms_out);

/* ---- LoD occupancy pyramid and first-active-voxel search ----------------------------------
 * The reference builds one NanoVDB grid per LoD from the voxelizer's point cloud, level k holding
 * voxel (x,y,z) >> k (rptr/cuda/neural-lod/neural_lod_learning_init.cu:194-267), and marches
 * index-space rays through it with nanovdb::TreeMarcher + DDA in first_active_voxel_intersection
 * (rptr/cuda/neural-lod/neural_lod_learning_common.cuh:783-832), called from raymarch_impl
 * (rptr/cuda/wavefront_neural_pt.cuh:89-141).  Here the pyramid is a bit-packed grid per level
 * (bit x + y*res + z*res^2, most significant bit first per uint32: the cuda_voxelizer output) and
 * the search returns the same voxel, t_near and t_far as NanoVDB's DDA in IEEE single precision. */
typedef struct nlod_lod_grid nlod_lod_grid;

/* Builds n_levels levels from a level-0 occupancy of res^3 voxels (device buffer, copied).
 * res must be a power of two <= 4096.  Synchronous. */
NLOD_API int nlod_lod_grid_create(const uint32_t* level0_bits, uint32_t res, uint32_t n_levels, void* stream,
                                  nlod_lod_grid** out);
NLOD_API void nlod_lod_grid_destroy(nlod_lod_grid* g);
/* Resolution, active voxel count, tight bbox (min xyz, max xyz) and NanoVDB leaf-node count. */
NLOD_API int nlod_lod_grid_level_info(const nlod_lod_grid* g, uint32_t level, int32_t* res, int32_t* n_active,
                                      int32_t* bbox6, uint32_t* n_leaves);
/* Device pointer to a level's occupancy bits (owned by the grid). */
NLOD_API const uint32_t* nlod_lod_grid_level_bits(const nlod_lod_grid* g, uint32_t level);
/* Copies a level's occupancy words (ceil(res^3/32) uint32) to host memory.  Synchronous. */
NLOD_API int nlod_lod_grid_copy_bits(const nlod_lod_grid* g, uint32_t level, uint32_t* host_dst);
/* For n index-space rays (origin, dir: [n][3]; t_min: [n] or NULL for 0; prev: [n][3] voxel to skip
 * or NULL for none) writes hit [n] (0/1), ijk [n][3], t_near [n], t_far [n] of the first active
 * voxel of `level` (first_active_voxel_intersection).  Asynchronous. */
NLOD_API int nlod_first_active_voxel(const nlod_lod_grid* g, uint32_t level, void* stream, uint32_t n,
                                     const float* origin, const float* dir, const float* t_min, const int32_t* prev,
                                     int32_t* hit, int32_t* ijk, float* t_near, float* t_far);
/* NLOD_ERR_TIMEOUT if a ray of an earlier search exceeded its step budget (reported as a miss). */
NLOD_API int nlod_lod_grid_sync_status(nlod_lod_grid* g, void* stream);

/* Device status word of the last launch sequence (NLOD_OK or NLOD_ERR_TIMEOUT); synchronises. */
NLOD_API int nlod_sync_status(nlod_module* m, void* stream);

/* ---- Conservative surface voxelization --------------------------------------------------------
 * The reference's cuda_voxelizer (run as `cuda_voxelizer -f mesh -s G -o obj_points -pad` by
 * results/scripts/voxelize.py:36): main.cpp:204-257 takes the trimesh bbox, cubes and pads it with
 * createMeshBBCube (util.h:87-112, epsilonPadding 1e-4, main.cpp:45) and launches voxelize_triangle
 * (voxelize.cu:58-190), which ORs bit x + y*G + z*G^2 (most significant bit first per uint32,
 * setBit voxelize.cu:50-55) for every voxel whose closed box overlaps a triangle.  Triangles are a
 * soup of n x 9 floats (v0 v1 v2, xyz each), like meshToGPU_thrust's buffer. */

/* Per-axis min / max of all vertices of n device triangles (trimesh's need_bbox). Synchronous. */
NLOD_API int nlod_mesh_bounds(const float* triangles, uint64_t n_triangles, void* stream, float mesh_min[3],
                              float mesh_max[3]);
/* createMeshBBCube + voxinfo on the host: the cube frame around [mesh_min, mesh_max] padded by
 * epsilon_padding * extent per side (0 for none), and the voxel size (bbox_max - bbox_min) / grid. */
NLOD_API int nlod_mesh_frame(const float mesh_min[3], const float mesh_max[3], uint32_t grid, float epsilon_padding,
                             float bbox_min[3], float bbox_max[3], float unit[3]);
/* ORs the conservative surface voxelization of n device triangles into `bits` (device,
 * ceil(grid^3 / 32) uint32 words, zeroed by the caller for a fresh grid); grid <= 4096.  The
 * voxel set equals voxelize_triangle's evaluated in IEEE single precision without contraction.
 * Asynchronous on `stream`. */
NLOD_API int nlod_voxelize(const float* triangles, uint64_t n_triangles, uint32_t grid, const float bbox_min[3],
                           const float unit[3], uint32_t* bits, void* stream);

/* ---- Wavefront render query ---------------------------------------------------------------------
 * Pinhole rays through one level of the LoD pyramid: every occupied voxel a ray enters is one
 * visibility query; an accepted voxel (visibility >= threshold) is one throughput query and a
 * bounce in a uniformly sampled direction; rays that leave the grid take the background (before
 * any bounce) or throughput x environment radiance.  This is the reference's wavefront loop
 * (rptr/cuda/neural-lod/wavefront_neural_throughput_visibility_lod.cu:470-720 with the per-ray
 * steps of rptr/cuda/wavefront_neural_pt.cuh: raymarch_impl, generate_*_inference_data_impl,
 * check_visibility, process_ray_bounce) without the host round trip per wavefront.  A frame is one
 * CUDA-graph launch, in one of two forms: the persistent form (tensor-core modules) is one kernel
 * whose tile pipelines refill their ray slots from a queue and run both networks on full tiles;
 * the wavefront form advances every ray by rounds (one round: a chain of visibility queries marched
 * ahead, or a throughput query), the rounds running in a conditional while node.  Both forms give
 * the same pixels and query counts.
 * Network inputs: visibility = (voxel-local entry point in [0,1]^3, (dir + 1) / 2) with
 * lod_max_level as the grid's max level; throughput = (voxel centre / res, (wi + 1) / 2,
 * (wo + 1) / 2, lod_input), wo = -dir.  Camera and radiance parameters are the renderer's. */
typedef struct nlod_renderer nlod_renderer;
typedef struct nlod_render_params {
    uint32_t width, height;        /* pixels (one ray per pixel) */
    uint32_t level;                /* pyramid level the rays traverse */
    uint32_t max_depth;            /* path vertices; a hit on the last one ends the path dark (reference: 4) */
    uint32_t max_vis_queries;      /* visibility queries per ray and bounce before the path is dropped */
    float threshold;               /* visibility >= threshold accepts the voxel */
    float eye[3], target[3], up[3];  /* camera in the grid's normalised coordinates [0,1]^3 */
    float fov_y_deg;
    float background[3];           /* radiance of rays that escape before the first bounce */
    float env_color[3];            /* radiance (times throughput) of rays that escape after one */
    float lod_max_level;           /* visibility network's max grid level fraction for this LoD */
    float lod_input;               /* throughput network's LoD input column for this LoD */
    uint64_t seed;                 /* direction sampling */
    uint32_t mode;                 /* NLOD_RENDER_AUTO: when both modules are tensor-core modules of one
                                      operand type, the faster of the persistent kernel (organisation
                                      autotuned) and the wavefront rounds, timed on this scene at
                                      creation; else the wavefront rounds.
                                      NLOD_RENDER_WAVEFRONT / NLOD_RENDER_PERSISTENT force one form;
                                      NLOD_RENDER_HOST_ROUNDS issues the wavefront rounds from the host.
                                      The wavefront form (AUTO, WAVEFRONT) also picks its modules'
                                      inference kernel organisations for this frame by timing frames
                                      at creation; the modules' own settings are unchanged */
    uint32_t max_chain;            /* wavefront forms: most visibility queries a ray marches ahead in one
                                      round (query k+1 is the march that follows query k's rejection; the
                                      queries past an accepted one are dropped, so pixels and counts do not
                                      depend on it).  Each round's chain length is the longest power of two
                                      up to this cap whose expected dropped queries stay near 3 %, from the
                                      last round's accepted fraction.  0: 8; at most 64; the cap also keeps
                                      the visibility rows within 2^23 (one query per round beyond that) */
} nlod_render_params;

#define NLOD_RENDER_AUTO 0
#define NLOD_RENDER_WAVEFRONT 1
#define NLOD_RENDER_PERSISTENT 2
/* The wavefront rounds issued one by one from the host, which reads the list sizes after every
 * round (the reference's wavefront loop synchronises with the host the same way): the same
 * kernels and pixels as NLOD_RENDER_WAVEFRONT, without the graph, so that a profiler sees every
 * launch.  nlod_render_frame then synchronises the stream. */
#define NLOD_RENDER_HOST_ROUNDS 3
/* The persistent form with one organisation forced instead of autotuned (tests and tuning):
 * f = 4 or 6 tile pipelines per CTA that march their own rays, or f = 8 or 16 marcher warps
 * feeding two tensor-core groups (warp-specialized). */
#define NLOD_RENDER_PERSISTENT_FORM(f) (0x100 | (f))

/* Index-space camera of a level with res voxels per axis: eye[3], right[3] (scaled by
 * tan(fov/2) * aspect), up[3] (scaled by tan(fov/2)), forward[3].  Host only. */
NLOD_API int nlod_render_camera(const nlod_render_params* p, uint32_t level_res, float* out12);
/* Builds the frame graph (allocates the ray state and query buffers); the modules and the grid
 * must outlive the renderer.  Synchronous.  NLOD_ERR_UNSUPPORTED when mode is
 * NLOD_RENDER_PERSISTENT and the modules cannot run the persistent form. */
NLOD_API int nlod_renderer_create(nlod_module* visibility, nlod_module* throughput, const nlod_lod_grid* grid,
                                  const nlod_render_params* p, nlod_renderer** out);
NLOD_API void nlod_renderer_destroy(nlod_renderer* r);
/* Renders one frame: image [height][width][3] FP32 device (NULL to skip the copy), ray_stats
 * [height*width][2] visibility / throughput queries per ray (NULL to skip).  Asynchronous. */
NLOD_API int nlod_render_frame(nlod_renderer* r, void* stream, float* image, uint32_t* ray_stats);
/* Totals of the last frame: visibility queries, throughput queries, rounds (persistent form: the
 * most tile iterations of one pipeline), rays dropped at the per-bounce cap.  Synchronises;
 * NLOD_ERR_TIMEOUT if a ray ran out of DDA steps, the frame hit its round or time bound, or a
 * tensor-core wait timed out. */
NLOD_API int nlod_render_stats(nlod_renderer* r, void* stream, uint64_t* out4);
/* The form the renderer runs: NLOD_RENDER_WAVEFRONT, NLOD_RENDER_HOST_ROUNDS, or
 * NLOD_RENDER_PERSISTENT_FORM(f) with the persistent organisation the autotune (or the caller)
 * chose. */
NLOD_API int nlod_renderer_mode(const nlod_renderer* r);

/* ---- Per-voxel visibility thresholds ----------------------------------------------------------
 * optimise_thresholds_for_voxel_grid (rptr/cuda/neural-lod/neural_lod_learning.cu:122-293, metrics
 * neural_lod_learning_common.cuh:836-927): for each voxel, the thresholds k/100 (k = 0..100) are
 * scored on its samples (reference 0/1, probability p, occluded when p > t) with the chosen metric,
 * and the middle of the run of best scores (equal within 1e-4) is kept.  Samples of voxel v are
 * entries [v * n_samples, (v + 1) * n_samples) of truth / proba (device); thresholds: [n_voxels]
 * device floats, the reference's optimal_thresholds/<lod>.bin contents.  Asynchronous. */
#define NLOD_METRIC_PRECISION               0
#define NLOD_METRIC_RECALL                  1
#define NLOD_METRIC_FSCORE                  2
#define NLOD_METRIC_FSCORE_MACRO            3
#define NLOD_METRIC_FSCORE_WEIGHTED         4
#define NLOD_METRIC_OPTIMAL_FSCORE_WEIGHTED 5   /* the reference's default */
#define NLOD_METRIC_MCC                     6
#define NLOD_METRIC_COHEN_KAPPA             7
#define NLOD_METRIC_ACCURACY                8
#define NLOD_METRIC_BALANCED_ACCURACY       9
#define NLOD_METRIC_FOWLKES_MALLOWS         10
#define NLOD_METRIC_YOUDEN_J                11
NLOD_API int nlod_optimal_thresholds(const float* truth, const float* proba, uint32_t n_samples, uint32_t n_voxels, int metric,
                                     float beta, float* thresholds, void* stream);

/* ---- Training-sample generation ---------------------------------------------------------------
 * The reference's sampler (rptr/cuda/neural-lod/neural_lod_learning_kernels.cuh:29-238, 364-569)
 * on the GPU, with exact-DDA stand-ins for its Vulkan ray queries (rptr/vulkan/raygen.rgen:
 * 505-730).  All buffers are device memory; all calls are asynchronous on `stream` and need no
 * host synchronisation between them (counts stay in device memory). */

/* RenderRayQuery (rptr/librender/render_params.glsl.h:165-172), same layout (48 bytes). */
typedef struct nlod_ray_query {
    float origin[3];
    int32_t mode_or_data;    /* throughput: path orders (max_throughput_depth); visibility: 0 */
    float dir[3];
    float t_max;             /* 1e20; -1 marks a sample whose rejection loops ran out */
    float voxel_center[3];
    float voxel_extent;      /* edge of the query box: voxel edge * (1 + max(dilation, bound_bias)) */
} nlod_ray_query;

/* Sampler settings (NeuralLodLearning::Params, rptr/cuda/neural-lod/neural_lod_learning.h:120-214;
 * reference defaults: dilation_outward 0.005, dilation_inward 0, min_dilation 1e-4, bound_bias 0,
 * pdf_strength 0, pdf_shift 0, increase_boundary_density 0, n_lods 7, grid_res 512). */
typedef struct nlod_sampler_params {
    float aabb_min[3];           /* voxel-grid AABB in world space */
    float aabb_max[3];
    float voxel_size;            /* level-0 voxel edge */
    uint32_t grid_res;           /* level-0 voxels per axis */
    uint32_t n_lods;             /* LoDs sampled, 1..16 */
    float dilation_outward;
    float dilation_inward;
    float min_dilation;
    float bound_bias;
    float pdf_strength;          /* shifted_square_pdf slope */
    float pdf_shift;             /* shifted_square_pdf shift */
    int32_t increase_boundary_density;
    uint32_t max_attempts;       /* bound of every rejection loop (the reference's are unbounded), > 0 */
} nlod_sampler_params;

/* Sorted Morton codes (encode_morton3, 10 bits per axis) of the set voxels of a res^3 bit grid
 * (bit x + y*res + z*res^2, most significant bit first; res a power of two <= 1024): the
 * reference's morton_sparse_voxel_idx_mapping (neural_lod_learning_init.cu:201-294).  Writes the
 * number of set voxels to *count (device) and the first `capacity` codes to `codes` (NULL: count
 * only). */
NLOD_API int nlod_morton_voxels(const uint32_t* bits, uint32_t res, uint32_t* codes, uint32_t capacity, uint32_t* count,
                                void* stream);

/* fill_ray_queries_visibility (kernels.cuh:364-569): sample i draws from the LCG stream
 * (batch_index * n, 0, i): a level-0 voxel of `morton` (*n_voxels codes, device count) and a LoD
 * (shifted_square_pdf), a direction wi, the dilation of the cube and a chord of it by rejection
 * sampling, ordered into (pi, po) by cube face.  input [n][6]: pi, po normalised to the AABB;
 * queries [n] (nullable): ray from pi towards po; lod [n] (nullable). */
NLOD_API int nlod_sample_visibility(const nlod_sampler_params* p, const uint32_t* morton, const uint32_t* n_voxels,
                                    uint32_t batch_index, uint32_t n, float* input, nlod_ray_query* queries, uint32_t* lod,
                                    void* stream);
/* The threshold-optimisation mode of the same kernel (kernels.cuh:392-413): n_samples samples for
 * each of voxels first_voxel .. first_voxel + n_voxels - 1 of a LoD's own sorted mapping
 * (nlod_morton_voxels of that pyramid level); sample s of voxel v is entry s + v * n_samples and
 * draws from the stream (first_voxel + v, 0, s). */
NLOD_API int nlod_sample_visibility_voxels(const nlod_sampler_params* p, const uint32_t* lod_morton, uint32_t first_voxel,
                                           uint32_t n_voxels, uint32_t n_samples, uint32_t lod, float* input,
                                           nlod_ray_query* queries, void* stream);
/* fill_ray_queries_throughput (kernels.cuh:100-238): voxel and LoD as above, wo uniform on the
 * sphere, the entry point of a rejection-sampled ray of direction -wo into the dilated cube.
 * input [n][9]: voxel centre normalised to the AABB, (wo + 1) / 2, then wi (written by
 * nlod_trace_throughput). */
NLOD_API int nlod_sample_throughput(const nlod_sampler_params* p, const uint32_t* morton, const uint32_t* n_voxels,
                                    uint32_t batch_index, uint32_t n, int32_t max_orders, float* input, nlod_ray_query* queries,
                                    uint32_t* lod, void* stream);

/* Visibility targets (main_visibility_optimisation, raygen.rgen:695-730, against the voxelized
 * scene): 1 when the query ray's first occupied level-0 voxel of `g` begins inside the query box,
 * else 0; -1 for an invalid query.  target [n]. */
NLOD_API int nlod_trace_visibility(const nlod_lod_grid* g, const nlod_sampler_params* p, const nlod_ray_query* queries, uint32_t n,
                                   float* target, void* stream);
/* Throughput targets (stand-in for the path-traced ray query, raygen.rgen:505-687, and
 * record_ray_query_results_throughput_optim, kernels.cuh:240-278): the query ray must meet an
 * occupied level-0 voxel inside the box, else every input and target of the sample is -1 and
 * *n_invalid (device, nullable) counts it; wi is uniform on the sphere (LCG stream
 * (batch_index * n, 1, i)), input[6..8] = (wi + 1) / 2 and target = the voxel's albedo if the ray
 * from the hit point along wi leaves the box without meeting another occupied voxel, else 0
 * (log(1 + target) when log_learning).  target [n][3]. */
NLOD_API int nlod_trace_throughput(const nlod_lod_grid* g, const nlod_sampler_params* p, const nlod_ray_query* queries, uint32_t n,
                                   uint32_t batch_index, int log_learning, float* input, float* target, uint32_t* n_invalid,
                                   void* stream);
/* copy_valid_results_throughput_optim (kernels.cuh:280-318): the samples whose first target value
 * is not -1, in index order, at most next_multiple(count, 128) - 128 of them (the reference's
 * training-batch rule); the number kept goes to *n_valid (device). */
NLOD_API int nlod_compact_samples(const float* input, const float* target, uint32_t n, uint32_t n_in, uint32_t n_out,
                                  float* valid_input, float* valid_target, uint32_t* n_valid, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* NLOD_H */
