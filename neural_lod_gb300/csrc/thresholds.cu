// Per-voxel visibility threshold optimisation: for every voxel, the 101 thresholds t = k / 100 are
// scored on that voxel's samples (reference value 0/1, network probability p, predicted occluded
// when p > t) and the best-scoring threshold is kept, the middle one of a run of equal scores.
// Restates compute_confusion_matrices, compute_scores and compute_optimal_thresholds
// (rptr/cuda/neural-lod/neural_lod_learning.cu:122-293) and the metric helpers
// (rptr/cuda/neural-lod/neural_lod_learning_common.cuh:836-927).
//
// One CTA per voxel: the voxel's samples are staged in shared memory, thread k counts the
// confusion matrix of threshold k with no atomics (the reference issues one global atomic per
// sample and threshold), scores it, and the argmax runs over shared memory.  This unit is built
// with -fmad=false so that the scores are the uncontracted float expressions of the host
// restatement: the chosen threshold is bit-identical.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>

#include "abi_util.h"
#include "nlod.h"

namespace nlod {
namespace {

constexpr uint32_t kThresholds = 101;
constexpr uint32_t kMaxSamples = 4096;

__device__ __forceinline__ float precision_score(uint32_t fp, uint32_t tp) { return tp == 0 ? 0.f : float(tp) / float(tp + fp); }
__device__ __forceinline__ float recall_score(uint32_t fn, uint32_t tp) { return tp == 0 ? 0.f : float(tp) / float(tp + fn); }
__device__ __forceinline__ float fscore(uint32_t tn, uint32_t fp, uint32_t fn, uint32_t tp, float beta) {
    const float p = precision_score(fp, tp), r = recall_score(fn, tp);
    if (p + r == 0.f) return 0.f;
    const float b2 = beta * beta;
    return ((1.f + b2) * p * r) / (b2 * p + r);
}

__device__ float score(int metric, uint32_t tn, uint32_t fp, uint32_t fn, uint32_t tp, uint32_t sup_pos, uint32_t sup_neg, float beta) {
    switch (metric) {
        case NLOD_METRIC_PRECISION: return precision_score(fp, tp);
        case NLOD_METRIC_RECALL: return recall_score(fn, tp);
        case NLOD_METRIC_FSCORE: return fscore(tn, fp, fn, tp, beta);
        case NLOD_METRIC_FSCORE_MACRO: return (fscore(tn, fp, fn, tp, beta) + fscore(tp, fn, fp, tn, beta)) * 0.5f;
        case NLOD_METRIC_FSCORE_WEIGHTED:
            return (fscore(tn, fp, fn, tp, beta) * sup_pos + fscore(tp, fn, fp, tn, beta) * sup_neg) / (sup_pos + sup_neg);
        case NLOD_METRIC_OPTIMAL_FSCORE_WEIGHTED:
            return (fscore(tn, fp, fn, tp, beta) * sup_pos + fscore(tp, fn, fp, tn, 1.f) * sup_neg) / (sup_pos + sup_neg);
        case NLOD_METRIC_MCC: {
            const float numer = float(tp * tn) - float(fp * fn);
            const float den = float(tp + fp) * float(tp + fn) * float(tn + fp) * float(tn + fn);
            return den == 0 ? 0.f : numer / sqrtf(den);
        }
        case NLOD_METRIC_COHEN_KAPPA: {
            const float numer = 2.f * (float(tp * tn) - float(fn * fp));
            const float den = float(tp + fp) * float(fp + tn) + float(tp + fn) * float(fn + tn);
            return den == 0 ? 0.f : numer / den;
        }
        case NLOD_METRIC_ACCURACY: {
            const float den = float(tp + tn + fp + fn);
            return den == 0 ? 0.f : float(tp + tn) / den;
        }
        case NLOD_METRIC_BALANCED_ACCURACY: {
            const float se = tp == 0 ? 0.0f : float(tp) / float(tp + fn), sp = tn == 0 ? 0.0f : float(tn) / float(tn + fp);
            return (se + sp) * 0.5f;
        }
        case NLOD_METRIC_FOWLKES_MALLOWS: return sqrtf(precision_score(fp, tp) * recall_score(fn, tp));
        case NLOD_METRIC_YOUDEN_J: {
            const float se = tp == 0 ? 0.0f : float(tp) / float(tp + fn), sp = tn == 0 ? 0.0f : float(tn) / float(tn + fp);
            return se + sp - 1.f;
        }
        default: return 0.f;
    }
}

__global__ void __launch_bounds__(128) k_optimal_thresholds(const float* __restrict__ truth, const float* __restrict__ proba,
                                                            uint32_t n_samples, uint32_t n_voxels, int metric, float beta,
                                                            float* __restrict__ out) {
    __shared__ float p_s[kMaxSamples];
    __shared__ uint8_t t_s[kMaxSamples];
    __shared__ float sc[kThresholds];
    const uint32_t v = blockIdx.x;
    if (v >= n_voxels) return;
    const uint32_t k = threadIdx.x;
    for (uint32_t i = k; i < n_samples; i += blockDim.x) {
        p_s[i] = proba[(size_t)v * n_samples + i];
        t_s[i] = truth[(size_t)v * n_samples + i] == 1.0f;
    }
    __syncthreads();
    uint32_t pos = 0;
    for (uint32_t i = 0; i < n_samples; ++i) pos += t_s[i];
    if (k < kThresholds) {
        const float th = k / (float)(kThresholds - 1);
        uint32_t tn = 0, fp = 0, fn = 0, tp = 0;
        for (uint32_t i = 0; i < n_samples; ++i) {
            const bool pred = p_s[i] > th;
            if (!t_s[i]) { if (pred) ++fp; else ++tn; }
            else { if (pred) ++tp; else ++fn; }
        }
        sc[k] = score(metric, tn, fp, fn, tp, pos, n_samples - pos, beta);
    }
    __syncthreads();
    if (k == 0) {
        float best = -10.0f;
        uint32_t opt = 0;
        for (uint32_t t = 0; t < kThresholds; ++t)
            if (sc[t] > best) { best = sc[t]; opt = t; }
        uint32_t eq = 0;
        // the reference compares the float difference with the double 1e-4 (neural_lod_learning.cu:
        // 257); 1e-4f is the largest float below 1e-4, so "<= 1e-4f" is the same test in float
        while (opt + eq < kThresholds && fabsf(sc[opt + eq] - sc[opt]) <= 1e-4f) ++eq;
        opt += eq / 2;
        out[v] = opt / (float)(kThresholds - 1);
    }
}

}  // namespace
}  // namespace nlod

using namespace nlod;

extern "C" int nlod_optimal_thresholds(const float* truth, const float* proba, uint32_t n_samples, uint32_t n_voxels, int metric,
                                       float beta, float* thresholds, void* stream) {
    return guarded([&] {
        if (n_voxels == 0) return;
        if (!truth || !proba || !thresholds) throw Error(NLOD_ERR_INVALID, "buffers must not be NULL");
        if (n_samples == 0 || n_samples > kMaxSamples) throw Error(NLOD_ERR_INVALID, "samples per voxel must be in [1, 4096]");
        if (metric < NLOD_METRIC_PRECISION || metric > NLOD_METRIC_YOUDEN_J) throw Error(NLOD_ERR_INVALID, "unknown metric");
        k_optimal_thresholds<<<n_voxels, 128, 0, (cudaStream_t)stream>>>(truth, proba, n_samples, n_voxels, metric, beta, thresholds);
        cuda_check(cudaGetLastError(), "optimal thresholds");
    });
}
