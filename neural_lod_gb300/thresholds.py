"""Per-voxel visibility thresholds (host-side mirror of nlod_optimal_thresholds) and the
reference's threshold file format (neural_lod/scenes/*/optimal_thresholds/*.bin: one float32 per
sparse voxel of a LoD, in the learner's voxel order, no header)."""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from ._lib import check, load

METRICS = {"precision": 0, "recall": 1, "fscore": 2, "fscore_macro": 3, "fscore_weighted": 4,
           "optimal_fscore_weighted": 5, "mcc": 6, "cohen_kappa": 7, "accuracy": 8, "balanced_accuracy": 9,
           "fowlkes_mallows": 10, "youden_j": 11}


def optimal_thresholds(truth, proba, n_samples: int, metric: str = "optimal_fscore_weighted", beta: float = 1.0, stream=None):
    """truth / proba: cuda float32 tensors of n_voxels * n_samples values (voxel-major).
    Returns the cuda float32 thresholds [n_voxels]."""
    import torch

    n_vox = truth.numel() // n_samples
    out = torch.empty(n_vox, dtype=torch.float32, device=truth.device)
    s = torch.cuda.current_stream().cuda_stream if stream is None else stream
    check(load().nlod_optimal_thresholds(truth.data_ptr(), proba.data_ptr(), int(n_samples), int(n_vox), METRICS[metric],
                                         C.c_float(beta), out.data_ptr(), s or None))
    return out


def save_bin(path, thresholds) -> None:
    np.ascontiguousarray(np.asarray(thresholds, dtype=np.float32)).tofile(Path(path))


def load_bin(path) -> np.ndarray:
    return np.fromfile(Path(path), dtype=np.float32)
