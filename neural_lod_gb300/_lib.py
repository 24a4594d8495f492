"""ctypes binding of libnlod.so (include/nlod.h).

The library is built in-tree by neural_lod_gb300.build; loading fails loudly when it is missing
(there is no CPU fallback).
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "libnlod.so"

NLOD_OK = 0
NLOD_ERR_INVALID = 1
NLOD_ERR_CUDA = 2
NLOD_ERR_ALLOC = 3
NLOD_ERR_UNSUPPORTED = 4
NLOD_ERR_TIMEOUT = 5
NLOD_ERR_STATE = 6

PRECISION = {"fp32": 0, "fp16": 1, "bf16": 2}

# (name, restype, argtypes) of every symbol declared in include/nlod.h
_vp = C.c_void_p
_u32 = C.c_uint32
_fp = C.c_void_p  # device/host float pointers are passed as integers
SIGNATURES = [
    ("nlod_last_error", C.c_char_p, []),
    ("nlod_version", C.c_char_p, []),
    ("nlod_module_create", C.c_int, [C.c_char_p, C.c_char_p, C.c_char_p, C.c_char_p, _u32, _u32, C.c_int, C.c_uint64, C.POINTER(_vp)]),
    ("nlod_layout_json", C.c_int, [C.c_char_p, C.c_char_p, _u32, _u32, C.POINTER(C.c_void_p)]),
    ("nlod_module_destroy", None, [_vp]),
    ("nlod_n_params", C.c_size_t, [_vp]),
    ("nlod_n_network_params", C.c_size_t, [_vp]),
    ("nlod_n_input_dims", _u32, [_vp]),
    ("nlod_n_output_dims", _u32, [_vp]),
    ("nlod_encoded_width", _u32, [_vp]),
    ("nlod_padded_output_width", _u32, [_vp]),
    ("nlod_precision", C.c_int, [_vp]),
    ("nlod_set_max_level_gpu", C.c_int, [_vp, _fp]),
    ("nlod_set_max_level", C.c_int, [_vp, C.c_float]),
    ("nlod_inference", C.c_int, [_vp, _vp, _u32, _fp, _fp]),
    ("nlod_inference_host", C.c_int, [_vp, _vp, _u32, _fp, _fp]),
    ("nlod_forward", C.c_int, [_vp, _vp, _u32, _fp, _fp, C.POINTER(_vp)]),
    ("nlod_backward", C.c_int, [_vp, _vp, _vp, _fp, _fp]),
    ("nlod_ctx_destroy", None, [_vp]),
    ("nlod_training_step", C.c_int, [_vp, _vp, _u32, _fp, _fp, _fp]),
    ("nlod_forward_backward_loss", C.c_int, [_vp, _vp, _u32, _fp, _fp, _fp]),
    ("nlod_training_step_noalloc", C.c_int, [_vp, _vp, _u32, _fp, _fp, _fp]),
    ("nlod_optimizer_step", C.c_int, [_vp, _vp]),
    ("nlod_optimizer_step_count", _u32, [_vp]),
    ("nlod_learning_rate", C.c_float, [_vp]),
    ("nlod_set_learning_rate", C.c_int, [_vp, C.c_float]),
    ("nlod_set_params", C.c_int, [_vp, _fp, C.c_size_t, C.c_int]),
    ("nlod_get_params", C.c_int, [_vp, _fp, C.c_size_t, C.c_int, C.c_int]),
    ("nlod_serialize", C.c_int, [_vp, C.c_int, C.POINTER(C.c_void_p)]),
    ("nlod_deserialize", C.c_int, [_vp, C.c_char_p]),
    ("nlod_free_string", None, [C.c_void_p]),
    ("nlod_kernel_variants", C.c_int, [_vp]),
    ("nlod_get_kernel_variant", C.c_int, [_vp]),
    ("nlod_set_kernel_variant", C.c_int, [_vp, C.c_int]),
    ("nlod_autotune", C.c_int, [_vp, _vp, _u32, _fp, _fp]),
    ("nlod_calib_gathers", C.c_int, [_vp, _vp, _u32, C.POINTER(C.c_float)]),
    ("nlod_calib_scatter", C.c_int, [_vp, _vp, _u32, C.POINTER(C.c_float)]),
    ("nlod_sync_status", C.c_int, [_vp, _vp]),
    ("nlod_lod_grid_create", C.c_int, [_fp, _u32, _u32, _vp, C.POINTER(_vp)]),
    ("nlod_lod_grid_destroy", None, [_vp]),
    ("nlod_lod_grid_level_info", C.c_int, [_vp, _u32, _fp, _fp, _fp, _fp]),
    ("nlod_lod_grid_level_bits", C.c_void_p, [_vp, _u32]),
    ("nlod_lod_grid_copy_bits", C.c_int, [_vp, _u32, _fp]),
    ("nlod_first_active_voxel", C.c_int, [_vp, _u32, _vp, _u32, _fp, _fp, _fp, _fp, _fp, _fp, _fp, _fp]),
    ("nlod_lod_grid_sync_status", C.c_int, [_vp, _vp]),
    ("nlod_mesh_bounds", C.c_int, [_fp, C.c_uint64, _vp, _fp, _fp]),
    ("nlod_mesh_frame", C.c_int, [_fp, _fp, _u32, C.c_float, _fp, _fp, _fp]),
    ("nlod_voxelize", C.c_int, [_fp, C.c_uint64, _u32, _fp, _fp, _fp, _vp]),
    ("nlod_render_camera", C.c_int, [_vp, _u32, _fp]),
    ("nlod_renderer_create", C.c_int, [_vp, _vp, _vp, _vp, C.POINTER(_vp)]),
    ("nlod_renderer_destroy", None, [_vp]),
    ("nlod_render_frame", C.c_int, [_vp, _vp, _fp, _fp]),
    ("nlod_render_stats", C.c_int, [_vp, _vp, _fp]),
    ("nlod_renderer_mode", C.c_int, [_vp]),
    ("nlod_optimal_thresholds", C.c_int, [_fp, _fp, _u32, _u32, C.c_int, C.c_float, _fp, _vp]),
    ("nlod_morton_voxels", C.c_int, [_fp, _u32, _fp, _u32, _fp, _vp]),
    ("nlod_sample_visibility", C.c_int, [_vp, _fp, _fp, _u32, _u32, _fp, _fp, _fp, _vp]),
    ("nlod_sample_visibility_voxels", C.c_int, [_vp, _fp, _u32, _u32, _u32, _u32, _fp, _fp, _vp]),
    ("nlod_sample_throughput", C.c_int, [_vp, _fp, _fp, _u32, _u32, C.c_int32, _fp, _fp, _fp, _vp]),
    ("nlod_trace_visibility", C.c_int, [_vp, _vp, _fp, _u32, _fp, _vp]),
    ("nlod_trace_throughput", C.c_int, [_vp, _vp, _fp, _u32, _u32, C.c_int, _fp, _fp, _fp, _vp]),
    ("nlod_compact_samples", C.c_int, [_fp, _fp, _u32, _u32, _u32, _fp, _fp, _fp, _vp]),
]

_lib = None


class NlodError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"[nlod status {code}] {message}")
        self.code = code


def load(path: str | os.PathLike | None = None) -> C.CDLL:
    """Loads libnlod.so and declares every entry point; raises if the library is missing."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise FileNotFoundError(
            f"{p} is missing: build it with `python -m neural_lod_gb300.build` (no CPU fallback exists)")
    lib = C.CDLL(str(p))
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def check(code: int) -> None:
    if code != NLOD_OK:
        msg = load().nlod_last_error()
        raise NlodError(code, msg.decode() if msg else "")
