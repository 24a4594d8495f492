"""ctypes binding of the reference voxelizer kernel (oracle/_ref/libvoxref_{fma,nofma}-<arch>.so,
built by oracle/build_ref.py from the staged cuda_voxelizer sources) -- TEST INFRASTRUCTURE ONLY.
Device buffers are torch CUDA tensors."""
from __future__ import annotations

import ctypes as C

import numpy as np

from .build_ref import VOXREF, build_voxelizer_ref, voxelizer_staged

_libs: dict = {}


def available() -> bool:
    return voxelizer_staged() or all(p.exists() for p in VOXREF.values())


def _lib(kind: str):
    if kind not in _libs:
        if voxelizer_staged():
            build_voxelizer_ref()
        lib = C.CDLL(str(VOXREF[kind]))
        lib.vref_voxelize.argtypes = [C.c_void_p, C.c_uint64, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        lib.vref_voxelize.restype = C.c_int
        lib.vref_unit.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p]
        lib.vref_unit.restype = None
        _libs[kind] = lib
    return _libs[kind]


def unit(bbox_min, bbox_max, grid: int, kind: str = "fma") -> np.ndarray:
    mn = np.ascontiguousarray(bbox_min, np.float32)
    mx = np.ascontiguousarray(bbox_max, np.float32)
    u = np.zeros(3, np.float32)
    _lib(kind).vref_unit(mn.ctypes.data, mx.ctypes.data, grid, u.ctypes.data)
    return u


def voxelize(triangles, grid: int, bbox_min, bbox_max, kind: str = "fma"):
    """cuda_voxelizer's voxelize_triangle over triangles (cuda float32 [n, 9]) into a fresh
    grid^3-bit table (cuda int32 words); kind "fma" (nvcc's default contraction, the reference's
    build) or "nofma" (-fmad=false)."""
    import torch

    t = triangles.reshape(-1, 9).contiguous()
    out = torch.zeros((grid ** 3 + 31) // 32, dtype=torch.int32, device=t.device)
    mn = np.ascontiguousarray(bbox_min, np.float32)
    mx = np.ascontiguousarray(bbox_max, np.float32)
    rc = _lib(kind).vref_voxelize(t.data_ptr(), t.shape[0], grid, mn.ctypes.data, mx.ctypes.data, out.data_ptr(),
                                  torch.cuda.current_stream().cuda_stream or None)
    if rc != 0:
        raise RuntimeError(f"reference voxelizer launch failed: cudaError {rc}")
    return out
