"""Conservative surface voxelization (host-side mirror of the nlod_voxelize C ABI).

    bits = voxelize(triangles, grid=1024)            # triangles: cuda float32 [n, 9] (or [n, 3, 3])

does what `cuda_voxelizer -f mesh -s 1024 -pad` does to a triangle soup (cuda_voxelizer/src/main.cpp:
204-257): mesh bbox, createMeshBBCube with 1e-4 padding, voxelize_triangle; the result is the
MSB-first bit-packed uint32 grid (as int32 words in a cuda tensor) that LodGrid takes as level 0.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import check, load

EPSILON_PADDING = 1e-4   # cuda_voxelizer/src/main.cpp:45


def _stream(stream):
    import torch

    if stream is None:
        return torch.cuda.current_stream().cuda_stream or None
    return stream if isinstance(stream, int) else (stream.cuda_stream or None)


def _tris(triangles):
    import torch

    if not isinstance(triangles, torch.Tensor) or not triangles.is_cuda or triangles.dtype != torch.float32:
        raise TypeError("triangles must be a cuda float32 tensor of shape [n, 9] or [n, 3, 3]")
    t = triangles.reshape(-1, 9)
    return t if t.is_contiguous() else t.contiguous()


def mesh_bounds(triangles, stream=None):
    """Per-axis (min, max) over all vertices, float32[3] each."""
    t = _tris(triangles)
    mn, mx = np.zeros(3, np.float32), np.zeros(3, np.float32)
    check(load().nlod_mesh_bounds(t.data_ptr(), t.shape[0], _stream(stream), mn.ctypes.data, mx.ctypes.data))
    return mn, mx


def mesh_frame(mesh_min, mesh_max, grid: int, epsilon_padding: float = EPSILON_PADDING):
    """createMeshBBCube + voxinfo: (bbox_min, bbox_max, unit), float32[3] each."""
    mn = np.ascontiguousarray(mesh_min, dtype=np.float32)
    mx = np.ascontiguousarray(mesh_max, dtype=np.float32)
    bmin, bmax, unit = (np.zeros(3, np.float32) for _ in range(3))
    check(load().nlod_mesh_frame(mn.ctypes.data, mx.ctypes.data, int(grid), C.c_float(epsilon_padding), bmin.ctypes.data,
                                 bmax.ctypes.data, unit.ctypes.data))
    return bmin, bmax, unit


def n_words(grid: int) -> int:
    return (grid ** 3 + 31) // 32


def voxelize(triangles, grid: int, bbox_min=None, unit=None, epsilon_padding: float = EPSILON_PADDING, out=None, stream=None):
    """Returns the grid^3 occupancy as int32 words (bit x + y*grid + z*grid^2, MSB first).

    Without bbox_min / unit the frame is the padded cube around the mesh bounds.  With `out`
    the voxels are OR-ed into it (no clearing)."""
    import torch

    t = _tris(triangles)
    if bbox_min is None or unit is None:
        mn, mx = mesh_bounds(t, stream)
        bbox_min, _, unit = mesh_frame(mn, mx, grid, epsilon_padding)
    bmin = np.ascontiguousarray(bbox_min, dtype=np.float32)
    u = np.ascontiguousarray(unit, dtype=np.float32)
    if out is None:
        out = torch.zeros(n_words(grid), dtype=torch.int32, device=t.device)
    elif out.numel() < n_words(grid) or out.dtype != torch.int32 or not out.is_contiguous():
        raise ValueError("out must be a contiguous int32 tensor of ceil(grid^3 / 32) words")
    check(load().nlod_voxelize(t.data_ptr(), t.shape[0], int(grid), bmin.ctypes.data, u.ctypes.data, out.data_ptr(),
                               _stream(stream)))
    return out
