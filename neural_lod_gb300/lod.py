"""LoD occupancy pyramid and first-active-voxel search (host-side mirror of the nlod_lod_grid C ABI).

    grid = LodGrid(bits0, res=512, n_levels=8)          # bits0: cuda uint32 words (or numpy)
    hit, ijk, t_near, t_far = grid.first_active_voxel(lod, origin, dir, t_min, prev)

The search is the reference's first_active_voxel_intersection over its NanoVDB LoD grids
(rptr/cuda/neural-lod/neural_lod_learning_common.cuh:783-832) on index-space rays.
"""
from __future__ import annotations

import ctypes as C

from ._lib import check, load


def _ptr(t):
    return None if t is None else t.data_ptr()


def _stream(stream):
    import torch

    if stream is None:
        return torch.cuda.current_stream().cuda_stream or None
    return stream if isinstance(stream, int) else (stream.cuda_stream or None)


class LodGrid:
    def __init__(self, bits0, res: int, n_levels: int, stream=None):
        import numpy as np
        import torch

        self._lib = load()
        if not isinstance(bits0, torch.Tensor):
            bits0 = torch.from_numpy(np.ascontiguousarray(np.asarray(bits0, dtype=np.uint32)).view(np.int32)).cuda()
        self._bits0 = bits0
        self._g = C.c_void_p()
        check(self._lib.nlod_lod_grid_create(bits0.data_ptr(), int(res), int(n_levels), _stream(stream), C.byref(self._g)))
        self.res = int(res)
        self.n_levels = int(n_levels)

    def level_info(self, level: int) -> dict:
        r, na, nl = C.c_int32(), C.c_int32(), C.c_uint32()
        bb = (C.c_int32 * 6)()
        check(self._lib.nlod_lod_grid_level_info(self._g, int(level), C.addressof(r), C.addressof(na), C.addressof(bb), C.addressof(nl)))
        return {"res": r.value, "n_active": na.value, "bbox_min": tuple(bb[:3]), "bbox_max": tuple(bb[3:]), "n_leaves": nl.value}

    def level_bits(self, level: int):
        """Host copy (numpy uint32) of a level's occupancy words."""
        import numpy as np

        r = self.res >> level
        out = np.empty((r ** 3 + 31) // 32, dtype=np.uint32)
        check(self._lib.nlod_lod_grid_copy_bits(self._g, int(level), out.ctypes.data))
        return out

    def first_active_voxel(self, level: int, origin, dir, t_min=None, prev=None, stream=None):
        import torch

        n = origin.shape[0]
        dev = origin.device
        hit = torch.empty(n, dtype=torch.int32, device=dev)
        ijk = torch.empty((n, 3), dtype=torch.int32, device=dev)
        tn = torch.empty(n, dtype=torch.float32, device=dev)
        tf = torch.empty(n, dtype=torch.float32, device=dev)
        check(self._lib.nlod_first_active_voxel(self._g, int(level), _stream(stream), n, _ptr(origin), _ptr(dir), _ptr(t_min),
                                                _ptr(prev), _ptr(hit), _ptr(ijk), _ptr(tn), _ptr(tf)))
        return hit, ijk, tn, tf

    def sync_status(self, stream=None) -> None:
        check(self._lib.nlod_lod_grid_sync_status(self._g, _stream(stream)))

    def close(self):
        if getattr(self, "_g", None) is not None and self._g.value:
            self._lib.nlod_lod_grid_destroy(self._g)
            self._g = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
