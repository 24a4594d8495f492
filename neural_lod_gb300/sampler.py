"""Training-sample generation on the GPU (host-side mirror of the nlod_sample_* / nlod_trace_* C ABI).

The reference draws its training samples with fill_ray_queries_visibility / _throughput
(rptr/cuda/neural-lod/neural_lod_learning_kernels.cuh:100-238, 364-569) and labels them with
Vulkan ray queries (rptr/vulkan/raygen.rgen:505-730).  Here the same sampler runs on the GPU and
the labels come from exact DDA against the voxelized scene (the LoD pyramid's level 0):

    sp = Sampler(grid, aabb_min=(0, 0, 0), aabb_max=(1, 1, 1))    # grid: LodGrid
    x, queries, lod = sp.sample_visibility(batch_index, n)         # x: [n, 6] (pi, po)
    y = sp.trace_visibility(queries)                               # [n, 1] occlusion 0/1
    x, queries, lod = sp.sample_throughput(batch_index, n)         # x: [n, 9] (centre, wo, wi)
    y, n_invalid = sp.trace_throughput(queries, x, batch_index)    # [n, 3], invalid rows -1
    xv, yv, n_valid = sp.compact(x, y)                             # training batch (multiple of 128)

Everything stays on the device; counts are device tensors.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from ._lib import check, load

# nlod_ray_query (48 bytes)
RAY_QUERY_DTYPE = np.dtype([("origin", "<f4", (3,)), ("mode_or_data", "<i4"), ("dir", "<f4", (3,)), ("t_max", "<f4"),
                            ("voxel_center", "<f4", (3,)), ("voxel_extent", "<f4")])


class SamplerParamsC(C.Structure):
    """nlod_sampler_params."""
    _fields_ = [("aabb_min", C.c_float * 3), ("aabb_max", C.c_float * 3), ("voxel_size", C.c_float), ("grid_res", C.c_uint32),
                ("n_lods", C.c_uint32), ("dilation_outward", C.c_float), ("dilation_inward", C.c_float),
                ("min_dilation", C.c_float), ("bound_bias", C.c_float), ("pdf_strength", C.c_float), ("pdf_shift", C.c_float),
                ("increase_boundary_density", C.c_int32), ("max_attempts", C.c_uint32)]


@dataclass
class SamplerParams:
    """Sampler settings; defaults are the reference's (NeuralLodLearning::Params,
    rptr/cuda/neural-lod/neural_lod_learning.h:120-214), except max_attempts, the bound this
    implementation puts on each rejection loop."""
    aabb_min: tuple = (0.0, 0.0, 0.0)
    aabb_max: tuple = (1.0, 1.0, 1.0)
    grid_res: int = 512
    n_lods: int = 7
    voxel_size: float | None = None        # default: AABB x extent / grid_res
    dilation_outward: float = 0.005
    dilation_inward: float = 0.0
    min_dilation: float = 1e-4
    bound_bias: float = 0.0
    pdf_strength: float = 0.0
    pdf_shift: float = 0.0
    increase_boundary_density: bool = False
    max_attempts: int = 256

    def to_c(self) -> SamplerParamsC:
        c = SamplerParamsC()
        c.aabb_min[:] = [float(v) for v in self.aabb_min]
        c.aabb_max[:] = [float(v) for v in self.aabb_max]
        vs = self.voxel_size
        if vs is None:
            vs = float(np.float32(np.float32(self.aabb_max[0]) - np.float32(self.aabb_min[0])) / np.float32(self.grid_res))
        c.voxel_size = vs
        c.grid_res = self.grid_res
        c.n_lods = self.n_lods
        c.dilation_outward = self.dilation_outward
        c.dilation_inward = self.dilation_inward
        c.min_dilation = self.min_dilation
        c.bound_bias = self.bound_bias
        c.pdf_strength = self.pdf_strength
        c.pdf_shift = self.pdf_shift
        c.increase_boundary_density = int(bool(self.increase_boundary_density))
        c.max_attempts = self.max_attempts
        return c


def _stream(stream):
    import torch

    if stream is None:
        return torch.cuda.current_stream().cuda_stream or None
    return stream if isinstance(stream, int) else (stream.cuda_stream or None)


def morton_voxels(bits, res: int, stream=None):
    """Sorted Morton codes of the set voxels of a res^3 bit grid (cuda int32 words): (codes [count]
    int32 tensor, count [1] int32 tensor).  Reads the count back once to size the output."""
    import torch

    lib = load()
    count = torch.zeros(1, dtype=torch.int32, device=bits.device)
    s = _stream(stream)
    check(lib.nlod_morton_voxels(bits.data_ptr(), int(res), None, 0, count.data_ptr(), s))
    n = int(count.item())
    codes = torch.empty(max(n, 1), dtype=torch.int32, device=bits.device)
    check(lib.nlod_morton_voxels(bits.data_ptr(), int(res), codes.data_ptr(), n, count.data_ptr(), s))
    return codes[:n], count


class Sampler:
    """The reference's training-sample generator over a LodGrid (level 0 = the voxelized scene)."""

    def __init__(self, grid, params: SamplerParams | None = None, **kw):
        import torch

        self._lib = load()
        self.grid = grid
        self.params = params or SamplerParams(grid_res=grid.res, **kw)
        if self.params.grid_res != grid.res:
            raise ValueError("params.grid_res must equal the grid's level-0 resolution")
        self._c = self.params.to_c()
        bits0 = torch.from_numpy(grid.level_bits(0).view(np.int32)).cuda()
        self.morton, self.count = morton_voxels(bits0, grid.res)
        self._lod_morton = {}

    def lod_morton(self, lod: int):
        """Sorted Morton codes of the occupied voxels of pyramid level `lod` (the reference's
        morton_sparse_voxel_idx_mappings[lod])."""
        import torch

        if lod not in self._lod_morton:
            bits = torch.from_numpy(self.grid.level_bits(lod).view(np.int32)).cuda()
            self._lod_morton[lod] = morton_voxels(bits, self.grid.res >> lod)
        return self._lod_morton[lod]

    def sample_visibility(self, batch_index: int, n: int, stream=None):
        import torch

        x = torch.empty((n, 6), dtype=torch.float32, device="cuda")
        q = torch.empty((n, 48), dtype=torch.uint8, device="cuda")
        lod = torch.empty(n, dtype=torch.int32, device="cuda")
        check(self._lib.nlod_sample_visibility(C.byref(self._c), self.morton.data_ptr(), self.count.data_ptr(), int(batch_index), n,
                                               x.data_ptr(), q.data_ptr(), lod.data_ptr(), _stream(stream)))
        return x, q, lod

    def sample_visibility_voxels(self, lod: int, first: int, n_voxels: int, n_samples: int, stream=None):
        import torch

        codes, _ = self.lod_morton(lod)
        if first + n_voxels > codes.shape[0]:
            raise ValueError("voxel range beyond the level's occupied voxels")
        n = n_voxels * n_samples
        x = torch.empty((n, 6), dtype=torch.float32, device="cuda")
        q = torch.empty((n, 48), dtype=torch.uint8, device="cuda")
        check(self._lib.nlod_sample_visibility_voxels(C.byref(self._c), codes.data_ptr(), int(first), int(n_voxels), int(n_samples),
                                                      int(lod), x.data_ptr(), q.data_ptr(), _stream(stream)))
        return x, q

    def sample_throughput(self, batch_index: int, n: int, max_orders: int = 1000, stream=None):
        import torch

        x = torch.empty((n, 9), dtype=torch.float32, device="cuda")
        q = torch.empty((n, 48), dtype=torch.uint8, device="cuda")
        lod = torch.empty(n, dtype=torch.int32, device="cuda")
        check(self._lib.nlod_sample_throughput(C.byref(self._c), self.morton.data_ptr(), self.count.data_ptr(), int(batch_index), n,
                                               int(max_orders), x.data_ptr(), q.data_ptr(), lod.data_ptr(), _stream(stream)))
        return x, q, lod

    def trace_visibility(self, queries, stream=None):
        import torch

        n = queries.shape[0]
        y = torch.empty((n, 1), dtype=torch.float32, device="cuda")
        check(self._lib.nlod_trace_visibility(self.grid._g, C.byref(self._c), queries.data_ptr(), n, y.data_ptr(), _stream(stream)))
        return y

    def trace_throughput(self, queries, x, batch_index: int, log_learning: bool = False, stream=None):
        import torch

        n = queries.shape[0]
        y = torch.empty((n, 3), dtype=torch.float32, device="cuda")
        bad = torch.zeros(1, dtype=torch.int32, device="cuda")
        check(self._lib.nlod_trace_throughput(self.grid._g, C.byref(self._c), queries.data_ptr(), n, int(batch_index),
                                              int(bool(log_learning)), x.data_ptr(), y.data_ptr(), bad.data_ptr(), _stream(stream)))
        return y, bad

    def compact(self, x, y, stream=None):
        """Valid samples (first target value not -1) in index order, at most the reference's
        next_multiple(count, 128) - 128: (x_valid, y_valid, n_valid [1] device int32); the first
        n_valid rows are the batch."""
        return compact(x, y, stream)

    def sync_status(self):
        self.grid.sync_status()


def compact(x, y, stream=None):
    import torch

    n, n_in = x.shape
    n_out = y.shape[1]
    xv = torch.empty_like(x)
    yv = torch.empty_like(y)
    nv = torch.zeros(1, dtype=torch.int32, device=x.device)
    check(load().nlod_compact_samples(x.data_ptr(), y.data_ptr(), n, n_in, n_out, xv.data_ptr(), yv.data_ptr(), nv.data_ptr(),
                                      _stream(stream)))
    return xv, yv, nv
