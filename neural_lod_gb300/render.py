"""Neural-LoD render query (host-side mirror of the nlod_renderer C ABI).

    r = Renderer(visibility_module, throughput_module, lod_grid, RenderParams(width=1024, height=1024, level=3))
    image = r.frame()                      # cuda float32 [height, width, 3]
    vis_q, thr_q, rounds, dropped = r.stats()

A frame is one CUDA-graph launch with no host round trip per wavefront (unlike the reference's
voxel_tracing loop in rptr/cuda/neural-lod/wavefront_neural_throughput_visibility_lod.cu:470-720),
in one of two forms that give the same pixels: one persistent kernel whose tile pipelines refill
their ray slots from a queue, or rounds in a conditional while node in which every ray advances
one query (MODE_WAVEFRONT, and the FP32 modules).  MODE_AUTO times both on the scene at creation
and keeps the faster.  MODE_HOST_ROUNDS issues the wavefront rounds from the host, as the reference
does (same pixels; every launch visible to a profiler).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

from ._lib import check, load


class _Params(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("level", C.c_uint32), ("max_depth", C.c_uint32),
                ("max_vis_queries", C.c_uint32), ("threshold", C.c_float), ("eye", C.c_float * 3), ("target", C.c_float * 3),
                ("up", C.c_float * 3), ("fov_y_deg", C.c_float), ("background", C.c_float * 3), ("env_color", C.c_float * 3),
                ("lod_max_level", C.c_float), ("lod_input", C.c_float), ("seed", C.c_uint64), ("mode", C.c_uint32),
                ("max_chain", C.c_uint32)]

MODE_AUTO, MODE_WAVEFRONT, MODE_PERSISTENT, MODE_HOST_ROUNDS = 0, 1, 2, 3     # NLOD_RENDER_*


def persistent_form(f: int) -> int:
    """NLOD_RENDER_PERSISTENT_FORM(f): f = 4 / 6 tile pipelines, 8 / 16 marcher warps."""
    return 0x100 | f


@dataclass
class RenderParams:
    width: int = 1024
    height: int = 1024
    level: int = 3
    max_depth: int = 4
    max_vis_queries: int = 64
    threshold: float = 0.5
    eye: tuple = (1.6, 1.25, 1.9)
    target: tuple = (0.5, 0.5, 0.5)
    up: tuple = (0.0, 1.0, 0.0)
    fov_y_deg: float = 40.0
    background: tuple = (0.05, 0.07, 0.10)
    env_color: tuple = (1.0, 0.95, 0.9)
    lod_max_level: float = 1000.0
    lod_input: float = 0.0
    seed: int = 1337
    mode: int = MODE_AUTO
    max_chain: int = 0      # most visibility queries a ray marches ahead per round (0: 8)
    extra: dict = field(default_factory=dict)

    def to_c(self) -> _Params:
        p = _Params()
        for k in ("width", "height", "level", "max_depth", "max_vis_queries", "threshold", "fov_y_deg", "lod_max_level",
                  "lod_input", "seed", "mode", "max_chain"):
            setattr(p, k, getattr(self, k))
        for k in ("eye", "target", "up", "background", "env_color"):
            getattr(p, k)[:] = [float(v) for v in getattr(self, k)]
        return p


def camera(params: RenderParams, level_res: int):
    """Index-space camera: (eye, right, up, forward) as 12 float32 (what the renderer uses)."""
    import numpy as np

    out = np.zeros(12, np.float32)
    p = params.to_c()
    check(load().nlod_render_camera(C.byref(p), int(level_res), out.ctypes.data))
    return out


def _stream(stream):
    import torch

    if stream is None:
        return torch.cuda.current_stream().cuda_stream or None
    return stream if isinstance(stream, int) else (stream.cuda_stream or None)


class Renderer:
    def __init__(self, visibility, throughput, grid, params: RenderParams):
        self._lib = load()
        self.params = params
        self._keep = (visibility, throughput, grid)
        self._r = C.c_void_p()
        p = params.to_c()
        check(self._lib.nlod_renderer_create(visibility.handle, throughput.handle, grid._g, C.byref(p), C.byref(self._r)))

    def frame(self, image=None, ray_stats=None, stream=None):
        import torch

        h, w = self.params.height, self.params.width
        if image is None:
            image = torch.empty((h, w, 3), dtype=torch.float32, device="cuda")
        check(self._lib.nlod_render_frame(self._r, _stream(stream), image.data_ptr(),
                                          None if ray_stats is None else ray_stats.data_ptr()))
        return image

    @property
    def mode(self) -> int:
        """MODE_WAVEFRONT (rounds), MODE_HOST_ROUNDS, or persistent_form(f) (one persistent kernel
        per frame)."""
        return int(self._lib.nlod_renderer_mode(self._r))

    @property
    def persistent(self) -> bool:
        return (self.mode & 0x100) != 0

    def stats(self, stream=None):
        """(visibility queries, throughput queries, rounds, dropped rays) of the last frame; syncs."""
        out = (C.c_uint64 * 4)()
        check(self._lib.nlod_render_stats(self._r, _stream(stream), out))
        return tuple(int(v) for v in out)

    def close(self):
        if getattr(self, "_r", None) is not None and self._r.value:
            self._lib.nlod_renderer_destroy(self._r)
            self._r = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
