"""CPU oracle of the neural-LoD hot path -- TEST INFRASTRUCTURE ONLY.

Imported only by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs, as the
checker; the product path (libnlod.so and neural_lod_gb300) never imports it.
The numerics live in nlod_oracle.c (FP64 restatement of tiny-cuda-nn's algorithms, citations in
nlod_oracle.h); this module builds it, fills its model description from oracle.layout and
exposes numpy-level helpers.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from .build import build_oracle
from .layout import grid_levels, model_spec

ORC_MAX_SLOTS, ORC_MAX_GRIDS, ORC_MAX_LEVELS, ORC_MAX_LAYERS = 8, 2, 32, 10
LOSS = {"BinaryCrossEntropy": 1, "RelativeL2": 2, "L2": 3}


class OrcGrid(C.Structure):
    _fields_ = [("n_levels", C.c_int32), ("hash", C.c_int32), ("kind", C.c_int32), ("interp", C.c_int32),
                ("param_offset", C.c_int64), ("offset", C.c_uint32 * (ORC_MAX_LEVELS + 1)),
                ("res", C.c_uint32 * ORC_MAX_LEVELS), ("scale", C.c_float * ORC_MAX_LEVELS)]


class OrcSlot(C.Structure):
    _fields_ = [("type", C.c_int32), ("in_begin", C.c_int32), ("n_in", C.c_int32), ("out_begin", C.c_int32),
                ("out_width", C.c_int32), ("n_pad", C.c_int32), ("grid", C.c_int32), ("degree", C.c_int32),
                ("n_bins", C.c_int32), ("scale", C.c_float), ("offset", C.c_float)]


class OrcModel(C.Structure):
    _fields_ = [("n_input", C.c_int32), ("n_output", C.c_int32), ("enc_width", C.c_int32), ("width", C.c_int32),
                ("n_layers", C.c_int32), ("act", C.c_int32), ("out_act", C.c_int32),
                ("layer_in", C.c_int32 * ORC_MAX_LAYERS), ("layer_out", C.c_int32 * ORC_MAX_LAYERS),
                ("layer_offset", C.c_int64 * ORC_MAX_LAYERS), ("n_slots", C.c_int32), ("n_grids", C.c_int32),
                ("slots", OrcSlot * ORC_MAX_SLOTS), ("grids", OrcGrid * ORC_MAX_GRIDS),
                ("n_params", C.c_int64), ("n_params_network", C.c_int64)]


class OrcAdam(C.Structure):
    _fields_ = [(k, C.c_float) for k in ("lr", "beta1", "beta2", "eps", "l2_reg", "rel_decay", "abs_decay", "clip",
                                         "non_matrix_lr_factor")] + \
               [("optimize_matrix", C.c_int32), ("optimize_non_matrix", C.c_int32),
                ("lower_lr_bound", C.c_float), ("upper_lr_bound", C.c_float), ("loss_scale", C.c_float)]


_lib = None


def declare(L):
    """Declares argument/return types (pointers must not be narrowed to C int)."""
    vp, i64, f32, ci = C.c_void_p, C.c_int64, C.c_float, C.c_int
    L.orc_grid_offsets.restype = C.c_uint32
    L.orc_grid_offsets.argtypes = [ci, C.c_uint32, C.c_uint32, f32, ci, vp, vp, vp]
    L.orc_sh.restype = None
    L.orc_sh.argtypes = [ci, C.c_double, C.c_double, C.c_double, vp]
    for name in ("orc_encode", "orc_forward"):
        fn = getattr(L, name)
        fn.restype = None
    L.orc_encode.argtypes = [vp, i64, vp, vp, vp, f32, vp]
    L.orc_forward.argtypes = [vp, i64, vp, vp, vp, f32, vp, vp]
    L.orc_loss.restype = None
    L.orc_loss.argtypes = [vp, ci, i64, vp, vp, C.c_double, vp, vp]
    L.orc_backward.restype = None
    L.orc_backward.argtypes = [vp, i64, vp, vp, vp, f32, vp, vp]
    L.orc_adam_step.restype = None
    L.orc_adam_step.argtypes = [vp, i64, i64, vp, vp, vp, vp, vp, vp, f32, f32, f32]
    L.orc_forward_f32.restype = ci
    L.orc_forward_f32.argtypes = [vp, i64, vp, vp, vp, f32, vp, ci]
    L.orc_lod_level.restype = None
    L.orc_lod_level.argtypes = [vp, C.c_int32, C.c_int32, vp, vp, vp, vp]
    L.orc_first_active_voxel_batch.restype = None
    L.orc_first_active_voxel_batch.argtypes = [vp, i64, vp, vp, vp, vp, vp, vp, vp, vp]
    L.orc_optimal_thresholds.restype = None
    L.orc_optimal_thresholds.argtypes = [vp, vp, C.c_uint32, C.c_uint32, ci, f32, vp]
    L.orc_render.restype = None
    L.orc_render.argtypes = [vp, vp, vp, vp, vp, vp, vp, vp, vp, vp]
    L.orc_mesh_frame.restype = None
    L.orc_mesh_frame.argtypes = [vp, vp, C.c_uint32, f32, vp, vp, vp]
    L.orc_voxelize.restype = None
    L.orc_voxelize.argtypes = [vp, i64, vp, vp, C.c_uint32, vp]
    u32 = C.c_uint32
    L.orc_morton_voxels.restype = u32
    L.orc_morton_voxels.argtypes = [vp, u32, vp, u32]
    L.orc_cos_sin.restype = None
    L.orc_cos_sin.argtypes = [f32, vp, vp]
    L.orc_sample_visibility.restype = None
    L.orc_sample_visibility.argtypes = [vp, vp, u32, u32, u32, vp, vp, vp]
    L.orc_sample_visibility_voxels.restype = None
    L.orc_sample_visibility_voxels.argtypes = [vp, vp, u32, u32, u32, u32, vp, vp]
    L.orc_sample_throughput.restype = None
    L.orc_sample_throughput.argtypes = [vp, vp, u32, u32, u32, C.c_int32, vp, vp, vp]
    L.orc_trace_visibility.restype = None
    L.orc_trace_visibility.argtypes = [vp, vp, vp, u32, vp]
    L.orc_trace_throughput.restype = u32
    L.orc_trace_throughput.argtypes = [vp, vp, vp, u32, u32, ci, vp, vp]
    L.orc_compact_samples.restype = u32
    L.orc_compact_samples.argtypes = [vp, vp, u32, u32, u32, vp, vp]
    return L


def lib():
    global _lib
    if _lib is None:
        _lib = declare(C.CDLL(str(build_oracle())))
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data


class Oracle:
    """FP64 oracle for one network-with-input-encoding configuration."""

    def __init__(self, encoding: dict, network: dict, n_input: int, n_output: int):
        self.spec = model_spec(encoding, network, n_input, n_output)
        s = self.spec
        m = OrcModel()
        m.n_input, m.n_output, m.enc_width, m.width = s["n_input"], s["n_output"], s["enc_width"], s["width"]
        m.n_layers, m.act, m.out_act = s["n_layers"], s["act"], s["out_act"]
        for i, l in enumerate(s["layers"]):
            m.layer_in[i], m.layer_out[i], m.layer_offset[i] = l["in"], l["out"], l["offset"]
        m.n_slots, m.n_grids = len(s["slots"]), len(s["grids"])
        for i, sl in enumerate(s["slots"]):
            o = m.slots[i]
            for k in ("type", "in_begin", "n_in", "out_begin", "out_width", "n_pad", "grid", "degree", "n_bins"):
                setattr(o, k, sl[k])
            o.scale, o.offset = sl["scale"], sl["offset"]
        for i, g in enumerate(s["grids"]):
            o = m.grids[i]
            o.n_levels, o.hash, o.kind, o.interp, o.param_offset = g["n_levels"], g["hash"], g["kind"], g["interp"], g["param_offset"]
            for j, v in enumerate(g["offset"]):
                o.offset[j] = v
            for j in range(g["n_levels"]):
                o.res[j] = g["res"][j]
                o.scale[j] = g["scale"][j]
        m.n_params, m.n_params_network = s["n_params"], s["n_params_network"]
        self.m = m
        self.n_params = s["n_params"]
        self.n_output = n_output
        self.n_input = n_input

    @staticmethod
    def _in(x):
        return np.ascontiguousarray(np.asarray(x, dtype=np.float32))

    def encode(self, x, params, max_level=None, max_level_scalar=1000.0):
        x = self._in(x)
        p = np.ascontiguousarray(params, dtype=np.float64)
        ml = None if max_level is None else self._in(max_level)
        out = np.empty((x.shape[0], self.spec["enc_width"]), dtype=np.float64)
        lib().orc_encode(C.byref(self.m), C.c_int64(x.shape[0]), _p(x), _p(p), _p(ml), C.c_float(max_level_scalar), _p(out))
        return out

    def forward(self, x, params, max_level=None, max_level_scalar=1000.0, with_y16=False):
        x = self._in(x)
        p = np.ascontiguousarray(params, dtype=np.float64)
        ml = None if max_level is None else self._in(max_level)
        out = np.empty((x.shape[0], self.n_output), dtype=np.float64)
        y16 = np.empty((x.shape[0], 16), dtype=np.float64) if with_y16 else None
        lib().orc_forward(C.byref(self.m), C.c_int64(x.shape[0]), _p(x), _p(p), _p(ml), C.c_float(max_level_scalar), _p(out), _p(y16))
        return (out, y16) if with_y16 else out

    def loss(self, loss_name, y16, target, loss_scale=1.0):
        y16 = np.ascontiguousarray(y16, dtype=np.float64)
        t = self._in(target)
        dz = np.empty_like(y16)
        val = C.c_double()
        lib().orc_loss(C.byref(self.m), LOSS[loss_name], C.c_int64(y16.shape[0]), _p(y16), _p(t), C.c_double(loss_scale),
                       C.byref(val), _p(dz))
        return val.value, dz

    def backward(self, x, params, dz16, max_level=None, max_level_scalar=1000.0):
        x = self._in(x)
        p = np.ascontiguousarray(params, dtype=np.float64)
        ml = None if max_level is None else self._in(max_level)
        dz = np.ascontiguousarray(dz16, dtype=np.float64)
        g = np.zeros(self.n_params, dtype=np.float64)
        lib().orc_backward(C.byref(self.m), C.c_int64(x.shape[0]), _p(x), _p(p), _p(ml), C.c_float(max_level_scalar), _p(dz), _p(g))
        return g

    def loss_and_grad(self, loss_name, x, params, target, max_level=None, loss_scale=1.0):
        _, y16 = self.forward(x, params, max_level=max_level, with_y16=True)
        val, dz = self.loss(loss_name, y16, target, loss_scale)
        return val, self.backward(x, params, dz, max_level=max_level)

    def forward_f32(self, x, params, max_level=None, max_level_scalar=1000.0, n_threads=0):
        """FP32 scalar host forward (the timed CPU baseline); returns (out, threads_used)."""
        x = self._in(x)
        p = np.ascontiguousarray(params, dtype=np.float32)
        ml = None if max_level is None else self._in(max_level)
        out = np.empty((x.shape[0], self.n_output), dtype=np.float32)
        used = lib().orc_forward_f32(C.byref(self.m), C.c_int64(x.shape[0]), _p(x), _p(p), _p(ml), C.c_float(max_level_scalar),
                                     _p(out), C.c_int(n_threads))
        return out, used


def adam_step(hp: dict, params, grads, m1, m2, steps, n_matrix, loss_scale=1.0, ema=None, ema_decay=0.0,
              ema_debias_old=0.0, ema_debias_new=1.0, lower=0.0, upper=3.4e38):
    """In-place FP32 Adam step (adam.h:47-119) on numpy arrays."""
    a = OrcAdam()
    a.lr = hp.get("learning_rate", 1e-3)
    a.beta1, a.beta2, a.eps = hp.get("beta1", 0.9), hp.get("beta2", 0.999), hp.get("epsilon", 1e-8)
    a.l2_reg = hp.get("l2_reg", 1e-8)
    a.rel_decay, a.abs_decay = hp.get("relative_decay", 0.0), hp.get("absolute_decay", 0.0)
    a.clip = hp.get("clipping_magnitude", 0.0)
    a.non_matrix_lr_factor = hp.get("non_matrix_learning_rate_factor", 1.0)
    a.optimize_matrix, a.optimize_non_matrix = 1, 1
    a.lower_lr_bound, a.upper_lr_bound, a.loss_scale = lower, upper, loss_scale
    lib().orc_adam_step(C.byref(a), C.c_int64(params.size), C.c_int64(n_matrix), _p(params), _p(grads), _p(m1), _p(m2),
                        _p(steps), _p(ema), C.c_float(ema_decay), C.c_float(ema_debias_old), C.c_float(ema_debias_new))


class OrcLodLevel(C.Structure):
    _fields_ = [("res", C.c_int32), ("n_active", C.c_int32), ("bbox_min", C.c_int32 * 3), ("bbox_max", C.c_int32 * 3),
                ("bits", C.c_void_p), ("leaf", C.c_void_p), ("lower", C.c_void_p)]


class LodLevel:
    """One level of the LoD occupancy pyramid (level-0 voxels >> lod), with the NanoVDB-style leaf
    (8^3) and lower-node (128^3) existence flags the first-active-voxel search needs."""

    def __init__(self, bits0: np.ndarray, res0: int, lod: int):
        r = res0 >> lod
        self.bits = np.zeros(((r ** 3) + 31) // 32, dtype=np.uint32)
        nb, nl = (r + 7) // 8, (r + 127) // 128
        self.leaf = np.zeros(nb ** 3, dtype=np.uint8)
        self.lower = np.zeros(nl ** 3, dtype=np.uint8)
        self.s = OrcLodLevel()
        b0 = np.ascontiguousarray(bits0, dtype=np.uint32)
        lib().orc_lod_level(b0.ctypes.data, res0, lod, self.bits.ctypes.data, self.leaf.ctypes.data,
                            self.lower.ctypes.data, C.byref(self.s))
        self.res = r

    @property
    def bbox(self):
        return tuple(self.s.bbox_min), tuple(self.s.bbox_max)

    def first_active_voxel(self, eye, dir, t_min=None, prev=None):
        """Batch search; returns (hit [n] int32, ijk [n,3] int32, t_near [n], t_far [n])."""
        eye = np.ascontiguousarray(eye, dtype=np.float32)
        d = np.ascontiguousarray(dir, dtype=np.float32)
        n = eye.shape[0]
        tm = None if t_min is None else np.ascontiguousarray(t_min, dtype=np.float32)
        pv = None if prev is None else np.ascontiguousarray(prev, dtype=np.int32)
        hit = np.empty(n, np.int32)
        ijk = np.empty((n, 3), np.int32)
        tn = np.empty(n, np.float32)
        tf = np.empty(n, np.float32)
        lib().orc_first_active_voxel_batch(C.byref(self.s), n, eye.ctypes.data, d.ctypes.data, _p(tm), _p(pv),
                                           hit.ctypes.data, ijk.ctypes.data, tn.ctypes.data, tf.ctypes.data)
        return hit, ijk, tn, tf


class OrcRenderParams(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("max_depth", C.c_uint32), ("max_vis", C.c_uint32),
                ("threshold", C.c_float), ("lod_max_level", C.c_float), ("lod_input", C.c_float),
                ("background", C.c_float * 3), ("env", C.c_float * 3), ("seed", C.c_uint64)]


def render(vis: "Oracle", vis_params, thr: "Oracle", thr_params, level: "LodLevel", params, cam):
    """Wavefront render restated on the host: returns (image [h,w,3] float32, ray_stats [h*w,2]
    uint32, totals (visibility queries, throughput queries, dropped rays)).  `params` has the
    fields of neural_lod_gb300.render.RenderParams; cam = the renderer's 12-float camera."""
    p = OrcRenderParams()
    p.width, p.height, p.max_depth, p.max_vis = params.width, params.height, params.max_depth, params.max_vis_queries
    p.threshold, p.lod_max_level, p.lod_input, p.seed = params.threshold, params.lod_max_level, params.lod_input, params.seed
    p.background[:] = list(params.background)
    p.env[:] = list(params.env_color)
    n = params.width * params.height
    image = np.zeros((n, 3), np.float32)
    stats = np.zeros((n, 2), np.uint32)
    totals = np.zeros(3, np.uint64)
    vp_ = np.ascontiguousarray(vis_params, dtype=np.float64)
    tp_ = np.ascontiguousarray(thr_params, dtype=np.float64)
    cam = np.ascontiguousarray(cam, dtype=np.float32)
    lib().orc_render(C.byref(vis.m), vp_.ctypes.data, C.byref(thr.m), tp_.ctypes.data, C.byref(level.s), C.byref(p),
                     cam.ctypes.data, image.ctypes.data, stats.ctypes.data, totals.ctypes.data)
    return image.reshape(params.height, params.width, 3), stats, tuple(int(v) for v in totals)


def optimal_thresholds(truth, proba, n_samples: int, metric: int = 5, beta: float = 1.0):
    """Per-voxel optimal visibility thresholds (the reference's threshold optimisation)."""
    t = np.ascontiguousarray(truth, dtype=np.float32).reshape(-1)
    p = np.ascontiguousarray(proba, dtype=np.float32).reshape(-1)
    n_vox = t.size // n_samples
    out = np.zeros(n_vox, np.float32)
    lib().orc_optimal_thresholds(t.ctypes.data, p.ctypes.data, n_samples, n_vox, metric, C.c_float(beta), out.ctypes.data)
    return out


def mesh_frame(mesh_min, mesh_max, grid: int, eps: float = 1e-4):
    """createMeshBBCube + voxinfo: (bbox_min, bbox_max, unit), each float32[3]."""
    mn = np.ascontiguousarray(mesh_min, dtype=np.float32)
    mx = np.ascontiguousarray(mesh_max, dtype=np.float32)
    bmin, bmax, unit = (np.zeros(3, np.float32) for _ in range(3))
    lib().orc_mesh_frame(mn.ctypes.data, mx.ctypes.data, grid, C.c_float(eps), bmin.ctypes.data, bmax.ctypes.data,
                         unit.ctypes.data)
    return bmin, bmax, unit


def voxelize(triangles, grid: int, bbox_min, unit, bits=None):
    """Conservative surface voxelization (voxelize_triangle); returns the grid^3 bit words."""
    t = np.ascontiguousarray(triangles, dtype=np.float32).reshape(-1, 9)
    if bits is None:
        bits = np.zeros((grid ** 3 + 31) // 32, dtype=np.uint32)
    bmin = np.ascontiguousarray(bbox_min, dtype=np.float32)
    u = np.ascontiguousarray(unit, dtype=np.float32)
    lib().orc_voxelize(t.ctypes.data, t.shape[0], bmin.ctypes.data, u.ctypes.data, grid, bits.ctypes.data)
    return bits


def sh(degree: int, x: float, y: float, z: float):
    out = (C.c_double * (degree * degree))()
    lib().orc_sh(C.c_int(degree), C.c_double(x), C.c_double(y), C.c_double(z), out)
    return np.array(out[:], dtype=np.float64)


__all__ = ["Oracle", "LodLevel", "adam_step", "sh", "grid_levels", "model_spec", "mesh_frame", "voxelize", "render", "optimal_thresholds"]


# ---- training-sample generator (nlod_sampler.c) ----

RAY_QUERY_DTYPE = np.dtype([("origin", "<f4", (3,)), ("mode_or_data", "<i4"), ("dir", "<f4", (3,)), ("t_max", "<f4"),
                            ("voxel_center", "<f4", (3,)), ("voxel_extent", "<f4")])


class SamplerParams(C.Structure):
    """OrcSamplerParams (the layout of nlod_sampler_params)."""
    _fields_ = [("aabb_min", C.c_float * 3), ("aabb_max", C.c_float * 3), ("voxel_size", C.c_float), ("grid_res", C.c_uint32),
                ("n_lods", C.c_uint32), ("dilation_outward", C.c_float), ("dilation_inward", C.c_float),
                ("min_dilation", C.c_float), ("bound_bias", C.c_float), ("pdf_strength", C.c_float), ("pdf_shift", C.c_float),
                ("increase_boundary_density", C.c_int32), ("max_attempts", C.c_uint32)]

    @classmethod
    def from_dict(cls, d: dict) -> "SamplerParams":
        p = cls()
        for k, v in d.items():
            if k in ("aabb_min", "aabb_max"):
                getattr(p, k)[:] = [float(x) for x in v]
            else:
                setattr(p, k, v)
        return p


def morton_voxels(bits, res: int):
    """Sorted Morton codes of the set voxels (uint32 array)."""
    b = np.ascontiguousarray(bits, dtype=np.uint32)
    n = lib().orc_morton_voxels(b.ctypes.data, res, None, 0)
    out = np.zeros(max(n, 1), np.uint32)
    lib().orc_morton_voxels(b.ctypes.data, res, out.ctypes.data, n)
    return out[:n]


def cos_sin(phi: float):
    c, s = C.c_float(), C.c_float()
    lib().orc_cos_sin(C.c_float(phi), C.byref(c), C.byref(s))
    return c.value, s.value


def sample_visibility(params: SamplerParams, morton, batch_index: int, n: int):
    """(input [n,6] float32, queries [n] RAY_QUERY_DTYPE, lod [n] uint32)."""
    m = np.ascontiguousarray(morton, dtype=np.uint32)
    x = np.zeros((n, 6), np.float32)
    q = np.zeros(n, RAY_QUERY_DTYPE)
    lod = np.zeros(n, np.uint32)
    lib().orc_sample_visibility(C.byref(params), m.ctypes.data, m.size, batch_index, n, x.ctypes.data, q.ctypes.data, lod.ctypes.data)
    return x, q, lod


def sample_visibility_voxels(params: SamplerParams, lod_morton, first: int, n_voxels: int, n_samples: int, lod: int):
    m = np.ascontiguousarray(lod_morton, dtype=np.uint32)
    n = n_voxels * n_samples
    x = np.zeros((n, 6), np.float32)
    q = np.zeros(n, RAY_QUERY_DTYPE)
    lib().orc_sample_visibility_voxels(C.byref(params), m.ctypes.data, first, n_voxels, n_samples, lod, x.ctypes.data, q.ctypes.data)
    return x, q


def sample_throughput(params: SamplerParams, morton, batch_index: int, n: int, max_orders: int = 1000):
    m = np.ascontiguousarray(morton, dtype=np.uint32)
    x = np.zeros((n, 9), np.float32)
    q = np.zeros(n, RAY_QUERY_DTYPE)
    lod = np.zeros(n, np.uint32)
    lib().orc_sample_throughput(C.byref(params), m.ctypes.data, m.size, batch_index, n, max_orders, x.ctypes.data, q.ctypes.data,
                                lod.ctypes.data)
    return x, q, lod


def trace_visibility(level0: "LodLevel", params: SamplerParams, queries):
    q = np.ascontiguousarray(queries, dtype=RAY_QUERY_DTYPE)
    y = np.zeros(q.size, np.float32)
    lib().orc_trace_visibility(C.byref(level0.s), C.byref(params), q.ctypes.data, q.size, y.ctypes.data)
    return y


def trace_throughput(level0: "LodLevel", params: SamplerParams, queries, x, batch_index: int, log_learning: bool = False):
    """Fills wi into x (in place) and returns (target [n,3], n_invalid)."""
    q = np.ascontiguousarray(queries, dtype=RAY_QUERY_DTYPE)
    assert x.dtype == np.float32 and x.flags.c_contiguous
    y = np.zeros((q.size, 3), np.float32)
    bad = lib().orc_trace_throughput(C.byref(level0.s), C.byref(params), q.ctypes.data, q.size, batch_index, int(log_learning),
                                     x.ctypes.data, y.ctypes.data)
    return y, bad


def compact_samples(x, y):
    x = np.ascontiguousarray(x, dtype=np.float32)
    y = np.ascontiguousarray(y, dtype=np.float32)
    xv = np.zeros_like(x)
    yv = np.zeros_like(y)
    k = lib().orc_compact_samples(x.ctypes.data, y.ctypes.data, x.shape[0], x.shape[1], y.shape[1], xv.ctypes.data, yv.ctypes.data)
    return xv[:k], yv[:k]
