"""GB300-native neural level-of-detail query and training (host-side Python mirror).

The compute lives in libnlod.so (hand-written sm_103a CUDA behind the C ABI of
include/nlod.h).  This module mirrors tiny-cuda-nn's NetworkWithInputEncoding + Trainer call
shape (rptr/ext/tiny-cuda-nn/include/tiny-cuda-nn/network_with_input_encoding.h,
trainer.h) for Python callers, with torch tensors as the device buffers:

    net = NetworkWithInputEncoding(n_input_dims, n_output_dims, encoding, network,
                                   loss=..., optimizer=..., precision="fp16", seed=1337)
    y = net.inference(x)                      # x: cuda float32 [n, n_input_dims]
    loss = net.training_step(x, target)       # fwd + loss + bwd + Adam, loss stays on device
"""
from __future__ import annotations

import ctypes as C
import json as _json
from typing import Any

from ._lib import NLOD_OK, PRECISION, NlodError, check, load

__all__ = ["NetworkWithInputEncoding", "NlodError", "layout", "load", "PRECISION"]


def _dump(cfg: Any) -> bytes | None:
    if cfg is None:
        return None
    if isinstance(cfg, (bytes, str)):
        return cfg.encode() if isinstance(cfg, str) else cfg
    return _json.dumps(cfg).encode()


def layout(encoding: Any, network: Any, n_input_dims: int, n_output_dims: int) -> dict:
    """Host-only layout of a configuration (nlod_layout_json); raises NlodError on bad configs."""
    lib = load()
    p = C.c_void_p()
    check(lib.nlod_layout_json(_dump(encoding), _dump(network), int(n_input_dims), int(n_output_dims), C.byref(p)))
    try:
        return _json.loads(C.string_at(p.value).decode())
    finally:
        lib.nlod_free_string(p)


def _stream_ptr(stream) -> int | None:
    import torch

    if stream is None:
        # torch's current stream on the current device, read as a raw handle where torch offers
        # that (it skips building a Stream object on every call of a small query)
        raw = getattr(torch._C, "_cuda_getCurrentRawStream", None)
        if raw is not None:
            return raw(torch.cuda.current_device()) or None
        return torch.cuda.current_stream().cuda_stream or None
    if isinstance(stream, int):
        return stream or None
    return stream.cuda_stream or None


def _ptr(t) -> int:
    return t.data_ptr() if t is not None else None


class NetworkWithInputEncoding:
    """Encoding -> fully fused MLP network plus its trainer (loss + optimizer).

    precision: "fp32" (plain FP32 form on CUDA cores), "fp16" or "bf16" (tcgen05 tensor-core
    form with FP32 accumulation, FP32 master weights / hash tables / optimizer moments).
    """

    def __init__(self, n_input_dims: int, n_output_dims: int, encoding: Any, network: Any,
                 loss: Any = None, optimizer: Any = None, precision: str = "fp16", seed: int = 1337):
        self._lib = load()
        self._m = C.c_void_p()
        self.precision = precision
        check(self._lib.nlod_module_create(_dump(encoding), _dump(network), _dump(loss), _dump(optimizer),
                                           int(n_input_dims), int(n_output_dims), PRECISION[precision],
                                           int(seed), C.byref(self._m)))
        self._max_level_ref = None

    # ---- sizes ------------------------------------------------------------------------------
    @property
    def handle(self) -> int:
        return self._m.value

    @property
    def n_params(self) -> int:
        return int(self._lib.nlod_n_params(self._m))

    @property
    def n_network_params(self) -> int:
        return int(self._lib.nlod_n_network_params(self._m))

    @property
    def n_input_dims(self) -> int:
        return int(self._lib.nlod_n_input_dims(self._m))

    @property
    def n_output_dims(self) -> int:
        return int(self._lib.nlod_n_output_dims(self._m))

    @property
    def encoded_width(self) -> int:
        return int(self._lib.nlod_encoded_width(self._m))

    @property
    def padded_output_width(self) -> int:
        return int(self._lib.nlod_padded_output_width(self._m))

    # ---- grid level masking (GridEncoding::set_max_level / set_max_level_gpu) ---------------
    def set_max_level(self, value: float) -> None:
        """One level fraction in [0,1] for every element (levels above it encode as zero)."""
        check(self._lib.nlod_set_max_level(self._m, float(value)))

    def set_max_level_gpu(self, per_element) -> None:
        """per_element: cuda float32 [n] of level fractions in [0,1], or None."""
        self._max_level_ref = per_element
        check(self._lib.nlod_set_max_level_gpu(self._m, _ptr(per_element)))

    # ---- compute ----------------------------------------------------------------------------
    def inference(self, x, out=None, stream=None):
        """network->inference(stream, X, Y): x cuda float32 [n][n_input_dims], n a multiple of 128;
        returns out, cuda float32 [n][n_output_dims] (asynchronous on `stream`, torch's current
        stream by default)."""
        import torch

        n = x.shape[0]
        if out is None:
            out = torch.empty((n, self.n_output_dims), device=x.device, dtype=torch.float32)
        check(self._lib.nlod_inference(self._m, _stream_ptr(stream), n, _ptr(x), _ptr(out)))
        return out

    def inference_host(self, x, out=None, stream=None):
        """Inference on a host (CPU) batch: pinned tensors are read in place by the kernel, others
        are staged; `out` (a CPU tensor, pinned when asynchrony matters) is valid once the stream
        has synchronised."""
        import torch

        if x.is_cuda or (out is not None and out.is_cuda):
            raise ValueError("inference_host takes host tensors; use inference() for device tensors")
        x = x.contiguous()
        if out is None:
            out = torch.empty((x.shape[0], self.n_output_dims), dtype=torch.float32, pin_memory=True)
        check(self._lib.nlod_inference_host(self._m, _stream_ptr(stream), x.shape[0], x.data_ptr(), out.data_ptr()))
        return out

    def training_step(self, x, target, loss_out=None, stream=None, run_optimizer: bool = True):
        """Returns a 1-element cuda tensor holding this step's mean loss (no host sync)."""
        import torch

        if loss_out is None:
            loss_out = torch.empty(1, device=x.device, dtype=torch.float32)
        fn = self._lib.nlod_training_step if run_optimizer else self._lib.nlod_forward_backward_loss
        check(fn(self._m, _stream_ptr(stream), x.shape[0], _ptr(x), _ptr(target), _ptr(loss_out)))
        return loss_out

    def optimizer_step(self, stream=None) -> None:
        """Applies the optimizer to the gradients of the last forward/backward (Trainer's
        optimizer step: loss scale divided out, Adam, ExponentialDecay and EMA wrappers)."""
        check(self._lib.nlod_optimizer_step(self._m, _stream_ptr(stream)))

    def forward(self, x, out=None, stream=None):
        """Training-mode forward; returns (out, ctx) for backward()."""
        import torch

        n = x.shape[0]
        if out is None:
            out = torch.empty((n, self.n_output_dims), device=x.device, dtype=torch.float32)
        ctx = C.c_void_p()
        check(self._lib.nlod_forward(self._m, _stream_ptr(stream), n, _ptr(x), _ptr(out), C.byref(ctx)))
        return out, _Ctx(self._lib, ctx)

    def backward(self, ctx, x, dL_dout, stream=None) -> None:
        """Accumulates parameter gradients from dL/d(output) [n][n_output_dims] into the module's
        gradient vector (read with get_params("gradients"))."""
        check(self._lib.nlod_backward(self._m, _stream_ptr(stream), ctx.handle, _ptr(x), _ptr(dL_dout)))

    # ---- kernel variants / autotuning ------------------------------------------------------
    @property
    def n_kernel_variants(self) -> int:
        return int(self._lib.nlod_kernel_variants(self._m))

    @property
    def kernel_variant(self) -> int:
        return int(self._lib.nlod_get_kernel_variant(self._m))

    @kernel_variant.setter
    def kernel_variant(self, v: int) -> None:
        check(self._lib.nlod_set_kernel_variant(self._m, int(v)))

    def autotune(self, x, out=None, stream=None) -> int:
        """Times every kernel variant on batch x and keeps the fastest; returns its index."""
        import torch

        if out is None:
            out = torch.empty((x.shape[0], self.n_output_dims), device=x.device, dtype=torch.float32)
        check(self._lib.nlod_autotune(self._m, _stream_ptr(stream), x.shape[0], _ptr(x), _ptr(out)))
        return self.kernel_variant

    def calib_gathers(self, n: int, stream=None) -> float:
        """Duration (ms) of the encoding's grid gathers alone for n seeded queries
        (nlod_calib_gathers): the memory-side floor of the query kernel."""
        ms = C.c_float()
        check(self._lib.nlod_calib_gathers(self._m, _stream_ptr(stream), n, C.byref(ms)))
        return ms.value

    def calib_scatter(self, n: int, stream=None) -> float:
        """Duration (ms) of the grid-gradient scatter alone for n seeded samples
        (nlod_calib_scatter; overwrites the gradient buffer): the floor of the fused training kernel."""
        ms = C.c_float()
        check(self._lib.nlod_calib_scatter(self._m, _stream_ptr(stream), n, C.byref(ms)))
        return ms.value

    def sync_status(self, stream=None) -> None:
        """Synchronises `stream` and raises NlodError if a kernel reported a device-side error
        (for example a wait that gave up) since the last check."""
        check(self._lib.nlod_sync_status(self._m, _stream_ptr(stream)))

    # ---- parameters -------------------------------------------------------------------------
    def get_params(self, which: str = "params"):
        """which: "params" (FP32 master), "inference" (EMA when enabled) or "gradients"."""
        import numpy as np

        code = {"params": 0, "inference": 1, "gradients": 2}[which]
        buf = np.empty(self.n_params, dtype=np.float32)
        check(self._lib.nlod_get_params(self._m, buf.ctypes.data, buf.size, code, 0))
        return buf

    def set_params(self, params) -> None:
        """Trainer::set_params_full_precision: the FP32 vector (network then encoding) from a numpy
        array or a cuda tensor; the EMA (inference) weights and the FP16/BF16 copies are set to it
        too."""
        import numpy as np

        if hasattr(params, "is_cuda") and params.is_cuda:
            check(self._lib.nlod_set_params(self._m, params.data_ptr(), params.numel(), 1))
            return
        arr = np.ascontiguousarray(np.asarray(params, dtype=np.float32))
        check(self._lib.nlod_set_params(self._m, arr.ctypes.data, arr.size, 0))

    @property
    def optimizer_step_count(self) -> int:
        return int(self._lib.nlod_optimizer_step_count(self._m))

    @property
    def learning_rate(self) -> float:
        return float(self._lib.nlod_learning_rate(self._m))

    @learning_rate.setter
    def learning_rate(self, value: float) -> None:
        check(self._lib.nlod_set_learning_rate(self._m, float(value)))

    # ---- checkpoints (Trainer::serialize / deserialize JSON) --------------------------------
    def serialize(self, half_precision: bool = True) -> str:
        """Trainer::serialize's parameter fields as JSON text: n_params, params_type and the
        inference parameters (the EMA when there is one) as `params_binary` bytes, FP16 when
        half_precision (as tiny-cuda-nn's half build writes them), else FP32."""
        p = C.c_void_p()
        check(self._lib.nlod_serialize(self._m, 1 if half_precision else 0, C.byref(p)))
        try:
            return C.string_at(p.value).decode()
        finally:
            self._lib.nlod_free_string(p)

    def deserialize(self, data: str | dict) -> None:
        """Trainer::deserialize: loads what serialize() (or tiny-cuda-nn's trainer) wrote."""
        s = data if isinstance(data, str) else _json.dumps(data)
        check(self._lib.nlod_deserialize(self._m, s.encode()))

    def close(self) -> None:
        if getattr(self, "_m", None) is not None and self._m.value:
            self._lib.nlod_module_destroy(self._m)
            self._m = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class _Ctx:
    def __init__(self, lib, handle):
        self._lib = lib
        self.handle = handle

    def __del__(self):
        try:
            if self.handle and self.handle.value:
                self._lib.nlod_ctx_destroy(self.handle)
                self.handle = None
        except Exception:
            pass
