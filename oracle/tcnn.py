"""ctypes binding of oracle/_ref/libtcnn_harness-<arch>.so -- TEST INFRASTRUCTURE ONLY.

tiny-cuda-nn built from the reference's vendored sources (oracle/build_tcnn.py) with the small C
ABI of oracle/tcnn_harness.cu.  Used by the parity tests, tests/golden/make_tcnn_golden.py and
the bench's comparison leg; never by the library.  Device buffers are torch CUDA tensors.
"""
from __future__ import annotations

import ctypes as C
import json
from pathlib import Path

import numpy as np

from .build_tcnn import LIB, built

_lib = None


def available() -> bool:
    return built()


def _load():
    global _lib
    if _lib is None:
        if not LIB.exists():
            raise FileNotFoundError(f"{LIB} is not built (python -m oracle.build_tcnn build)")
        lib = C.CDLL(str(LIB))
        vp, u32, sz = C.c_void_p, C.c_uint32, C.c_size_t
        lib.tch_last_error.restype = C.c_char_p
        lib.tch_create.argtypes = [C.c_char_p, u32, u32, C.POINTER(vp)]
        lib.tch_destroy.argtypes = [vp]
        lib.tch_destroy.restype = None
        lib.tch_n_params.argtypes = [vp]
        lib.tch_n_params.restype = sz
        lib.tch_padded_output_width.argtypes = [vp]
        lib.tch_padded_output_width.restype = u32
        lib.tch_encoded_width.argtypes = [vp]
        lib.tch_encoded_width.restype = u32
        lib.tch_set_params.argtypes = [vp, vp, sz]
        lib.tch_get_params.argtypes = [vp, vp, sz]
        lib.tch_set_max_level_gpu.argtypes = [vp, vp]
        lib.tch_inference.argtypes = [vp, vp, u32, vp, vp]
        lib.tch_training_step.argtypes = [vp, vp, u32, vp, vp, C.c_int]
        lib.tch_loss.argtypes = [vp, vp, C.POINTER(C.c_float)]
        lib.tch_get_gradients.argtypes = [vp, vp, sz]
        _lib = lib
    return _lib


def _check(rc: int) -> None:
    if rc != 0:
        raise RuntimeError(f"tiny-cuda-nn: {_lib.tch_last_error().decode()}")


def _stream() -> int | None:
    import torch

    return torch.cuda.current_stream().cuda_stream or None


class TcnnModel:
    """tcnn::create_from_config(n_in, n_out, {encoding, network, loss, optimizer})."""

    def __init__(self, n_in: int, n_out: int, encoding: dict, network: dict, loss: dict | None = None,
                 optimizer: dict | None = None):
        lib = _load()
        cfg = {"encoding": encoding, "network": network}
        if loss is not None:
            cfg["loss"] = loss
        if optimizer is not None:
            cfg["optimizer"] = optimizer
        self._h = C.c_void_p()
        _check(lib.tch_create(json.dumps(cfg).encode(), n_in, n_out, C.byref(self._h)))
        self.n_in, self.n_out = n_in, n_out
        self._keep = None

    def __del__(self):
        if getattr(self, "_h", None) and self._h.value and _lib is not None:
            _lib.tch_destroy(self._h)
            self._h = C.c_void_p()

    @property
    def n_params(self) -> int:
        return int(_lib.tch_n_params(self._h))

    @property
    def encoded_width(self) -> int:
        return int(_lib.tch_encoded_width(self._h))

    @property
    def padded_output_width(self) -> int:
        return int(_lib.tch_padded_output_width(self._h))

    def set_params(self, params: np.ndarray) -> None:
        p = np.ascontiguousarray(params, dtype=np.float32)
        _check(_lib.tch_set_params(self._h, p.ctypes.data, p.size))

    def get_params(self) -> np.ndarray:
        p = np.empty(self.n_params, np.float32)
        _check(_lib.tch_get_params(self._h, p.ctypes.data, p.size))
        return p

    def set_max_level_gpu(self, levels) -> None:
        """levels: cuda float32 [n] of per-element level fractions (kept alive here), or None."""
        self._keep = levels
        _check(_lib.tch_set_max_level_gpu(self._h, levels.data_ptr() if levels is not None else None))

    def inference(self, x, out=None):
        import torch

        n = x.shape[0]
        if out is None:
            out = torch.empty((n, self.n_out), dtype=torch.float32, device=x.device)
        _check(_lib.tch_inference(self._h, _stream(), n, x.data_ptr(), out.data_ptr()))
        return out

    def training_step(self, x, target, run_optimizer: bool = True) -> None:
        _check(_lib.tch_training_step(self._h, _stream(), x.shape[0], x.data_ptr(), target.data_ptr(),
                                      1 if run_optimizer else 0))

    def loss(self) -> float:
        v = C.c_float()
        _check(_lib.tch_loss(self._h, _stream(), C.byref(v)))
        return float(v.value)

    def gradients(self) -> np.ndarray:
        g = np.empty(self.n_params, np.float32)
        _check(_lib.tch_get_gradients(self._h, g.ctypes.data, g.size))
        return g
