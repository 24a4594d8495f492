"""nlod_training_step_noalloc: the training step for callers that cannot allocate device memory
while they train (for example an online learner inside a real-time frame loop).  It runs the plain
FP32 step whatever precision the module was created with, so it must give the same result as
nlod_training_step on the module's FP32 form, call after call, from its fixed scratch instead of a
cudaMalloc'ed workspace.  Both entry points are called through the C ABI.

The first call in a device's context is the set-up call (under lazy module loading it loads the
scratch array and the step's kernels); the no-allocation check applies from the second call on.
It reads the device-wide free memory, so it assumes that no other process allocates on this GPU
while the test runs (the GPU is leased to this test run alone).

This file is named so that pytest collects it last."""
import ctypes as C

import numpy as np
import pytest

import oracle
from neural_lod_gb300 import NetworkWithInputEncoding, workloads as W

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.linalg.norm(a.astype(np.float64) - b) / max(np.linalg.norm(b.astype(np.float64)), 1e-30))


@pytest.mark.parametrize("precision", ["fp32", "fp16"])
def test_training_step_noalloc_matches_training_step(cuda, nlod_lib, precision):
    import torch

    enc, net = W.visibility_configs(16)
    spec = oracle.model_spec(enc, net, 6, 1)
    params = W.test_params(spec, seed=21, grid_scale=0.3)
    n = 4096
    x, _, _ = W.visibility_inputs(n, seed=22)
    t = (np.random.default_rng(23).random((n, 1)) < 0.4).astype(np.float32)
    xd, td = torch.from_numpy(x).to(cuda), torch.from_numpy(t).to(cuda)
    ref = NetworkWithInputEncoding(6, 1, enc, net, loss=W.VISIBILITY_LOSS, optimizer=W.VISIBILITY_OPTIMIZER, precision="fp32")
    noa = NetworkWithInputEncoding(6, 1, enc, net, loss=W.VISIBILITY_LOSS, optimizer=W.VISIBILITY_OPTIMIZER, precision=precision)
    ref.set_params(params)
    noa.set_params(params)
    loss_ref = torch.zeros(1, device=cuda)
    loss_noa = torch.zeros(1, device=cuda)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream or None)
    p_prev = params.copy()
    for call in range(2):
        assert nlod_lib.nlod_training_step(ref.handle, stream, n, xd.data_ptr(), td.data_ptr(), loss_ref.data_ptr()) == 0
        free_before = torch.cuda.mem_get_info()[0]
        assert nlod_lib.nlod_training_step_noalloc(noa.handle, stream, n, xd.data_ptr(), td.data_ptr(), loss_noa.data_ptr()) == 0, \
            nlod_lib.nlod_last_error()
        torch.cuda.synchronize()
        if call >= 1:   # after the set-up call: nothing allocated by the call
            assert torch.cuda.mem_get_info()[0] == free_before
        assert loss_noa.item() == pytest.approx(loss_ref.item(), rel=1e-5)
        g_ref, g_noa = ref.get_params("gradients"), noa.get_params("gradients")
        assert _rel(g_noa, g_ref) <= 1e-3
        p_ref, p_noa = ref.get_params("params"), noa.get_params("params")
        # parameters agree to 1e-3 of the step's own update
        assert np.linalg.norm(p_noa.astype(np.float64) - p_ref) <= 1e-3 * np.linalg.norm(p_ref.astype(np.float64) - p_prev)
        p_prev = p_ref
        assert ref.optimizer_step_count == noa.optimizer_step_count == call + 1


def test_training_step_noalloc_rejects_batches_beyond_its_scratch(cuda, nlod_lib):
    import torch

    enc, net = W.visibility_configs(16)
    m = NetworkWithInputEncoding(6, 1, enc, net, loss=W.VISIBILITY_LOSS, optimizer=W.VISIBILITY_OPTIMIZER, precision="fp16")
    n = 1 << 16
    x = torch.zeros((n, 6), device=cuda)
    t = torch.zeros((n, 1), device=cuda)
    code = nlod_lib.nlod_training_step_noalloc(m.handle, None, n, x.data_ptr(), t.data_ptr(), None)
    assert code == 1
    msg = nlod_lib.nlod_last_error().decode()
    assert "16 MiB" in msg and "10880" in msg
    # a batch that is not a multiple of 128 is rejected too, before any launch
    assert nlod_lib.nlod_training_step_noalloc(m.handle, None, 100, x.data_ptr(), t.data_ptr(), None) == 1
    assert m.optimizer_step_count == 0
