"""Parity of the training path (loss, backward, Adam, EMA/decay, checkpoints) against the
FP64 oracle.  Gradient tolerance of the plain FP32 form: relative L2 error <= 1e-3 of the FP64
oracle's gradient per parameter block (network matrices, grid tables); loss within 1e-4 relative."""
import json

import numpy as np
import pytest

import oracle
from neural_lod_gb300 import NetworkWithInputEncoding, workloads as W

pytestmark = pytest.mark.gpu


def _setup(precision, n=4096, seed=3, loss=W.VISIBILITY_LOSS, opt=W.VISIBILITY_OPTIMIZER, cfg=None):
    enc, net = cfg or W.visibility_configs(16)
    spec = oracle.model_spec(enc, net, 6, 1)
    params = W.test_params(spec, seed=seed, grid_scale=0.3)
    m = NetworkWithInputEncoding(6, 1, enc, net, loss=loss, optimizer=opt, precision=precision)
    m.set_params(params)
    x, _, _ = W.visibility_inputs(n, seed=seed + 10)
    t = (np.random.default_rng(seed).random((n, 1)) < 0.4).astype(np.float32)
    return m, oracle.Oracle(enc, net, 6, 1), params, x, t, spec


def _rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)


@pytest.mark.parametrize("precision", ["fp32"])
def test_loss_and_gradients_match_oracle(cuda, nlod_lib, precision):
    """The plain FP32 form (the FP16 / BF16 forms run the fused kernel: test_gpu_train_tc.py)."""
    import torch

    m, orc, params, x, t, spec = _setup(precision)
    xd, td = torch.from_numpy(x).to(cuda), torch.from_numpy(t).to(cuda)
    loss = m.training_step(xd, td, run_optimizer=False).item()
    g = m.get_params("gradients").astype(np.float64)
    ref_loss, ref_g = orc.loss_and_grad("BinaryCrossEntropy", x, params, t)
    assert loss == pytest.approx(ref_loss, rel=1e-4)
    n_net = spec["n_params_network"]
    assert _rel(g[:n_net], ref_g[:n_net]) <= 1e-3
    assert _rel(g[n_net:], ref_g[n_net:]) <= 1e-3
    # untouched grid entries have exactly zero gradient (Adam's sparse skip depends on it)
    assert np.array_equal(g[n_net:] == 0, ref_g[n_net:] == 0)


def test_module_forward_backward_api(cuda, nlod_lib):
    import torch

    m, orc, params, x, _, spec = _setup("fp32", n=2048)
    xd = torch.from_numpy(x).to(cuda)
    out, ctx = m.forward(xd)
    dl = np.random.default_rng(1).standard_normal((2048, 1)).astype(np.float32)
    m.backward(ctx, xd, torch.from_numpy(dl).to(cuda))
    g = m.get_params("gradients").astype(np.float64)
    _, y16 = orc.forward(x, params, with_y16=True)
    np.testing.assert_allclose(out.cpu().numpy(), y16[:, :1], atol=1e-5)
    dz = np.zeros((2048, 16))
    dz[:, 0] = dl[:, 0] * y16[:, 0] * (1 - y16[:, 0])
    ref_g = orc.backward(x, params, dz)
    assert _rel(g, ref_g) <= 1e-4


def test_adam_step_matches_oracle(cuda, nlod_lib):
    import torch

    m, orc, params, x, t, spec = _setup("fp32")
    xd, td = torch.from_numpy(x).to(cuda), torch.from_numpy(t).to(cuda)
    m.training_step(xd, td, run_optimizer=False)
    g_unscaled = m.get_params("gradients")
    m.optimizer_step()
    p_gpu = m.get_params("params")
    p = params.copy()
    m1 = np.zeros_like(p); m2 = np.zeros_like(p); steps = np.zeros(p.size, dtype=np.uint32)
    g_scaled = (g_unscaled.astype(np.float32) * np.float32(128.0)).astype(np.float32)
    oracle.adam_step(W.VISIBILITY_OPTIMIZER, p, g_scaled, m1, m2, steps, spec["n_params_network"], loss_scale=128.0)
    np.testing.assert_allclose(p_gpu, p, rtol=1e-5, atol=1e-7)
    # encoding entries with zero gradient were skipped: unchanged
    n_net = spec["n_params_network"]
    zero = g_unscaled[n_net:] == 0
    assert zero.any()
    assert np.array_equal(p_gpu[n_net:][zero], params[n_net:][zero])


def test_training_reduces_loss(cuda, nlod_lib):
    import torch

    m, orc, params, x, t, spec = _setup("fp16", n=1 << 14)
    xd, td = torch.from_numpy(x).to(cuda), torch.from_numpy(t).to(cuda)
    first = m.training_step(xd, td).item()
    for _ in range(50):
        last = m.training_step(xd, td)
    assert last.item() < first
    assert m.optimizer_step_count == 51


def test_ema_and_decay_schedule(cuda, nlod_lib):
    """Ema(ExponentialDecay(Adam)) as the neural_lod throughput trainer builds it."""
    import torch

    opt = {"otype": "Ema", "decay": 0.9, "nested": {"otype": "ExponentialDecay", "decay_start": 2, "decay_interval": 2,
                                                   "decay_base": 0.5, "nested": dict(W.VISIBILITY_OPTIMIZER)}}
    m, orc, params, x, t, spec = _setup("fp32", opt=opt)
    # before any step the EMA (inference) weights are what set_params wrote
    np.testing.assert_array_equal(m.get_params("inference"), params)
    xd, td = torch.from_numpy(x).to(cuda), torch.from_numpy(t).to(cuda)
    lrs = []
    ema = params.copy()
    p_prev = params.copy()
    for step in range(1, 6):
        lrs.append(m.learning_rate)
        m.training_step(xd, td)
        p = m.get_params("params")
        d_old = 1 - 0.9 ** (step - 1)
        d_new = 1 / (1 - 0.9 ** step)
        ema = ((ema * np.float32(0.9) * np.float32(d_old) + p * np.float32(0.1)) * np.float32(d_new)).astype(np.float32)
        np.testing.assert_allclose(m.get_params("inference"), ema, rtol=1e-5, atol=1e-7)
        p_prev = p
    # factor multiplies by 0.5 at steps 2 and 4 (counted before increment): lr sequence
    assert lrs[0] == pytest.approx(1e-2)
    assert m.learning_rate == pytest.approx(1e-2 * 0.25)


def test_checkpoint_round_trip(cuda, nlod_lib):
    import torch

    m, orc, params, x, t, spec = _setup("fp16")
    for half in (False, True):
        s = m.serialize(half_precision=half)
        d = json.loads(s)
        assert d["n_params"] == spec["n_params"]
        assert d["params_type"] == ("__half" if half else "float")
        m2 = NetworkWithInputEncoding(6, 1, *W.visibility_configs(16), precision="fp16")
        m2.deserialize(s)
        p2 = m2.get_params("params")
        if half:
            np.testing.assert_allclose(p2, params.astype(np.float16).astype(np.float32), rtol=0, atol=0)
        else:
            np.testing.assert_array_equal(p2, params)
    xd = torch.from_numpy(x).to(cuda)
    np.testing.assert_allclose(m.inference(xd).cpu().numpy(), m2.inference(xd).cpu().numpy(), atol=2e-3)
