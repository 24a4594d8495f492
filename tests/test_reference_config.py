"""The throughput network shipped with the reference's arcade scene runs through the module:
its restated configuration matches the shipped JSON's layout (CPU, when the reference's files are
staged), and on the GPU its FP32 and FP16 inference agree with the FP64 oracle, it trains, and a
checkpoint round trip reproduces it."""
import json

import numpy as np
import pytest

import oracle
from neural_lod_gb300 import workloads as W
from oracle.build_ref import ARCADE_CONFIG as SHIPPED   # the shipped JSON, staged from the reference


def test_restated_config_matches_shipped_json():
    import neural_lod_gb300 as N

    if not SHIPPED.exists():
        pytest.skip("the shipped configuration is not staged (python -m oracle.build_ref stage)")
    cfg = json.loads(SHIPPED.read_text())
    enc, net, loss, opt = W.arcade_throughput_configs()
    assert N.layout(cfg["encoding"], cfg["network"], 9, 3) == N.layout(enc, net, 9, 3)
    assert cfg["loss"] == loss
    a, b = cfg["optimizer"], opt
    assert a["otype"] == b["otype"] and a["decay"] == b["decay"]
    for k in ("decay_base", "decay_interval", "decay_start"):
        assert np.float32(a["nested"][k]) == np.float32(b["nested"][k])
    for k in ("learning_rate", "beta1", "beta2", "epsilon", "l2_reg"):
        assert np.float32(a["nested"]["nested"][k]) == np.float32(b["nested"]["nested"][k])


def test_layout_of_shipped_config():
    import neural_lod_gb300 as N

    enc, net, _, _ = W.arcade_throughput_configs()
    L = N.layout(enc, net, 9, 3)
    assert L["enc_width"] == 144 and L["width"] == 128 and L["n_layers"] == 5
    assert [s["out_width"] for s in L["slots"]] == [14, 64, 66]   # 7 levels x 2, SH 8^2, SH 8^2 + pad to 16


@pytest.mark.gpu
def test_shipped_config_inference_training_checkpoint(cuda, nlod_lib):
    import torch

    import neural_lod_gb300 as N

    enc, net, loss, opt = W.arcade_throughput_configs()
    spec = N.layout(enc, net, 9, 3)
    params = W.test_params(spec, seed=21, grid_scale=0.3)
    rng = np.random.Generator(np.random.PCG64(5))
    n = 8192
    pos = rng.random((n, 3)).astype(np.float32)
    wo = (W._unit_dirs(rng, n) + 1) * 0.5
    wi = (W._unit_dirs(rng, n) + 1) * 0.5
    x = np.concatenate([pos, wo, wi], 1).astype(np.float32)
    ref = oracle.Oracle(enc, net, 9, 3).forward(x, params.astype(np.float64))
    scale = float(np.abs(ref).mean())
    xd = torch.from_numpy(x).to(cuda)
    outs = {}
    for prec, tol in (("fp32", 1e-5), ("fp16", 2e-2)):
        m = N.NetworkWithInputEncoding(9, 3, enc, net, loss=loss, optimizer=opt, precision=prec)
        m.set_params(params)
        y = torch.empty((n, 3), device=cuda)
        m.inference(xd, y)
        m.sync_status()
        err = float(np.abs(y.cpu().numpy() - ref).mean())
        assert err <= tol * max(scale, 1.0), (prec, err, scale)
        outs[prec] = m
    # training: a few steps on a smooth target lower the loss
    m = outs["fp16"]
    t = torch.from_numpy((0.5 + 0.4 * np.sin(3 * x[:, :3])).astype(np.float32)).to(cuda)
    lo = torch.empty(1, device=cuda)
    losses = []
    for _ in range(30):
        m.training_step(xd, t, lo)
        losses.append(float(lo.item()))
    m.sync_status()
    assert np.isfinite(losses).all() and losses[-1] < losses[0]
    # checkpoint round trip reproduces the inference outputs
    blob = m.serialize(half_precision=False)
    m2 = N.NetworkWithInputEncoding(9, 3, enc, net, loss=loss, optimizer=opt, precision="fp16")
    m2.deserialize(blob)
    y1 = torch.empty((n, 3), device=cuda)
    y2 = torch.empty((n, 3), device=cuda)
    m.inference(xd, y1)
    m2.inference(xd, y2)
    assert torch.equal(y1, y2)
