"""This library against tiny-cuda-nn itself, on the GPU.

tiny-cuda-nn is compiled from the reference's vendored sources (oracle/build_tcnn.py) and was run
on a GB300 with the same FP32 parameter vectors, inputs and targets (tests/golden/
make_tcnn_golden.py, fixture tests/golden/tcnn_golden.npz).  Here the same cases run through this
library's C ABI (nlod_inference, nlod_training_step, nlod_forward_backward_loss) and are compared
with tiny-cuda-nn's results and with the FP64 oracle.

tiny-cuda-nn's half-precision path keeps FP16 activations and FP16 hidden-layer accumulators
(fully_fused_mlp.cu:68, 595) and FP16 gradient atomics (grid.h:411-417); this library's FP16 form
accumulates in FP32.  Stated and checked, per case:
  outputs     mean |ours - tcnn| <= 2e-3 * mean |y| + 2e-4, and this library's FP16 error against
              FP64 is at most tiny-cuda-nn's (FP32 form: at most a tenth of it)
  gradients   relative L2 |ours - tcnn| <= 6e-2 per parameter block, this library's FP16 error
              against FP64 at most 1.25x tiny-cuda-nn's
  Adam        the first step's update has the sign of tiny-cuda-nn's on >= 99 % of the changed
              entries and the same size (about lr) to 1e-3; zero-gradient grid entries stay put
  EMA         after three steps, inference (EMA weights) within 5e-3 * mean |y| of tiny-cuda-nn
When tiny-cuda-nn is built on this machine (oracle/_ref), the live tests repeat the query and
gradient comparisons on 2^16-element batches of fresh seeds.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

import oracle
from neural_lod_gb300 import NetworkWithInputEncoding, workloads as W

GOLDEN = Path(__file__).resolve().parent / "golden" / "tcnn_golden.npz"
sys.path.insert(0, str(GOLDEN.parent))

import make_tcnn_golden as G  # noqa: E402

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gold():
    if not GOLDEN.exists():
        pytest.skip("tiny-cuda-nn golden vectors not generated")
    return np.load(GOLDEN)


def _rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


def _module(name, precision):
    enc, net, spec, params = G.case_params(name)
    c = G.CASES[name]
    m = NetworkWithInputEncoding(c["n_in"], c["n_out"], enc, net, loss=c.get("loss"), optimizer=c.get("optimizer"), precision=precision)
    m.set_params(params)
    return m, enc, net, spec, params


@pytest.mark.parametrize("precision", ["fp16", "fp32"])
@pytest.mark.parametrize("name", ["vis_query", "thr_query", "arcade_query"])
def test_queries_match_tcnn(cuda, nlod_lib, gold, name, precision):
    import torch

    m, enc, net, spec, params = _module(name, precision)
    x, ml, _ = G.case_inputs(name)
    c = G.CASES[name]
    orc = oracle.Oracle(enc, net, c["n_in"], c["n_out"])
    xd = torch.from_numpy(x).to(cuda)
    cases = [("out", None)] + ([("out_masked", ml)] if ml is not None else [])
    for key, lv in cases:
        if lv is not None:
            m.set_max_level_gpu(torch.from_numpy(lv).to(cuda))
        ours = m.inference(xd).cpu().numpy().astype(np.float64)
        m.sync_status()
        tc = gold[f"{name}/{key}"].astype(np.float64)
        ref = orc.forward(x, params, max_level=lv)
        scale = np.abs(ref).mean()
        e_ot, e_t, e_o = np.abs(ours - tc).mean(), np.abs(tc - ref).mean(), np.abs(ours - ref).mean()
        print(f"\n{name}/{key} {precision}: |ours-tcnn| {e_ot:.2e}  |tcnn-fp64| {e_t:.2e}  |ours-fp64| {e_o:.2e}  (mean |y| {scale:.3f})")
        assert e_ot <= 2e-3 * scale + 2e-4
        assert e_o <= (e_t if precision == "fp16" else 0.1 * e_t)


def test_one_hot_and_identity_forms_agree(cuda, nlod_lib):
    """The throughput network with its LoD as this library's one-hot encoding (10 inputs) and as 8
    identity inputs (17 inputs, the form tiny-cuda-nn builds) gives the same bits.  The two forms
    differ only in the 8 padding columns of the 80-wide encoded row (the one-hot encoding pads with
    0, the identity encoding with 1 as in identity.h:62-66), so their first-layer weights are set
    to zero here."""
    import torch

    enc1, net = W.throughput_configs()
    enc2, _ = W.thr_identity_configs()
    spec = oracle.model_spec(enc1, net, 10, 3)
    assert spec["n_params"] == oracle.model_spec(enc2, net, 17, 3)["n_params"]
    params = W.test_params(spec, seed=6, grid_scale=0.2)
    L0 = spec["layers"][0]
    w0 = params[L0["offset"]:L0["offset"] + L0["in"] * L0["out"]].reshape(L0["out"], L0["in"])
    w0[:, 72:] = 0.0
    x10 = W.throughput_inputs(4096, seed=22)
    x17 = W.thr_identity_inputs(4096, seed=22)
    for precision in ("fp16", "fp32"):
        a = NetworkWithInputEncoding(10, 3, enc1, net, precision=precision)
        b = NetworkWithInputEncoding(17, 3, enc2, net, precision=precision)
        a.set_params(params)
        b.set_params(params)
        ya = a.inference(torch.from_numpy(x10).to(cuda)).cpu().numpy()
        yb = b.inference(torch.from_numpy(x17).to(cuda)).cpu().numpy()
        assert np.array_equal(ya, yb)


def test_visibility_gradients_match_tcnn(cuda, nlod_lib, gold):
    import torch

    name = "vis_train"
    m, enc, net, spec, params = _module(name, "fp16")
    x, _, t = G.case_inputs(name)
    loss = m.training_step(torch.from_numpy(x).to(cuda), torch.from_numpy(t).to(cuda), run_optimizer=False).item()
    m.sync_status()
    g = m.get_params("gradients").astype(np.float64)
    ref_loss, ref_g = oracle.Oracle(enc, net, 6, 1).loss_and_grad("BinaryCrossEntropy", x, params, t)
    assert abs(loss - float(gold[f"{name}/loss"])) <= 2e-3 * abs(ref_loss)
    n_net = spec["n_params_network"]
    idx = gold[f"{name}/grid_idx"]
    blocks = [(f"W{k}", slice(L["offset"], L["offset"] + L["in"] * L["out"])) for k, L in enumerate(spec["layers"])]
    tg_net = gold[f"{name}/grad_net"].astype(np.float64)
    for label, sl in blocks:
        e_ot, e_t, e_o = _rel(g[sl], tg_net[sl]), _rel(tg_net[sl], ref_g[sl]), _rel(g[sl], ref_g[sl])
        print(f"\n{label}: |ours-tcnn| {e_ot:.2e}  |tcnn-fp64| {e_t:.2e}  |ours-fp64| {e_o:.2e}")
        assert e_ot <= 6e-2
        assert e_o <= 1.25 * e_t
    tg_grid = gold[f"{name}/grad_grid"].astype(np.float64)
    e_ot, e_t, e_o = _rel(g[idx], tg_grid), _rel(tg_grid, ref_g[idx]), _rel(g[idx], ref_g[idx])
    print(f"grid: |ours-tcnn| {e_ot:.2e}  |tcnn-fp64| {e_t:.2e}  |ours-fp64| {e_o:.2e}")
    assert e_ot <= 6e-2
    assert e_o <= 1.25 * e_t


def test_adam_step_matches_tcnn(cuda, nlod_lib, gold):
    import torch

    name = "vis_train"
    m, enc, net, spec, params = _module(name, "fp16")
    x, _, t = G.case_inputs(name)
    m.training_step(torch.from_numpy(x).to(cuda), torch.from_numpy(t).to(cuda))
    m.sync_status()
    p1 = m.get_params("params").astype(np.float64)
    n_net = spec["n_params_network"]
    idx = gold[f"{name}/grid_idx"]
    for ours, theirs, before in ((p1[:n_net], gold[f"{name}/params1_net"], params[:n_net]),
                                 (p1[idx], gold[f"{name}/params1_grid"], params[idx])):
        d_o = ours - before
        d_t = np.asarray(theirs, np.float64) - before
        moved = np.abs(d_o) > 1e-4
        assert moved.sum() > 0
        assert (np.sign(d_o[moved]) == np.sign(d_t[moved])).mean() >= 0.99
        assert np.abs(np.abs(d_o[moved]) - np.abs(d_t[moved])).mean() <= 1e-3
        assert np.all(np.abs(d_t[d_o == 0]) <= 1e-6)


def test_ema_training_matches_tcnn(cuda, nlod_lib, gold):
    import torch

    name = "thr_train"
    m, enc, net, spec, params = _module(name, "fp16")
    x, _, t = G.case_inputs(name)
    xd, td = torch.from_numpy(x).to(cuda), torch.from_numpy(t).to(cuda)
    for _ in range(3):
        m.training_step(xd, td)
    out = m.inference(xd).cpu().numpy().astype(np.float64)
    m.sync_status()
    tc = gold[f"{name}/out3"].astype(np.float64)
    assert np.abs(out - tc).mean() <= 5e-3 * np.abs(tc).mean()


# ---- live comparisons against a tiny-cuda-nn build on this machine ----------------------------

def _tcnn():
    from oracle import tcnn as T

    if not T.available():
        pytest.skip("tiny-cuda-nn is not built here (python -m oracle.build_tcnn build)")
    return T


@pytest.mark.parametrize("name", ["vis_query", "thr_query"])
def test_live_queries_match_tcnn(cuda, nlod_lib, name):
    import torch

    T = _tcnn()
    enc, net, spec, params = G.case_params(name)
    c = G.CASES[name]
    n = 1 << 16
    if name == "vis_query":
        x, _, ml = W.visibility_inputs(n, seed=91)
    else:
        x, ml = W.thr_identity_inputs(n, seed=92), None
    xd = torch.from_numpy(x).to(cuda)
    tm = T.TcnnModel(c["n_in"], c["n_out"], enc, net)
    tm.set_params(params)
    m = NetworkWithInputEncoding(c["n_in"], c["n_out"], enc, net, precision="fp16")
    m.set_params(params)
    if ml is not None:
        mld = torch.from_numpy(ml).to(cuda)
        tm.set_max_level_gpu(mld)
        m.set_max_level_gpu(mld)
    tc = tm.inference(xd).cpu().numpy().astype(np.float64)
    ours = m.inference(xd).cpu().numpy().astype(np.float64)
    m.sync_status()
    ref = oracle.Oracle(enc, net, c["n_in"], c["n_out"]).forward(x[:8192], params, max_level=None if ml is None else ml[:8192])
    scale = np.abs(tc).mean()
    assert np.abs(ours - tc).mean() <= 2e-3 * scale + 2e-4
    assert np.abs(ours[:8192] - ref).mean() <= np.abs(tc[:8192] - ref).mean()


def test_live_gradients_match_tcnn(cuda, nlod_lib):
    import torch

    T = _tcnn()
    enc, net, spec, params = G.case_params("vis_train")
    n = 1 << 16
    x, _, _ = W.visibility_inputs(n, seed=93, n_grid_levels=16)
    t = W.binary_targets(n, 94)
    xd, td = torch.from_numpy(x).to(cuda), torch.from_numpy(t).to(cuda)
    tm = T.TcnnModel(6, 1, enc, net, W.VISIBILITY_LOSS, W.VISIBILITY_OPTIMIZER)
    tm.set_params(params)
    tm.training_step(xd, td, run_optimizer=False)
    tg = tm.gradients().astype(np.float64)
    m = NetworkWithInputEncoding(6, 1, enc, net, loss=W.VISIBILITY_LOSS, optimizer=W.VISIBILITY_OPTIMIZER, precision="fp16")
    m.set_params(params)
    m.training_step(xd, td, run_optimizer=False)
    m.sync_status()
    g = m.get_params("gradients").astype(np.float64)
    n_net = spec["n_params_network"]
    assert _rel(g[:n_net], tg[:n_net]) <= 6e-2
    assert _rel(g[n_net:], tg[n_net:]) <= 6e-2
