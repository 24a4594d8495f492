"""The FP64 oracle against tiny-cuda-nn itself (CPU).

tests/golden/tcnn_golden.npz holds outputs, gradients and updated parameters of tiny-cuda-nn,
compiled from the reference's vendored sources and run on a GB300 with the FP32 parameter vectors,
inputs and targets that tests/golden/make_tcnn_golden.py regenerates here from its seeds.  This
pins the oracle's reading of tiny-cuda-nn's semantics (parameter layout network-then-encoding, row-major
[out][in] matrices with the output layer padded to 16 rows, grid offsets and hashing, SH and
composite padding, per-element max level, loss normalisation and the static loss scale, Adam's
sparse skip and per-parameter steps, EMA inference weights) to the reference's own results.

Tolerances come from tiny-cuda-nn's precision, not the oracle's: its FullyFusedMLP keeps FP16
parameters, FP16 activations and FP16 hidden-layer accumulators (fully_fused_mlp.cu:68, 595), and its
grid gradients are FP16 atomics (grid.h:411-417), so its results differ from the FP64 oracle by
FP16 rounding.  A misread of any semantic above shows up as an error of the order of the values
themselves (1e-1 and more), far above these bounds:
  query outputs       mean |tcnn - fp64| <= 2e-3 * mean |fp64| + 2e-4 (with the max level, too)
  loss                |tcnn - fp64| <= 2e-3 * |fp64|
  MLP gradients       relative L2 <= 3e-2
  grid gradients      relative L2 <= 6e-2 on a seeded sample of 8,192 entries
  params after Adam   the update's sign agrees on >= 99 % of the changed entries; entries with
                      a zero gradient are unchanged (Adam skips them, adam.h:76-79)
  EMA after 3 steps   inference outputs: mean |tcnn - fp64| <= 5e-3 * mean |fp64|
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

import oracle
from neural_lod_gb300 import workloads as W

GOLDEN = Path(__file__).resolve().parent / "golden" / "tcnn_golden.npz"
sys.path.insert(0, str(GOLDEN.parent))

import make_tcnn_golden as G  # noqa: E402

pytestmark = pytest.mark.skipif(not GOLDEN.exists(), reason="tiny-cuda-nn golden vectors not generated")


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLDEN)


def _rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


@pytest.mark.parametrize("name", ["vis_query", "thr_query", "arcade_query"])
def test_oracle_matches_tcnn_query(gold, name):
    enc, net, spec, params = G.case_params(name)
    x, ml, _ = G.case_inputs(name)
    c = G.CASES[name]
    orc = oracle.Oracle(enc, net, c["n_in"], c["n_out"])
    ref = orc.forward(x, params)
    t = gold[f"{name}/out"].astype(np.float64)
    assert t.shape == ref.shape
    err = np.abs(t - ref).mean()
    assert err <= 2e-3 * np.abs(ref).mean() + 2e-4, (name, err, np.abs(ref).mean())
    if ml is not None:
        refm = orc.forward(x, params, max_level=ml)
        tm = gold[f"{name}/out_masked"].astype(np.float64)
        errm = np.abs(tm - refm).mean()
        assert errm <= 2e-3 * np.abs(refm).mean() + 2e-4, (name, errm)
        # the masked and unmasked outputs differ: the max level is not vacuous in either library
        assert np.abs(tm - t).mean() > 20 * errm


def test_oracle_matches_tcnn_visibility_gradients(gold):
    name = "vis_train"
    enc, net, spec, params = G.case_params(name)
    x, _, t = G.case_inputs(name)
    orc = oracle.Oracle(enc, net, 6, 1)
    loss, g = orc.loss_and_grad("BinaryCrossEntropy", x, params, t)
    assert abs(float(gold[f"{name}/loss"]) - loss) <= 2e-3 * abs(loss)
    n_net = spec["n_params_network"]
    assert _rel(gold[f"{name}/grad_net"], g[:n_net]) <= 3e-2
    idx = gold[f"{name}/grid_idx"]
    assert _rel(gold[f"{name}/grad_grid"], g[idx]) <= 6e-2


def _adam(hp, p, g, state, n_net):
    """One in-place FP32 Adam step of the oracle (adam.h:47-119) on p with loss-scaled gradients g."""
    m1, m2, steps = state
    oracle.adam_step(hp, p, np.ascontiguousarray(g, np.float32), m1, m2, steps, n_net, loss_scale=128.0)


def test_oracle_adam_step_matches_tcnn(gold):
    name = "vis_train"
    enc, net, spec, params = G.case_params(name)
    x, _, t = G.case_inputs(name)
    orc = oracle.Oracle(enc, net, 6, 1)
    _, g = orc.loss_and_grad("BinaryCrossEntropy", x, params, t, loss_scale=128.0)
    n = params.size
    n_net = spec["n_params_network"]
    p1 = params.astype(np.float32).copy()
    _adam(W.VISIBILITY_OPTIMIZER, p1, g, (np.zeros(n, np.float32), np.zeros(n, np.float32), np.zeros(n, np.uint32)), n_net)
    idx = gold[f"{name}/grid_idx"]
    for ours, theirs, before in ((p1[:n_net], gold[f"{name}/params1_net"], params[:n_net]),
                                 (p1[idx], gold[f"{name}/params1_grid"], params[idx])):
        d_ours = np.asarray(ours, np.float64) - before
        d_theirs = np.asarray(theirs, np.float64) - before
        moved = np.abs(d_ours) > 1e-4
        assert moved.sum() > 0
        agree = np.sign(d_ours[moved]) == np.sign(d_theirs[moved])
        assert agree.mean() >= 0.99, agree.mean()
        # the first Adam step moves an entry by about lr, whatever its gradient's size
        assert np.abs(np.abs(d_theirs[moved]) - np.abs(d_ours[moved])).mean() <= 1e-3
        # untouched entries (zero gradient) stay put in both
        still = np.abs(d_ours) == 0
        assert np.all(np.abs(d_theirs[still]) <= 1e-6)


def test_oracle_ema_training_matches_tcnn(gold):
    name = "thr_train"
    enc, net, spec, params = G.case_params(name)
    x, _, t = G.case_inputs(name)
    orc = oracle.Oracle(enc, net, 17, 3)
    n = params.size
    n_net = spec["n_params_network"]
    ema_decay = W.THROUGHPUT_OPTIMIZER["decay"]
    adam = W.THROUGHPUT_OPTIMIZER["nested"]["nested"]          # no decay before step 8000
    p = params.astype(np.float32).copy()
    ema = p.copy()
    state = (np.zeros(n, np.float32), np.zeros(n, np.float32), np.zeros(n, np.uint32))
    for step in range(1, 4):
        _, g = orc.loss_and_grad("RelativeL2", x, p, t, loss_scale=128.0)
        _adam(adam, p, g, state, n_net)
        d_old = np.float32(1 - ema_decay ** (step - 1))
        d_new = np.float32(1 / (1 - ema_decay ** step))
        ema = ((ema * np.float32(ema_decay) * d_old + p * np.float32(1 - ema_decay)) * d_new).astype(np.float32)
    ref = orc.forward(x, ema)
    out = gold[f"{name}/out3"].astype(np.float64)
    assert np.abs(out - ref).mean() <= 5e-3 * np.abs(ref).mean()
