"""CPU tests of the oracle itself: its gradients against FP64 central finite differences (the
reference's own check of the grid encoding is torch gradcheck, rptr/ext/tiny-cuda-nn/scripts/
test_grid_bwdbwd.py:104-199), its spherical harmonics against the generated FP32 polynomials the
kernels use, its loss / Adam formulas against direct restatements, and its FP32 baseline
against its FP64 forward."""
import re
from pathlib import Path

import numpy as np
import pytest

import oracle
from neural_lod_gb300 import workloads as W

ROOT = Path(__file__).resolve().parents[1]


def test_sh_matches_reference_polynomials_golden():
    """oracle.sh (associated-Legendre recurrence) against the 64 polynomials of the reference's
    kernel_sh, evaluated by tests/golden/make_sh_golden.py from spherical_harmonics.h."""
    from pathlib import Path

    g = np.load(Path(__file__).resolve().parent / "golden" / "sh_golden.npz")
    for d, v in zip(g["dirs"], g["values"]):
        for degree in (1, 2, 4, 8):
            np.testing.assert_allclose(oracle.sh(degree, *d), v[: degree * degree], rtol=0, atol=1e-12)


def test_sh_recurrence_matches_generated_polynomials():
    src = (ROOT / "neural_lod_gb300" / "csrc" / "sh_basis.inc").read_text()
    exprs = {int(m.group(1)): m.group(2) for m in re.finditer(r"OUT\((\d+), \((.*?)\)\); \\", src)}
    assert len(exprs) == 64
    rng = np.random.default_rng(0)
    for _ in range(200):
        v = rng.standard_normal(3)
        v /= np.linalg.norm(v)
        ref = oracle.sh(8, *v)
        for i in range(64):
            val = eval(exprs[i].replace("f", ""), {"x": v[0], "y": v[1], "z": v[2]})
            assert abs(val - ref[i]) < 1e-12


def test_sh_low_degree_closed_forms():
    x, y, z = 0.3, -0.5, np.sqrt(1 - 0.34)
    s = oracle.sh(3, x, y, z)
    c0 = 0.5 / np.sqrt(np.pi)
    c1 = np.sqrt(3 / (4 * np.pi))
    assert s[0] == pytest.approx(c0)
    assert s[1:4] == pytest.approx([-c1 * y, c1 * z, -c1 * x])
    assert s[6] == pytest.approx(np.sqrt(5 / (16 * np.pi)) * (3 * z * z - 1))


def _small_model():
    enc = {"otype": "Composite", "nested": [
        {"otype": "HashGrid", "n_dims_to_encode": 3, "n_levels": 4, "log2_hashmap_size": 10, "base_resolution": 4,
         "per_level_scale": 1.5},
        {"otype": "SphericalHarmonics", "n_dims_to_encode": 3, "degree": 3}]}
    net = {"otype": "FullyFusedMLP", "n_neurons": 16, "n_hidden_layers": 2, "activation": "ReLU",
           "output_activation": "Sigmoid"}
    return enc, net


def _fd_check(orc, params, x, objective, g, rng, h=1e-4):
    # 1,024 sampled parameters (network weights + touched grid entries), central differences
    touched = np.nonzero(g)[0]
    idx = rng.choice(touched, size=min(1024, touched.size), replace=False)
    errs = []
    for i in idx:
        p = params.copy()
        p[i] += h
        fp = objective(p)
        p[i] -= 2 * h
        fm = objective(p)
        fd = (fp - fm) / (2 * h)
        errs.append(abs(fd - g[i]) / max(abs(g[i]), 1e-6))
    errs = np.array(errs)
    # ReLU kinks make a handful of samples non-differentiable at h; the bulk must agree
    assert np.median(errs) < 1e-6
    assert np.mean(errs < 1e-3) > 0.99


@pytest.mark.parametrize("loss", ["BinaryCrossEntropy", "RelativeL2", "L2"])
def test_oracle_backward_vs_central_differences(loss):
    """Backward of the loss gradient convention: d/dparams of sum_i c_i y_i(params) with
    c = dL/dy held fixed (tiny-cuda-nn's RelativeL2 treats its denominator y^2 + 0.01 as a
    constant, relative_l2.h:67-70, so its gradient is not the derivative of its value)."""
    enc, net = _small_model()
    orc = oracle.Oracle(enc, net, 6, 1)
    rng = np.random.default_rng(1)
    params = W.test_params(orc.spec, seed=2, grid_scale=0.5).astype(np.float64)
    x, _, _ = W.visibility_inputs(64, seed=3)
    t = rng.random((64, 1)).astype(np.float32)
    _, y16 = orc.forward(x, params, with_y16=True)
    _, dz = orc.loss(loss, y16, t)
    g = orc.backward(x, params, dz)
    y = y16[:, 0]
    c = dz[:, 0] / (y * (1 - y))  # undo the sigmoid derivative: c = dL/dy

    def objective(p):
        return float((c * orc.forward(x, p)[:, 0]).sum())

    _fd_check(orc, params, x, objective, g, rng)


@pytest.mark.parametrize("loss", ["BinaryCrossEntropy", "L2"])
def test_oracle_loss_gradient_vs_central_differences(loss):
    enc, net = _small_model()
    orc = oracle.Oracle(enc, net, 6, 1)
    rng = np.random.default_rng(4)
    params = W.test_params(orc.spec, seed=5, grid_scale=0.5).astype(np.float64)
    x, _, _ = W.visibility_inputs(64, seed=6)
    t = rng.random((64, 1)).astype(np.float32)
    _, g = orc.loss_and_grad(loss, x, params, t)

    def objective(p):
        _, y16 = orc.forward(x, p, with_y16=True)
        return orc.loss(loss, y16, t)[0]

    _fd_check(orc, params, x, objective, g, rng)


def test_oracle_large_batch_and_f32_baseline():
    enc, net = W.throughput_configs()
    orc = oracle.Oracle(enc, net, 10, 3)
    params = W.test_params(orc.spec, seed=3, grid_scale=0.2)
    x = W.throughput_inputs(1 << 14, seed=5)
    ref = orc.forward(x, params)
    out, threads = orc.forward_f32(x, params)
    assert threads >= 1
    assert np.abs(out - ref).max() < 1e-4


def test_loss_values_match_formulas():
    enc, net = _small_model()
    orc = oracle.Oracle(enc, net, 6, 1)
    y16 = np.zeros((4, 16))
    y16[:, 0] = [0.2, 0.7, 1.0, 0.0]
    t = np.array([[0.0], [1.0], [1.0], [0.0]], dtype=np.float32)
    val, dz = orc.loss("BinaryCrossEntropy", y16, t, loss_scale=128.0)
    eps = np.float64(np.float32(1e-5))
    p = np.clip(y16[:, 0], eps, 1 - eps)
    ref = -(t[:, 0] * np.log(p) + (1 - t[:, 0]) * np.log(1 - p)).mean()
    assert val == pytest.approx(ref)
    g = -(t[:, 0] - p) / (p - p * p) * 128 / 4 * (y16[:, 0] * (1 - y16[:, 0]))
    assert dz[:, 0] == pytest.approx(g)
    assert np.all(dz[:, 1:] == 0)


def test_adam_skips_zero_gradient_encoding_params():
    hp = dict(W.VISIBILITY_OPTIMIZER)
    p = np.ones(8, dtype=np.float32)
    g = np.array([1, 0, 2, 0, 0, 3, 0, 1], dtype=np.float32)
    m1 = np.zeros(8, np.float32); m2 = np.zeros(8, np.float32); st = np.zeros(8, np.uint32)
    oracle.adam_step(hp, p, g, m1, m2, st, n_matrix=4)
    # matrix params (first 4) always step; non-matrix params with zero gradient are skipped
    assert list(st) == [1, 1, 1, 1, 0, 1, 0, 1]
    assert p[4] == 1.0 and p[6] == 1.0
    # first Adam step moves every stepped parameter by ~lr against the gradient sign
    assert p[0] == pytest.approx(1 - 1e-2, rel=1e-4)
