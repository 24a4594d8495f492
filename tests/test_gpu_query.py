"""Parity of the fused query forward (nlod_inference) against the FP64 oracle.

Tolerances (stated per form, vs the FP64 oracle on identical FP32 weights and inputs):
  fp32  max |err| <= 2e-5 * (1 + |y|)
  fp16  mean |err| <= 1e-3, max |err| <= 1e-2 * (1 + |y|)
  bf16  mean |err| <= 1e-2, max |err| <= 6e-2 * (1 + |y|)
"""
import numpy as np
import pytest

import oracle
from neural_lod_gb300 import NetworkWithInputEncoding, NlodError, workloads as W

pytestmark = pytest.mark.gpu

TOL = {"fp32": (2e-5, 2e-5), "fp16": (1e-3, 1e-2), "bf16": (1e-2, 6e-2)}


def _check(out, ref, precision):
    mean_tol, max_tol = TOL[precision]
    err = np.abs(out.astype(np.float64) - ref)
    bound = max_tol * (1.0 + np.abs(ref))
    assert np.all(np.isfinite(out))
    if precision == "fp32":
        assert np.all(err <= bound), f"max err {err.max()}"
    else:
        assert err.mean() <= mean_tol, f"mean err {err.mean()}"
        assert np.all(err <= bound), f"max err {err.max()}"
    return err


def _net(cfg, n_in, n_out, precision, seed=3, grid_scale=0.5):
    enc, net = cfg
    spec = oracle.model_spec(enc, net, n_in, n_out)
    params = W.test_params(spec, seed=seed, grid_scale=grid_scale)
    m = NetworkWithInputEncoding(n_in, n_out, enc, net, precision=precision)
    m.set_params(params)
    return m, oracle.Oracle(enc, net, n_in, n_out), params


@pytest.mark.parametrize("precision", ["fp32", "fp16", "bf16"])
def test_visibility_query_with_lod_mask(cuda, nlod_lib, precision):
    import torch

    n = 8192
    m, orc, params = _net(W.visibility_configs(), 6, 1, precision)
    x, lod, frac = W.visibility_inputs(n, seed=11)
    ref = orc.forward(x, params, max_level=frac)
    xd = torch.from_numpy(x).to(cuda)
    fd = torch.from_numpy(frac).to(cuda)
    m.set_max_level_gpu(fd)
    out = m.inference(xd).cpu().numpy()
    m.sync_status()
    _check(out, ref, precision)
    # masking changes the result (the test is not vacuous)
    assert np.abs(orc.forward(x, params) - ref).max() > 1e-3


@pytest.mark.parametrize("precision", ["fp32", "fp16", "bf16"])
def test_throughput_query(cuda, nlod_lib, precision):
    import torch

    n = 16384
    m, orc, params = _net(W.throughput_configs(), 10, 3, precision, grid_scale=0.2)
    x = W.throughput_inputs(n, seed=5)
    ref = orc.forward(x, params)
    out = m.inference(torch.from_numpy(x).to(cuda)).cpu().numpy()
    m.sync_status()
    err = _check(out, ref, precision)
    # per-channel error is reported by the test log
    print(precision, "per-channel mean abs err", err.mean(axis=0))


@pytest.mark.parametrize("precision", ["fp32", "fp16"])
def test_visibility16_query(cuda, nlod_lib, precision):
    import torch

    n = 4096
    m, orc, params = _net(W.visibility_configs(16), 6, 1, precision)
    x, _, _ = W.visibility_inputs(n, seed=2)
    ref = orc.forward(x, params)
    out = m.inference(torch.from_numpy(x).to(cuda)).cpu().numpy()
    _check(out, ref, precision)


@pytest.mark.parametrize("precision", ["fp32", "fp16", "bf16"])
def test_identity_hidden_activation(cuda, nlod_lib, precision):
    """Hidden activation "None": the identity branch of every hidden epilogue."""
    import torch

    enc, net = W.throughput_configs()
    net = dict(net, activation="None", output_activation="Sigmoid")
    m, orc, params = _net((enc, net), 10, 3, precision)
    x = W.throughput_inputs(4096, seed=21)
    ref = orc.forward(x, params)
    out = m.inference(torch.from_numpy(x).to(cuda)).cpu().numpy()
    _check(out, ref, precision)


@pytest.mark.parametrize("precision", ["fp32", "fp16"])
def test_width128_sh8_config(cuda, nlod_lib, precision):
    """The shipped arcade throughput configuration shape: 7-level grid (base 8, scale 2),
    two degree-8 SH encodings (the second one padded first), 128-wide MLP."""
    import torch

    enc = {"otype": "Composite", "nested": [
        {"otype": "HashGrid", "n_dims_to_encode": 3, "n_levels": 7, "n_features_per_level": 2, "log2_hashmap_size": 19,
         "base_resolution": 8, "per_level_scale": 2.0},
        {"otype": "SphericalHarmonics", "n_dims_to_encode": 3, "degree": 8},
        {"otype": "SphericalHarmonics", "n_dims_to_encode": 3, "degree": 8}]}
    net = {"otype": "FullyFusedMLP", "n_neurons": 128, "n_hidden_layers": 4, "activation": "ReLU", "output_activation": "None"}
    m, orc, params = _net((enc, net), 9, 3, precision, grid_scale=0.3)
    rng = np.random.default_rng(4)
    d1 = rng.standard_normal((2048, 3)); d1 /= np.linalg.norm(d1, axis=1, keepdims=True)
    d2 = rng.standard_normal((2048, 3)); d2 /= np.linalg.norm(d2, axis=1, keepdims=True)
    x = np.concatenate([rng.random((2048, 3)), (d1 + 1) / 2, (d2 + 1) / 2], axis=1).astype(np.float32)
    ref = orc.forward(x, params)
    out = m.inference(torch.from_numpy(x).to(cuda)).cpu().numpy()
    _check(out, ref, precision)


def test_dense_and_nearest_grids(cuda, nlod_lib):
    import torch

    enc = {"otype": "Composite", "nested": [
        {"otype": "DenseGrid", "n_dims_to_encode": 3, "n_levels": 4, "base_resolution": 8, "per_level_scale": 1.7,
         "interpolation": "Nearest"},
        {"otype": "HashGrid", "n_dims_to_encode": 3, "n_levels": 4, "log2_hashmap_size": 12, "hash": "Prime",
         "interpolation": "Smoothstep"},
        {"otype": "Identity", "n_dims_to_encode": 2, "scale": 2.0, "offset": -1.0}]}
    net = {"otype": "FullyFusedMLP", "n_neurons": 64, "n_hidden_layers": 3, "activation": "ReLU", "output_activation": "None"}
    for precision in ("fp32", "fp16"):
        m, orc, params = _net((enc, net), 8, 2, precision, grid_scale=0.5)
        x = np.random.default_rng(9).random((1024, 8)).astype(np.float32) * 1.2 - 0.1  # some inputs outside [0,1]
        ref = orc.forward(x, params)
        out = m.inference(torch.from_numpy(x).to(cuda)).cpu().numpy()
        _check(out, ref, precision)


def test_dense_level_cell_table(cuda, nlod_lib):
    """The FP16 form reads the corners of a dense level's cell from the cell table (one 32-byte
    record per cell, rebuilt with the FP16 tables); positions on the grid's far faces (whose
    corners wrap past the level's last entry), outside [0,1] (no record: the corners are gathered)
    and inside all match the oracle, and the leading dense levels of a hash grid too."""
    import torch

    enc = {"otype": "Composite", "nested": [
        {"otype": "DenseGrid", "n_dims_to_encode": 3, "n_levels": 3, "base_resolution": 6, "per_level_scale": 1.5},
        {"otype": "Identity", "n_dims_to_encode": 1}]}
    net = {"otype": "FullyFusedMLP", "n_neurons": 64, "n_hidden_layers": 2, "activation": "ReLU", "output_activation": "None"}
    rng = np.random.default_rng(12)
    x = rng.random((2048, 4)).astype(np.float32)
    x[:256, :3] = rng.integers(0, 2, (256, 3)).astype(np.float32)      # cube corners and faces
    x[256:512, :3] = x[256:512, :3] * 1.3 - 0.15                        # outside [0,1]
    for cfg, n_in, xs in (((enc, net), 4, x), (W.throughput_configs(), 10, W.throughput_inputs(2048, seed=13))):
        m, orc, params = _net(cfg, n_in, 3 if n_in == 10 else 1, "fp16", grid_scale=0.5)
        ref = orc.forward(xs, params)
        out = m.inference(torch.from_numpy(xs).to(cuda)).cpu().numpy()
        m.sync_status()
        _check(out, ref, "fp16")


@pytest.mark.parametrize("precision", ["fp16", "bf16"])
def test_every_kernel_variant_and_autotune(cuda, nlod_lib, precision):
    """Each tensor-core kernel organisation the autotuner may pick computes the same result."""
    import torch

    m, orc, params = _net(W.throughput_configs(), 10, 3, precision, grid_scale=0.2)
    x = W.throughput_inputs(8192 + 128 * 5, seed=6)   # tile count not a multiple of any group count
    ref = orc.forward(x, params)
    xd = torch.from_numpy(x).to(cuda)
    outs = []
    assert m.n_kernel_variants >= 4
    for v in range(m.n_kernel_variants):
        try:
            m.kernel_variant = v
        except NlodError as e:
            assert e.code == 4  # variant does not fit this network
            continue
        out = m.inference(xd).cpu().numpy()
        m.sync_status()
        _check(out, ref, precision)
        outs.append(out)
    assert len(outs) >= 4
    for o in outs[1:]:
        assert np.array_equal(o, outs[0])  # same arithmetic in every organisation
    best = m.autotune(xd)
    assert 0 <= best < m.n_kernel_variants


@pytest.mark.parametrize("precision", ["fp16", "bf16"])
def test_every_kernel_variant_visibility_with_lod_mask(cuda, nlod_lib, precision):
    """The same on the visibility network with a per-element max level: organisations that split a
    tile row's grid levels between two threads (the LoD mask then falls on either part) compute
    the same bits as the others."""
    import torch

    m, orc, params = _net(W.visibility_configs(), 6, 1, precision, grid_scale=0.3)
    x, _, frac = W.visibility_inputs(4096 + 128 * 3, seed=7)
    ref = orc.forward(x, params, max_level=frac)
    m.set_max_level_gpu(torch.from_numpy(frac).to(cuda))
    xd = torch.from_numpy(x).to(cuda)
    outs = []
    for v in range(m.n_kernel_variants):
        try:
            m.kernel_variant = v
        except NlodError as e:
            assert e.code == 4
            continue
        out = m.inference(xd).cpu().numpy()
        m.sync_status()
        _check(out, ref, precision)
        outs.append(out)
    assert len(outs) >= 10
    for o in outs[1:]:
        assert np.array_equal(o, outs[0])


def test_batch_must_be_multiple_of_128(cuda, nlod_lib):
    import torch

    m, _, _ = _net(W.visibility_configs(), 6, 1, "fp16")
    x = torch.zeros((100, 6), device=cuda)
    with pytest.raises(NlodError) as e:
        m.inference(x)
    assert e.value.code == 1
    # empty batch is a no-op
    m.inference(torch.zeros((0, 6), device=cuda))


def test_deterministic(cuda, nlod_lib):
    import torch

    m, _, _ = _net(W.throughput_configs(), 10, 3, "fp16", grid_scale=0.2)
    x = torch.from_numpy(W.throughput_inputs(4096, seed=8)).to(cuda)
    a = m.inference(x).cpu().numpy()
    b = m.inference(x).cpu().numpy()
    assert np.array_equal(a, b)


@pytest.mark.parametrize("precision", ["fp16", "fp32"])
def test_inference_from_host_buffers(cuda, nlod_lib, precision):
    """nlod_inference_host: a pinned input read in place, a pageable one staged; pinned and
    pageable outputs; every combination gives the device call's outputs bit for bit."""
    import torch

    m, _, _ = _net(W.throughput_configs(), 10, 3, precision, grid_scale=0.2)
    xh = torch.from_numpy(W.throughput_inputs(8192, seed=9))
    ref = m.inference(xh.to(cuda)).cpu()
    pinned = m.inference_host(xh.pin_memory())
    torch.cuda.synchronize()
    assert pinned.is_pinned() and torch.equal(pinned, ref)
    out = torch.zeros((8192, 3), dtype=torch.float32)        # pageable output and input
    m.inference_host(xh.clone(), out)
    torch.cuda.synchronize()
    assert torch.equal(out, ref)
    out2 = torch.zeros((8192, 3), dtype=torch.float32)       # pinned input, pageable output
    m.inference_host(xh.pin_memory(), out2)
    torch.cuda.synchronize()
    assert torch.equal(out2, ref)
    out3 = torch.zeros((8192, 3), dtype=torch.float32).pin_memory()   # pageable input, pinned output
    m.inference_host(xh.clone(), out3)
    torch.cuda.synchronize()
    assert torch.equal(out3, ref)
    with pytest.raises(ValueError):
        m.inference_host(xh.to(cuda))
    # a large batch
    nb = (1 << 19) + 128 * 7
    xb = torch.from_numpy(W.throughput_inputs(nb, seed=10))
    refb = m.inference(xb.to(cuda)).cpu()
    outb = m.inference_host(xb.pin_memory())
    torch.cuda.synchronize()
    assert torch.equal(outb, refb)


@pytest.mark.parametrize("with_ema", [False, True])
def test_inference_after_training_reads_current_grid_tables(cuda, nlod_lib, with_ema):
    """The FP16 form gathers from an FP16 copy of the grid tables that the optimizer step refreshes
    in place: after training, inference equals a fresh module loaded with the inference
    parameters, bit for bit."""
    import torch

    enc, net = W.throughput_configs()
    opt = W.THROUGHPUT_OPTIMIZER if with_ema else W.THROUGHPUT_OPTIMIZER["nested"]["nested"]
    m = NetworkWithInputEncoding(10, 3, enc, net, loss=W.THROUGHPUT_LOSS, optimizer=opt, precision="fp16")
    spec = oracle.model_spec(enc, net, 10, 3)
    m.set_params(W.test_params(spec, seed=4, grid_scale=0.2))
    x = torch.from_numpy(W.throughput_inputs(4096, seed=10)).to(cuda)
    t = torch.rand((4096, 3), device=cuda)
    y0 = m.inference(x).clone()
    for _ in range(3):
        m.training_step(x, t)
    y1 = m.inference(x)
    m.sync_status()
    assert not torch.equal(y0, y1)
    fresh = NetworkWithInputEncoding(10, 3, enc, net, precision="fp16")
    fresh.set_params(m.get_params("inference"))
    assert torch.equal(fresh.inference(x), y1)


def test_calibration_floors(cuda, nlod_lib):
    """The gather and scatter floors run on a module's grid and take less time than the kernels
    they bound: the query kernel does the same gathers and more, the training step the same
    scatter and more."""
    import torch

    enc, net = W.throughput_configs()
    m = NetworkWithInputEncoding(10, 3, enc, net, loss=W.THROUGHPUT_LOSS, optimizer=W.THROUGHPUT_OPTIMIZER, precision="fp16")
    m.set_params(W.xavier_params(oracle.model_spec(enc, net, 10, 3), seed=10))
    n = 1 << 17
    x = torch.from_numpy(W.throughput_inputs(n, seed=1)).to(cuda)
    out = torch.empty((n, 3), device=cuda)
    for _ in range(2):
        g = m.calib_gathers(n)
        s = m.calib_scatter(n)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    m.inference(x, out)
    e0.record()
    m.inference(x, out)
    e1.record()
    e1.synchronize()
    q = e0.elapsed_time(e1)
    m.sync_status()
    print(f"\ngathers {g:.4f} ms, scatter {s:.4f} ms, query {q:.4f} ms for {n} elements")
    assert 0.0 < g < 1.5 * q
    assert s > 0.0
    # the scatter left the gradients dirty: a training step starts from cleared gradients
    t = torch.rand((n, 3), device=cuda)
    loss = m.training_step(x, t).item()
    m.sync_status()
    assert np.isfinite(loss)


def test_captured_inference_after_training_without_cell_rebuild(cuda, nlod_lib):
    """Inference captured in a CUDA graph before training still reads current values when it is
    replayed after an optimizer step that nothing has rebuilt the cell table for since: the step
    marks the table out of date on the device and the kernel then gathers the corners."""
    import torch

    enc, net = W.throughput_configs()
    opt = W.THROUGHPUT_OPTIMIZER["nested"]["nested"]
    m = NetworkWithInputEncoding(10, 3, enc, net, loss=W.THROUGHPUT_LOSS, optimizer=opt, precision="fp16")
    spec = oracle.model_spec(enc, net, 10, 3)
    m.set_params(W.test_params(spec, seed=5, grid_scale=0.2))
    x = torch.from_numpy(W.throughput_inputs(4096, seed=11)).to(cuda)
    t = torch.rand((4096, 3), device=cuda)
    out = torch.empty((4096, 3), device=cuda)
    side = torch.cuda.Stream()
    with torch.cuda.stream(side):
        m.inference(x, out)                      # cell table current: nothing to rebuild in the capture
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=side):
            m.inference(x, out)
    torch.cuda.synchronize()
    y0 = out.clone()
    m.training_step(x, t)
    torch.cuda.synchronize()
    g.replay()
    torch.cuda.synchronize()
    m.sync_status()
    y1 = out.clone()
    assert not torch.equal(y0, y1)
    fresh = NetworkWithInputEncoding(10, 3, enc, net, precision="fp16")
    fresh.set_params(m.get_params("inference"))
    assert torch.equal(fresh.inference(x), y1)
    assert torch.equal(m.inference(x), y1)     # rebuilt table, same values
