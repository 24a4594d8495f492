"""The oracle's grid encoding against a second, independent restatement written in numpy directly
from tiny-cuda-nn's grid.h (paths relative to rptr/ext/tiny-cuda-nn/include/tiny-cuda-nn/):
encodings/grid.h:111-135 (lcg_hash and its prime tables), :170-187 (grid_index: dense index while
the stride fits, hash beyond, modulo the level size), :236-265 (per-element max_level masking) and
:266-392 (n-linear interpolation over the 8 corners); common_device.h:437-464 (pos_fract,
p = x * scale + 0.5 fused, cell = floor(p)).

Both restatements take the level offsets, resolutions and scales from the layout (whose sizes are
pinned separately by the reference's offset-table totals); this test pins the indexing, hashing,
interpolation and masking.  A wrong corner entry changes a feature by O(0.1): the tolerance is
1e-12."""
import numpy as np
import pytest

import oracle
from neural_lod_gb300 import workloads as W

_PRIMES = {0: (1, 2654435761, 805459861), 1: (1958374283, 2654435761, 805459861),
           2: (2165219737, 1434869437, 2097192037)}


def _pos_fract(x, scale):
    # fmaf(x, scale, 0.5f): the product of two floats is exact in float64; one rounding to float32
    p = (x.astype(np.float64) * np.float64(scale) + 0.5).astype(np.float32)
    cell = np.floor(p)
    return (p - cell).astype(np.float32), cell.astype(np.int64).astype(np.uint32)


def _index(g, level, pos):
    size = np.uint64(g["offset"][level + 1] - g["offset"][level])
    res = np.uint64(g["res"][level])
    stride, index = np.uint64(1), np.zeros(pos.shape[0], np.uint64)
    for d in range(3):
        if stride > size:
            break
        index = (index + pos[:, d].astype(np.uint64) * stride) & np.uint64(0xFFFFFFFF)
        stride = stride * res
    if g["kind"] == 0 and size < stride:
        pr = _PRIMES[g["hash"]]
        h = np.zeros(pos.shape[0], np.uint64)
        for d in range(3):
            h ^= (pos[:, d].astype(np.uint64) * np.uint64(pr[d])) & np.uint64(0xFFFFFFFF)
        index = h
    return (index % size).astype(np.int64)


def _encode_grid(g, xyz, table, ml):
    n_lv = g["n_levels"]
    out = np.zeros((xyz.shape[0], 2 * n_lv))
    max_level = (ml * np.float32(2 * n_lv)) / np.float32(2)
    for level in range(n_lv):
        live = ~(np.float32(level) >= max_level + np.float32(1e-3))
        frac, cell = zip(*(_pos_fract(xyz[:, d], np.float32(g["scale"][level])) for d in range(3)))
        frac, cell = np.stack(frac, 1).astype(np.float64), np.stack(cell, 1)
        lv = table[2 * g["offset"][level]:2 * g["offset"][level + 1]].reshape(-1, 2)
        if g["interp"] == 1:
            val = lv[_index(g, level, cell)]
        else:
            t = frac if g["interp"] == 0 else frac * frac * (3.0 - 2.0 * frac)
            val = np.zeros((xyz.shape[0], 2))
            for c in range(8):
                w = np.ones(xyz.shape[0])
                q = cell.copy()
                for d in range(3):
                    if c >> d & 1:
                        w *= t[:, d]
                        q[:, d] += np.uint32(1)
                    else:
                        w *= 1.0 - t[:, d]
                val += w[:, None] * lv[_index(g, level, q)]
        out[:, 2 * level:2 * level + 2] = np.where(live[:, None], val, 0.0)
    return out


CONFIGS = {
    "visibility_16": (W.visibility_configs(16), 6, 1),
    "throughput": (W.throughput_configs(), 10, 3),
    "dense_nearest_prime_smoothstep": (({"otype": "Composite", "nested": [
        {"otype": "DenseGrid", "n_dims_to_encode": 3, "n_levels": 4, "base_resolution": 8, "per_level_scale": 1.7,
         "interpolation": "Nearest"},
        {"otype": "HashGrid", "n_dims_to_encode": 3, "n_levels": 4, "log2_hashmap_size": 12, "hash": "Prime",
         "interpolation": "Smoothstep"}]},
        {"otype": "FullyFusedMLP", "n_neurons": 64, "n_hidden_layers": 1, "activation": "ReLU", "output_activation": "None"}), 6, 1),
    "reversed_prime_and_tiled": (({"otype": "Composite", "nested": [
        {"otype": "HashGrid", "n_dims_to_encode": 3, "n_levels": 5, "log2_hashmap_size": 10, "hash": "ReversedPrime",
         "base_resolution": 8},
        {"otype": "TiledGrid", "n_dims_to_encode": 3, "n_levels": 3, "base_resolution": 6, "per_level_scale": 2.0}]},
        {"otype": "FullyFusedMLP", "n_neurons": 64, "n_hidden_layers": 1, "activation": "ReLU", "output_activation": "None"}), 6, 1),
}


@pytest.mark.parametrize("name", sorted(CONFIGS))
def test_grid_encoding_matches_independent_restatement(name):
    (enc, net), n_in, n_out = CONFIGS[name]
    orc = oracle.Oracle(enc, net, n_in, n_out)
    spec = orc.spec
    rng = np.random.Generator(np.random.PCG64(17))
    n = 2048
    x = rng.random((n, n_in)).astype(np.float32) * np.float32(1.2) - np.float32(0.1)  # some outside [0, 1]
    ml = rng.random(n).astype(np.float32)
    params = W.test_params(spec, seed=5, grid_scale=0.5)
    got = orc.encode(x, params, max_level=ml)
    n_grid_slots = 0
    for s in spec["slots"]:
        if s["type"] != 0:
            continue
        n_grid_slots += 1
        g = spec["grids"][s["grid"]]
        table = params[g["param_offset"]:g["param_offset"] + g["n_params"]].astype(np.float64)
        ref = _encode_grid(g, x[:, s["in_begin"]:s["in_begin"] + 3], table, ml)
        cols = slice(s["out_begin"], s["out_begin"] + 2 * g["n_levels"])
        np.testing.assert_allclose(got[:, cols], ref, rtol=0, atol=1e-12, err_msg=f"{name} slot at {s['out_begin']}")
    assert n_grid_slots >= 1
