"""Network configurations and seeded synthetic inputs of the neural-LoD workloads.

Configurations are tiny-cuda-nn style JSON (the form neural_lod builds in
rptr/cuda/neural-lod/neural_lod_learning_init.cu:577-676, 822-911), sized as:

  visibility_query   position U[0,1]^3 + direction on S^2 (fed as (d+1)/2) + LoD in {0..7}
                     applied as a per-element grid max-level (GridEncoding::set_max_level_gpu);
                     8-level hash grid (F=2, 2^16 entries/level, base 16, scale 1.5) + SH degree 4;
                     MLP 32 -> 64 -> 64 -> 1 (sigmoid); batch 65,536.
  throughput_query   position + wi + wo + LoD one-hot over 8; 16-level hash grid (2^19 entries),
                     SH degree 4 for each direction; MLP 72 (padded to 80) -> 4 x 64 -> 3 (exp);
                     batch 2^21.
  visibility_train   visibility_query's architecture with 16 levels (input 48), BCE loss,
                     Adam lr 1e-2, beta 0.9/0.99, eps 1e-15; batch 2^18.
Inputs are generated from one uint64 seed with numpy's PCG64 so every run and the oracle see
identical data.  These seeded synthetic inputs stand in for the paper's scenes, which are not
available.
"""
from __future__ import annotations

import numpy as np


def visibility_configs(n_levels: int = 8, log2T: int = 16):
    encoding = {
        "otype": "Composite",
        "nested": [
            {"otype": "HashGrid", "n_dims_to_encode": 3, "n_levels": n_levels, "n_features_per_level": 2,
             "log2_hashmap_size": log2T, "base_resolution": 16, "per_level_scale": 1.5},
            {"otype": "SphericalHarmonics", "n_dims_to_encode": 3, "degree": 4},
        ],
    }
    network = {"otype": "FullyFusedMLP", "n_neurons": 64, "n_hidden_layers": 2, "activation": "ReLU",
               "output_activation": "Sigmoid"}
    return encoding, network


def throughput_configs():
    encoding = {
        "otype": "Composite",
        "nested": [
            {"otype": "HashGrid", "n_dims_to_encode": 3, "n_levels": 16, "n_features_per_level": 2,
             "log2_hashmap_size": 19, "base_resolution": 16, "per_level_scale": 1.5},
            {"otype": "SphericalHarmonics", "n_dims_to_encode": 3, "degree": 4},
            {"otype": "SphericalHarmonics", "n_dims_to_encode": 3, "degree": 4},
            {"otype": "OneHot", "n_dims_to_encode": 1, "n_bins": 8},
        ],
    }
    network = {"otype": "FullyFusedMLP", "n_neurons": 64, "n_hidden_layers": 4, "activation": "ReLU",
               "output_activation": "Exponential"}
    return encoding, network


def arcade_throughput_configs():
    """The throughput network shipped with the reference's arcade scene
    (neural_lod/scenes/arcade/learned_weights/arcade_world_final_512_throughput_config.json):
    position hash grid (7 levels, base 8, scale 2, 2^19 entries) + SH degree 8 for wo and for wi ->
    128 x 4 ReLU -> 3 linear; RelativeL2; Ema(0.95) of ExponentialDecay(0.33 every 4000 from 8000)
    of Adam (lr 5e-3, beta 0.9/0.99, eps 1e-15, l2 1e-8).  Returns (encoding, network, loss,
    optimizer) for a 9-input, 3-output module."""
    encoding = {"otype": "Composite", "nested": [
        {"otype": "HashGrid", "n_dims_to_encode": 3, "n_levels": 7, "n_features_per_level": 2, "log2_hashmap_size": 19,
         "base_resolution": 8, "per_level_scale": 2.0, "interpolation": "Linear"},
        {"otype": "SphericalHarmonics", "n_dims_to_encode": 3, "degree": 8},
        {"otype": "SphericalHarmonics", "n_dims_to_encode": 3, "degree": 8},
    ]}
    network = {"otype": "FullyFusedMLP", "activation": "ReLU", "output_activation": "None", "n_neurons": 128, "n_hidden_layers": 4}
    loss = {"otype": "RelativeL2"}
    optimizer = {"otype": "Ema", "decay": 0.95, "nested": {
        "otype": "ExponentialDecay", "decay_base": 0.33, "decay_interval": 4000, "decay_start": 8000, "nested": {
            "otype": "Adam", "learning_rate": 5e-3, "beta1": 0.9, "beta2": 0.99, "epsilon": 1e-15, "l2_reg": 1e-8,
            "relative_decay": 0.0, "absolute_decay": 0.0, "adabound": False}}}
    return encoding, network, loss, optimizer


VISIBILITY_LOSS = {"otype": "BinaryCrossEntropy"}
VISIBILITY_OPTIMIZER = {"otype": "Adam", "learning_rate": 1e-2, "beta1": 0.9, "beta2": 0.99, "epsilon": 1e-15,
                        "l2_reg": 1e-8}
THROUGHPUT_LOSS = {"otype": "RelativeL2"}
THROUGHPUT_OPTIMIZER = {"otype": "Ema", "decay": 0.95, "nested": {
    "otype": "ExponentialDecay", "decay_start": 8000, "decay_interval": 4000, "decay_base": 0.33,
    "nested": {"otype": "Adam", "learning_rate": 5e-3, "beta1": 0.9, "beta2": 0.99, "epsilon": 1e-15,
               "l2_reg": 1e-8}}}

WORKLOADS = {
    "visibility_query": {"batch": 65536, "n_input": 6, "n_output": 1},
    "throughput_query": {"batch": 1 << 21, "n_input": 10, "n_output": 3},
    "visibility_train": {"batch": 1 << 18, "n_input": 6, "n_output": 1},
}


def pack_bits(occ: np.ndarray) -> np.ndarray:
    """[res,res,res] bool indexed [z,y,x] -> uint32 words, bit x + y*res + z*res^2, most
    significant bit first (the cuda_voxelizer grid layout, rptr voxelize.cu:50-55)."""
    flat = np.ascontiguousarray(occ, dtype=bool).reshape(-1)
    pad = (-flat.size) % 32
    if pad:
        flat = np.concatenate([flat, np.zeros(pad, bool)])
    return np.packbits(flat.reshape(-1, 32), axis=1, bitorder="big").view(">u4").reshape(-1).astype(np.uint32)


def unpack_bits(words: np.ndarray, res: int) -> np.ndarray:
    b = np.unpackbits(np.asarray(words, dtype=np.uint32).astype(">u4").view(np.uint8), bitorder="big")
    return b[: res ** 3].astype(bool).reshape(res, res, res)


def value_noise_occupancy(res: int, seed: int = 0, spacing: int = 16, density: float = 0.3) -> np.ndarray:
    """Seeded occupancy [z,y,x]: a lattice of U[0,1] values every `spacing` voxels, trilinearly
    interpolated at voxel centres and thresholded so that `density` of the voxels are occupied."""
    rng = np.random.Generator(np.random.PCG64(seed))
    n = res // spacing + 2
    lat = rng.random((n, n, n))
    c = (np.arange(res) + 0.5) / spacing
    i0 = np.floor(c).astype(np.int64)
    f = c - i0
    # separable trilinear interpolation along x, then y, then z
    a = lat[:, :, i0] * (1 - f) + lat[:, :, i0 + 1] * f
    a = a[:, i0, :] * (1 - f)[None, :, None] + a[:, i0 + 1, :] * f[None, :, None]
    a = a[i0, :, :] * (1 - f)[:, None, None] + a[i0 + 1, :, :] * f[:, None, None]
    thr = np.quantile(a, 1.0 - density)
    return a > thr


def _unit_dirs(rng: np.random.Generator, n: int) -> np.ndarray:
    v = rng.standard_normal((n, 3))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    return v


def visibility_inputs(n: int, seed: int = 0, n_grid_levels: int = 8):
    """Returns (x [n,6] float32, lod [n] int32, max_level_frac [n] float32).

    LoD k keeps grid levels 0..(n_grid_levels-1-k): fraction (n_grid_levels-1-k)/n_grid_levels.
    """
    rng = np.random.Generator(np.random.PCG64(seed))
    pos = rng.random((n, 3))
    d = _unit_dirs(rng, n)
    lod = rng.integers(0, 8, size=n).astype(np.int32)
    x = np.concatenate([pos, (d + 1.0) * 0.5], axis=1).astype(np.float32)
    frac = (np.float32(n_grid_levels - 1) - lod.astype(np.float32)).clip(0) / np.float32(n_grid_levels)
    return x, lod, frac.astype(np.float32)


def throughput_inputs(n: int, seed: int = 1):
    """Returns x [n,10] float32: position, (wi+1)/2, (wo+1)/2, (lod + 0.5)/8."""
    rng = np.random.Generator(np.random.PCG64(seed))
    pos = rng.random((n, 3))
    wi = _unit_dirs(rng, n)
    wo = _unit_dirs(rng, n)
    lod = rng.integers(0, 8, size=n)
    x = np.concatenate([pos, (wi + 1.0) * 0.5, (wo + 1.0) * 0.5, ((lod + 0.5) / 8.0)[:, None]], axis=1)
    return x.astype(np.float32)


def thr_identity_configs():
    """The throughput network with the LoD one-hot given as 8 identity inputs (17 inputs: position,
    wi, wo, one-hot).  The encoded input is the same 72 columns as throughput_configs(); this is the
    form tiny-cuda-nn can build, since it has no one-hot encoding."""
    enc, net = throughput_configs()
    enc = {"otype": "Composite", "nested": enc["nested"][:3] + [{"otype": "Identity", "n_dims_to_encode": 8}]}
    return enc, net


def thr_identity_inputs(n: int, seed: int = 1) -> np.ndarray:
    """throughput_inputs(n, seed) with the LoD column expanded to its one-hot row: float32 [n, 17]."""
    x = throughput_inputs(n, seed=seed)
    lod = np.floor(x[:, 9] * 8).astype(np.int64)
    onehot = np.zeros((n, 8), np.float32)
    onehot[np.arange(n), lod] = 1.0
    return np.concatenate([x[:, :9], onehot], axis=1).astype(np.float32)


def binary_targets(n: int, seed: int) -> np.ndarray:
    """Seeded 0/1 visibility targets, float32 [n, 1]."""
    return (np.random.default_rng(seed).random((n, 1)) < 0.5).astype(np.float32)


def rgb_targets(n: int, seed: int) -> np.ndarray:
    """Seeded RGB throughput targets U[0.05, 1], float32 [n, 3]."""
    return np.random.default_rng(seed).uniform(0.05, 1.0, (n, 3)).astype(np.float32)


def xavier_params(spec: dict, seed: int = 7) -> np.ndarray:
    """FP32 parameter vector for a layout spec: Xavier-uniform matrices (gpu_matrix.h:291-306),
    grid entries U[-1e-4, 1e-4] (grid.h:1353-1356), scaled up by `grid_gain` for test signal."""
    rng = np.random.Generator(np.random.PCG64(seed))
    p = np.empty(spec["n_params"], dtype=np.float32)
    for l in spec["layers"]:
        s = np.sqrt(6.0 / (l["in"] + l["out"]))
        p[l["offset"]:l["offset"] + l["in"] * l["out"]] = rng.uniform(-s, s, l["in"] * l["out"])
    n_net = spec["n_params_network"]
    p[n_net:] = rng.uniform(-1e-4, 1e-4, spec["n_params"] - n_net)
    return p


def test_params(spec: dict, seed: int = 7, grid_scale: float = 0.5) -> np.ndarray:
    """Like xavier_params but with grid entries U[-grid_scale, grid_scale], so the grid features
    carry signal through the MLP (used by the parity tests)."""
    p = xavier_params(spec, seed)
    rng = np.random.Generator(np.random.PCG64(seed + 1))
    n_net = spec["n_params_network"]
    p[n_net:] = rng.uniform(-grid_scale, grid_scale, spec["n_params"] - n_net)
    return p


def _rotations(rng: np.random.Generator, n: int) -> np.ndarray:
    """n random rotation matrices [n,3,3] (QR of Gaussian matrices, sign-fixed)."""
    q, r = np.linalg.qr(rng.standard_normal((n, 3, 3)))
    q *= np.sign(np.diagonal(r, axis1=1, axis2=2))[:, None, :]
    return q


def ellipsoid_shells(n: int, seed: int = 0, slices: int = 8, stacks: int = 4, radius=(0.004, 0.02)) -> np.ndarray:
    """n randomly placed, oriented and scaled ellipsoid shells inside the unit cube, each a UV
    sphere of 2*slices*(stacks-1) triangles.  Returns float32 [n*tris, 9]."""
    rng = np.random.Generator(np.random.PCG64(seed))
    th = np.pi * np.arange(1, stacks) / stacks
    ph = 2 * np.pi * np.arange(slices) / slices
    ring = np.stack([np.sin(th)[:, None] * np.cos(ph)[None], np.sin(th)[:, None] * np.sin(ph)[None],
                     np.broadcast_to(np.cos(th)[:, None], (stacks - 1, slices))], -1).reshape(-1, 3)
    verts = np.concatenate([[[0, 0, 1]], ring, [[0, 0, -1]]])            # [2 + slices*(stacks-1), 3]
    top, bot = 0, len(verts) - 1
    idx = lambda s, j: 1 + s * slices + (j % slices)
    tri = [(top, idx(0, j), idx(0, j + 1)) for j in range(slices)]
    for s in range(stacks - 2):
        for j in range(slices):
            tri += [(idx(s, j), idx(s + 1, j), idx(s + 1, j + 1)), (idx(s, j), idx(s + 1, j + 1), idx(s, j + 1))]
    tri += [(idx(stacks - 2, j), bot, idx(stacks - 2, j + 1)) for j in range(slices)]
    tri = np.asarray(tri)
    radii = rng.uniform(radius[0], radius[1], (n, 3))
    centre = rng.uniform(radius[1], 1 - radius[1], (n, 3))
    rot = _rotations(rng, n)
    local = verts[None, :, :] * radii[:, None, :]                          # [n, V, 3]
    world = np.einsum("nij,nvj->nvi", rot, local) + centre[:, None, :]
    return world[:, tri, :].reshape(-1, 9).astype(np.float32)


def foliage_quads(n: int, seed: int = 1, side=(1e-3, 1e-2)) -> np.ndarray:
    """n randomly oriented rectangles with sides U[side] inside the unit cube, two triangles each.
    Returns float32 [2n, 9]."""
    rng = np.random.Generator(np.random.PCG64(seed))
    rot = _rotations(rng, n)
    a = rng.uniform(side[0], side[1], (n, 1)) * rot[:, :, 0]
    b = rng.uniform(side[0], side[1], (n, 1)) * rot[:, :, 1]
    m = side[1]
    c = rng.uniform(m, 1 - m, (n, 3))
    p00, p10, p11, p01 = c - (a + b) / 2, c + (a - b) / 2, c + (a + b) / 2, c + (b - a) / 2
    t = np.stack([np.concatenate([p00, p10, p11], 1), np.concatenate([p00, p11, p01], 1)], 1)
    return t.reshape(-1, 9).astype(np.float32)


def synthetic_mesh(n_ellipsoids: int = 20_000, n_quads: int = 520_000, seed: int = 0) -> np.ndarray:
    """The voxelize+train scene: ellipsoid shells (48 triangles each) plus foliage-like quads in the
    unit cube; defaults give 20k shells + 0.52M quads = 2.0M triangles.  float32 [n, 9]."""
    parts = [ellipsoid_shells(n_ellipsoids, seed=seed), foliage_quads(n_quads, seed=seed + 1)]
    return np.concatenate(parts, 0)
