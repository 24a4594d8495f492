"""Training-sample generation for the visibility and throughput networks with exact-DDA targets.

The reference generates training samples with Vulkan ray queries against the scene
(rptr/cuda/neural-lod/neural_lod_learning_kernels.cuh:100-238, 364-569: voxel + LoD sampling, then
visibility / throughput targets traced in the renderer).  Here the targets come from the LoD
pyramid itself through the bit-exact first-active-voxel search (LodGrid.first_active_voxel), which
is what "exact DDA transmittance" means for a voxelized scene:

  * visibility: a segment of length U[0, max_len] (normalised units) from a uniform position in a
    uniform direction; target 1 when no occupied voxel of the sample's LoD begins before the
    segment ends, else 0.  Input: position, (dir + 1) / 2; per-element max level (7 - lod) / 8.
  * throughput: the centre of a uniformly chosen occupied voxel of LoD k, wi and wo uniform on the
    sphere; target = albedo(centre) * T, T = 1 when the ray from the centre along wi meets no other
    occupied voxel of LoD k that begins closer than `min_dist` voxels (the voxel's own surface
    sheet - its immediate neighbours - does not shadow it).  Input: centre, (wi+1)/2, (wo+1)/2,
    (k+0.5)/8.
"""
from __future__ import annotations

import numpy as np

from .workloads import _unit_dirs


def _bit_set(words: np.ndarray, res: int, ijk: np.ndarray) -> np.ndarray:
    idx = ijk[:, 0].astype(np.int64) + ijk[:, 1].astype(np.int64) * res + ijk[:, 2].astype(np.int64) * res * res
    return ((words[idx >> 5] >> (31 - (idx & 31)).astype(np.uint32)) & 1).astype(bool)


def occupied_voxels(words: np.ndarray, res: int, n: int, rng: np.random.Generator, max_rounds: int = 64) -> np.ndarray:
    """n voxel coordinates drawn uniformly among the occupied voxels (rejection sampling)."""
    out = np.zeros((0, 3), np.int32)
    for _ in range(max_rounds):
        cand = rng.integers(0, res, size=(max(4 * n, 1 << 16), 3), dtype=np.int32)
        out = np.concatenate([out, cand[_bit_set(words, res, cand)]])
        if len(out) >= n:
            return out[:n]
    raise RuntimeError("occupancy too sparse for rejection sampling")


def _dda_first_hit(grid, level, origin_idx, dirs, t_min=None, prev=None):
    import torch

    o = torch.from_numpy(np.ascontiguousarray(origin_idx, dtype=np.float32)).cuda()
    d = torch.from_numpy(np.ascontiguousarray(dirs, dtype=np.float32)).cuda()
    tm = None if t_min is None else torch.from_numpy(np.ascontiguousarray(t_min, dtype=np.float32)).cuda()
    pv = None if prev is None else torch.from_numpy(np.ascontiguousarray(prev, dtype=np.int32)).cuda()
    hit, _, tn, _ = grid.first_active_voxel(level, o, d, tm, pv)
    grid.sync_status()
    return hit.cpu().numpy(), tn.cpu().numpy()


def visibility_batch(grid, n: int, seed: int = 0, max_len: float = 0.1, n_lods: int = 8):
    """(x [n,6], max_level_frac [n], target [n,1]) with exact-DDA binary transmittance targets."""
    rng = np.random.Generator(np.random.PCG64(seed))
    pos = rng.random((n, 3)).astype(np.float32)
    d = _unit_dirs(rng, n).astype(np.float32)
    length = rng.uniform(0.0, max_len, n).astype(np.float32)
    lod = rng.integers(0, min(n_lods, grid.n_levels), size=n)
    target = np.zeros(n, np.float32)
    for k in np.unique(lod):
        sel = lod == k
        res = grid.res >> int(k)
        hit, tn = _dda_first_hit(grid, int(k), pos[sel] * np.float32(res), d[sel])
        target[sel] = ((hit == 0) | (tn >= length[sel] * np.float32(res))).astype(np.float32)
    x = np.concatenate([pos, (d + 1.0) * 0.5], axis=1).astype(np.float32)
    frac = ((np.float32(n_lods - 1) - lod.astype(np.float32)).clip(0) / np.float32(n_lods)).astype(np.float32)
    return x, frac, target[:, None]


def albedo(p: np.ndarray, seed: int = 7) -> np.ndarray:
    """Seeded smooth RGB albedo field in [0.1, 0.9] over the unit cube."""
    rng = np.random.Generator(np.random.PCG64(seed))
    f = rng.normal(0.0, 3.0, (3, 3))
    ph = rng.uniform(0, 2 * np.pi, 3)
    return (0.5 + 0.4 * np.sin(2 * np.pi * (p @ f.T) + ph)).astype(np.float32)


def throughput_batch(grid, n: int, seed: int = 0, n_lods: int = 8, min_dist: float = 2.0):
    """(x [n,10], target [n,3]): centres of occupied voxels, wi / wo uniform, albedo x transmittance."""
    rng = np.random.Generator(np.random.PCG64(seed))
    lod = rng.integers(0, min(n_lods, grid.n_levels), size=n)
    x = np.zeros((n, 10), np.float32)
    target = np.zeros((n, 3), np.float32)
    for k in np.unique(lod):
        sel = np.nonzero(lod == k)[0]
        res = grid.res >> int(k)
        words = grid.level_bits(int(k))
        vox = occupied_voxels(words, res, len(sel), rng)
        centre = ((vox.astype(np.float32) + np.float32(0.5)) / np.float32(res)).astype(np.float32)
        wi = _unit_dirs(rng, len(sel)).astype(np.float32)
        wo = _unit_dirs(rng, len(sel)).astype(np.float32)
        hit, tn = _dda_first_hit(grid, int(k), centre * np.float32(res), wi, prev=vox)
        x[sel, 0:3] = centre
        x[sel, 3:6] = (wi + 1.0) * 0.5
        x[sel, 6:9] = (wo + 1.0) * 0.5
        x[sel, 9] = (k + 0.5) / 8.0
        target[sel] = albedo(centre) * ((hit == 0) | (tn >= np.float32(min_dist)))[:, None]
    return x, target
