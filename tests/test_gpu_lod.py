"""GPU parity of the LoD pyramid and the first-active-voxel search: bit-exact against the golden
vectors of the reference's own NanoVDB DDA, and bit-exact against the oracle on larger seeded
pyramids (512^3 level 0, eight levels down to 4^3) and ray batches."""
from pathlib import Path

import numpy as np
import pytest

import oracle
from neural_lod_gb300 import NlodError, workloads as W
from neural_lod_gb300.lod import LodGrid

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden" / "dda_golden.npz"


def _run(grid, lod, rays, cuda):
    import torch

    o = torch.from_numpy(np.ascontiguousarray(rays["eye"])).to(cuda)
    d = torch.from_numpy(np.ascontiguousarray(rays["dir"])).to(cuda)
    t = torch.from_numpy(np.ascontiguousarray(rays["tmin"])).to(cuda)
    p = torch.from_numpy(np.ascontiguousarray(rays["prev"])).to(cuda)
    hit, ijk, tn, tf = grid.first_active_voxel(lod, o, d, t, p)
    grid.sync_status()
    return hit.cpu().numpy(), ijk.cpu().numpy(), tn.cpu().numpy(), tf.cpu().numpy()


def _same(hit, ijk, tn, tf, ref_hit, ref_ijk, ref_tn, ref_tf):
    assert np.array_equal(hit, ref_hit)
    h = hit == 1
    assert np.array_equal(ijk[h], ref_ijk[h])
    assert np.array_equal(tn[h].view(np.uint32), ref_tn[h].view(np.uint32))
    assert np.array_equal(tf[h].view(np.uint32), ref_tf[h].view(np.uint32))


@pytest.mark.parametrize("case", [0, 1])
def test_first_active_voxel_matches_nanovdb_golden(cuda, nlod_lib, case):
    g = np.load(GOLDEN)
    res, n_levels = int(g[f"c{case}_res"]), int(g[f"c{case}_n_levels"])
    bits, levels, rays, out = g[f"c{case}_bits"], g[f"c{case}_levels"], g[f"c{case}_rays"], g[f"c{case}_out"]
    grid = LodGrid(bits, res, n_levels)
    for lod in range(n_levels):
        info = grid.level_info(lod)
        assert info["bbox_min"] == tuple(levels[lod][:3]) and info["bbox_max"] == tuple(levels[lod][3:6])
        assert info["n_leaves"] == levels[lod][6] and info["n_active"] == levels[lod][7]
        sel = rays["lod"] == lod
        _same(*_run(grid, lod, rays[sel], cuda), out[sel]["hit"], out[sel]["ijk"], out[sel]["t_near"], out[sel]["t_far"])


def _random_rays(rng, r, n):
    rays = np.zeros(n, dtype=[("eye", "<f4", 3), ("dir", "<f4", 3), ("tmin", "<f4"), ("prev", "<i4", 3)])
    u = rng.standard_normal((n, 3))
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    outside = rng.random(n) < 0.6
    eye = np.where(outside[:, None], r / 2 + u * r * rng.uniform(0.8, 1.6, (n, 1)), rng.uniform(0, r, (n, 3)))
    tgt = rng.uniform(0, r, (n, 3))
    d = np.where(outside[:, None], tgt - eye, rng.standard_normal((n, 3)))
    zero = rng.random((n, 3)) < 0.05
    d[zero] = 0.0
    d[~d.any(axis=1), 0] = 1.0
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays["eye"], rays["dir"], rays["prev"] = eye, d, -1
    return rays


def test_pyramid_512_eight_levels_bit_exact_vs_oracle(cuda, nlod_lib):
    res, n_levels = 512, 8
    occ = W.value_noise_occupancy(res, seed=5, spacing=32, density=0.02)
    bits = W.pack_bits(occ)
    grid = LodGrid(bits, res, n_levels)
    rng = np.random.Generator(np.random.PCG64(6))
    for lod in range(n_levels):
        L = oracle.LodLevel(bits, res, lod)
        assert np.array_equal(grid.level_bits(lod), L.bits)
        info = grid.level_info(lod)
        assert (info["bbox_min"], info["bbox_max"]) == L.bbox
        assert info["n_leaves"] == int(L.leaf.sum())
        rays = _random_rays(rng, res >> lod, 4000)
        ref = L.first_active_voxel(rays["eye"], rays["dir"], rays["tmin"], rays["prev"])
        got = _run(grid, lod, rays, cuda)
        _same(*got, *ref)
        # re-query from the middle of each hit, skipping it (the renderer's pattern)
        h = ref[0] == 1
        re = rays[h].copy()
        re["tmin"] = (ref[2][h] + ref[3][h]) * np.float32(0.5)
        re["prev"] = ref[1][h]
        _same(*_run(grid, lod, re, cuda), *L.first_active_voxel(re["eye"], re["dir"], re["tmin"], re["prev"]))


def test_empty_and_invalid(cuda, nlod_lib):
    import torch

    bits = W.pack_bits(np.zeros((16, 16, 16), bool))
    grid = LodGrid(bits, 16, 2)
    o = torch.zeros((128, 3), device=cuda)
    d = torch.ones((128, 3), device=cuda) / 3 ** 0.5
    hit, _, _, _ = grid.first_active_voxel(0, o, d)
    assert int(hit.sum()) == 0
    with pytest.raises(NlodError):
        LodGrid(bits, 24, 1)       # not a power of two
    with pytest.raises(NlodError):
        grid.first_active_voxel(5, o, d)
