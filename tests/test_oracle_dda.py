"""CPU tests: the oracle's LoD pyramid and first-active-voxel search against golden vectors made by
running the reference's own NanoVDB TreeMarcher / DDA (tests/golden/make_dda_golden.py)."""
from pathlib import Path

import numpy as np
import pytest

import oracle
from neural_lod_gb300 import workloads as W

GOLDEN = Path(__file__).resolve().parent / "golden" / "dda_golden.npz"


def _cases():
    g = np.load(GOLDEN)
    for c in range(int(g["n_cases"])):
        yield (int(g[f"c{c}_res"]), int(g[f"c{c}_n_levels"]), g[f"c{c}_bits"], g[f"c{c}_levels"], g[f"c{c}_rays"],
               g[f"c{c}_out"])


def test_golden_file_present():
    assert GOLDEN.exists()


@pytest.mark.parametrize("case", [0, 1])
def test_oracle_pyramid_matches_nanovdb_grids(case):
    res, n_levels, bits, levels, _, _ = list(_cases())[case]
    for lod in range(n_levels):
        L = oracle.LodLevel(bits, res, lod)
        bmin, bmax = L.bbox
        assert tuple(levels[lod][:3]) == bmin and tuple(levels[lod][3:6]) == bmax
        assert int(L.leaf.sum()) == int(levels[lod][6])           # NanoVDB leaf count
        assert int(L.s.n_active) == int(levels[lod][7])           # NanoVDB active voxel count


@pytest.mark.parametrize("case", [0, 1])
def test_oracle_first_active_voxel_bit_exact(case):
    res, n_levels, bits, _, rays, out = list(_cases())[case]
    for lod in range(n_levels):
        sel = rays["lod"] == lod
        r, o = rays[sel], out[sel]
        L = oracle.LodLevel(bits, res, lod)
        hit, ijk, tn, tf = L.first_active_voxel(r["eye"], r["dir"], r["tmin"], r["prev"])
        assert np.array_equal(hit, o["hit"])
        h = hit == 1
        assert np.array_equal(ijk[h], o["ijk"][h])
        # bit-exact times (compare bit patterns)
        assert np.array_equal(tn[h].view(np.uint32), o["t_near"][h].view(np.uint32))
        assert np.array_equal(tf[h].view(np.uint32), o["t_far"][h].view(np.uint32))


def test_pyramid_is_or_downsampling():
    occ = W.value_noise_occupancy(32, seed=3, spacing=8, density=0.05)
    bits = W.pack_bits(occ)
    for lod in range(1, 4):
        L = oracle.LodLevel(bits, 32, lod)
        r = 32 >> lod
        down = occ.reshape(r, 1 << lod, r, 1 << lod, r, 1 << lod).any(axis=(1, 3, 5))
        assert np.array_equal(W.unpack_bits(L.bits, r), down)
