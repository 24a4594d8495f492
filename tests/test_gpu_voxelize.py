"""GPU parity of the conservative voxelizer: bit-exact against the oracle (orc_voxelize) on random
soups that exercise both the per-lane and the per-warp triangle paths, on special triangles, and on
the full 2M-triangle voxelize+train scene at 1024^3; mesh bounds and frame bit-exact."""
import numpy as np
import pytest

import oracle
from neural_lod_gb300 import NlodError, workloads as W
from neural_lod_gb300 import voxelize as V
from neural_lod_gb300.lod import LodGrid

pytestmark = pytest.mark.gpu


def _words(t):
    return t.cpu().numpy().view(np.uint32)


def _soup(rng, n, scales):
    c = rng.uniform(0.0, 1.0, (n, 1, 3))
    s = rng.choice(scales, (n, 1, 1))
    return (c + rng.uniform(-1, 1, (n, 3, 3)) * s).reshape(n, 9).astype(np.float32)


@pytest.mark.parametrize("grid", [32, 100, 256])
def test_random_soup_bit_exact(cuda, nlod_lib, grid):
    import torch

    rng = np.random.Generator(np.random.PCG64(grid))
    tris = _soup(rng, 5000, [0.2 / grid, 2.0 / grid, 8.0 / grid, 0.3])
    # a few degenerate ones (repeated vertex, collinear) and some outside the unit cube
    tris[:50, 3:6] = tris[:50, 0:3]
    tris[50:100, 6:9] = 0.5 * (tris[50:100, 0:3] + tris[50:100, 3:6])
    tris[100:150] += 1.5
    bmin = np.zeros(3, np.float32)
    unit = np.full(3, 1.0 / grid, np.float32)
    got = _words(V.voxelize(torch.from_numpy(tris).to(cuda), grid, bmin, unit))
    ref = oracle.voxelize(tris, grid, bmin, unit)
    assert np.array_equal(got, ref)
    assert ref.any()


def test_mesh_bounds_and_frame(cuda, nlod_lib):
    import torch

    mesh = W.synthetic_mesh(n_ellipsoids=500, n_quads=5000, seed=4)
    mesh[7, 4] = -3.25
    mn, mx = V.mesh_bounds(torch.from_numpy(mesh).to(cuda))
    v = mesh.reshape(-1, 3)
    assert np.array_equal(mn, v.min(0)) and np.array_equal(mx, v.max(0))
    for g, eps in [(1024, 1e-4), (512, 0.0), (100, 1e-3)]:
        got = V.mesh_frame(mn, mx, g, eps)
        ref = oracle.mesh_frame(mn, mx, g, eps)
        for a, b in zip(got, ref):
            assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_voxelize_train_scene_1024(cuda, nlod_lib):
    """The full scene: 20k ellipsoid shells + 0.52M quads (2.0M triangles) at 1024^3."""
    import torch

    mesh = W.synthetic_mesh()
    t = torch.from_numpy(mesh).to(cuda)
    got = _words(V.voxelize(t, 1024))
    v = mesh.reshape(-1, 3)
    bmin, _, unit = oracle.mesh_frame(v.min(0), v.max(0), 1024, V.EPSILON_PADDING)
    ref = oracle.voxelize(mesh, 1024, bmin, unit)
    assert np.array_equal(got, ref)
    assert int(np.unpackbits(ref.view(np.uint8)).sum()) > 1_000_000


def test_or_into_and_pyramid(cuda, nlod_lib):
    import torch

    mesh = W.synthetic_mesh(n_ellipsoids=300, n_quads=3000, seed=2)
    t = torch.from_numpy(mesh).to(cuda)
    mn, mx = V.mesh_bounds(t)
    bmin, _, unit = V.mesh_frame(mn, mx, 256)
    whole = V.voxelize(t, 256, bmin, unit)
    part = V.voxelize(t[: len(mesh) // 3], 256, bmin, unit)
    V.voxelize(t[len(mesh) // 3:], 256, bmin, unit, out=part)
    assert torch.equal(whole, part)
    V.voxelize(t, 256, bmin, unit, out=part)   # idempotent
    assert torch.equal(whole, part)
    # the voxelizer's grid is the pyramid's level 0
    g = LodGrid(whole, 256, 3)
    assert np.array_equal(g.level_bits(0), _words(whole))
    assert np.array_equal(g.level_bits(2), oracle.LodLevel(_words(whole), 256, 2).bits)


def test_empty_and_invalid(cuda, nlod_lib):
    import torch

    empty = torch.zeros((0, 9), device=cuda)
    out = V.voxelize(empty, 16, np.zeros(3), np.ones(3))
    assert int(out.abs().sum()) == 0
    tri = torch.rand((4, 9), device=cuda)
    with pytest.raises(NlodError):
        V.voxelize(tri, 0, np.zeros(3), np.ones(3))
    with pytest.raises(NlodError):
        V.voxelize(tri, 8192, np.zeros(3), np.ones(3))
    with pytest.raises(NlodError):
        V.voxelize(tri, 16, np.zeros(3), np.array([1, 0, 1]))
    with pytest.raises(NlodError):
        V.mesh_frame([0, 0, 0], [0, 0, 0], 16)
