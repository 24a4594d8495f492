"""The voxelizer against the reference voxelizer kernel itself, bit for bit.

cuda_voxelizer's voxelize_triangle (neural_lod/cuda_voxelizer/src/voxelize.cu:58-190) is compiled
from the reference's own source (staged and built by oracle/build_ref.py, GLM supplied by
oracle/glm_shim) in two forms: with nvcc's default contraction of multiply-adds into FMAs, which is
how the reference's CMake builds it, and with -fmad=false.  Each runs on the same triangles, grid
and frame as nlod_voxelize, and the bit grids are compared word for word.

Checked: nlod_voxelize is bit-exact with the reference kernel as the reference builds it (the
contracted form), on random soups and on the 2.0 M-triangle scene at 1024^3.  It evaluates the
overlap tests with the fused multiply-adds that nvcc puts into that kernel, each written out.  The
uncontracted build differs on the voxels whose test is decided by the last bit of a fused
product (about 1e-5 .. 2e-4 of the set voxels); that count is reported.
"""
import numpy as np
import pytest

import oracle.voxref as VR
from neural_lod_gb300 import workloads as W
from neural_lod_gb300 import voxelize as V

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not VR.available(), reason="reference voxelizer not staged or built")]


def _bits(t):
    return t.cpu().numpy().view(np.uint32)


def _ndiff(a, b):
    return int(np.unpackbits((a ^ b).view(np.uint8)).sum())


def _nset(a):
    return int(np.unpackbits(a.view(np.uint8)).sum())


def _compare(tris_d, grid, bmin, bmax, unit):
    ours = _bits(V.voxelize(tris_d, grid, bmin, unit))
    fma = _bits(VR.voxelize(tris_d, grid, bmin, bmax, "fma"))
    nofma = _bits(VR.voxelize(tris_d, grid, bmin, bmax, "nofma"))
    return ours, fma, nofma


def test_frame_unit_matches_reference(cuda, nlod_lib):
    mesh = W.synthetic_mesh(n_ellipsoids=200, n_quads=2000, seed=9)
    v = mesh.reshape(-1, 3)
    for grid in (64, 1000, 1024):
        bmin, bmax, unit = V.mesh_frame(v.min(0), v.max(0), grid)
        for kind in ("fma", "nofma"):
            assert np.array_equal(VR.unit(bmin, bmax, grid, kind).view(np.uint32), unit.view(np.uint32))


@pytest.mark.parametrize("grid", [32, 100, 256])
def test_random_soup_against_reference_kernel(cuda, nlod_lib, grid):
    import torch

    rng = np.random.Generator(np.random.PCG64(100 + grid))
    c = rng.uniform(0.0, 1.0, (4000, 1, 3))
    s = rng.choice([0.2 / grid, 2.0 / grid, 8.0 / grid, 0.1], (4000, 1, 1))
    tris = (c + rng.uniform(-1, 1, (4000, 3, 3)) * s).reshape(-1, 9).astype(np.float32)
    tris[:40, 3:6] = tris[:40, 0:3]                                  # repeated vertex
    tris[40:80, 6:9] = 0.5 * (tris[40:80, 0:3] + tris[40:80, 3:6])    # collinear
    v = tris.reshape(-1, 3)
    bmin, bmax, unit = V.mesh_frame(v.min(0), v.max(0), grid)
    ours, fma, nofma = _compare(torch.from_numpy(tris).to(cuda), grid, bmin, bmax, unit)
    assert _nset(fma) > 1000
    assert np.array_equal(ours, fma), f"{_ndiff(ours, fma)} voxels differ from the reference kernel as built"
    print(f"grid {grid}: {_nset(fma)} voxels set by the reference kernel, {_ndiff(ours, nofma)} differ from its -fmad=false build")


def test_voxelize_train_scene_against_reference_kernel(cuda, nlod_lib):
    """The 2.0M-triangle voxelize+train scene at 1024^3."""
    import torch

    mesh = W.synthetic_mesh()
    t = torch.from_numpy(mesh).to(cuda)
    mn, mx = V.mesh_bounds(t)
    bmin, bmax, unit = V.mesh_frame(mn, mx, 1024)
    ours, fma, nofma = _compare(t, 1024, bmin, bmax, unit)
    n = _nset(fma)
    assert n > 1_000_000
    assert np.array_equal(ours, fma), f"{_ndiff(ours, fma)} voxels differ from the reference kernel as built"
    print(f"1024^3 scene: {n} voxels set by the reference kernel, {_ndiff(fma, nofma)} differ between its two builds")
