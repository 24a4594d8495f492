"""The voxelizer oracle (oracle/nlod_oracle.c: orc_mesh_frame, orc_voxelize) pinned by known
answers, by an independent FP64 separating-axis overlap test, and by the reference kernel's bits.

The reference voxelizer ships no test or golden output.  Its kernel is compiled from its own source
(oracle/build_ref.py, GLM from oracle/glm_shim) and run on a GPU to make
tests/golden/voxelizer_golden.npz; the oracle must reproduce those bits exactly.  The other pins:
the createMeshBBCube example of its own comment (cuda_voxelizer/src/util.h:77-85), hand-derived
voxel sets, the MSB-first bit order of setBit (voxelize.cu:50-55), and agreement with the exact
triangle/box overlap (13-axis separating-axis test in float64) everywhere except within rounding
distance of a touching contact.
"""
import numpy as np
import pytest

import oracle
from neural_lod_gb300 import workloads as W


def _vox_set(bits, g):
    occ = W.unpack_bits(bits, g)
    return {(int(x), int(y), int(z)) for z, y, x in zip(*np.nonzero(occ))}


def test_mesh_frame_cube_example():
    # util.h comment: (1,2,3)-(4,4,4) becomes (1,1.5,2)-(4,4.5,5)
    bmin, bmax, unit = oracle.mesh_frame([1, 2, 3], [4, 4, 4], 8, 0.0)
    assert bmin.tolist() == [1.0, 1.5, 2.0] and bmax.tolist() == [4.0, 4.5, 5.0]
    assert unit.tolist() == [np.float32(3) / np.float32(8)] * 3
    bmin, bmax, unit = oracle.mesh_frame([0, 0, 0], [1, 1, 1], 4, 0.25)
    assert bmin.tolist() == [-0.25] * 3 and bmax.tolist() == [1.25] * 3 and unit.tolist() == [0.375] * 3


def test_bit_order_msb_first():
    g = 4
    tri = np.array([[0.1, 0.1, 0.1, 0.2, 0.1, 0.1, 0.1, 0.2, 0.1]], np.float32)
    bits = oracle.voxelize(tri, g, [0, 0, 0], [1, 1, 1])
    assert bits[0] == 0x80000000 and not bits[1:].any()
    tri[0, 0::3] += 1.0   # voxel (1, 0, 0) -> bit 1 -> second most significant bit
    assert oracle.voxelize(tri, g, [0, 0, 0], [1, 1, 1])[0] == 0x40000000


def test_right_triangle_known_voxels():
    # plane z = 0.5, legs along x and y: covers x, y >= 0.5, x + y <= 3; the closed voxel boxes
    # overlapping it have min corners with x + y <= 3 (corner contacts at (2,1) and (1,2) included)
    tri = np.array([[0.5, 0.5, 0.5, 2.5, 0.5, 0.5, 0.5, 2.5, 0.5]], np.float32)
    got = _vox_set(oracle.voxelize(tri, 4, [0, 0, 0], [1, 1, 1]), 4)
    assert got == {(x, y, 0) for x in range(3) for y in range(3) if x + y <= 3}


def test_triangle_inside_one_voxel_and_outside_grid():
    tri = np.array([[2.2, 1.3, 3.4, 2.7, 1.4, 3.5, 2.3, 1.8, 3.6]], np.float32)
    assert _vox_set(oracle.voxelize(tri, 8, [0, 0, 0], [1, 1, 1]), 8) == {(2, 1, 3)}
    # a triangle beyond the grid is clamped onto the boundary layer like the reference's bbox clamp
    far = tri + np.float32(20)
    got = _vox_set(oracle.voxelize(far, 8, [0, 0, 0], [1, 1, 1]), 8)
    assert got <= {(7, 7, 7)}


def _sat_margin(tri, lo, hi):
    """Largest separation (>0 separated, <=0 overlapping) of a triangle and a closed box over the
    13 separating axes, each normalised to a unit axis (float64)."""
    v = tri.reshape(3, 3).astype(np.float64)
    e = [v[1] - v[0], v[2] - v[1], v[0] - v[2]]
    axes = [np.eye(3)[i] for i in range(3)] + [np.cross(e[0], e[1])]
    axes += [np.cross(ei, np.eye(3)[j]) for ei in e for j in range(3)]
    c, h = (lo + hi) / 2, (hi - lo) / 2
    worst = -np.inf
    for a in axes:
        na = np.linalg.norm(a)
        if na < 1e-12:
            continue
        a = a / na
        p = v @ a
        r = np.abs(a) @ h
        s = max(p.min() - (c @ a + r), (c @ a - r) - p.max())
        worst = max(worst, s)
    return worst


def test_agrees_with_exact_overlap_fp64():
    rng = np.random.Generator(np.random.PCG64(3))
    g, tol = 16, 1e-4
    bmin = np.zeros(3, np.float32)
    unit = np.full(3, np.float32(1.0 / g), np.float32)
    n_checked = n_marked = 0
    for t in range(120):
        scale = [0.02, 0.1, 0.4][t % 3]
        c = rng.uniform(0.1, 0.9, 3)
        tri = (c + rng.uniform(-scale, scale, (3, 3))).astype(np.float32).reshape(1, 9)
        got = _vox_set(oracle.voxelize(tri, g, bmin, unit), g)
        v = tri.reshape(3, 3)
        lo = np.clip((v.min(0) - bmin) / unit, 0, g - 1).astype(np.int64)
        hi = np.clip((v.max(0) - bmin) / unit, 0, g - 1).astype(np.int64)
        for z in range(lo[2], hi[2] + 1):
            for y in range(lo[1], hi[1] + 1):
                for x in range(lo[0], hi[0] + 1):
                    bl = np.array([x, y, z], np.float64) / g
                    m = _sat_margin(tri, bl, bl + 1.0 / g)
                    if abs(m) < tol / g:
                        continue
                    n_checked += 1
                    n_marked += m <= 0
                    assert ((x, y, z) in got) == (m <= 0), (t, x, y, z, m)
        assert all(lo[0] <= x <= hi[0] and lo[1] <= y <= hi[1] and lo[2] <= z <= hi[2] for x, y, z in got)
    assert n_checked > 10000 and n_marked > 1000


def test_or_into_and_order_independence():
    mesh = W.synthetic_mesh(n_ellipsoids=60, n_quads=400, seed=9)
    v = mesh.reshape(-1, 3)
    bmin, _, unit = oracle.mesh_frame(v.min(0), v.max(0), 128, 1e-4)
    whole = oracle.voxelize(mesh, 128, bmin, unit)
    half = oracle.voxelize(mesh[: len(mesh) // 2], 128, bmin, unit)
    both = oracle.voxelize(mesh[len(mesh) // 2:][::-1].copy(), 128, bmin, unit, bits=half)
    assert np.array_equal(whole, both)
    assert whole.any()


@pytest.mark.parametrize("shape", ["degenerate", "axis_plane"])
def test_special_triangles(shape):
    g = 8
    if shape == "degenerate":
        # zero area: the normal is NaN, the plane test never rejects, the edge tests keep the segment
        tri = np.array([[1.5, 1.5, 1.5, 3.5, 3.5, 3.5, 2.5, 2.5, 2.5]], np.float32)
        got = _vox_set(oracle.voxelize(tri, g, [0, 0, 0], [1, 1, 1]), g)
        assert {(1, 1, 1), (2, 2, 2), (3, 3, 3)} <= got
    else:
        # triangle in the plane x = 3 exactly: only the x = 3 layer is a candidate (floor bbox)
        tri = np.array([[3, 0.5, 0.5, 3, 2.5, 0.5, 3, 0.5, 2.5]], np.float32)
        got = _vox_set(oracle.voxelize(tri, g, [0, 0, 0], [1, 1, 1]), g)
        assert got and all(x == 3 for x, _, _ in got)


def test_oracle_matches_reference_kernel_build():
    """The host restatement against the reference voxelizer kernel itself, compiled from its source
    the way the reference builds it (nvcc's default multiply-add contraction) and run on a GB300
    (tests/golden/make_voxelizer_golden.py): the same bits on a 20,000-triangle soup at 100^3."""
    import sys
    from pathlib import Path

    golden = Path(__file__).resolve().parent / "golden" / "voxelizer_golden.npz"
    if not golden.exists():
        pytest.skip("reference voxelizer golden vectors not generated")
    sys.path.insert(0, str(golden.parent))
    import make_voxelizer_golden as M

    g = np.load(golden)
    tris = M.soup(int(g["n"]), int(g["grid"]), int(g["seed"]))
    got = oracle.voxelize(tris, int(g["grid"]), g["bbox_min"], g["unit"])
    assert int(np.unpackbits(g["bits"].view(np.uint8)).sum()) > 100_000
    assert np.array_equal(got, g["bits"])
