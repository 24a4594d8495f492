"""Training-sample generator on the GPU against the host restatement, bit for bit: the sorted
Morton voxel list, the visibility and throughput samplers (every parameter branch: inward and
outward dilation, boundary-density rejection, LoD pdf), the threshold-optimisation per-voxel
mode, the exact-DDA targets and the stable compaction."""
import numpy as np
import pytest

import oracle
from neural_lod_gb300 import sampler as SM
from neural_lod_gb300 import workloads as W
from neural_lod_gb300.lod import LodGrid

pytestmark = pytest.mark.gpu

RES = 64
PARAM_SETS = {
    "reference_defaults": {},
    "inward_boundary_pdf": {"dilation_inward": 0.003, "increase_boundary_density": True, "pdf_strength": 3.0, "pdf_shift": 0.2,
                            "bound_bias": 0.002},
    "strong_dilation": {"dilation_outward": 0.3, "dilation_inward": 0.2, "min_dilation": 0.01, "pdf_strength": 8.0, "pdf_shift": -0.3},
}


def occupancy(res=RES, seed=3):
    return W.value_noise_occupancy(res, seed=seed, spacing=8, density=0.25)


@pytest.fixture(scope="module")
def scene(cuda, nlod_lib):
    occ = occupancy()
    bits = W.pack_bits(occ)
    grid = LodGrid(bits, RES, 5)
    return occ, bits, grid


def params(kind, aabb=((-1.0, 0.5, 2.0), (3.0, 4.5, 6.0))):
    base = dict(aabb_min=aabb[0], aabb_max=aabb[1], grid_res=RES, n_lods=5)
    base.update(PARAM_SETS[kind])
    gp = SM.SamplerParams(**base)
    c = gp.to_c()
    op = oracle.SamplerParams.from_dict({k: getattr(c, k) if k not in ("aabb_min", "aabb_max") else list(getattr(c, k))
                                         for k, _ in oracle.SamplerParams._fields_})
    return gp, op


def q_host(t):
    return t.cpu().numpy().view(oracle.RAY_QUERY_DTYPE).reshape(-1)


def test_morton_voxels_match(scene):
    import torch

    occ, bits, grid = scene
    codes, count = SM.morton_voxels(torch.from_numpy(bits.view(np.int32)).cuda(), RES)
    ref = oracle.morton_voxels(bits, RES)
    assert int(count.item()) == ref.size == int(occ.sum())
    assert np.array_equal(codes.cpu().numpy().view(np.uint32), ref)
    # an empty grid and a full grid
    empty = torch.zeros(RES ** 3 // 32, dtype=torch.int32, device="cuda")
    c0, n0 = SM.morton_voxels(empty, RES)
    assert int(n0.item()) == 0 and c0.numel() == 0
    full = torch.full((8 ** 3 // 32,), -1, dtype=torch.int32, device="cuda")
    c1, n1 = SM.morton_voxels(full, 8)
    assert np.array_equal(c1.cpu().numpy(), np.arange(512))


@pytest.mark.parametrize("kind", list(PARAM_SETS))
def test_visibility_samples_match(scene, kind):
    occ, bits, grid = scene
    gp, op = params(kind)
    s = SM.Sampler(grid, gp)
    ref_m = oracle.morton_voxels(bits, RES)
    for batch_index, n in ((0, 4096), (7, 3000)):
        x, q, lod = s.sample_visibility(batch_index, n)
        rx, rq, rl = oracle.sample_visibility(op, ref_m, batch_index, n)
        assert np.array_equal(x.cpu().numpy(), rx)
        assert np.array_equal(lod.cpu().numpy().view(np.uint32), rl)
        gq = q_host(q)
        assert gq.tobytes() == rq.tobytes()
        assert (rq["t_max"] < 0).sum() == 0
        # targets
        y = s.trace_visibility(q)
        L0 = oracle.LodLevel(bits, RES, 0)
        ry = oracle.trace_visibility(L0, op, rq)
        assert np.array_equal(y.cpu().numpy().reshape(-1), ry)
        assert 0.05 < ry.mean() < 0.95
    s.sync_status()


def test_visibility_voxels_mode_matches(scene):
    occ, bits, grid = scene
    gp, op = params("inward_boundary_pdf")
    s = SM.Sampler(grid, gp)
    lod = 2
    codes, count = s.lod_morton(lod)
    ref_codes = oracle.morton_voxels(grid.level_bits(lod), RES >> lod)
    assert np.array_equal(codes.cpu().numpy().view(np.uint32), ref_codes)
    first, nv, ns = 3, min(40, ref_codes.size - 3), 37
    x, q = s.sample_visibility_voxels(lod, first, nv, ns)
    rx, rq = oracle.sample_visibility_voxels(op, ref_codes, first, nv, ns, lod)
    assert np.array_equal(x.cpu().numpy(), rx)
    assert q_host(q).tobytes() == rq.tobytes()


@pytest.mark.parametrize("kind", ["reference_defaults", "strong_dilation"])
@pytest.mark.parametrize("log_learning", [False, True])
def test_throughput_samples_targets_and_compaction(scene, kind, log_learning):
    occ, bits, grid = scene
    gp, op = params(kind)
    s = SM.Sampler(grid, gp)
    ref_m = oracle.morton_voxels(bits, RES)
    n, bi = 5000, 11
    x, q, lod = s.sample_throughput(bi, n, max_orders=17)
    rx, rq, rl = oracle.sample_throughput(op, ref_m, bi, n, 17)
    assert np.array_equal(x.cpu().numpy(), rx)
    assert np.array_equal(lod.cpu().numpy().view(np.uint32), rl)
    assert q_host(q).tobytes() == rq.tobytes()
    assert (rq["mode_or_data"] == 17).all()
    y, bad = s.trace_throughput(q, x, bi, log_learning)
    L0 = oracle.LodLevel(bits, RES, 0)
    ry, rbad = oracle.trace_throughput(L0, op, rq, rx, bi, log_learning)
    gx, gy = x.cpu().numpy(), y.cpu().numpy()
    assert int(bad.item()) == rbad and 0 < rbad < n
    assert np.array_equal(gx, rx)
    if log_learning:
        # logf on the device and on the host may differ in the last place
        np.testing.assert_allclose(gy, ry, rtol=2e-7, atol=0)
    else:
        assert np.array_equal(gy, ry)
    xv, yv, nv = s.compact(x, y)
    rxv, ryv = oracle.compact_samples(gx, gy)
    k = int(nv.item())
    assert k == rxv.shape[0] and k % 128 == 0 and k > 0
    assert np.array_equal(xv[:k].cpu().numpy(), rxv) and np.array_equal(yv[:k].cpu().numpy(), ryv)
    assert (ryv[:, 0] != -1).all()
    s.sync_status()


def test_empty_grid_marks_every_sample_invalid(cuda, nlod_lib):
    bits = np.zeros(RES ** 3 // 32, np.uint32)
    bits[0] = 0x80000000   # one voxel, so the pyramid is non-empty
    grid = LodGrid(bits, RES, 3)
    gp, _ = params("reference_defaults")
    s = SM.Sampler(grid, gp)
    import torch

    s.count = torch.zeros(1, dtype=torch.int32, device="cuda")   # as if nothing were occupied
    x, q, _ = s.sample_visibility(0, 256)
    assert (x.cpu().numpy() == -1).all() and (q_host(q)["t_max"] < 0).all()
    y = s.trace_visibility(q)
    assert (y.cpu().numpy() == -1).all()
    xv, yv, nv = s.compact(x, y)
    assert int(nv.item()) == 0
