"""Host restatement of the training-sample generator: its sine/cosine against float64, its Morton
list against an independent numpy construction, and the sampler's geometric invariants (chord
end points on the dilated cube, deterministic pi/po order, LoD distribution, compaction rule).
Also checks that the C ABI rejects bad sampler parameters before touching the GPU."""
import ctypes as C

import numpy as np
import pytest

import oracle
from neural_lod_gb300 import workloads as W

RES = 32


def morton_np(xyz):
    def part(v):
        v = v.astype(np.uint64) & 0x3FF
        out = np.zeros_like(v)
        for b in range(10):
            out |= ((v >> b) & 1) << (3 * b)
        return out
    return (part(xyz[:, 2]) << 2) + (part(xyz[:, 1]) << 1) + part(xyz[:, 0])


def defaults(**kw):
    d = dict(aabb_min=(0.0, 0.0, 0.0), aabb_max=(1.0, 1.0, 1.0), voxel_size=np.float32(1.0 / RES), grid_res=RES, n_lods=4,
             dilation_outward=0.005, dilation_inward=0.0, min_dilation=1e-4, bound_bias=0.0, pdf_strength=0.0, pdf_shift=0.0,
             increase_boundary_density=0, max_attempts=256)
    d.update(kw)
    return oracle.SamplerParams.from_dict(d)


def test_cos_sin_is_correctly_rounded():
    phi = np.linspace(0.0, 2 * np.pi, 20001, dtype=np.float32)
    got = np.array([oracle.cos_sin(float(p)) for p in phi], dtype=np.float32)
    ref = np.stack([np.cos(phi.astype(np.float64)), np.sin(phi.astype(np.float64))], 1).astype(np.float32)
    assert np.array_equal(got, ref)


def test_morton_list_matches_numpy():
    occ = W.value_noise_occupancy(RES, seed=9, spacing=8, density=0.3)
    codes = oracle.morton_voxels(W.pack_bits(occ), RES)
    z, y, x = np.nonzero(occ)
    ref = np.sort(morton_np(np.stack([x, y, z], 1)))
    assert np.array_equal(codes.astype(np.uint64), ref)


def test_visibility_sampler_invariants():
    occ = W.value_noise_occupancy(RES, seed=9, spacing=8, density=0.3)
    bits = W.pack_bits(occ)
    m = oracle.morton_voxels(bits, RES)
    p = defaults()
    x, q, lod = oracle.sample_visibility(p, m, 0, 20000)
    assert (q["t_max"] > 0).all()
    # chord end points lie on the dilated cube: |p - c|_inf = extent (1 + dil) / 2 = voxel_extent / 2
    for pt in (x[:, :3], x[:, 3:]):
        d = np.abs(pt - q["voxel_center"]).max(1)
        np.testing.assert_allclose(d, q["voxel_extent"] / 2, rtol=2e-5)
    # the query starts at pi and points at po
    np.testing.assert_allclose(q["origin"], x[:, :3], rtol=0, atol=0)
    dirn = x[:, 3:] - x[:, :3]
    ln = np.linalg.norm(dirn, axis=1, keepdims=True)
    long_chord = ln[:, 0] > 0.05 * q["voxel_extent"]   # short chords lose the direction to input rounding
    assert long_chord.mean() > 0.95
    np.testing.assert_allclose(q["dir"][long_chord], (dirn / ln)[long_chord], atol=2e-4)
    # pi lies on the lower-numbered cube face
    def face(v):
        a = np.abs(v).argmax(1)
        return np.where(v[np.arange(len(v)), a] > 0, 2 * a, 2 * a + 1)
    lc = (x[:, :3] - q["voxel_center"]), (x[:, 3:] - q["voxel_center"])
    assert (face(lc[0]) <= face(lc[1])).all()
    # the dilation stays in [min, outward]
    dil = q["voxel_extent"] / (2.0 ** lod.astype(np.float32) / RES) - 1
    assert dil.min() > 1e-4 * 0.99 and dil.max() < 0.005 * 1.01
    # uniform LoD pdf with strength 0
    h = np.bincount(lod, minlength=4) / len(lod)
    assert np.abs(h - 0.25).max() < 0.02


def test_lod_pdf_follows_shifted_square():
    bits = W.pack_bits(np.ones((RES, RES, RES), bool))
    m = oracle.morton_voxels(bits, RES)
    s, d, n_lods = 6.0, 0.1, 4
    p = defaults(pdf_strength=s, pdf_shift=d)
    _, _, lod = oracle.sample_visibility(p, m, 3, 40000)
    xl = np.arange(n_lods) / n_lods + d - 0.5 + 0.0625
    pdf = 1 + s * xl * xl
    pdf /= pdf.sum()
    h = np.bincount(lod, minlength=n_lods) / len(lod)
    assert np.abs(h - pdf).max() < 0.015


def test_compaction_rule():
    x = np.arange(1000 * 2, dtype=np.float32).reshape(1000, 2)
    y = np.zeros((1000, 1), np.float32)
    y[::3] = -1.0
    xv, yv = oracle.compact_samples(x, y)
    valid = 1000 - len(range(0, 1000, 3))
    assert xv.shape[0] == (valid + 127) // 128 * 128 - 128
    assert np.array_equal(xv, x[y[:, 0] != -1][: xv.shape[0]])


def test_c_abi_rejects_bad_sampler_params():
    from neural_lod_gb300 import sampler as SM
    from neural_lod_gb300._lib import NLOD_ERR_INVALID, load

    lib = load()
    good = SM.SamplerParams(grid_res=64).to_c()
    for field, value in (("n_lods", 0), ("n_lods", 17), ("voxel_size", 0.0), ("max_attempts", 0)):
        bad = SM.SamplerParams(grid_res=64).to_c()
        setattr(bad, field, value)
        assert lib.nlod_sample_visibility(C.byref(bad), 8, 8, 0, 1, 8, None, None, None) == NLOD_ERR_INVALID
    bad = SM.SamplerParams(grid_res=64, aabb_max=(0.0, 1.0, 1.0)).to_c()
    assert lib.nlod_sample_throughput(C.byref(bad), 8, 8, 0, 1, 1, 8, None, None, None) == NLOD_ERR_INVALID
    assert lib.nlod_sample_visibility(C.byref(good), None, None, 0, 1, None, None, None, None) == NLOD_ERR_INVALID
    assert lib.nlod_morton_voxels(8, 48, None, 0, 8, None) == NLOD_ERR_INVALID   # not a power of two
    assert lib.nlod_compact_samples(None, None, 4, 0, 1, None, None, 8, None) == NLOD_ERR_INVALID
