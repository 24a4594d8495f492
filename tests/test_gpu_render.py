"""GPU parity of the wavefront render query (nlod_renderer: one CUDA-graph launch per frame with a
conditional while loop over rounds) against the host restatement oracle.render.

Rays, voxel traversal and direction sampling are bit-identical on both sides; the networks are
FP32 / FP16 on the GPU and FP64 on the host, so a ray's path can differ only where a visibility
value lies within the networks' rounding distance of the threshold.  Tolerances: FP32 form -
per-ray query counts equal for >= 99.5% of the rays and their pixels within 1e-3 relative;
FP16 form - counts equal for >= 97% of the rays and those pixels within 2e-2 relative."""
import numpy as np
import pytest

import oracle
from neural_lod_gb300 import NetworkWithInputEncoding, workloads as W
from neural_lod_gb300.lod import LodGrid
from neural_lod_gb300.render import RenderParams, Renderer, camera

pytestmark = pytest.mark.gpu


def _scene(res=64, levels=3, density=0.3, seed=11):
    occ = W.value_noise_occupancy(res, seed=seed, spacing=8, density=density)
    return W.pack_bits(occ), res, levels


def _nets(precision):
    venc, vnet = W.visibility_configs()
    henc, hnet = W.throughput_configs()
    vo, to = oracle.Oracle(venc, vnet, 6, 1), oracle.Oracle(henc, hnet, 10, 3)
    vp, tp = W.xavier_params(vo.spec, seed=31), W.test_params(to.spec, seed=32, grid_scale=0.2)
    vm = NetworkWithInputEncoding(6, 1, venc, vnet, precision=precision)
    tm = NetworkWithInputEncoding(10, 3, henc, hnet, precision=precision)
    vm.set_params(vp)
    tm.set_params(tp)
    return vm, tm, vo, to, vp, tp


def _render_both(precision, params, bits, res, levels):
    import torch

    vm, tm, vo, to, vp, tp = _nets(precision)
    grid = LodGrid(bits, res, levels)
    r = Renderer(vm, tm, grid, params)
    n = params.width * params.height
    stats = torch.zeros((n, 2), dtype=torch.int32, device="cuda")
    img = r.frame(ray_stats=stats).cpu().numpy()
    tot = r.stats()
    img2 = r.frame().cpu().numpy()             # a second frame of the same graph is identical
    assert np.array_equal(img, img2)
    level = oracle.LodLevel(bits, res, params.level)
    cam = camera(params, res >> params.level)
    ref_img, ref_stats, ref_tot = oracle.render(vo, vp, to, tp, level, params, cam)
    return img, stats.cpu().numpy().astype(np.uint32), tot, ref_img, ref_stats, ref_tot


@pytest.mark.parametrize("precision,frac,rel", [("fp32", 0.995, 1e-3), ("fp16", 0.97, 2e-2)])
def test_render_matches_oracle(cuda, nlod_lib, precision, frac, rel):
    bits, res, levels = _scene()
    params = RenderParams(width=96, height=64, level=1, max_depth=4, max_vis_queries=24, lod_max_level=6 / 8, lod_input=1.5 / 8)
    img, st, tot, ref_img, ref_st, ref_tot = _render_both(precision, params, bits, res, levels)
    same = np.all(st == ref_st, axis=1)
    print(precision, "rays with identical query counts", same.mean(), "totals", tot, ref_tot)
    assert same.mean() >= frac
    a, b = img.reshape(-1, 3)[same], ref_img.reshape(-1, 3)[same]
    close = np.abs(a - b) <= rel * np.maximum(np.abs(b), 1e-3)
    assert np.all(close)
    assert tot[0] == int(st[:, 0].sum()) and tot[1] == int(st[:, 1].sum())
    assert ref_tot[0] > 2 * params.width * params.height and ref_tot[1] > 0     # the scene exercises both networks
    assert tot[2] >= 2                                                           # rounds


def test_render_empty_grid_and_query_cap(cuda, nlod_lib):
    res, levels = 32, 2
    empty = W.pack_bits(np.zeros((res, res, res), bool))
    params = RenderParams(width=32, height=32, level=0, background=(0.25, 0.5, 0.75))
    img, st, tot, ref_img, ref_st, ref_tot = _render_both("fp32", params, empty, res, levels)
    assert np.allclose(img, np.array([0.25, 0.5, 0.75], np.float32)) and tot[0] == tot[1] == 0
    # threshold above any sigmoid: no voxel is accepted; rays stop at the per-bounce query cap
    full = W.pack_bits(np.ones((res, res, res), bool))
    params = RenderParams(width=32, height=32, level=0, threshold=2.0, max_vis_queries=5)
    img, st, tot, ref_img, ref_st, ref_tot = _render_both("fp32", params, full, res, levels)
    assert tot[1] == 0 and ref_tot[1] == 0
    assert np.array_equal(st, ref_st)
    assert tot[3] == ref_tot[2] > 0          # dropped rays
    assert np.array_equal(img, ref_img)
