"""GPU parity of the render query (nlod_renderer: one CUDA-graph launch per frame, either the
persistent kernel or rounds in a conditional while loop) against the host restatement
oracle.render, and of the two forms against each other.

Rays, voxel traversal and direction sampling are bit-identical on both sides; the networks are
FP32 / FP16 on the GPU and FP64 on the host, so a ray's path can differ only where a visibility
value lies within the networks' rounding distance of the threshold.  Tolerances: FP32 form -
per-ray query counts equal for >= 99.5% of the rays and their pixels within 1e-3 relative;
FP16 form - counts equal for >= 97% of the rays and those pixels within 2e-2 relative.
The persistent form and the wavefront form run the same per-ray steps and network arithmetic, so
their pixels, per-ray query counts and totals are identical bits (FP16 and BF16 modules)."""
import numpy as np
import pytest

import oracle
from neural_lod_gb300 import NetworkWithInputEncoding, workloads as W
from neural_lod_gb300.lod import LodGrid
from neural_lod_gb300 import NlodError
from neural_lod_gb300.render import MODE_HOST_ROUNDS, MODE_PERSISTENT, MODE_WAVEFRONT, RenderParams, Renderer, camera, persistent_form

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
    assert r.persistent == (precision != "fp32" and params.mode != MODE_WAVEFRONT)
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


@pytest.mark.parametrize("precision,frac,rel,mode", [("fp32", 0.995, 1e-3, 0), ("fp16", 0.97, 2e-2, MODE_PERSISTENT),
                                                      ("fp16", 0.97, 2e-2, MODE_WAVEFRONT)])
def test_render_matches_oracle(cuda, nlod_lib, precision, frac, rel, mode):
    bits, res, levels = _scene()
    params = RenderParams(width=96, height=64, level=1, max_depth=4, max_vis_queries=24, lod_max_level=6 / 8, lod_input=1.5 / 8,
                          mode=mode)
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


def _frame(precision, params, grid, mode):
    import torch

    vm, tm, vo, to, vp, tp = _nets(precision)
    p = RenderParams(**{**params.__dict__, "mode": mode})
    r = Renderer(vm, tm, grid, p)
    assert r.mode == mode
    n = p.width * p.height
    stats = torch.zeros((n, 2), dtype=torch.int32, device="cuda")
    img = r.frame(ray_stats=stats).cpu().numpy()
    tot = r.stats()
    img2 = r.frame().cpu().numpy()
    assert np.array_equal(img, img2)
    r.close()
    return img, stats.cpu().numpy(), tot


@pytest.mark.parametrize("form", [4, 6, 8, 16])
@pytest.mark.parametrize("precision", ["fp16", "bf16"])
@pytest.mark.parametrize("shape", [(96, 64, 1, 24), (257, 131, 0, 9)])
def test_persistent_form_matches_wavefront_form(cuda, nlod_lib, precision, shape, form):
    """Every persistent organisation (tile pipelines marching their own rays; marcher warps feeding
    two tensor-core groups) against the wavefront rounds: same pixels, same per-ray query counts,
    same totals; ray counts that are not a multiple of a tile and a query cap that drops rays
    included."""
    w, h, level, cap = shape
    bits, res, levels = _scene()
    grid = LodGrid(bits, res, levels)
    params = RenderParams(width=w, height=h, level=level, max_depth=4, max_vis_queries=cap, lod_max_level=6 / 8, lod_input=1.5 / 8)
    img_p, st_p, tot_p = _frame(precision, params, grid, persistent_form(form))
    img_w, st_w, tot_w = _frame(precision, params, grid, MODE_WAVEFRONT)
    print(f"{precision} {w}x{h}: persistent totals {tot_p}, wavefront {tot_w}")
    assert np.array_equal(st_p, st_w)
    assert np.array_equal(img_p.view(np.uint32), img_w.view(np.uint32))
    assert tot_p[0] == tot_w[0] and tot_p[1] == tot_w[1] and tot_p[3] == tot_w[3]
    assert tot_p[1] > 0


@pytest.mark.parametrize("precision", ["fp16", "fp32"])
def test_host_rounds_match_graph_rounds(cuda, nlod_lib, precision):
    """The wavefront rounds issued from the host (one list-size read per round) against the same
    rounds in the frame graph's conditional loop: same pixels, per-ray query counts and totals,
    rounds included; a query cap that drops rays included."""
    bits, res, levels = _scene()
    grid = LodGrid(bits, res, levels)
    params = RenderParams(width=96, height=64, level=1, max_depth=4, max_vis_queries=24, lod_max_level=6 / 8, lod_input=1.5 / 8)
    img_h, st_h, tot_h = _frame(precision, params, grid, MODE_HOST_ROUNDS)
    img_g, st_g, tot_g = _frame(precision, params, grid, MODE_WAVEFRONT)
    assert np.array_equal(st_h, st_g)
    assert np.array_equal(img_h.view(np.uint32), img_g.view(np.uint32))
    assert tot_h == tot_g and tot_h[2] >= 2


def test_persistent_form_needs_tensor_core_modules(cuda, nlod_lib):
    bits, res, levels = _scene()
    grid = LodGrid(bits, res, levels)
    vm, tm, *_ = _nets("fp32")
    with pytest.raises(NlodError):
        Renderer(vm, tm, grid, RenderParams(width=32, height=32, level=1, mode=MODE_PERSISTENT))


@pytest.mark.parametrize("precision", ["fp16", "fp32"])
@pytest.mark.parametrize("threshold,cap", [(0.5, 24), (0.8, 24), (0.8, 7)])
def test_query_chains_match_single_queries(cuda, nlod_lib, precision, threshold, cap):
    """Wavefront rounds with chains of visibility queries marched ahead (max_chain 0: up to 8, and
    3) against one query per ray and round (max_chain 1): the same pixels, per-ray query counts and
    totals; a threshold that rejects most voxels makes the chains long (fewer rounds), and a small
    per-bounce cap drops rays inside chains."""
    bits, res, levels = _scene()
    grid = LodGrid(bits, res, levels)
    params = RenderParams(width=96, height=64, level=1, max_depth=4, max_vis_queries=cap, lod_max_level=6 / 8, lod_input=1.5 / 8,
                          threshold=threshold)
    img1, st1, tot1 = _frame(precision, RenderParams(**{**params.__dict__, "max_chain": 1}), grid, MODE_WAVEFRONT)
    for mc in (0, 3):
        img, st, tot = _frame(precision, RenderParams(**{**params.__dict__, "max_chain": mc}), grid, MODE_WAVEFRONT)
        print(f"{precision} threshold {threshold} cap {cap} max_chain {mc}: totals {tot}, one query per round {tot1}")
        assert np.array_equal(st, st1)
        assert np.array_equal(img.view(np.uint32), img1.view(np.uint32))
        assert tot[0] == tot1[0] and tot[1] == tot1[1] and tot[3] == tot1[3]
        assert tot[2] <= tot1[2]
        if threshold == 0.8:
            assert tot[2] < tot1[2]
    if cap == 7:
        assert tot1[3] > 0
