"""The host restatement of the wavefront render query (oracle.render) on small scenes: escaped
rays take the background, no voxel is accepted above a threshold of 1, per-ray query counts obey
the caps, and results do not depend on the thread schedule."""
import numpy as np

import oracle
from neural_lod_gb300 import workloads as W
from neural_lod_gb300.render import RenderParams

CAM = np.array([51.2, 40.0, 60.8, 0.26, 0.0, -0.22, -0.04, 0.34, -0.05, -0.56, -0.39, -0.73], np.float32)


def _nets():
    venc, vnet = W.visibility_configs()
    henc, hnet = W.throughput_configs()
    vo, to = oracle.Oracle(venc, vnet, 6, 1), oracle.Oracle(henc, hnet, 10, 3)
    return vo, W.xavier_params(vo.spec, seed=1), to, W.test_params(to.spec, seed=2, grid_scale=0.2)


def test_background_and_caps():
    vo, vp, to, tp = _nets()
    lvl = oracle.LodLevel(W.pack_bits(np.zeros((32, 32, 32), bool)), 32, 0)
    P = RenderParams(width=24, height=16, level=0, background=(0.1, 0.2, 0.3))
    img, st, tot = oracle.render(vo, vp, to, tp, lvl, P, CAM)
    assert np.allclose(img, [0.1, 0.2, 0.3]) and tot == (0, 0, 0)
    occ = W.value_noise_occupancy(32, seed=3, spacing=4, density=0.3)
    lvl = oracle.LodLevel(W.pack_bits(occ), 32, 0)
    P = RenderParams(width=24, height=16, level=0, threshold=1.5, max_vis_queries=3)
    img, st, tot = oracle.render(vo, vp, to, tp, lvl, P, CAM)
    assert tot[1] == 0 and st[:, 0].max() <= 3 and tot[2] > 0
    P = RenderParams(width=24, height=16, level=0, max_depth=3, max_vis_queries=40)
    img, st, tot = oracle.render(vo, vp, to, tp, lvl, P, CAM)
    assert st[:, 1].max() <= 2                      # throughput queries only before the last vertex
    assert tot[0] > 0 and tot[1] > 0
    img2, st2, _ = oracle.render(vo, vp, to, tp, lvl, P, CAM)
    assert np.array_equal(img, img2) and np.array_equal(st, st2)


def test_render_params_validation_on_the_host(nlod_lib):
    """nlod_render_camera validates the parameters without a GPU: the query-chain cap accepts 0-64
    (0: the default of 8), the struct keeps its size with the cap in the former padding."""
    import ctypes as C

    from neural_lod_gb300 import NlodError
    from neural_lod_gb300.render import _Params, camera

    assert C.sizeof(_Params) == 112
    for mc in (0, 1, 8, 64):
        cam = camera(RenderParams(width=16, height=8, level=0, max_chain=mc), 32)
        assert np.all(np.isfinite(cam))
    try:
        camera(RenderParams(width=16, height=8, level=0, max_chain=65), 32)
    except NlodError as e:
        assert e.code == 1 and "max_chain" in str(e)
    else:
        raise AssertionError("max_chain 65 accepted")
