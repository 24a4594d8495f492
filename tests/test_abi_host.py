"""Host-side tests of the C ABI (no GPU): the library loads, exports every declared symbol,
computes the same layouts as the oracle's independent restatement, and rejects bad configs
before any launch."""
import re
from pathlib import Path

import pytest

import oracle
from neural_lod_gb300 import NlodError, layout, workloads as W

ROOT = Path(__file__).resolve().parents[1]


def declared_symbols():
    text = (ROOT / "include" / "nlod.h").read_text()
    return sorted(set(re.findall(r"NLOD_API[^;(]*?\b(nlod_\w+)\s*\(", text)))


def test_library_exports_every_declared_symbol(nlod_lib):
    import subprocess

    syms = declared_symbols()
    assert len(syms) >= 25
    out = subprocess.run(["nm", "-D", "--defined-only", str(ROOT / "neural_lod_gb300" / "libnlod.so")],
                         capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\b(nlod_\w+)\b", out))
    missing = [s for s in syms if s not in exported]
    assert not missing, missing
    for s in syms:
        getattr(nlod_lib, s)


def test_python_binding_covers_header(nlod_lib):
    from neural_lod_gb300._lib import SIGNATURES

    bound = {name for name, _, _ in SIGNATURES}
    assert set(declared_symbols()) <= bound


CONFIGS = [
    ("visibility_query", W.visibility_configs(), 6, 1),
    ("throughput_query", W.throughput_configs(), 10, 3),
    ("visibility_train", W.visibility_configs(16), 6, 1),
]


@pytest.mark.parametrize("name,cfg,n_in,n_out", CONFIGS, ids=[c[0] for c in CONFIGS])
def test_layout_matches_oracle(nlod_lib, name, cfg, n_in, n_out):
    enc, net = cfg
    got = layout(enc, net, n_in, n_out)
    ref = oracle.model_spec(enc, net, n_in, n_out)
    for k in ("enc_width", "width", "n_layers", "n_params_network", "n_params", "act", "out_act"):
        assert got[k] == ref[k], k
    assert [(l["in"], l["out"], l["offset"]) for l in got["layers"]] == [(l["in"], l["out"], l["offset"]) for l in ref["layers"]]
    for a, b in zip(got["slots"], ref["slots"], strict=True):
        for k in ("type", "in_begin", "n_in", "out_begin", "out_width", "n_pad", "degree", "n_bins"):
            assert a[k] == b[k], (k, a, b)
    for a, b in zip(got["grids"], ref["grids"], strict=True):
        assert a["offset"] == b["offset"]
        assert a["res"] == b["res"]
        assert a["param_offset"] == b["param_offset"]
        assert [float(x) for x in a["scale"]] == pytest.approx(b["scale"], rel=0, abs=0)


def test_known_sizes():
    # Parameter counts of the three workloads (grid entries from the offset tables).
    assert layout(*W.visibility_configs(), 6, 1)["grids"][0]["offset"][-1] == 392256
    assert layout(*W.throughput_configs(), 10, 3)["grids"][0]["offset"][-1] == 6513496
    assert layout(*W.visibility_configs(16), 6, 1)["grids"][0]["offset"][-1] == 916544
    assert layout(*W.throughput_configs(), 10, 3)["enc_width"] == 80


def test_sh_padding_goes_first_and_composite_pads_last_nested():
    enc = {"otype": "Composite", "nested": [
        {"otype": "HashGrid", "n_dims_to_encode": 3, "n_levels": 7, "base_resolution": 8, "per_level_scale": 2.0},
        {"otype": "SphericalHarmonics", "n_dims_to_encode": 3, "degree": 8},
        {"otype": "SphericalHarmonics", "n_dims_to_encode": 3, "degree": 8}]}
    net = {"otype": "FullyFusedMLP", "n_neurons": 128, "n_hidden_layers": 4, "activation": "ReLU", "output_activation": "None"}
    got = layout(enc, net, 9, 3)
    assert got["enc_width"] == 144
    assert [s["n_pad"] for s in got["slots"]] == [0, 0, 2]
    assert got["slots"][2]["out_begin"] == 14 + 64


@pytest.mark.parametrize("enc,net,n_in,n_out,msg", [
    ({"otype": "HashGrid", "n_features_per_level": 3}, {"otype": "FullyFusedMLP", "n_neurons": 64}, 3, 1, "n_features_per_level"),
    ({"otype": "HashGrid"}, {"otype": "FullyFusedMLP", "n_neurons": 48}, 3, 1, "16, 32, 64, and 128"),
    ({"otype": "SphericalHarmonics", "degree": 9}, {"otype": "FullyFusedMLP", "n_neurons": 64}, 3, 1, "degree 8"),
    ({"otype": "SphericalHarmonics"}, {"otype": "FullyFusedMLP", "n_neurons": 64}, 2, 1, "3D directions"),
    ({"otype": "Frequency"}, {"otype": "FullyFusedMLP", "n_neurons": 64}, 3, 1, "Unsupported encoding"),
    ({"otype": "HashGrid"}, {"otype": "FullyFusedMLP", "n_neurons": 64, "n_hidden_layers": 0}, 3, 1, "at least 1 hidden"),
    ({"otype": "HashGrid"}, {"otype": "FullyFusedMLP", "n_neurons": 64}, 3, 17, "n_output_dims"),
    ({"otype": "Composite", "nested": [{"otype": "HashGrid", "n_dims_to_encode": 4}]}, {"otype": "FullyFusedMLP"}, 3, 1, "more dims"),
    ("{not json", {"otype": "FullyFusedMLP"}, 3, 1, "json"),
    # the fused kernels' hidden epilogues implement exactly these two activations
    ({"otype": "HashGrid"}, {"otype": "FullyFusedMLP", "n_neurons": 64, "activation": "Sigmoid"}, 3, 1, "ReLU or None"),
    ({"otype": "HashGrid"}, {"otype": "FullyFusedMLP", "n_neurons": 64, "activation": "Exponential"}, 3, 1, "ReLU or None"),
])
def test_bad_configs_are_rejected(nlod_lib, enc, net, n_in, n_out, msg):
    with pytest.raises(NlodError) as e:
        layout(enc, net, n_in, n_out)
    assert e.value.code == 1
    assert msg.lower() in str(e.value).lower()


def test_module_create_rejects_bad_config_before_touching_the_gpu(nlod_lib):
    from neural_lod_gb300 import NetworkWithInputEncoding

    with pytest.raises(NlodError) as e:
        NetworkWithInputEncoding(3, 1, {"otype": "HashGrid"}, {"otype": "FullyFusedMLP", "n_neurons": 48})
    assert e.value.code == 1
    with pytest.raises(NlodError):
        NetworkWithInputEncoding(3, 1, {"otype": "HashGrid"}, {"otype": "FullyFusedMLP", "n_neurons": 64},
                                 loss={"otype": "Hinge"})
    with pytest.raises(NlodError):
        NetworkWithInputEncoding(3, 1, {"otype": "HashGrid"}, {"otype": "FullyFusedMLP", "n_neurons": 64},
                                 optimizer={"otype": "Shampoo"})


def test_entry_points_reject_null_arguments_before_touching_the_gpu(nlod_lib):
    """Every call returns NLOD_ERR_INVALID (1) with a message for a NULL module or buffer, and
    never throws across the boundary."""
    import ctypes as C

    L = nlod_lib
    out = C.c_void_p()
    calls = {
        "nlod_inference": lambda: L.nlod_inference(None, None, 128, None, None),
        "nlod_inference_host": lambda: L.nlod_inference_host(None, None, 128, None, None),
        "nlod_training_step": lambda: L.nlod_training_step(None, None, 128, None, None, None),
        "nlod_training_step_noalloc": lambda: L.nlod_training_step_noalloc(None, None, 128, None, None, None),
        "nlod_training_step_noalloc (batch 100)": lambda: L.nlod_training_step_noalloc(None, None, 100, None, None, None),
        "nlod_forward": lambda: L.nlod_forward(None, None, 128, None, None, None),
        "nlod_optimizer_step": lambda: L.nlod_optimizer_step(None, None),
        "nlod_autotune": lambda: L.nlod_autotune(None, None, 128, None, None),
        "nlod_calib_gathers": lambda: L.nlod_calib_gathers(None, None, 128, None),
        "nlod_calib_scatter": lambda: L.nlod_calib_scatter(None, None, 128, None),
        "nlod_serialize": lambda: L.nlod_serialize(None, 1, C.byref(out)),
        "nlod_deserialize": lambda: L.nlod_deserialize(None, b"{}"),
        "nlod_set_params": lambda: L.nlod_set_params(None, None, 0, 0),
        "nlod_lod_grid_create": lambda: L.nlod_lod_grid_create(None, 64, 4, None, C.byref(out)),
        "nlod_first_active_voxel": lambda: L.nlod_first_active_voxel(None, 0, None, 128, *([None] * 8)),
        "nlod_voxelize": lambda: L.nlod_voxelize(None, 10, 64, None, None, None, None),
        "nlod_renderer_create": lambda: L.nlod_renderer_create(None, None, None, None, C.byref(out)),
        "nlod_render_frame": lambda: L.nlod_render_frame(None, None, None, None),
        "nlod_optimal_thresholds": lambda: L.nlod_optimal_thresholds(None, None, 16, 4, 0, C.c_float(1.0), None, None),
        "nlod_morton_voxels": lambda: L.nlod_morton_voxels(None, 64, None, 0, None, None),
        "nlod_sample_visibility": lambda: L.nlod_sample_visibility(None, None, None, 0, 128, None, None, None, None),
        "nlod_trace_visibility": lambda: L.nlod_trace_visibility(None, None, None, 128, None, None),
    }
    for name, call in calls.items():
        assert call() == 1, name
        assert L.nlod_last_error(), name
    assert L.nlod_n_params(None) == 0


def test_last_error_is_per_thread(nlod_lib):
    """nlod_last_error() reports the calling thread's last failure only."""
    import threading

    L = nlod_lib
    seen = {}

    def worker():
        assert L.nlod_inference(None, None, 128, None, None) == 1
        seen["worker"] = L.nlod_last_error()

    t = threading.Thread(target=worker)
    t.start()
    t.join()
    assert seen["worker"] == b"module is NULL"
    # this thread made no failing call since its own last one: a different message or none
    assert L.nlod_set_params(None, None, 0, 0) == 1
    mine = L.nlod_last_error()
    t2 = threading.Thread(target=worker)
    t2.start()
    t2.join()
    assert L.nlod_last_error() == mine
