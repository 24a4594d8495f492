"""Golden vectors from tiny-cuda-nn itself, for the network path.

    python -m oracle.build_tcnn build                 # on a GPU machine, sources staged first
    python tests/golden/make_tcnn_golden.py OUT.npz   # writes the fixture (committed as tcnn_golden.npz)

tiny-cuda-nn is the one compiled from the reference's vendored sources (rptr/ext/tiny-cuda-nn)
behind oracle/tcnn_harness.cu.  Every case injects the same FP32 parameter vector into it
(Trainer::set_params_full_precision, trainer.h:234-246) that the tests give the FP64 oracle and
this library; inputs, targets and parameters are regenerated from the seeds stored here, so the
fixture holds only tiny-cuda-nn's outputs:

  vis_query      visibility query network (8-level grid, SH 4, 32->64->64->1 sigmoid), 4,096
                 queries, with and without the per-element max level (GridEncoding::
                 set_max_level_gpu) that carries the LoD index
  thr_query      throughput query network (16-level grid with 2^19 entries, SH 4 for wi and wo,
                 the LoD one-hot given as 8 identity inputs; 72->80 -> 4x64 -> 3 exp), 4,096
  arcade_query   the reference's shipped arcade throughput configuration (7 levels, SH 8 x2,
                 128-wide, no output activation), 2,048 queries
  vis_train      visibility training network (16 levels, BCE, Adam lr 1e-2 beta 0.9/0.99
                 eps 1e-15), 4,096 samples: the loss and the gradients of one step
                 (Trainer::training_step without the optimizer), and the parameters after one
                 full step (with the optimizer) from the same start
  thr_train      throughput network with RelativeL2 and EMA(0.95) of ExponentialDecay of Adam,
                 4,096 samples: three full steps, then the inference outputs (EMA weights)
Gradients are stored for every MLP parameter and for a seeded sample of grid entries.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402
from neural_lod_gb300 import workloads as W  # noqa: E402

N_QUERY = 4096
N_ARCADE = 2048
N_TRAIN = 4096
N_GRID_SAMPLE = 8192


def grid_sample(spec: dict, seed: int) -> np.ndarray:
    n_net = spec["n_params_network"]
    return np.sort(np.random.default_rng(seed).choice(np.arange(n_net, spec["n_params"]), N_GRID_SAMPLE, replace=False))


# Every case: (name, configs, n_in, n_out, params seed, grid_scale, input maker)
CASES = {
    "vis_query": dict(cfg=lambda: W.visibility_configs(8), n_in=6, n_out=1, seed=5, grid_scale=0.5),
    "thr_query": dict(cfg=W.thr_identity_configs, n_in=17, n_out=3, seed=6, grid_scale=0.2),
    "arcade_query": dict(cfg=lambda: W.arcade_throughput_configs()[:2], n_in=9, n_out=3, seed=7, grid_scale=0.2),
    "vis_train": dict(cfg=lambda: W.visibility_configs(16), n_in=6, n_out=1, seed=8, grid_scale=0.3,
                      loss=W.VISIBILITY_LOSS, optimizer=W.VISIBILITY_OPTIMIZER),
    "thr_train": dict(cfg=W.thr_identity_configs, n_in=17, n_out=3, seed=9, grid_scale=0.2,
                      loss=W.THROUGHPUT_LOSS, optimizer=W.THROUGHPUT_OPTIMIZER),
}


def case_params(name: str):
    c = CASES[name]
    enc, net = c["cfg"]()
    spec = oracle.model_spec(enc, net, c["n_in"], c["n_out"])
    return enc, net, spec, W.test_params(spec, seed=c["seed"], grid_scale=c["grid_scale"])


def case_inputs(name: str):
    """(x, per-element max level or None, target or None) of a case."""
    if name == "vis_query":
        x, _, frac = W.visibility_inputs(N_QUERY, seed=21)
        return x, frac, None
    if name == "thr_query":
        return W.thr_identity_inputs(N_QUERY, seed=22), None, None
    if name == "arcade_query":
        rng = np.random.default_rng(23)
        pos = rng.random((N_ARCADE, 3))
        d = rng.standard_normal((N_ARCADE, 6))
        d[:, :3] /= np.linalg.norm(d[:, :3], axis=1, keepdims=True)
        d[:, 3:] /= np.linalg.norm(d[:, 3:], axis=1, keepdims=True)
        return np.concatenate([pos, (d + 1) / 2], axis=1).astype(np.float32), None, None
    if name == "vis_train":
        x, _, _ = W.visibility_inputs(N_TRAIN, seed=24, n_grid_levels=16)
        return x, None, W.binary_targets(N_TRAIN, 25)
    if name == "thr_train":
        return W.thr_identity_inputs(N_TRAIN, seed=26), None, W.rgb_targets(N_TRAIN, 27)
    raise KeyError(name)


def main(out_path: str) -> None:
    import torch

    from oracle.tcnn import TcnnModel

    dev = torch.device("cuda:0")
    res = {}
    for name, c in CASES.items():
        enc, net, spec, params = case_params(name)
        x, ml, t = case_inputs(name)
        m = TcnnModel(c["n_in"], c["n_out"], enc, net, c.get("loss"), c.get("optimizer"))
        assert m.n_params == spec["n_params"], (name, m.n_params, spec["n_params"])
        assert m.encoded_width == spec["enc_width"], (name, m.encoded_width, spec["enc_width"])
        m.set_params(params)
        xd = torch.from_numpy(x).to(dev)
        if name.endswith("_query"):
            res[f"{name}/out"] = m.inference(xd).cpu().numpy()
            if ml is not None:
                md = torch.from_numpy(ml).to(dev)
                m.set_max_level_gpu(md)
                res[f"{name}/out_masked"] = m.inference(xd).cpu().numpy()
                m.set_max_level_gpu(None)
        elif name == "vis_train":
            td = torch.from_numpy(t).to(dev)
            m.training_step(xd, td, run_optimizer=False)
            res[f"{name}/loss"] = np.float64(m.loss())
            g = m.gradients()
            idx = grid_sample(spec, 31)
            res[f"{name}/grad_net"] = g[: spec["n_params_network"]]
            res[f"{name}/grid_idx"] = idx
            res[f"{name}/grad_grid"] = g[idx]
            m.set_params(params)
            m.training_step(xd, td, run_optimizer=True)
            torch.cuda.synchronize()
            p1 = m.get_params()
            res[f"{name}/params1_net"] = p1[: spec["n_params_network"]]
            res[f"{name}/params1_grid"] = p1[idx]
        elif name == "thr_train":
            td = torch.from_numpy(t).to(dev)
            for _ in range(3):
                m.training_step(xd, td, run_optimizer=True)
            res[f"{name}/loss3"] = np.float64(m.loss())
            res[f"{name}/out3"] = m.inference(xd).cpu().numpy()
        torch.cuda.synchronize()
        print(name, "ok", flush=True)
    res["meta/torch"] = np.array(torch.__version__)
    res["meta/gpu"] = np.array(torch.cuda.get_device_name(0))
    np.savez_compressed(out_path, **res)
    print("wrote", out_path, sorted(res))


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else str(Path(__file__).with_name("tcnn_golden.npz")))
