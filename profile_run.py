"""Small, self-contained runs of single kernels of the hot path, for ncu captures.

    python profile_run.py query  [--precision fp16] [--n 2097152] [--iters 3] [--variant v]
    python profile_run.py visq   [--n 65536] [--ml 0.5] [--variant v]
    python profile_run.py train  [--precision fp16] [--n 262144]  [--iters 3]
    python profile_run.py render [--precision fp16] [--iters 3] [--mode 0|1|2|3|256+f] [--size 1024]
    python profile_run.py voxelize [--iters 3]
    python profile_run.py sampler  [--iters 3]
    python profile_run.py calib    [--n 2097152] [--iters 5]   # gather / scatter floors

`query` runs the throughput-query forward (the bench's headline kernel) `iters` times on the
bench's inputs; `train` runs visibility training steps.  Each run ends with a status check, so a
capture only starts after a clean run (the same command without ncu exits 0 first).
"""
from __future__ import annotations

import argparse
import sys
from pathlib import Path

sys.path.insert(0, str(Path(__file__).resolve().parent))


def pick_variant(N, m, x, out, a, dev):
    """--variant, or every variant's median time per call (L2 flushed before each launch) and then
    the autotuner's pick."""
    import torch

    if a.variant >= 0:
        m.kernel_variant = a.variant
    elif a.precision != "fp32":
        flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
        for v in range(m.n_kernel_variants):
            try:
                m.kernel_variant = v
            except N.NlodError:
                continue
            ts = []
            for _ in range(15):
                flush.fill_(1)
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                m.inference(x, out)
                e1.record()
                e1.synchronize()
                ts.append(e0.elapsed_time(e1))
            print(f"variant {v}: {sorted(ts)[7]:.4f} ms")
        m.autotune(x, out)
    print("variant", m.kernel_variant)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("what", choices=["query", "train", "train_thr", "visq", "render", "voxelize", "sampler", "calib"])
    ap.add_argument("--precision", default="fp16")
    ap.add_argument("--n", type=int, default=0)
    ap.add_argument("--iters", type=int, default=3)
    ap.add_argument("--variant", type=int, default=-1, help="tensor-core kernel variant (-1: autotune)")
    ap.add_argument("--mode", type=int, default=0,
                    help="render form: 0 auto, 1 wavefront, 2 persistent, 3 host-issued rounds, 256+f one persistent organisation")
    ap.add_argument("--size", type=int, default=1024, help="render image width and height")
    ap.add_argument("--ml", type=float, default=-1.0, help="visq: one max level fraction for the batch (default: per element)")
    a = ap.parse_args()

    import numpy as np
    import torch

    import neural_lod_gb300 as N
    from neural_lod_gb300 import workloads as W
    from neural_lod_gb300.build import build_library

    build_library()
    dev = torch.device("cuda:0")
    if a.what == "query":
        n = a.n or W.WORKLOADS["throughput_query"]["batch"]
        enc, net = W.throughput_configs()
        m = N.NetworkWithInputEncoding(10, 3, enc, net, precision=a.precision)
        x = torch.from_numpy(W.throughput_inputs(n, seed=1)).to(dev)
        out = torch.empty((n, 3), device=dev)
        pick_variant(N, m, x, out, a, dev)
        for _ in range(a.iters):
            m.inference(x, out)
    elif a.what == "visq":
        n = a.n or W.WORKLOADS["visibility_query"]["batch"]
        enc, net = W.visibility_configs()
        m = N.NetworkWithInputEncoding(6, 1, enc, net, precision=a.precision)
        xv, _, frac = W.visibility_inputs(n, seed=2)
        x = torch.from_numpy(xv).to(dev)
        if a.ml >= 0:
            m.set_max_level(a.ml)   # one max level for the batch (the renderer's queries)
        else:
            m.set_max_level_gpu(torch.from_numpy(frac).to(dev))
        out = torch.empty((n, 1), device=dev)
        pick_variant(N, m, x, out, a, dev)
        for _ in range(a.iters):
            m.inference(x, out)
    elif a.what == "render":
        from neural_lod_gb300.lod import LodGrid
        from neural_lod_gb300.render import RenderParams, Renderer

        occ = W.value_noise_occupancy(256, seed=5, spacing=16, density=0.3)
        pyr = LodGrid(W.pack_bits(occ.repeat(2, 0).repeat(2, 1).repeat(2, 2)), 512, 8)
        venc, vnet = W.visibility_configs()
        henc, hnet = W.throughput_configs()
        rv = N.NetworkWithInputEncoding(6, 1, venc, vnet, precision=a.precision)
        rt = N.NetworkWithInputEncoding(10, 3, henc, hnet, precision=a.precision)
        rv.set_params(W.xavier_params(N.layout(venc, vnet, 6, 1), seed=12))
        rt.set_params(W.xavier_params(N.layout(henc, hnet, 10, 3), seed=13))
        p = RenderParams(width=a.size, height=a.size, level=3, lod_max_level=4 / 8, lod_input=3.5 / 8, seed=42, mode=a.mode)
        if a.precision != "fp32":
            # the bench's kernel organisations for the frame's rounds
            rv.set_max_level(p.lod_max_level)
            rv.autotune(torch.from_numpy(W.visibility_inputs(1 << 20, seed=6)[0]).to(dev), torch.empty((1 << 20, 1), device=dev))
            rt.autotune(torch.from_numpy(W.throughput_inputs(1 << 16, seed=6)).to(dev), torch.empty((1 << 16, 3), device=dev))
            print("variants", rv.kernel_variant, rt.kernel_variant)
        r = Renderer(rv, rt, pyr, p)
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(2 * a.iters)]
        for i in range(a.iters):
            ev[2 * i].record()
            r.frame()
            ev[2 * i + 1].record()
        torch.cuda.synchronize()
        print("stats", r.stats(), "form", r.mode, "frame ms", [round(ev[2 * i].elapsed_time(ev[2 * i + 1]), 3) for i in range(a.iters)])
        n = p.width * p.height
        m = rv
    elif a.what == "sampler":
        # the bench's generator workload: reference sampler defaults on the 512^3 value-noise scene,
        # 2^18 visibility samples with targets, 2^20 throughput samples with targets and compaction
        from neural_lod_gb300.lod import LodGrid
        from neural_lod_gb300.sampler import Sampler, SamplerParams

        occ = W.value_noise_occupancy(256, seed=5, spacing=16, density=0.3)
        pyr = LodGrid(W.pack_bits(occ.repeat(2, 0).repeat(2, 1).repeat(2, 2)), 512, 8)
        sp = Sampler(pyr, SamplerParams(grid_res=512, n_lods=7))
        for it in range(a.iters):
            xg, qg, _ = sp.sample_visibility(it, 1 << 18)
            sp.trace_visibility(qg)
            xt, qt, _ = sp.sample_throughput(it, 1 << 20)
            yt, _ = sp.trace_throughput(qt, xt, it)
            sp.compact(xt, yt)
        sp.sync_status()
        torch.cuda.synchronize()
        print("ok sampler")
        return
    elif a.what == "calib":
        # the memory-side floors on the bench's grids: the throughput query's gathers (2^21 queries,
        # FP16 tables) and the training scatters (throughput 2^20, visibility 2^18 samples)
        import statistics

        enc, net = W.throughput_configs()
        m = N.NetworkWithInputEncoding(10, 3, enc, net, loss=W.THROUGHPUT_LOSS, optimizer=W.THROUGHPUT_OPTIMIZER, precision="fp16")
        m.set_params(W.xavier_params(N.layout(enc, net, 10, 3), seed=10))
        nq = a.n or W.WORKLOADS["throughput_query"]["batch"]
        g = [m.calib_gathers(nq) for _ in range(max(3, a.iters))]
        st = [m.calib_scatter(1 << 20) for _ in range(max(3, a.iters))]
        venc, vnet = W.visibility_configs(16)
        mv = N.NetworkWithInputEncoding(6, 1, venc, vnet, loss=W.VISIBILITY_LOSS, optimizer=W.VISIBILITY_OPTIMIZER, precision="fp16")
        mv.set_params(W.xavier_params(N.layout(venc, vnet, 6, 1), seed=11))
        sv = [mv.calib_scatter(1 << 18) for _ in range(max(3, a.iters))]
        print(f"gathers of {nq} throughput queries: median {statistics.median(g):.4f} ms ({[round(v, 4) for v in g]})")
        print(f"scatter of 2^20 throughput samples: median {statistics.median(st):.4f} ms")
        print(f"scatter of 2^18 visibility samples: median {statistics.median(sv):.4f} ms")
        m.sync_status()
        mv.sync_status()
        return
    elif a.what == "voxelize":
        from neural_lod_gb300 import voxelize as V

        mesh = torch.from_numpy(W.synthetic_mesh()).to(dev)
        for _ in range(a.iters):
            bits = V.voxelize(mesh, 1024)
        n = mesh.shape[0]
        torch.cuda.synchronize()
        print("ok voxelize", n)
        return
    elif a.what == "train_thr":
        # the throughput network's training step: 2^20 samples, RelativeL2, Ema(0.95) of
        # ExponentialDecay(Adam) (the bench's throughput_train workload)
        n = a.n or (1 << 20)
        enc, net = W.throughput_configs()
        m = N.NetworkWithInputEncoding(10, 3, enc, net, loss=W.THROUGHPUT_LOSS, optimizer=W.THROUGHPUT_OPTIMIZER,
                                       precision=a.precision)
        m.set_params(W.xavier_params(N.layout(enc, net, 10, 3), seed=10))
        x = torch.from_numpy(W.throughput_inputs(n, seed=4)).to(dev)
        td = torch.from_numpy(np.random.default_rng(4).random((n, 3)).astype(np.float32)).to(dev)
        for _ in range(a.iters):
            m.training_step(x, td)
    else:
        n = a.n or W.WORKLOADS["visibility_train"]["batch"]
        enc, net = W.visibility_configs(16)
        m = N.NetworkWithInputEncoding(6, 1, enc, net, loss=W.VISIBILITY_LOSS, optimizer=W.VISIBILITY_OPTIMIZER,
                                       precision=a.precision)
        xv, _, _ = W.visibility_inputs(n, seed=3)
        t = (np.random.default_rng(3).random((n, 1)) < 0.3).astype(np.float32)
        x, td = torch.from_numpy(xv).to(dev), torch.from_numpy(t).to(dev)
        for _ in range(a.iters):
            m.training_step(x, td)
    m.sync_status()
    torch.cuda.synchronize()
    print("ok", a.what, a.precision, n)


if __name__ == "__main__":
    main()
