"""Benchmark of the neural-LoD hot path on GB300 (one JSON line on stdout, rank 0).

Headline workload: the throughput query forward at batch 2^21 (16-level hash grid with 2^19
entries/level + two degree-4 SH encodings + LoD one-hot -> 80-wide input -> 4 x 64 ReLU -> 3
exp outputs), FP16 tcgen05 form, inputs resident in HBM.  A "step" is one fused query launch
over the whole batch.  Also reported: the same workload in the plain FP32 form, the end-to-end
call from pinned host buffers, the visibility query (batch 65,536), the visibility and throughput
training steps (fwd + loss + bwd + Adam), the render frame, the sample generator, the voxelizer,
the voxelize + train run, the FP64-oracle error, a scalar FP32 CPU baseline of the same encoding
+ MLP, and tiny-cuda-nn built from the reference's sources on the same GPU and workloads (live
when oracle/_ref holds its build, else the figures committed in profiles/tcnn_comparison.md).
Times are the median of the timed steps (p99 and mean beside the headline), each step between
CUDA events on the launching stream.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Under torchrun (N > 1) every rank runs an independent replica of the workload on its own GPU
(the path has no data exchange); value = total queries of all ranks / max-over-ranks time.
Between timed steps the L2 cache is flushed by writing a 256 MiB buffer (outside the events).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "queries/s fwd & samples/s train, FP16-TC vs plain FP32, 1 GB300, err≤1e-3 vs FP64"
UNIT = "queries/s"
FLOP_PER_QUERY = 34176          # 2 * (72*64 + 3*64*64 + 64*3), real (unpadded) layers
BYTES_PER_QUERY = 52            # 40 B input + 12 B output
TRAIN_FLOP_PER_SAMPLE = 43392   # visibility_train fwd 14,464 + bwd 28,928


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": d["hbm_gbs"], "bf16_tflops": d["bf16_tflops"], "source": "measured"}
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "source": "fallback"}


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 20 ms while the timed region runs; entering
    waits (up to 3 s) for the first sample, so that the samples cover the region."""

    FIELDS = "index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown," \
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap"

    def __init__(self, device_index: int):
        self.proc = None
        self.dev = device_index
        self.out_path = Path(os.environ.get("TMPDIR", "/tmp")) / f"nlod_clocks_{os.getpid()}.csv"

    def __enter__(self):
        try:
            self.fh = open(self.out_path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-lms", "20", "-i", str(self.dev)], stdout=self.fh, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
            return self
        t0 = time.perf_counter()
        while time.perf_counter() - t0 < 3.0 and self.proc.poll() is None:
            try:
                if self.out_path.stat().st_size > 0:
                    break
            except OSError:
                pass
            time.sleep(0.01)
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.fh.close()

    def summary(self):
        if self.proc is None or not self.out_path.exists():
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.out_path.read_text().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        try:
            self.out_path.unlink()
        except OSError:
            pass
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "samples": len(sm),
                "reasons": sorted(reasons)}


def time_steps(fn, steps, warmup, flush=None, stream=None, barrier=None):
    """Per-step CUDA-event durations (ms) of fn() on the current stream, L2 flushed in between.
    `barrier` (the process group's, for several ranks) brackets exactly the timed steps, each
    side after a device synchronisation."""
    import torch

    for _ in range(warmup):
        if flush is not None:
            flush()
        fn()
    torch.cuda.synchronize()
    if barrier is not None:
        barrier()
    times = []
    for _ in range(steps):
        if flush is not None:
            flush()
        s = torch.cuda.Event(enable_timing=True)
        e = torch.cuda.Event(enable_timing=True)
        s.record()
        fn()
        e.record()
        times.append((s, e))
    torch.cuda.synchronize()
    if barrier is not None:
        barrier()
    return [s.elapsed_time(e) for s, e in times]


def max_over_ranks(values, dist_mod, device):
    """Element-wise maximum of a list of floats over every rank of the default process group."""
    import torch

    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    dist_mod.all_reduce(t, op=dist_mod.ReduceOp.MAX)
    return [float(v) for v in t]


def traffic_from_profile():
    """DRAM bytes per launch of the fused query kernel from the committed ncu summary."""
    p = ROOT / "profiles" / "forward_tc_throughput_query.md"
    if not p.exists():
        return None
    for line in p.read_text().splitlines():
        if line.strip().startswith("traffic_bytes_per_launch:"):
            try:
                return float(line.split(":", 1)[1].strip().split()[0])
            except ValueError:
                return None
    return None


def cpu_baseline(enc, net, n_in, n_out, params, x_all, target_cpu_seconds=12.0):
    """Scalar FP32 host evaluation of the same encoding + MLP over all host threads, on a bounded
    sample of the workload's inputs sized to ~target_cpu_seconds of CPU work."""
    import numpy as np

    import oracle

    orc = oracle.Oracle(enc, net, n_in, n_out)
    probe = x_all[:4096]
    t0 = time.perf_counter()
    _, threads = orc.forward_f32(probe, params)
    dt = time.perf_counter() - t0
    per_query_cpu = dt * threads / probe.shape[0]
    n = int(min(x_all.shape[0], max(4096, target_cpu_seconds / max(per_query_cpu, 1e-9))))
    n = n // 128 * 128
    sample = np.ascontiguousarray(x_all[:n])
    t0 = time.perf_counter()
    _, threads = orc.forward_f32(sample, params)
    dt = time.perf_counter() - t0
    return {"value": n / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"first {n} queries of the throughput_query batch (same inputs and weights), FP32 scalar, {threads} threads"}


def tcnn_comparison(dev, flush, args):
    """tiny-cuda-nn, built from the reference's vendored sources (oracle/build_tcnn.py), on the same
    GPU, workloads and timing as this library's legs: FP16 fully fused MLP + grid encoding, weights
    injected from the same FP32 vectors.  tiny-cuda-nn has no one-hot encoding, so the throughput
    network takes the LoD as 8 identity inputs (17 inputs, the same 72 encoded columns); this
    library is timed on that same form beside it.  Returns None when the build is absent."""
    import torch

    from oracle import tcnn as T
    if not T.available():
        return None
    # a non-default stream, so tiny-cuda-nn's trainer captures its forward + backward in a CUDA
    # graph as it does in the application (trainer.h:175-180); both libraries run on it
    with torch.cuda.stream(torch.cuda.Stream(dev)):
        return _tcnn_comparison(dev, flush, args, T)


def _tcnn_comparison(dev, flush, args, T):
    import numpy as np
    import torch

    import oracle
    from neural_lod_gb300 import NetworkWithInputEncoding, layout, workloads as W

    res = {"live": True, "build": "rptr/ext/tiny-cuda-nn, 11 units + oracle/tcnn_harness.cu, nvcc -O3 sm_103a, TCNN_MIN_GPU_ARCH=103"}
    steps = max(3, args.steps // 2)

    # throughput query, 2^21, 17-input identity form
    n = W.WORKLOADS["throughput_query"]["batch"]
    enc, net = W.thr_identity_configs()
    spec = layout(enc, net, 17, 3)
    params = W.xavier_params(spec, seed=7)
    xh = W.thr_identity_inputs(n, seed=1)
    x = torch.from_numpy(xh).to(dev)
    out = torch.empty((n, 3), device=dev)
    tm = T.TcnnModel(17, 3, enc, net)
    tm.set_params(params)
    t_tc = statistics.median(time_steps(lambda: tm.inference(x, out), steps, 3, flush))
    ref = oracle.Oracle(enc, net, 17, 3).forward(xh[:4096], params)
    err_tc = float(np.abs(tm.inference(x[:4096]).cpu().numpy() - ref).mean())
    del tm
    mo = NetworkWithInputEncoding(17, 3, enc, net, precision="fp16")
    mo.set_params(params)
    mo.autotune(x, out)
    t_ours = statistics.median(time_steps(lambda: mo.inference(x, out), steps, 3, flush))
    err_ours = float(np.abs(mo.inference(x[:4096]).cpu().numpy() - ref).mean())
    del mo
    res["throughput_query"] = {"batch": n, "tcnn_queries_per_s": n / (t_tc * 1e-3), "ours_queries_per_s": n / (t_ours * 1e-3),
                               "ours_over_tcnn": t_tc / t_ours, "tcnn_err_vs_fp64_mean_abs": err_tc,
                               "ours_err_vs_fp64_mean_abs": err_ours}

    # visibility query, 65,536, per-element max level
    nv = W.WORKLOADS["visibility_query"]["batch"]
    venc, vnet = W.visibility_configs()
    vparams = W.xavier_params(layout(venc, vnet, 6, 1), seed=8)
    xv, _, frac = W.visibility_inputs(nv, seed=2)
    xvd, fd = torch.from_numpy(xv).to(dev), torch.from_numpy(frac).to(dev)
    ov = torch.empty((nv, 1), device=dev)
    tm = T.TcnnModel(6, 1, venc, vnet)
    tm.set_params(vparams)
    tm.set_max_level_gpu(fd)
    t_tc = statistics.median(time_steps(lambda: tm.inference(xvd, ov), args.steps, 3, flush))
    del tm
    mo = NetworkWithInputEncoding(6, 1, venc, vnet, precision="fp16")
    mo.set_params(vparams)
    mo.set_max_level_gpu(fd)
    mo.autotune(xvd, ov)
    t_ours = statistics.median(time_steps(lambda: mo.inference(xvd, ov), args.steps, 3, flush))
    del mo
    res["visibility_query"] = {"batch": nv, "tcnn_queries_per_s": nv / (t_tc * 1e-3), "ours_queries_per_s": nv / (t_ours * 1e-3),
                               "ours_over_tcnn": t_tc / t_ours}

    # training steps: visibility 2^18 (BCE, Adam) and throughput 2^20 (RelativeL2, EMA of decay of Adam)
    def train_pair(enc_, net_, n_in, n_out, loss, opt, xt, tt, seed):
        pr = W.xavier_params(layout(enc_, net_, n_in, n_out), seed=seed)
        xd_, td_ = torch.from_numpy(xt).to(dev), torch.from_numpy(tt).to(dev)
        tm_ = T.TcnnModel(n_in, n_out, enc_, net_, loss, opt)
        tm_.set_params(pr)
        t1 = statistics.median(time_steps(lambda: tm_.training_step(xd_, td_), steps, 3, flush))
        del tm_
        mo_ = NetworkWithInputEncoding(n_in, n_out, enc_, net_, loss=loss, optimizer=opt, precision="fp16")
        mo_.set_params(pr)
        lo = torch.empty(1, device=dev)
        t2 = statistics.median(time_steps(lambda: mo_.training_step(xd_, td_, lo), steps, 3, flush))
        del mo_
        nb = xt.shape[0]
        return {"batch": nb, "tcnn_samples_per_s": nb / (t1 * 1e-3), "ours_samples_per_s": nb / (t2 * 1e-3),
                "ours_over_tcnn": t1 / t2}

    nt = W.WORKLOADS["visibility_train"]["batch"]
    tenc, tnet = W.visibility_configs(16)
    xt, _, _ = W.visibility_inputs(nt, seed=3, n_grid_levels=16)
    tt = (np.random.default_rng(3).random((nt, 1)) < 0.5).astype(np.float32)
    res["visibility_train"] = train_pair(tenc, tnet, 6, 1, W.VISIBILITY_LOSS, W.VISIBILITY_OPTIMIZER, xt, tt, 9)
    ntt = 1 << 20
    res["throughput_train"] = train_pair(enc, net, 17, 3, W.THROUGHPUT_LOSS, W.THROUGHPUT_OPTIMIZER,
                                         W.thr_identity_inputs(ntt, seed=4), W.rgb_targets(ntt, 4), 10)
    return res


def committed_tcnn_figures():
    """The tiny-cuda-nn comparison measured earlier on this GPU model (profiles/tcnn_comparison.md,
    its JSON block), for runs where oracle/_ref holds no tiny-cuda-nn build."""
    p = ROOT / "profiles" / "tcnn_comparison.md"
    reason = "tiny-cuda-nn is not built here (python -m oracle.build_tcnn build; about 10 minutes of nvcc)"
    if not p.exists():
        return {"live": False, "reason": reason}
    text = p.read_text()
    try:
        block = text.split("```json", 1)[1].split("```", 1)[0]
        return {"live": False, "reason": reason, "source": "profiles/tcnn_comparison.md", **json.loads(block)}
    except (IndexError, ValueError):
        return {"live": False, "reason": reason}


def run_reference(args, world, rank):
    """Reference arm: the reference's CPU implementation of the path.  tiny-cuda-nn has no CPU
    path, so this times the FP32 restatement of its encoding + MLP (oracle port) on the host
    cores, each step a bounded sample of the throughput_query workload."""
    if rank != 0:
        return
    import numpy as np

    import oracle
    from neural_lod_gb300 import workloads as W

    enc, net = W.throughput_configs()
    orc = oracle.Oracle(enc, net, 10, 3)
    params = W.xavier_params(orc.spec, seed=7)
    n = 1 << 15
    x = W.throughput_inputs(n, seed=1)
    for _ in range(max(args.warmup, 0)):
        orc.forward_f32(x[:4096], params)
    times = []
    threads = 1
    for _ in range(args.steps):
        t0 = time.perf_counter()
        _, threads = orc.forward_f32(x, params)
        times.append(time.perf_counter() - t0)
    total = sum(times)
    value = n * args.steps / total
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic (seeded)", "impl": "reference",
            "config": {"workload": "throughput_query (bounded sample)", "global_batch": n, "precision": "fp32-cpu",
                       "l2": "n/a (host)"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"{n} queries of the throughput_query workload per step, FP32 scalar restatement"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "gpu_launches": 0}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    world, rank, local = dist_env()

    if args.impl == "reference":
        run_reference(args, world, rank)
        return

    import numpy as np
    import torch

    import __graft_entry__

    __graft_entry__.build()
    import oracle
    from neural_lod_gb300 import NetworkWithInputEncoding, layout, workloads as W

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    pg = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=dev)
        pg = dist

    # ---- headline: throughput query forward, batch 2^21 ----
    n = W.WORKLOADS["throughput_query"]["batch"]
    enc, net = W.throughput_configs()
    spec = layout(enc, net, 10, 3)
    params = W.xavier_params(spec, seed=7 + rank)
    x_host = W.throughput_inputs(n, seed=1 + rank)
    x = torch.from_numpy(x_host).to(dev)
    out = torch.empty((n, 3), device=dev)
    m16 = NetworkWithInputEncoding(10, 3, enc, net, precision="fp16")
    m16.set_params(params)
    variant = m16.autotune(x, out)   # picks the fastest tensor-core kernel organisation
    m32 = NetworkWithInputEncoding(10, 3, enc, net, precision="fp32")
    m32.set_params(params)
    flush_buf = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    def flush():
        flush_buf.fill_(1)

    # accuracy vs the FP64 oracle on a sample of the same batch
    ns = 4096
    ref = oracle.Oracle(enc, net, 10, 3).forward(x_host[:ns], params)
    m16.inference(x[:ns], out[:ns])
    err16 = float(np.abs(out[:ns].cpu().numpy() - ref).mean())
    m32.inference(x[:ns], out[:ns])
    err32 = float(np.abs(out[:ns].cpu().numpy() - ref).mean())

    if pg:
        pg.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        t_wall0 = time.perf_counter()
        times16 = time_steps(lambda: m16.inference(x, out), args.steps, args.warmup, flush, barrier=pg.barrier if pg else None)
        t_wall = time.perf_counter() - t_wall0
    clocks = clk.summary()
    torch.cuda.synchronize()
    m16.sync_status()
    ms16 = statistics.median(times16)
    t_sorted = sorted(times16)
    ms16_p99 = t_sorted[min(len(t_sorted) - 1, int(round(0.99 * (len(t_sorted) - 1))))]
    ms16_mean = statistics.mean(times16)
    times32 = time_steps(lambda: m32.inference(x, out), max(3, args.steps // 4), 3, flush)
    ms32 = statistics.median(times32)

    # ---- end to end through the public API from pinned host buffers ----
    # (nlod_inference_host: the kernel reads the pinned input in place over NVLink-C2C, the output
    # comes back with one device-to-host copy; every byte crosses the host link inside the timed region)
    x_pin = torch.from_numpy(x_host).pin_memory()
    out_pin = torch.empty((n, 3), dtype=torch.float32).pin_memory()

    def e2e_step():
        m16.inference_host(x_pin, out_pin)

    times_e2e = time_steps(e2e_step, max(3, args.steps // 2), 3, flush, barrier=pg.barrier if pg else None)
    ms_e2e = statistics.median(times_e2e)

    # ---- visibility query, batch 65,536 ----
    nv = W.WORKLOADS["visibility_query"]["batch"]
    venc, vnet = W.visibility_configs()
    vspec = layout(venc, vnet, 6, 1)
    vparams = W.xavier_params(vspec, seed=8)
    xv, _, frac = W.visibility_inputs(nv, seed=2)
    xvd, fracd = torch.from_numpy(xv).to(dev), torch.from_numpy(frac).to(dev)
    vis = {}
    for prec in ("fp16", "fp32"):
        mv = NetworkWithInputEncoding(6, 1, venc, vnet, precision=prec)
        mv.set_params(vparams)
        mv.set_max_level_gpu(fracd)
        ov = torch.empty((nv, 1), device=dev)
        if prec != "fp32":
            vis["variant"] = mv.autotune(xvd, ov)     # the kernel organisation for this batch size
        tv = time_steps(lambda: mv.inference(xvd, ov), args.steps, 3, flush)
        vis[prec] = nv / (statistics.median(tv) * 1e-3)
        del mv

    # ---- training steps: visibility (2^18, BCE) and throughput (2^20, RelativeL2, EMA/decay Adam) ----
    def train_times(enc_, net_, n_in, n_out, loss, opt, x_np, t_np, seed, precs):
        sp = layout(enc_, net_, n_in, n_out)
        pr = W.xavier_params(sp, seed=seed)
        xd_, td_ = torch.from_numpy(x_np).to(dev), torch.from_numpy(t_np).to(dev)
        res = {}
        for prec in precs:
            mt = NetworkWithInputEncoding(n_in, n_out, enc_, net_, loss=loss, optimizer=opt, precision=prec)
            mt.set_params(pr)
            lo = torch.empty(1, device=dev)
            steps = max(3, args.steps // 2) if prec != "fp32" else max(3, args.steps // 4)
            tr = time_steps(lambda: mt.training_step(xd_, td_, lo), steps, 3, flush)
            mt.sync_status()
            res[prec] = statistics.median(tr)
            del mt
        return res

    from neural_lod_gb300 import samples as S
    from neural_lod_gb300.lod import LodGrid

    nt = W.WORKLOADS["visibility_train"]["batch"]
    tenc, tnet = W.visibility_configs(16)
    noise256 = W.value_noise_occupancy(256, seed=5, spacing=16, density=0.3)
    grid256 = LodGrid(W.pack_bits(noise256), 256, 8)
    xt, _, tt = S.visibility_batch(grid256, nt, seed=3)     # exact-DDA segment transmittance targets
    del grid256
    train = train_times(tenc, tnet, 6, 1, W.VISIBILITY_LOSS, W.VISIBILITY_OPTIMIZER, xt, tt, 9, ("fp16", "bf16", "fp32"))
    ntt = 1 << 20
    henc, hnet = W.throughput_configs()
    xh = W.throughput_inputs(ntt, seed=4)
    th = np.random.default_rng(4).random((ntt, 3)).astype(np.float32)
    ttrain = train_times(henc, hnet, 10, 3, W.THROUGHPUT_LOSS, W.THROUGHPUT_OPTIMIZER, xh, th, 10, ("fp16", "bf16", "fp32"))

    # ---- voxelize + train: 2.0M triangles at 1024^3, pyramid, exact-DDA targets, 1,000 steps at 2^20 ----
    from neural_lod_gb300 import voxelize as V
    mesh = torch.from_numpy(W.synthetic_mesh()).to(dev)
    vmin, vmax = V.mesh_bounds(mesh)
    vb, _, vu = V.mesh_frame(vmin, vmax, 1024)
    vbits = torch.zeros(V.n_words(1024), dtype=torch.int32, device=dev)

    def vox_step():
        vbits.zero_()
        V.voxelize(mesh, 1024, vb, vu, out=vbits)

    tvox = statistics.median(time_steps(vox_step, max(3, args.steps // 2), 3, flush))
    vox_step()
    del mesh
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    grid1024 = LodGrid(vbits, 1024, 8)
    torch.cuda.synchronize()
    t_pyr = time.perf_counter() - t0
    n4 = 1 << 20
    n_batches = 2
    batches = [S.throughput_batch(grid1024, n4, seed=100 + b) for b in range(n_batches)]
    del grid1024, vbits
    xb = [torch.from_numpy(x_).to(dev) for x_, _ in batches]
    tb = [torch.from_numpy(t_).to(dev) for _, t_ in batches]
    x_eval = batches[0][0][:4096]
    e2e4 = {}
    n_steps4 = 1000
    for prec in ("fp16", "bf16", "fp32"):
        m4 = NetworkWithInputEncoding(10, 3, henc, hnet, loss=W.THROUGHPUT_LOSS, optimizer=W.THROUGHPUT_OPTIMIZER, precision=prec,
                                      seed=11)
        lo = torch.empty(1, device=dev)
        losses = []
        s0, s1 = torch.cuda.Event(True), torch.cuda.Event(True)
        torch.cuda.synchronize()
        s0.record()
        for i in range(n_steps4):
            m4.training_step(xb[i % n_batches], tb[i % n_batches], lo)
            if i >= n_steps4 - 10:
                losses.append(lo.clone())
        s1.record()
        s1.synchronize()
        m4.sync_status()
        ms4 = s0.elapsed_time(s1)
        out4 = m4.inference(torch.from_numpy(x_eval).to(dev)).cpu().numpy()
        ref4 = oracle.Oracle(henc, hnet, 10, 3).forward(x_eval, m4.get_params("inference").astype(np.float64))
        e2e4[prec] = {"steps": n_steps4, "ms_total": ms4, "samples_per_s": n_steps4 * n4 / (ms4 * 1e-3),
                      "final_loss": float(torch.stack(losses).mean()), "err_vs_fp64_mean_abs": float(np.abs(out4 - ref4).mean())}
        del m4

    # ---- wavefront render query: 1024^2 rays, LoD pyramid 512^3 -> 4^3, 4 path vertices ----
    from neural_lod_gb300.render import RenderParams, Renderer, camera

    occ = noise256.repeat(2, 0).repeat(2, 1).repeat(2, 2)
    pyr = LodGrid(W.pack_bits(occ), 512, 8)
    del occ
    rlevel = 3
    rparams = RenderParams(width=1024, height=1024, level=rlevel, max_depth=4, max_vis_queries=64,
                           lod_max_level=(7 - rlevel) / 8, lod_input=(rlevel + 0.5) / 8, seed=42)
    venc, vnet = W.visibility_configs()
    henc, hnet = W.throughput_configs()
    rv_params = W.xavier_params(layout(venc, vnet, 6, 1), seed=12)
    rt_params = W.xavier_params(layout(henc, hnet, 10, 3), seed=13)
    render = {}
    from neural_lod_gb300.render import MODE_WAVEFRONT
    for form in ("fp16", "fp16_wavefront", "fp32"):
        prec = form.split("_")[0]
        rv = NetworkWithInputEncoding(6, 1, venc, vnet, precision=prec)
        rt = NetworkWithInputEncoding(10, 3, henc, hnet, precision=prec)
        rv.set_params(rv_params)
        rt.set_params(rt_params)
        if prec != "fp32":
            # kernel organisations for the frame's large rounds (0.5-0.8 M visibility queries at the
            # frame's max level; throughput lists are evaluated from 32 K rows up)
            xa = torch.from_numpy(W.visibility_inputs(1 << 20, seed=6)[0]).to(dev)
            rv.set_max_level(rparams.lod_max_level)
            rv.autotune(xa, torch.empty((1 << 20, 1), device=dev))
            xb = torch.from_numpy(W.throughput_inputs(1 << 16, seed=6)).to(dev)
            rt.autotune(xb, torch.empty((1 << 16, 3), device=dev))
        rr = Renderer(rv, rt, pyr, RenderParams(**{**rparams.__dict__, "mode": MODE_WAVEFRONT}) if "wavefront" in form else rparams)
        frame = torch.empty((1024, 1024, 3), device=dev)
        ft = time_steps(lambda: rr.frame(frame), max(5, args.steps) if prec != "fp32" else 5, 3, flush)
        q = rr.stats()
        ft_sorted = sorted(ft)
        p50 = ft_sorted[len(ft) // 2]
        p99 = ft_sorted[min(len(ft) - 1, int(round(0.99 * (len(ft) - 1))))]
        render[form] = {"p50_ms": p50, "p99_ms": p99, "frames": len(ft), "vis_queries": q[0], "thr_queries": q[1],
                        "rounds": q[2], "dropped_rays": q[3], "queries_per_s": (q[0] + q[1]) / (statistics.median(ft) * 1e-3),
                        "form": (f"persistent kernel, organisation {rr.mode & 0xFF}" if rr.persistent else "wavefront rounds")}
        rr.close()
        del rv, rt
    # host restatement on a bounded sample of the same frame (FP64 networks, all host threads)
    rsmall = RenderParams(**{**rparams.__dict__, "width": 96, "height": 96})
    t0 = time.perf_counter()
    _, _, rtot = oracle.render(oracle.Oracle(venc, vnet, 6, 1), rv_params, oracle.Oracle(henc, hnet, 10, 3), rt_params,
                               oracle.LodLevel(pyr.level_bits(rlevel), 512 >> rlevel, 0), rsmall, camera(rsmall, 512 >> rlevel))
    cpu_render_s = time.perf_counter() - t0

    # ---- training-sample generator: the reference's samplers + exact-DDA targets on the 512^3 scene ----
    from neural_lod_gb300.sampler import Sampler, SamplerParams

    gsp = Sampler(pyr, SamplerParams(grid_res=512, n_lods=7))
    n_gv, n_gt = 1 << 18, 1 << 20

    def gen_vis():
        xg, qg, _ = gsp.sample_visibility(5, n_gv)
        return xg, gsp.trace_visibility(qg)

    def gen_thr():
        xg, qg, _ = gsp.sample_throughput(5, n_gt)
        yg, _ = gsp.trace_throughput(qg, xg, 5)
        return gsp.compact(xg, yg)

    t_gv = statistics.median(time_steps(gen_vis, max(3, args.steps // 2), 3, flush))
    t_gt = statistics.median(time_steps(gen_thr, max(3, args.steps // 2), 3, flush))
    _, yv_ = gen_vis()
    occluded = float(yv_.mean())
    _, _, nv_ = gen_thr()
    n_valid_thr = int(nv_.item())
    gsp.sync_status()
    op_ = oracle.SamplerParams.from_dict({k: (list(getattr(gsp._c, k)) if k in ("aabb_min", "aabb_max") else getattr(gsp._c, k))
                                          for k, _ in oracle.SamplerParams._fields_})
    m_host = gsp.morton.cpu().numpy().view(np.uint32)
    t0 = time.perf_counter()
    _, q_host, _ = oracle.sample_visibility(op_, m_host, 5, 1 << 14)
    oracle.trace_visibility(oracle.LodLevel(pyr.level_bits(0), 512, 0), op_, q_host)
    cpu_gen_s = time.perf_counter() - t0
    generator = {"scene": "512^3 value noise (30% occupied), 7 LoDs, unit AABB, reference sampler defaults",
                 "visibility": {"batch": n_gv, "ms": t_gv, "samples_per_s": n_gv / (t_gv * 1e-3), "occluded_fraction": occluded},
                 "throughput": {"batch": n_gt, "ms": t_gt, "samples_per_s": n_gt / (t_gt * 1e-3),
                                "training_batch_after_compaction": n_valid_thr},
                 "cpu_visibility_samples_per_s": (1 << 14) / cpu_gen_s,
                 "cpu_sample": "2^14 visibility samples + targets, host restatement, one thread"}
    del gsp, pyr

    # ---- tiny-cuda-nn built from the reference's sources, same GPU and workloads ----
    tcnn = tcnn_comparison(dev, flush, args) if rank == 0 else None
    if tcnn is None:
        tcnn = committed_tcnn_figures()

    # ---- aggregate over ranks ----
    total_queries = n * world
    t_step = ms16
    if pg:
        t_step, ms_e2e = max_over_ranks([ms16, ms_e2e], pg, dev)
    value = total_queries / (t_step * 1e-3)
    e2e_value = total_queries / (ms_e2e * 1e-3)

    if rank != 0:
        if pg:
            pg.barrier()
        return

    pk = peaks()
    achieved_tflops = FLOP_PER_QUERY * n / (ms16 * 1e-3) / 1e12

    def roof(bound, work, ms, note):
        """Roofline entry of a leg: algorithmic FLOPs (tensor) or bytes (hbm) per step over its time."""
        if bound == "tensor":
            a = work / (ms * 1e-3) / 1e12
            return {"bound": "tensor", "achieved": a, "peak": pk["bf16_tflops"], "unit": "TFLOP/s", "frac": a / pk["bf16_tflops"],
                    "work_per_step": work, "note": note}
        a = work / (ms * 1e-3) / 1e9
        return {"bound": "hbm", "achieved": a, "peak": pk["hbm_gbs"], "unit": "GB/s", "frac": a / pk["hbm_gbs"], "work_per_step": work,
                "note": note}

    vis_train_params = 1_841_280           # 16-level visibility grid (1,833,088) + MLP (8,192)
    thr_train_params = 13_045_424          # 16-level throughput grid (13,026,992) + MLP (18,432)
    render_flop = {k: 12416 * v["vis_queries"] + FLOP_PER_QUERY * v["thr_queries"] for k, v in render.items()}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": t_step, "ms_per_step_p99": ms16_p99, "ms_per_step_mean": ms16_mean, "timing": "median of the timed steps",
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "fp16", "data": "synthetic (seeded PCG64 inputs, Xavier/U[-1e-4,1e-4] weights)",
        "config": {"workload": "throughput_query", "global_batch": n * world, "per_gpu_batch": n,
                   "encoding": "hashgrid L16 F2 T2^19 base16 s1.5 + SH4 x2 + onehot8 (80 wide)",
                   "mlp": "80-64-64-64-64-3 ReLU/exp", "precision": "fp16 tcgen05, fp32 accumulate",
                   "l2": "flushed between timed steps (256 MiB write)", "parallelism": f"replicas x{world}"},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(x_host.nbytes),
                "d2h_bytes_per_step": int(n * 3 * 4)},
        "roofline": {"bound": "tensor", "achieved": achieved_tflops, "peak": pk["bf16_tflops"], "unit": "TFLOP/s",
                     "frac": achieved_tflops / pk["bf16_tflops"], "traffic": traffic_from_profile(),
                     "peak_source": pk["source"], "flop_per_query": FLOP_PER_QUERY,
                     "hbm_frac": BYTES_PER_QUERY * n / (ms16 * 1e-3) / 1e9 / pk["hbm_gbs"]},
        "fp32_form": {"value": n / (ms32 * 1e-3), "unit": UNIT, "ms_per_step": ms32},
        "speedup_fp16_vs_fp32": ms32 / ms16,
        "err_vs_fp64": {"fp16_mean_abs": err16, "fp32_mean_abs": err32, "sample": ns},
        "visibility_query": {"batch": nv, "fp16_queries_per_s": vis["fp16"], "fp32_queries_per_s": vis["fp32"],
                             "fp16_kernel_variant": vis["variant"]},
        "visibility_train": {"batch": nt, "unit": "samples/s", "flop_per_sample": TRAIN_FLOP_PER_SAMPLE,
                             **{f"{p}_samples_per_s": nt / (t * 1e-3) for p, t in train.items()},
                             **{f"{p}_ms_per_step": t for p, t in train.items()},
                             "speedup_fp16_vs_fp32": train["fp32"] / train["fp16"],
                             "roofline": roof("tensor", TRAIN_FLOP_PER_SAMPLE * nt, train["fp16"],
                                              f"fwd + bwd FLOPs of the FP16 step; Adam moves 33 B x {vis_train_params} params "
                                              f"= {33 * vis_train_params / 1e6:.1f} MB per step; the fused kernel is bound by the "
                                              "L2 reduction rate of the grid-gradient scatter")},
        "throughput_train": {"batch": ntt, "unit": "samples/s", "flop_per_sample": 3 * FLOP_PER_QUERY,
                             "optimizer": "Ema(0.95) of ExponentialDecay(Adam lr 5e-3)", "loss": "RelativeL2",
                             **{f"{p}_samples_per_s": ntt / (t * 1e-3) for p, t in ttrain.items()},
                             **{f"{p}_ms_per_step": t for p, t in ttrain.items()},
                             "speedup_fp16_vs_fp32": ttrain["fp32"] / ttrain["fp16"],
                             "roofline": roof("tensor", 3 * FLOP_PER_QUERY * ntt, ttrain["fp16"],
                                              f"fwd + bwd FLOPs of the FP16 step; Adam + EMA move about 41 B x {thr_train_params} "
                                              "params per step; bound by the L2 reduction rate of the grid-gradient scatter")},
        "render": {"workload": "1024x1024 pinhole rays, level 3 (64^3) of a 512^3->4^3 pyramid (256^3 value noise, "
                               "30% occupied, upsampled x2), 4 path vertices, <= 64 visibility queries per bounce",
                   "frame": "one CUDA-graph launch: the persistent kernel (fp16) or rounds in a conditional while node "
                            "(fp16_wavefront, fp32)", **render,
                   "roofline": {k: roof("tensor", render_flop[k], v["p50_ms"], "12,416 FLOP per visibility query + 34,176 per "
                                        "throughput query over the p50 frame") for k, v in render.items()},
                   "cpu_queries_per_s": (rtot[0] + rtot[1]) / cpu_render_s,
                   "cpu_sample": "96x96 rays of the same camera, FP64 host restatement, all host threads"},
        "sample_generator": generator,
        "voxelize": {"triangles": 2_000_000, "grid": 1024, "ms": tvox, "triangles_per_s": 2e6 / (tvox * 1e-3),
                     "scene": "20k ellipsoid shells (48 tris) + 0.52M quads, unit cube, 1e-4 padding",
                     "roofline": roof("hbm", 36 * 2_000_000 + (1 << 27), tvox, "36 B per triangle read + the 128 MiB grid "
                                      "written once; the kernel is instruction-issue bound (per-voxel overlap tests)")},
        "voxelize_train": {"pyramid_ms": t_pyr * 1e3, "batch": n4, "batches": n_batches, **e2e4,
                           "targets": "albedo(voxel centre) x exact-DDA transmittance along wi, LoD 0-7 of the 1024^3 pyramid",
                           "loss": "RelativeL2", "optimizer": "Ema(0.95) of ExponentialDecay(Adam lr 5e-3)"},
        "tcnn": tcnn,
        "clocks": clocks,
        "gpu_launches": len(times16),
        "kernel_variant": variant,
        "wall_s_timed_region": t_wall,
    }
    if world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(enc, net, 10, 3, params, x_host)
    print(json.dumps(line), flush=True)
    if pg:
        pg.barrier()


if __name__ == "__main__":
    main()
