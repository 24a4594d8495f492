"""Generates tests/golden/dda_golden.npz: first-active-voxel results of the reference's own NanoVDB
DDA / TreeMarcher on a seeded occupancy pyramid.

    python tests/golden/make_dda_golden.py

Runs oracle/_ref/nanovdb_ref (oracle/nanovdb_ref_harness.cpp compiled against the reference's
NanoVDB headers by oracle/build_ref.py; needs the reference checkout).  The occupancy is a 64^3
value-noise grid at 30% density, pyramid levels 0..3 (64^3 .. 8^3) by >> lod, and per level a
mix of rays: from outside the grid towards it, from inside, axis-parallel (zero direction
components), and re-queries that start mid-way through the previous hit with that voxel skipped
(the renderer's pattern, rptr/cuda/wavefront_neural_pt.cuh:111-118).
"""
from __future__ import annotations

import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from neural_lod_gb300 import workloads as W  # noqa: E402
from oracle.build_ref import build_nanovdb_ref  # noqa: E402

# (resolution, levels, seed, lattice spacing, density, rays per level)
CASES = [(64, 4, 11, 8, 0.30, 700), (256, 3, 12, 32, 0.01, 500)]
RAY_DTYPE = np.dtype([("lod", "<i4"), ("eye", "<f4", 3), ("dir", "<f4", 3), ("tmin", "<f4"), ("prev", "<i4", 3)])
OUT_DTYPE = np.dtype([("hit", "<i4"), ("ijk", "<i4", 3), ("t_near", "<f4"), ("t_far", "<f4")])


def make_rays(rng, res, lod, n):
    r = res >> lod
    rays = np.zeros(n, RAY_DTYPE)
    rays["lod"] = lod
    rays["prev"] = -1
    kind = rng.integers(0, 10, size=n)
    for i in range(n):
        if kind[i] < 6:   # from outside, aimed at a random point of the grid
            u = rng.standard_normal(3)
            eye = r / 2 + u / np.linalg.norm(u) * r * rng.uniform(0.8, 1.6)
            target = rng.uniform(0, r, 3)
            d = target - eye
        else:             # from inside
            eye = rng.uniform(0, r, 3)
            d = rng.standard_normal(3)
        if kind[i] >= 8:  # axis-parallel components
            d[rng.integers(0, 3)] = 0.0
            if kind[i] == 9:
                d[rng.integers(0, 3)] = 0.0
            if not np.any(d):
                d[0] = 1.0
        d = d / np.linalg.norm(d)
        rays[i]["eye"] = eye
        rays[i]["dir"] = d
    return rays


def run(exe, res, n_levels, bits, rays):
    with tempfile.TemporaryDirectory() as td:
        fin, fout = Path(td) / "in.bin", Path(td) / "out.bin"
        with open(fin, "wb") as f:
            np.array([res, n_levels, len(rays)], "<u4").tofile(f)
            bits.astype("<u4").tofile(f)
            rays.tofile(f)
        subprocess.run([str(exe), str(fin), str(fout)], check=True)
        raw = np.fromfile(fout, dtype=np.uint8)
    head = raw[: n_levels * 32].view("<i4").reshape(n_levels, 8)
    out = raw[n_levels * 32:].view(OUT_DTYPE)
    return head, out


def main():
    exe = build_nanovdb_ref()
    if exe is None:
        raise SystemExit("reference checkout not found: cannot run the NanoVDB harness")
    arrays = {}
    for ci, (res, n_levels, seed, spacing, density, per_level) in enumerate(CASES):
        rng = np.random.Generator(np.random.PCG64(seed))
        occ = W.value_noise_occupancy(res, seed=seed, spacing=spacing, density=density)
        bits = W.pack_bits(occ)
        rays = np.concatenate([make_rays(rng, res, lod, per_level) for lod in range(n_levels)])
        head, out = run(exe, res, n_levels, bits, rays)
        # re-queries: start mid-way through the previous hit and skip that voxel
        sel = np.nonzero(out["hit"] == 1)[0][: per_level]
        re = rays[sel].copy()
        re["tmin"] = (out["t_near"][sel] + out["t_far"][sel]) * np.float32(0.5)
        re["prev"] = out["ijk"][sel]
        _, out2 = run(exe, res, n_levels, bits, re)
        arrays.update({f"c{ci}_res": res, f"c{ci}_n_levels": n_levels, f"c{ci}_bits": bits, f"c{ci}_levels": head,
                       f"c{ci}_rays": np.concatenate([rays, re]), f"c{ci}_out": np.concatenate([out, out2])})
        print("case", ci, "res", res, "rays", len(rays) + len(re), "hits", int(out["hit"].sum() + out2["hit"].sum()),
              "levels", head.tolist())
    np.savez_compressed(Path(__file__).with_name("dda_golden.npz"), n_cases=len(CASES), **arrays)


if __name__ == "__main__":
    main()
