"""Stages reference sources and builds the reference-backed checkers into oracle/_ref/ -- TEST
INFRASTRUCTURE ONLY.

    python -m oracle.build_ref stage --reference <reference checkout>   # or NLOD_REFERENCE=<dir>
    python -m oracle.build_ref build

`stage` copies, from the reference checkout, the NanoVDB headers (rptr/ext/nanovdb/nanovdb), the
arcade scene's shipped throughput configuration, cuda_voxelizer's kernel sources with the trimesh2
headers they include, and the parts of tiny-cuda-nn that a build needs (oracle/build_tcnn.py) into
oracle/_ref/.  That folder is ignored by git, so no reference source
enters the repository's history, while the working tree carries the staged copy to machines that
have no reference checkout.

oracle/_ref/nanovdb_ref: oracle/nanovdb_ref_harness.cpp compiled with g++ against the staged
NanoVDB headers.  IEEE single precision without contraction (-ffp-contract=off), so the float
expressions of NanoVDB's DDA/HDDA are each rounded once per operation on every host.  Without a
staged copy the build is skipped (the golden vectors made from it are committed under
tests/golden/).

oracle/_ref/libvoxref_{fma,nofma}-<arch>.so: the reference voxelizer kernel (cuda_voxelizer's
voxelize.cu, compiled from the staged source through oracle/voxelizer_ref_harness.cu, with
oracle/glm_shim standing in for GLM), once with nvcc's default FMA contraction -- the way the
reference's CMake builds it -- and once with -fmad=false.  About half a minute of nvcc each.
"""
from __future__ import annotations

import argparse
import os
import platform
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
NANOVDB = OUT / "nanovdb"
ARCADE_CONFIG = OUT / "arcade_world_final_512_throughput_config.json"
ARCADE_CONFIG_REL = "neural_lod/scenes/arcade/learned_weights/arcade_world_final_512_throughput_config.json"
VOXELIZER = OUT / "voxelizer"
VOXELIZER_FILES = ["voxelize.cu", "voxelize.cuh", "util.h", "util_cuda.h", "morton_LUTs.h", "libs/cuda/helper_cuda.h",
                   "libs/cuda/helper_string.h"]
ARCH = platform.machine()
VOXREF = {"fma": OUT / f"libvoxref_fma-{ARCH}.so", "nofma": OUT / f"libvoxref_nofma-{ARCH}.so"}


def available() -> bool:
    return (NANOVDB / "nanovdb" / "NanoVDB.h").exists()


def stage(reference: Path) -> None:
    reference = Path(reference)
    src = reference / "rptr" / "ext" / "nanovdb" / "nanovdb"
    if not (src / "NanoVDB.h").exists():
        raise SystemExit(f"no NanoVDB under {src}")
    if NANOVDB.exists():
        shutil.rmtree(NANOVDB)
    (NANOVDB / "nanovdb").mkdir(parents=True)
    shutil.copy2(src / "NanoVDB.h", NANOVDB / "nanovdb" / "NanoVDB.h")
    shutil.copytree(src / "util", NANOVDB / "nanovdb" / "util")
    shutil.copyfile(reference / ARCADE_CONFIG_REL, ARCADE_CONFIG)
    if VOXELIZER.exists():
        shutil.rmtree(VOXELIZER)
    vsrc = reference / "neural_lod" / "cuda_voxelizer" / "src"
    for f in VOXELIZER_FILES:
        (VOXELIZER / "src" / f).parent.mkdir(parents=True, exist_ok=True)
        shutil.copyfile(vsrc / f, VOXELIZER / "src" / f)
    shutil.copytree(reference / "neural_lod" / "trimesh2" / "include", VOXELIZER / "trimesh2")
    from .build_tcnn import stage as stage_tcnn

    stage_tcnn(reference)


def build_nanovdb_ref(force: bool = False) -> Path | None:
    if not available():
        return None
    OUT.mkdir(exist_ok=True)
    exe = OUT / "nanovdb_ref"
    src = HERE / "nanovdb_ref_harness.cpp"
    if not force and exe.exists() and exe.stat().st_mtime >= src.stat().st_mtime:
        return exe
    cmd = [os.environ.get("CXX", "g++"), "-std=c++17", "-O2", "-ffp-contract=off", "-I", str(NANOVDB),
           str(src), "-o", str(exe), "-lpthread"]
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError(f"nanovdb_ref build failed:\n{' '.join(cmd)}\n{p.stderr}")
    return exe


def voxelizer_staged() -> bool:
    return (VOXELIZER / "src" / "voxelize.cu").exists()


def build_voxelizer_ref(force: bool = False) -> dict | None:
    """Builds both forms of the reference voxelizer kernel; None without a staged copy."""
    if not voxelizer_staged():
        return None
    src = HERE / "voxelizer_ref_harness.cu"
    nvcc = os.environ.get("NVCC", "nvcc")
    base = [nvcc, "-O3", "-std=c++17", "-gencode", "arch=compute_103a,code=sm_103a", "-shared", "-Xcompiler", "-fPIC",
            "-I", str(HERE / "glm_shim"), "-I", str(VOXELIZER / "src"), "-I", str(VOXELIZER / "trimesh2"), str(src)]

    def one(kind):
        lib = VOXREF[kind]
        if not force and lib.exists() and lib.stat().st_mtime >= src.stat().st_mtime:
            return
        cmd = base + (["-fmad=false"] if kind == "nofma" else []) + ["-o", str(lib)]
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError(f"reference voxelizer build failed:\n{' '.join(cmd)}\n{p.stderr[-4000:]}")

    with ThreadPoolExecutor(2) as ex:
        list(ex.map(one, VOXREF))
    return dict(VOXREF)


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("what", choices=["stage", "build"])
    ap.add_argument("--reference", default=os.environ.get("NLOD_REFERENCE"))
    ap.add_argument("--force", action="store_true")
    a = ap.parse_args()
    if a.what == "stage":
        if not a.reference:
            raise SystemExit("give --reference <reference checkout> (or set NLOD_REFERENCE)")
        stage(Path(a.reference))
        print(f"staged into {OUT}")
    else:
        print(build_nanovdb_ref(force=a.force))
        print(build_voxelizer_ref(force=a.force))
