"""Stages reference sources and builds the reference-backed checkers into oracle/_ref/ -- TEST
INFRASTRUCTURE ONLY.

    python -m oracle.build_ref stage --reference <reference checkout>   # or NLOD_REFERENCE=<dir>
    python -m oracle.build_ref build

`stage` copies, from the reference checkout, the NanoVDB headers (rptr/ext/nanovdb/nanovdb), the
arcade scene's shipped throughput configuration and the parts of tiny-cuda-nn that a build needs
(oracle/build_tcnn.py) into oracle/_ref/.  That folder is ignored by git, so no reference source
enters the repository's history, while the working tree carries the staged copy to machines that
have no reference checkout.

oracle/_ref/nanovdb_ref: oracle/nanovdb_ref_harness.cpp compiled with g++ against the staged
NanoVDB headers.  IEEE single precision without contraction (-ffp-contract=off), so the float
expressions of NanoVDB's DDA/HDDA are each rounded once per operation on every host.  Without a
staged copy the build is skipped (the golden vectors made from it are committed under
tests/golden/).
"""
from __future__ import annotations

import argparse
import os
import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
NANOVDB = OUT / "nanovdb"
ARCADE_CONFIG = OUT / "arcade_world_final_512_throughput_config.json"
ARCADE_CONFIG_REL = "neural_lod/scenes/arcade/learned_weights/arcade_world_final_512_throughput_config.json"


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
    shutil.copy2(reference / ARCADE_CONFIG_REL, ARCADE_CONFIG)
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
