"""Builds the reference-backed checkers into oracle/_ref/ -- TEST INFRASTRUCTURE ONLY.

    python -m oracle.build_ref

oracle/_ref/nanovdb_ref: oracle/nanovdb_ref_harness.cpp compiled with g++ against the
reference's own NanoVDB headers where they lie (rptr/ext/nanovdb under the reference checkout).
IEEE single precision without contraction (-ffp-contract=off), so the float expressions of
NanoVDB's DDA/HDDA are each rounded once per operation on every host.  Needs the reference
checkout; on machines without it the build is skipped (the golden vectors made from it are
committed under tests/golden/).
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
REFERENCE = Path(os.environ.get("NLOD_REFERENCE", "/root/reference"))
NANOVDB = REFERENCE / "rptr" / "ext" / "nanovdb"


def available() -> bool:
    return (NANOVDB / "nanovdb" / "NanoVDB.h").exists()


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
    print(build_nanovdb_ref(force="--force" in sys.argv))
