"""Builds the CPU oracle (test infrastructure): oracle/_build/liborc.so from nlod_oracle.c and
nlod_sampler.c.

    python -m oracle.build
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT_DIR = HERE / "_build"
LIB = OUT_DIR / "liborc.so"
SRC = HERE / "nlod_oracle.c"
SOURCES = [SRC, HERE / "nlod_sampler.c"]


def build_oracle(force: bool = False) -> Path:
    OUT_DIR.mkdir(exist_ok=True)
    if not force and LIB.exists() and LIB.stat().st_mtime >= max(*(f.stat().st_mtime for f in SOURCES), (HERE / "nlod_oracle.h").stat().st_mtime):
        return LIB
    cc = os.environ.get("CC", "gcc")
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [cc, "-O2", "-std=c11", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared", "-Wall",
           *map(str, SOURCES), "-o", str(tmp), "-lm"]
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{' '.join(cmd)}\n{p.stdout}\n{p.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
