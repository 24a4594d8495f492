"""Stages and builds tiny-cuda-nn from the reference's vendored sources -- TEST INFRASTRUCTURE ONLY.

    python -m oracle.build_tcnn stage --reference <reference checkout>   # where the reference is
    python -m oracle.build_tcnn build [-j N]                              # on a machine with nvcc

`stage` copies the parts of rptr/ext/tiny-cuda-nn that a build needs (src/, include/, and from
dependencies/ the CUTLASS, fmt, nlohmann-json and pcg32 headers) into oracle/_ref/tcnn/.  That
folder is ignored by git: reference sources never enter the repository's history, but the
working tree carries them to a GPU machine that has no reference checkout.

`build` compiles tiny-cuda-nn's eleven translation units (src/CMakeLists.txt:28-43) and
oracle/tcnn_harness.cu with nvcc, in parallel, for sm_103a, and links them into
oracle/_ref/libtcnn_harness-<arch>.so.  The flags are those of tiny-cuda-nn's own CMakeLists.txt
(:151-171) for a GPU whose lowest architecture is 103, without the x86-only -mf16c (the GPU
machines are aarch64) and without TCNN_SHAMPOO (an optimizer this path does not use, which would
pull in cuBLAS).  Nothing here is run by the library: the tests, the golden-vector script and the
bench's comparison leg load the result when it exists.
"""
from __future__ import annotations

import argparse
import os
import platform
import shutil
import subprocess
import sys
import time
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
STAGE = OUT / "tcnn"
# one build per machine architecture (the GPU machines are aarch64, this tree may also be built on x86)
ARCH = platform.machine()
LIB = OUT / f"libtcnn_harness-{ARCH}.so"
HARNESS = HERE / "tcnn_harness.cu"

TCNN_SOURCES = ["common", "common_device", "cpp_api", "cutlass_mlp", "encoding", "fully_fused_mlp", "loss",
                "network", "object", "optimizer", "reduce_sum"]
# (path inside rptr/ext/tiny-cuda-nn, what it is)
STAGED = [
    ("src", "tiny-cuda-nn sources"),
    ("include", "tiny-cuda-nn headers"),
    ("dependencies/cutlass/include", "CUTLASS 2.x headers"),
    ("dependencies/cutlass/tools/util/include", "CUTLASS util headers"),
    ("dependencies/fmt/include", "fmt headers"),
    ("dependencies/json", "nlohmann json"),
    ("dependencies/pcg32", "pcg32"),
]


def staged() -> bool:
    return (STAGE / "include" / "tiny-cuda-nn" / "common.h").exists() and (STAGE / "src" / "network.cu").exists()


def built() -> bool:
    return LIB.exists()


def stage(reference: Path) -> Path:
    tcnn = Path(reference) / "rptr" / "ext" / "tiny-cuda-nn"
    if not (tcnn / "include" / "tiny-cuda-nn" / "common.h").exists():
        raise SystemExit(f"no tiny-cuda-nn under {tcnn}")
    if STAGE.exists():
        shutil.rmtree(STAGE)
    for rel, _ in STAGED:
        shutil.copytree(tcnn / rel, STAGE / rel)
    return STAGE


def _flags() -> list[str]:
    inc = [STAGE / "include", STAGE / "dependencies", STAGE / "dependencies/cutlass/include",
           STAGE / "dependencies/cutlass/tools/util/include", STAGE / "dependencies/fmt/include"]
    # -split-compile=0 runs nvcc's optimiser over all cores of the machine within one unit (it
    # cuts fully_fused_mlp.cu, the longest unit, from about 11 to about 4 minutes on 8 cores)
    return ["-std=c++17", "-O3", "-split-compile=0", "-gencode", "arch=compute_103a,code=sm_103a", "-DTCNN_MIN_GPU_ARCH=103",
            "-DFMT_HEADER_ONLY", "--extended-lambda", "--expt-relaxed-constexpr", "-Xcompiler=-fPIC",
            "-Xcompiler=-Wno-float-conversion", "-Xcompiler=-fno-strict-aliasing",
            "-Xcudafe=--diag_suppress=unrecognized_gcc_pragma", *[f"-I{p}" for p in inc]]


def build(jobs: int | None = None, force: bool = False) -> Path:
    if not staged():
        raise SystemExit("oracle/_ref/tcnn is not staged: run `python -m oracle.build_tcnn stage --reference <dir>` "
                         "where the reference checkout is")
    if built() and not force:
        return LIB
    obj_dir = OUT / f"tcnn_obj-{ARCH}"
    obj_dir.mkdir(parents=True, exist_ok=True)
    nvcc = os.environ.get("NVCC", "nvcc")
    units = [(STAGE / "src" / f"{s}.cu", obj_dir / f"{s}.o") for s in TCNN_SOURCES] + [(HARNESS, obj_dir / "tcnn_harness.o")]
    # the longest unit first, so the pool's tail is short
    units.sort(key=lambda u: u[0].name != "fully_fused_mlp.cu")

    def compile_one(unit):
        src, obj = unit
        if obj.exists() and not force and obj.stat().st_mtime >= src.stat().st_mtime:
            return src.name, 0.0
        t0 = time.time()
        cmd = [nvcc, "-c", str(src), "-o", str(obj), *_flags()]
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError(f"{' '.join(cmd)}\n{p.stdout}\n{p.stderr}")
        return src.name, time.time() - t0

    with ThreadPoolExecutor(max_workers=jobs or os.cpu_count() or 4) as ex:
        for name, dt in ex.map(compile_one, units):
            print(f"  {name}: {dt:.0f} s", flush=True)
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc, "-shared", "-o", str(tmp), *[str(o) for _, o in units], "-lcuda"]
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError(f"{' '.join(cmd)}\n{p.stdout}\n{p.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("what", choices=["stage", "build"])
    ap.add_argument("--reference", default=os.environ.get("NLOD_REFERENCE"))
    ap.add_argument("-j", type=int, default=None)
    ap.add_argument("--force", action="store_true")
    a = ap.parse_args()
    if a.what == "stage":
        if not a.reference:
            raise SystemExit("give --reference <reference checkout> (or set NLOD_REFERENCE)")
        print(stage(Path(a.reference)))
    else:
        t0 = time.time()
        print(build(a.j, a.force), f"({time.time() - t0:.0f} s)")
        sys.stdout.flush()
