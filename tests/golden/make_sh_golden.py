"""Generates tests/golden/sh_golden.npz: real spherical-harmonics values computed from the
polynomials of the reference's own SH encoding (rptr/ext/tiny-cuda-nn/include/tiny-cuda-nn/
encodings/spherical_harmonics.h, kernel_sh: the `data_out(k) = ...;` lines), evaluated in float64
at seeded directions.  Run where the reference sources are present:

    python tests/golden/make_sh_golden.py <reference checkout>     # or NLOD_REFERENCE=<dir>
"""
import os
import re
import sys
from pathlib import Path

import numpy as np

_ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("NLOD_REFERENCE")
if not _ref:
    raise SystemExit("give the reference checkout as the argument (or set NLOD_REFERENCE)")
SRC = Path(_ref) / "rptr/ext/tiny-cuda-nn/include/tiny-cuda-nn/encodings/spherical_harmonics.h"


def reference_polynomials():
    text = SRC.read_text()
    start = text.index("auto write_sh = [&]() {")
    body = text[start:text.index("};", start)]
    polys = {}
    for m in re.finditer(r"data_out\((\d+)\)\s*=\s*([^;]+);", body):
        expr = re.sub(r"(\d(?:\.\d*)?(?:[eE][-+]?\d+)?)f\b", r"\1", m.group(2))
        polys[int(m.group(1))] = expr.strip()
    return polys


def main():
    polys = reference_polynomials()
    assert sorted(polys) == list(range(64)), f"expected 64 SH polynomials, found {len(polys)}"
    rng = np.random.Generator(np.random.PCG64(2024))
    d = rng.standard_normal((256, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    d = np.concatenate([d, np.eye(3), -np.eye(3)])           # plus the axis directions
    x, y, z = d[:, 0], d[:, 1], d[:, 2]
    env = dict(x=x, y=y, z=z, xy=x * y, xz=x * z, yz=y * z, x2=x * x, y2=y * y, z2=z * z)
    env.update(x4=env["x2"] ** 2, y4=env["y2"] ** 2, z4=env["z2"] ** 2)
    env.update(x6=env["x4"] * env["x2"], y6=env["y4"] * env["y2"], z6=env["z4"] * env["z2"])
    vals = np.zeros((d.shape[0], 64))
    for k, expr in polys.items():
        vals[:, k] = np.broadcast_to(eval(expr, {"__builtins__": {}}, env), d.shape[0])
    out = Path(__file__).resolve().parent / "sh_golden.npz"
    np.savez_compressed(out, dirs=d, values=vals, source=str(SRC.relative_to(Path(_ref))))
    print(out, vals.shape)


if __name__ == "__main__":
    main()
