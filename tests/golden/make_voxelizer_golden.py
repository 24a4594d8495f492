"""Golden vectors of the reference voxelizer kernel as the reference builds it.

    python tests/golden/make_voxelizer_golden.py OUT.npz     # on a GPU machine, sources staged

cuda_voxelizer's voxelize_triangle (neural_lod/cuda_voxelizer/src/voxelize.cu:58-190) is compiled
from its own source with nvcc's default contraction of multiply-adds (oracle/build_ref.py, the
"fma" form: the reference's CMake passes no -fmad flag) and run on a seeded random triangle soup
at 100^3.  The fixture keeps the frame and the bit grid; the triangles are regenerated from the
seed by soup() below, so that the host oracle can be held to the reference build on the CPU.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

GRID = 100
N_TRIANGLES = 20000
SEED = 88172645463325252


def soup(n: int = N_TRIANGLES, grid: int = GRID, seed: int = SEED) -> np.ndarray:
    """n triangles [n, 9] float32: a centre U[0,1)^3 per triangle and vertices at centre +
    U(-1,1) * s, s cycling through 0.2 / grid, 2 / grid, 8 / grid and 0.05 (xorshift64 stream)."""
    mask = (1 << 64) - 1
    state = seed

    def rnd():
        nonlocal state
        state ^= (state << 13) & mask
        state ^= state >> 7
        state ^= (state << 17) & mask
        return (state >> 11) * (1.0 / 9007199254740992.0)

    scales = (0.2 / grid, 2.0 / grid, 8.0 / grid, 0.05)
    out = np.empty((n, 9), np.float32)
    for t in range(n):
        s = scales[t % 4]
        c = (rnd(), rnd(), rnd())
        for k in range(3):
            for i in range(3):
                out[t, 3 * k + i] = np.float32(c[i] + (2.0 * rnd() - 1.0) * s)
    return out


def main(out_path: str) -> None:
    import torch

    import oracle.voxref as VR
    from neural_lod_gb300 import voxelize as V

    tris = soup()
    v = tris.reshape(-1, 3)
    bmin, bmax, unit = V.mesh_frame(v.min(0), v.max(0), GRID)
    bits = VR.voxelize(torch.from_numpy(tris).cuda(), GRID, bmin, bmax, "fma").cpu().numpy().view(np.uint32)
    np.savez_compressed(out_path, grid=GRID, n=N_TRIANGLES, seed=np.uint64(SEED), bbox_min=bmin, bbox_max=bmax, unit=unit, bits=bits)
    print("wrote", out_path, int(np.unpackbits(bits.view(np.uint8)).sum()), "voxels")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else str(Path(__file__).with_name("voxelizer_golden.npz")))
