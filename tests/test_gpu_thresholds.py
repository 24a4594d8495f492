"""Per-voxel threshold optimisation on the GPU against the host restatement (every metric,
including runs of tied scores), plus the .bin format round trip."""
import numpy as np
import pytest

import oracle
from neural_lod_gb300 import thresholds as TH

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("metric", list(TH.METRICS))
def test_thresholds_match_oracle(cuda, nlod_lib, metric, tmp_path):
    import torch

    rng = np.random.Generator(np.random.PCG64(TH.METRICS[metric]))
    n_vox, n_s = 700, 192
    truth = (rng.random((n_vox, n_s)) < rng.random((n_vox, 1))).astype(np.float32)
    # probabilities correlated with the truth, quantised so that many scores tie
    p = np.clip(0.5 * truth + rng.normal(0.25, 0.2, (n_vox, n_s)), 0, 1)
    p[: n_vox // 2] = np.round(p[: n_vox // 2] * 20) / 20
    p = p.astype(np.float32)
    got = TH.optimal_thresholds(torch.from_numpy(truth).to(cuda), torch.from_numpy(p).to(cuda), n_s, metric, beta=0.7).cpu().numpy()
    ref = oracle.optimal_thresholds(truth, p, n_s, TH.METRICS[metric], beta=0.7)
    assert np.array_equal(got, ref)
    assert 0.0 <= got.min() and got.max() <= 1.0 and len(np.unique(got)) > 3
    TH.save_bin(tmp_path / "lod0.bin", got)
    assert np.array_equal(TH.load_bin(tmp_path / "lod0.bin"), got)


def test_perfectly_separable_voxel(cuda, nlod_lib):
    import torch

    p = np.linspace(0.0, 1.0, 64, dtype=np.float32)
    truth = (p > 0.6).astype(np.float32)
    got = TH.optimal_thresholds(torch.from_numpy(truth).to(cuda), torch.from_numpy(p).to(cuda), 64, "accuracy").cpu().numpy()
    # every threshold between the last negative (0.6-) and the first positive (0.6+) scores 1
    assert 0.58 <= got[0] <= 0.62
