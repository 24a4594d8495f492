"""The host restatement of the per-voxel threshold optimisation: metric known answers and the
tie rule (middle of the run of best scores)."""
import numpy as np

import oracle


def test_separable_and_tie_rule():
    p = np.linspace(0.0, 1.0, 64, dtype=np.float32)
    t = (p > 0.6).astype(np.float32)
    # accuracy is 1 for every threshold in [0.6, 0.61]: the middle of that run
    assert oracle.optimal_thresholds(t, p, 64, 8)[0] == np.float32(0.6)
    # all-negative voxel: precision is 0 everywhere -> the run of equal scores is all thresholds
    assert oracle.optimal_thresholds(np.zeros(32, np.float32), p[:32], 32, 0)[0] == np.float32(0.5)


def test_metrics_bounded_and_deterministic():
    rng = np.random.Generator(np.random.PCG64(0))
    t = (rng.random((50, 100)) < 0.5).astype(np.float32)
    p = rng.random((50, 100)).astype(np.float32)
    for m in range(12):
        a = oracle.optimal_thresholds(t, p, 100, m)
        assert a.shape == (50,) and (a >= 0).all() and (a <= 1).all()
        assert np.array_equal(a, oracle.optimal_thresholds(t, p, 100, m))
