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


# --- an independent restatement of the reference's scores and selection, in numpy float32 -------
# (rptr/cuda/neural-lod/neural_lod_learning_common.cuh:836-927 metrics, neural_lod_learning.cu:
# 122-165 confusion counts, :234-266 argmax and the middle of the plateau)

_F = np.float32


def _div(a, b):
    return _F(a) / _F(b)


def _prec(fp, tp):
    return _F(0) if tp == 0 else _div(tp, tp + fp)


def _rec(fn, tp):
    return _F(0) if tp == 0 else _div(tp, tp + fn)


def _f(tn, fp, fn, tp, beta):
    p, r = _prec(fp, tp), _rec(fn, tp)
    if p + r == _F(0):
        return _F(0)
    b2 = _F(beta) * _F(beta)
    return ((_F(1) + b2) * p * r) / (b2 * p + r)


def _score(metric, tn, fp, fn, tp, sp, sn, beta):
    if metric == 0:
        return _prec(fp, tp)
    if metric == 1:
        return _rec(fn, tp)
    if metric == 2:
        return _f(tn, fp, fn, tp, beta)
    if metric == 3:
        return (_f(tn, fp, fn, tp, beta) + _f(tp, fn, fp, tn, beta)) * _F(0.5)
    if metric in (4, 5):
        fneg = _f(tp, fn, fp, tn, beta if metric == 4 else 1.0)
        return (_f(tn, fp, fn, tp, beta) * _F(sp) + fneg * _F(sn)) / _F(sp + sn)
    if metric == 6:
        num = _F(tp * tn) - _F(fp * fn)
        den = _F(tp + fp) * _F(tp + fn) * _F(tn + fp) * _F(tn + fn)
        return _F(0) if den == 0 else num / np.sqrt(den)
    if metric == 7:
        num = _F(2) * (_F(tp * tn) - _F(fn * fp))
        den = _F(tp + fp) * _F(fp + tn) + _F(tp + fn) * _F(fn + tn)
        return _F(0) if den == 0 else num / den
    if metric == 8:
        den = _F(tp + tn + fp + fn)
        return _F(0) if den == 0 else _F(tp + tn) / den
    se = _F(0) if tp == 0 else _div(tp, tp + fn)
    spc = _F(0) if tn == 0 else _div(tn, tn + fp)
    if metric == 9:
        return (se + spc) * _F(0.5)
    if metric == 10:
        return np.sqrt(_prec(fp, tp) * _rec(fn, tp))
    return se + spc - _F(1)


def _restated_thresholds(truth, proba, metric, beta=1.0, n_thresholds=101):
    out = []
    for t, p in zip(truth, proba):
        pos = int((t == 1.0).sum())
        scores = []
        for k in range(n_thresholds):
            th = _F(k) / _F(n_thresholds - 1)
            pred = p > th
            tv = t == 1.0
            tp, fp = int((pred & tv).sum()), int((pred & ~tv).sum())
            fn, tn = int((~pred & tv).sum()), int((~pred & ~tv).sum())
            scores.append(_score(metric, tn, fp, fn, tp, pos, len(t) - pos, beta))
        best, opt = -10.0, 0
        for k, s in enumerate(scores):
            if s > best:
                best, opt = s, k
        eq = 0
        # the reference compares the float difference with the double 1e-4
        while opt + eq < n_thresholds and float(abs(scores[opt + eq] - scores[opt])) < 1e-4:
            eq += 1
        out.append(_F(opt + eq // 2) / _F(n_thresholds - 1))
    return np.array(out, dtype=np.float32)


def test_every_metric_matches_an_independent_restatement():
    rng = np.random.Generator(np.random.PCG64(11))
    n_vox, n_s = 12, 64
    t = (rng.random((n_vox, n_s)) < rng.random((n_vox, 1))).astype(np.float32)
    # probabilities correlated with the truth, quantised so that ties and plateaus occur
    p = np.clip(0.6 * t + 0.5 * rng.random((n_vox, n_s)), 0, 1)
    p = (np.round(p * 40) / 40).astype(np.float32)
    t[0] = 0.0          # a voxel without positives
    t[1] = 1.0          # and one without negatives
    for m in range(12):
        for beta in (1.0, 0.5):
            got = oracle.optimal_thresholds(t, p, n_s, m, beta)
            np.testing.assert_array_equal(got, _restated_thresholds(t, p, m, beta), err_msg=f"metric {m} beta {beta}")
